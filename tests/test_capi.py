"""CPU tests of the C-ABI library: it loads, exports every symbol the public
header declares, and its host-only entry points behave (no GPU calls)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np

import nwchem_gb300 as ng
from nwchem_gb300 import _capi

HEADER = Path(__file__).resolve().parents[1] / "include" / "sdt_gb300.h"


def declared_symbols() -> set[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set()
    for fam in ("s1", "d1", "d2"):
        if f"SDT_{fam.upper()}_DECL" in text:
            names |= {f"sd_t_{fam}_{k}_cuda_" for k in range(1, 10)}
    lines, keep, in_define = text.splitlines(), [], False
    for ln in lines:
        if ln.lstrip().startswith("#define") or in_define:
            in_define = ln.rstrip().endswith("\\")
            continue
        keep.append(ln)
    body = "\n".join(keep)
    for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", body):
        name = m.group(1)
        if name in {"if", "for", "while", "sizeof", "return", "SDT_S1_DECL", "SDT_D1_DECL", "SDT_D2_DECL"}:
            continue
        names.add(name)
    return names


def test_library_exports_every_declared_symbol():
    lib = _capi.lib()
    names = declared_symbols()
    assert len(names) >= 27 + 12
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_reference_abi_names_present():
    lib = _capi.lib()
    for fam in ("s1", "d1", "d2"):
        for k in range(1, 10):
            assert hasattr(lib, f"sd_t_{fam}_{k}_cuda_")
    for n in ("compute_en_", "dev_mem_d_", "dev_mem_s_", "dev_release_", "initmemmodule_",
              "finalizememmodule_", "check_device_", "device_init_"):
        assert hasattr(lib, n)


def test_check_device_uses_local_rank(monkeypatch):
    lib = _capi.lib()
    monkeypatch.setenv("SDT_LOCAL_RANK", "2")
    assert lib.check_device_(C.byref(C.c_long(2))) == 0
    assert lib.check_device_(C.byref(C.c_long(3))) == 1


def test_error_mode_and_bad_arguments():
    lib = _capi.lib()
    lib.sdt_set_error_mode(1)
    assert lib.sdt_tasks_list(None, 0, None) == 1
    code, msg = _capi.last_error()
    assert code == 1 and "bad argument" in msg
    assert _capi.last_error()[0] == 0  # cleared


def test_bad_tiling_rejected():
    lib = _capi.lib()
    lib.sdt_set_error_mode(1)
    t = ng.Tiling([4], [6]).with_evl(0)
    ts = t.struct()
    ts.offset[1] = 5  # tiles must be contiguous
    assert lib.sdt_tasks_count(C.byref(ts)) < 0
    _capi.last_error()


def test_synth_file_layout():
    """Blocks are canonical, keys ascending, offsets contiguous (tce_hash layout)."""
    t = ng.Tiling([2, 3], [3, 4]).with_evl(0)
    for kind in (ng.FILE_T1, ng.FILE_T2, ng.FILE_V2):
        f = ng.synth_file(t, kind, 9)
        n = int(f.hash[0])
        keys, offs = f.hash[1:n + 1], f.hash[n + 1:2 * n + 1]
        assert (np.diff(keys) > 0).all()
        assert offs[0] == 0 and (np.diff(offs) > 0).all()
        assert f.lookup(int(keys[-1])) == int(offs[-1])
        assert f.lookup(-5) == -1


def test_task_list_writes_only_its_rows():
    """Canary-padded output: sdt_tasks_list fills exactly 7 * n int64 values."""
    t = ng.Tiling([3, 5, 2], [4, 6, 4, 3], occ_sym=[0, 1, 1], vir_sym=[1, 0, 1, 0])
    lib = _capi.lib()
    ts = t.struct()
    n = lib.sdt_tasks_count(C.byref(ts))
    assert n > 0
    canary = np.int64(-0x5A5A5A5A5A5A5A5B)
    buf = np.full(7 * n + 64, canary, dtype=np.int64)
    assert lib.sdt_tasks_list(C.byref(ts), n, buf.ctypes.data_as(_capi.PI64)) == 0
    assert np.all(buf[7 * n:] == canary)
    assert np.array_equal(buf[:7 * n].reshape(n, 7), ng.task_list(t))
