"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle restates NWChem's (T) Fortran in C (sdt_oracle.c).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg import this module;
the nwchem_gb300 package never does.  Parity status: pinned by
self-consistency known answers (re-tiling invariance, antisymmetry, the dense
closed form) in tests/golden/, not by reference-executed vectors.
"""
from __future__ import annotations

import ctypes as C
import subprocess
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libsdt_oracle.so"
_lock = threading.Lock()
_lib = None

I64 = C.c_int64
PI64 = C.POINTER(C.c_int64)
PD = C.POINTER(C.c_double)


class OrcTiling(C.Structure):
    _fields_ = [("noab", I64), ("nvab", I64), ("range", PI64), ("spin", PI64), ("sym", PI64),
                ("offset", PI64), ("alpha", PI64), ("evl_sorted", PD), ("restricted", I64),
                ("irrep_t", I64), ("irrep_v", I64)]


class OrcFile(C.Structure):
    _fields_ = [("hash", PI64), ("data", PD)]


HOOK = C.CFUNCTYPE(None, C.c_void_p, I64, PI64, PD, PD)


class OrcHooks(C.Structure):
    _fields_ = [("user", C.c_void_p), ("s1", HOOK), ("d1", HOOK), ("d2", HOOK)]


def build() -> Path:
    """Compiles the oracle with its Makefile (gcc, OpenMP)."""
    res = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    return LIB


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            _lib = C.CDLL(str(LIB))
            _lib.orc_ccsd_t.restype = I64
            _lib.orc_ccsd_t.argtypes = [C.POINTER(OrcTiling), C.POINTER(OrcFile), C.POINTER(OrcFile),
                                        C.POINTER(OrcFile), PI64, I64, PI64, I64, PD, PD, PI64]
            _lib.orc_6tasks.restype = I64
            _lib.orc_6tasks.argtypes = [C.POINTER(OrcTiling)]
            _lib.orc_neword.restype = I64
            _lib.orc_neword.argtypes = [C.POINTER(OrcTiling), I64, PI64]
            _lib.orc_tuple_tiles.restype = I64
            _lib.orc_tuple_tiles.argtypes = [C.POINTER(OrcTiling), C.POINTER(OrcFile), C.POINTER(OrcFile),
                                             C.POINTER(OrcFile), PI64, PD, PD]
            _lib.orc_tuple_drive.restype = I64
            _lib.orc_tuple_drive.argtypes = [C.POINTER(OrcTiling), C.POINTER(OrcFile), C.POINTER(OrcFile),
                                             C.POINTER(OrcFile), PI64, C.POINTER(OrcHooks), PI64]
            for name, nd in (("orc_sd_t_s1", 6), ("orc_sd_t_d1", 7), ("orc_sd_t_d2", 7)):
                f = getattr(_lib, name)
                f.restype = None
                f.argtypes = [I64] + [I64] * nd + [PD, PD, PD]
            _lib.orc_tce_sort_4.restype = None
            _lib.orc_tce_sort_4.argtypes = [PD, PD] + [I64] * 8 + [C.c_double]
            _lib.orc_tce_sort_2.restype = None
            _lib.orc_tce_sort_2.argtypes = [PD, PD] + [I64] * 4 + [C.c_double]
            _lib.orc_tce_hash.restype = I64
            _lib.orc_tce_hash.argtypes = [PI64, I64]
            _lib.orc_synth_evl.restype = None
            _lib.orc_synth_evl.argtypes = [I64, I64, C.c_uint64, PD]
            _lib.orc_synth_file.restype = I64
            _lib.orc_synth_file.argtypes = [C.POINTER(OrcTiling), C.c_int, C.c_uint64, PI64, PI64, PI64, PD]
            _lib.orc_tasks_flops.restype = C.c_double
            _lib.orc_tasks_flops.argtypes = [C.POINTER(OrcTiling), PI64, I64]
        return _lib


def _pd(a: np.ndarray):
    return a.ctypes.data_as(PD)


def _pi(a: np.ndarray):
    return a.ctypes.data_as(PI64)


class Problem:
    """A tiling plus its three TCE files, viewed through the oracle's structs.

    `tiling` is any object with numpy arrays range, spin, sym, offset, evl,
    alpha_arr (or None), noab, nvab, restricted; files are objects with
    numpy `hash` and `data` (nwchem_gb300.TceFile fits).
    """

    def __init__(self, tiling, t1, t2, v2):
        self.tiling, self.files = tiling, (t1, t2, v2)
        al = tiling.alpha_arr
        self.ts = OrcTiling(tiling.noab, tiling.nvab, _pi(tiling.range), _pi(tiling.spin), _pi(tiling.sym),
                            _pi(tiling.offset), _pi(al) if al is not None else C.cast(None, PI64),
                            _pd(tiling.evl), 1 if tiling.restricted else 0, 0, 0)
        self.fs = [OrcFile(_pi(f.hash), _pd(f.data)) for f in (t1, t2, v2)]

    def task_list(self) -> np.ndarray:
        L = lib()
        n = L.orc_6tasks(C.byref(self.ts))
        kl = np.empty((max(n, 1), 7), dtype=np.int64)
        rc = L.orc_neword(C.byref(self.ts), n, _pi(kl))
        if rc != 0:
            raise RuntimeError(f"orc_neword failed ({rc})")
        return kl[:n]

    def ccsd_t(self, klist: np.ndarray | None = None, task_ids=None):
        """(E[T], E(T), per_task (n,2), kernel_calls (n,3)) over the chosen tasks."""
        L = lib()
        kl = np.ascontiguousarray(self.task_list() if klist is None else klist, dtype=np.int64)
        ids = None if task_ids is None else np.ascontiguousarray(task_ids, dtype=np.int64)
        n = len(kl) if ids is None else len(ids)
        e = np.zeros(2)
        pt = np.zeros((max(n, 1), 2))
        kc = np.zeros((max(n, 1), 3), dtype=np.int64)
        rc = L.orc_ccsd_t(C.byref(self.ts), C.byref(self.fs[0]), C.byref(self.fs[1]), C.byref(self.fs[2]),
                          _pi(kl), len(kl), _pi(ids) if ids is not None else None, n, _pd(e), _pd(pt), _pi(kc))
        if rc != 0:
            raise RuntimeError(f"orc_ccsd_t failed ({rc})")
        return float(e[0]), float(e[1]), pt[:n], kc[:n]

    def tuple_tiles(self, tuple6) -> tuple[np.ndarray, np.ndarray]:
        """(singles, doubles) triples tiles of one tuple, Fortran (h3,h2,h1,p6,p5,p4)."""
        tp = np.ascontiguousarray(tuple6[:6], dtype=np.int64)
        r = self.tiling.range
        shape = tuple(int(r[b - 1]) for b in tp[[5, 4, 3, 2, 1, 0]])  # (h3,h2,h1,p6,p5,p4)
        n = int(np.prod(shape))
        s, d = np.zeros(n), np.zeros(n)
        rc = lib().orc_tuple_tiles(C.byref(self.ts), C.byref(self.fs[0]), C.byref(self.fs[1]),
                                   C.byref(self.fs[2]), _pi(tp), _pd(s), _pd(d))
        if rc != 0:
            raise RuntimeError(f"orc_tuple_tiles failed ({rc})")
        return s.reshape(shape, order="F"), d.reshape(shape, order="F")

    def drive(self, tuple6, s1, d1, d2) -> np.ndarray:
        """Runs the reference driver logic for one tuple with the kernels
        replaced by Python callables f(k, dims, sub_a, sub_b) receiving numpy
        views of the sorted sub-blocks.  Returns the (s1, d1, d2) call counts."""
        def wrap(fn, nd):
            def cb(user, k, dims, a, b):
                dd = [int(dims[i]) for i in range(nd)]
                fn(int(k), dd, a, b)
            return HOOK(cb)
        keep = [wrap(s1, 6), wrap(d1, 7), wrap(d2, 7)]
        hooks = OrcHooks(None, *keep)
        tp = np.ascontiguousarray(tuple6[:6], dtype=np.int64)
        calls = np.zeros(3, dtype=np.int64)
        rc = lib().orc_tuple_drive(C.byref(self.ts), C.byref(self.fs[0]), C.byref(self.fs[1]),
                                   C.byref(self.fs[2]), _pi(tp), C.byref(hooks), _pi(calls))
        if rc != 0:
            raise RuntimeError(f"orc_tuple_drive failed ({rc})")
        return calls


class Tiling:
    """A tiling with the attributes Problem reads (spin-orbital, unrestricted,
    irreps optional), built without the product library."""

    def __init__(self, occ, vir, occ_sym=None, vir_sym=None, seed: int = 0, name: str = "custom"):
        self.occ, self.vir, self.name = [int(x) for x in occ], [int(x) for x in vir], name
        self.noab, self.nvab = len(self.occ), len(self.vir)
        self.range = np.array(self.occ + self.vir, dtype=np.int64)
        self.spin = np.ones(self.noab + self.nvab, dtype=np.int64)
        self.sym = np.array(list(occ_sym or [0] * self.noab) + list(vir_sym or [0] * self.nvab), dtype=np.int64)
        self.offset = np.concatenate([[0], np.cumsum(self.range)[:-1]]).astype(np.int64)
        self.alpha_arr, self.restricted = None, False
        self.nocc, self.nvir = int(sum(self.occ)), int(sum(self.vir))
        self.evl = np.empty(self.nocc + self.nvir)
        lib().orc_synth_evl(self.nocc, self.nvir, seed, _pd(self.evl))
        self._ts = OrcTiling(self.noab, self.nvab, _pi(self.range), _pi(self.spin), _pi(self.sym),
                             _pi(self.offset), C.cast(None, PI64), _pd(self.evl), 0, 0, 0)


def config_tiling(config: int) -> Tiling:
    """The benchmark workloads' tilings, with their seeded orbital energies:
    0 o=10/v=40 one tile each; 1 o=40 as 8/12/20, v=300 as 20,24x5,30x4,40;
    2 o=64 as 2x32, v=512 as 8x64; 3 blocked symmetry, 8 occupied tiles
    (irreps 0..7) from {8,12,16,24,32} and 12 virtual tiles (irreps
    0..7,0..3) from {16,24,32,48,64}, drawn by numpy's PCG64 with seed 3."""
    if config == 0:
        return Tiling([10], [40], seed=0, name="o10v40")
    if config == 1:
        return Tiling([8, 12, 20], [20, 24, 24, 24, 24, 24, 30, 30, 30, 30, 40], seed=1, name="o40v300")
    if config == 2:
        return Tiling([32, 32], [64] * 8, seed=2, name="o64v512")
    if config == 3:
        rng = np.random.default_rng(3)
        occ = [int(x) for x in rng.choice([8, 12, 16, 24, 32], 8)]
        vir = [int(x) for x in rng.choice([16, 24, 32, 48, 64], 12)]
        return Tiling(occ, vir, [q % 8 for q in range(8)], [q % 8 for q in range(12)], seed=3,
                      name="sym8_o%dv%d" % (sum(occ), sum(vir)))
    raise ValueError(f"no tiling for workload {config}")


class File:
    """One TCE file: tce_hash table and block data."""

    def __init__(self, hash_: np.ndarray, data: np.ndarray):
        self.hash, self.data = hash_, data

    @property
    def nbytes(self) -> int:
        return int(self.hash.nbytes + self.data.nbytes)


def synth_inputs(tiling: Tiling, seed: int) -> tuple[File, File, File]:
    """The workloads' seeded T1, T2 and V2 files (orc_synth.c)."""
    L, out = lib(), []
    for kind in range(3):
        nb, nd = C.c_int64(), C.c_int64()
        if L.orc_synth_file(C.byref(tiling._ts), kind, seed, C.byref(nb), C.byref(nd), None, None) != 0:
            raise RuntimeError("orc_synth_file failed")
        h, d = np.empty(2 * nb.value + 1, dtype=np.int64), np.empty(nd.value)
        if L.orc_synth_file(C.byref(tiling._ts), kind, seed, C.byref(nb), C.byref(nd), _pi(h), _pd(d)) != 0:
            raise RuntimeError("orc_synth_file failed")
        out.append(File(h, d))
    return tuple(out)


def flops(tiling, klist: np.ndarray) -> float:
    """Algorithmic FLOPs of a tuple list (orc_tasks_flops)."""
    kl = np.ascontiguousarray(klist, dtype=np.int64).reshape(-1, 7)
    p = Problem.__new__(Problem)
    Problem.__init__(p, tiling, *(File(np.zeros(1, dtype=np.int64), np.zeros(1)),) * 3)
    return float(lib().orc_tasks_flops(C.byref(p.ts), _pi(kl), len(kl)))


def slab_retiling(occ, vir, tup, cut_p4: int, cut_h1: int):
    """(occ, vir, tuple) of the same orbital spaces re-tiled so that the
    first cut_p4 orbitals of the tuple's p4 tile and the first cut_h1 of its
    h1 tile are tiles of their own, and the tuple of those two tiles with
    the tuple's other tiles.  Its triples elements are the original tuple's
    elements with p4 < cut_p4 and h1 < cut_h1 (the amplitudes are functions
    of the orbital indices, and the contractions still run over every
    orbital), and its multiplicity factor is the original's when neither
    tile repeats in the tuple, so its energy is the energy of that slab of
    the original tuple.  Tiles are 1-based, occupied first."""
    occ, vir = [int(x) for x in occ], [int(x) for x in vir]
    noab = len(occ)
    p4, h1 = tup[0] - noab - 1, tup[3] - 1
    if tup[0] in tup[1:3] or tup[3] in tup[4:6]:
        raise ValueError("the p4 and h1 tiles must not repeat in the tuple")
    occ2 = occ[:h1] + [cut_h1, occ[h1] - cut_h1] + occ[h1 + 1:]
    vir2 = vir[:p4] + [cut_p4, vir[p4] - cut_p4] + vir[p4 + 1:]
    no2 = len(occ2)
    omap = lambda b: b + (1 if b - 1 > h1 else 0)
    vmap = lambda b: no2 + (b - noab) + (1 if b - noab - 1 > p4 else 0)
    return occ2, vir2, [vmap(tup[0]), vmap(tup[1]), vmap(tup[2]), omap(tup[3]), omap(tup[4]), omap(tup[5])]


def kernel(family: str, k: int, dims_fortran, triplesx: np.ndarray, a: np.ndarray, b: np.ndarray) -> None:
    """One oracle tile kernel, Fortran CPU dialect dims (h3d,h2d,h1d,p6d,p5d,p4d[,k7d])."""
    f = getattr(lib(), f"orc_sd_t_{family}")
    f(k, *[int(x) for x in dims_fortran], _pd(triplesx), _pd(a), _pd(b))
