"""GPU test of sdt_compute_en_noalloc, the energy reduction for callers that
own the triples tiles in their own device memory and cannot allocate
(a memory pool that already holds the budget, or device data owned by a
Fortran offload runtime).  It must give compute_en_'s energies for the same
tiles, on two calls in a row (the fixed scratch array is reused), and the
device's free memory (cudaMemGetInfo) must not move across its calls once
the first call has loaded the library's module."""
import ctypes as C

import numpy as np
import pytest

import nwchem_gb300 as ng
from nwchem_gb300 import _capi
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _refs(vals):
    return [C.byref(C.c_int64(int(v))) for v in vals]


def _pd(a):
    return a.ctypes.data_as(_capi.PD)


def test_noalloc_energy_matches_compute_en_twice(cuda_device):
    import torch
    lib = _capi.lib()
    lib.sdt_set_error_mode(1)
    t = ng.Tiling([3, 5], [4, 6, 5]).with_evl(31)
    P = orc.Problem(t, *ng.synth_inputs(t, 31))
    kl = P.task_list()
    r = t.range
    for q in (0, len(kl) - 1):                       # a large and a small tuple
        tup = [int(x) for x in kl[q, :6]]
        td = [int(r[b - 1]) for b in (tup[3], tup[4], tup[5], tup[0], tup[1], tup[2])]
        # Fill the library's tuple tiles through the reference tile ABI.
        lib.initmemmodule_()
        lib.dev_mem_s_(*_refs(td))
        lib.dev_mem_d_(*_refs(td))
        P.drive(tup,
                lambda k, d, a, b: getattr(lib, f"sd_t_s1_{k}_cuda_")(*_refs(d), None, a, b),
                lambda k, d, a, b: getattr(lib, f"sd_t_d1_{k}_cuda_")(*_refs(d), None, a, b),
                lambda k, d, a, b: getattr(lib, f"sd_t_d2_{k}_cuda_")(*_refs(d), None, a, b))
        ev = [np.ascontiguousarray(t.evl[t.offset[b - 1]:t.offset[b - 1] + r[b - 1]])
              for b in (tup[3], tup[4], tup[5], tup[0], tup[1], tup[2])]
        f = 0.5 if tup[3] == tup[4] else 1.0
        ref = np.zeros(2)
        lib.compute_en_(C.byref(C.c_double(f)), _pd(ref), *[_pd(x) for x in ev], *_refs(td), None, None)
        nt = int(np.prod(td))
        d_host, s_host = np.empty(nt), np.empty(nt)
        _capi.check(lib.sdt_tile_download(_pd(d_host), _pd(s_host)))
        lib.dev_release_()
        lib.finalizememmodule_()
        assert _capi.last_error()[0] == 0
        # The same tiles in caller-owned device memory (torch here).
        d_dev = torch.from_numpy(d_host).to(cuda_device)
        s_dev = torch.from_numpy(s_host).to(cuda_device)
        torch.cuda.synchronize()
        # The first call in a process may load the library's module (and its
        # fixed array); after that, free device memory must stay put.
        free0 = torch.cuda.mem_get_info(cuda_device)[0] if q > 0 else None
        for _ in range(2):
            got = np.full(2, np.nan)
            rc = lib.sdt_compute_en_noalloc(f, _pd(got), *[_pd(x) for x in ev], *td,
                                            C.c_void_p(d_dev.data_ptr()), C.c_void_p(s_dev.data_ptr()),
                                            None)
            _capi.check(rc, "sdt_compute_en_noalloc")
            torch.cuda.synchronize()
            free = torch.cuda.mem_get_info(cuda_device)[0]
            if free0 is None:
                free0 = free                             # after the first call (module loaded)
            else:
                assert free == free0, f"free device memory moved by {free - free0} bytes"
            assert got[0] == pytest.approx(ref[0], rel=1e-12, abs=1e-300)
            assert got[1] == pytest.approx(ref[1], rel=1e-12, abs=1e-300)


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda_device):
    lib = _capi.lib()
    lib.sdt_set_error_mode(1)
    ev = np.zeros(8192)
    big = [2000, 2000, 2000, 2000, 100, 100]      # 8200 orbital energies > 8192
    e = np.zeros(2)
    rc = lib.sdt_compute_en_noalloc(1.0, _pd(e), *[_pd(ev)] * 6, *big, C.c_void_p(1), None, None)
    code, msg = _capi.last_error()
    assert rc == 1 and code == 1 and "8192" in msg
