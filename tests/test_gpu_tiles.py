"""GPU parity of the reference tile-level ABI (sd_t_*_cuda_, compute_en_,
dev_mem_*): each of the 27 kernels against the oracle's restatement of
ccsd_t_kernels_omp.F, and whole tuples driven by the reference driver logic.

Tolerance: FP64 with a different summation order (DMMA fused products) --
1e-13 of the tile's largest element, 1e-12 relative on energies."""
import ctypes as C

import numpy as np
import pytest

import nwchem_gb300 as ng
from nwchem_gb300 import _capi
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

I64 = C.c_int64


def _refs(vals):
    return [C.byref(I64(int(v))) for v in vals]


def _pd(a):
    return a.ctypes.data_as(_capi.PD)


@pytest.fixture(scope="module")
def lib(cuda_device):
    L = _capi.lib()
    L.sdt_set_error_mode(1)
    L.initmemmodule_()
    yield L
    L.dev_release_()
    L.finalizememmodule_()


DIMS = [
    # (h1d, h2d, h3d, p4d, p5d, p6d, k7d)
    (3, 4, 2, 5, 3, 4, 6),
    (8, 8, 8, 12, 12, 12, 20),
    (5, 7, 6, 9, 11, 10, 13),
]


@pytest.mark.parametrize("dims", DIMS)
@pytest.mark.parametrize("family", ["s1", "d1", "d2"])
def test_each_tile_kernel_matches_oracle(lib, family, dims):
    rng = np.random.default_rng(hash((family, dims)) & 0xffff)
    h1, h2, h3, p4, p5, p6, k7 = dims
    nt = h1 * h2 * h3 * p4 * p5 * p6
    for k in range(1, 10):
        if family == "s1":
            a = rng.standard_normal(p4 * h1)
            b = rng.standard_normal(h3 * h2 * p6 * p5)
            abi = (h1, h2, h3, p4, p5, p6)
        elif family == "d1":
            a = rng.standard_normal(k7 * p4 * p5 * h1)
            b = rng.standard_normal(h3 * h2 * p6 * k7)
            abi = (h1, h2, h3, k7, p4, p5, p6)
        else:
            a = rng.standard_normal(k7 * p4 * h1 * h2)
            b = rng.standard_normal(k7 * h3 * p6 * p5)
            abi = (h1, h2, h3, p4, p5, p6, k7)
        tdims = _refs((h1, h2, h3, p4, p5, p6))
        (lib.dev_mem_s_ if family == "s1" else lib.dev_mem_d_)(*tdims)
        getattr(lib, f"sd_t_{family}_{k}_cuda_")(*_refs(abi), None, _pd(a), _pd(b))
        got = np.empty(nt)
        if family == "s1":
            _capi.check(lib.sdt_tile_download(None, _pd(got)))
        else:
            _capi.check(lib.sdt_tile_download(_pd(got), None))
        want = np.zeros(nt)
        fdims = (h3, h2, h1, p6, p5, p4) + (() if family == "s1" else (k7,))
        orc.kernel(family, k, fdims, want, a, b)
        scale = np.abs(want).max()
        assert scale > 0
        assert np.abs(got - want).max() <= 1e-13 * scale, (family, k, dims)
    code, msg = _capi.last_error()
    assert code == 0, msg


def _drive_tuple(lib, P, t, tup):
    """The reference CUDA driver sequence for one tuple (ccsd_t_gpu.F:122-220)."""
    r = t.range
    td = [int(r[b - 1]) for b in (tup[3], tup[4], tup[5], tup[0], tup[1], tup[2])]  # h1..p6
    lib.dev_mem_s_(*_refs(td))
    lib.dev_mem_d_(*_refs(td))

    def s1(k, dims, a, b):
        getattr(lib, f"sd_t_s1_{k}_cuda_")(*_refs(dims), None, a, b)

    def d1(k, dims, a, b):
        getattr(lib, f"sd_t_d1_{k}_cuda_")(*_refs(dims), None, a, b)

    def d2(k, dims, a, b):
        getattr(lib, f"sd_t_d2_{k}_cuda_")(*_refs(dims), None, a, b)

    calls = P.drive(tup, s1, d1, d2)
    f = 1.0
    if tup[0] == tup[1] == tup[2]:
        f /= 6
    elif tup[0] == tup[1] or tup[1] == tup[2]:
        f /= 2
    if tup[3] == tup[4] == tup[5]:
        f /= 6
    elif tup[3] == tup[4] or tup[4] == tup[5]:
        f /= 2
    ev = [np.ascontiguousarray(t.evl[t.offset[b - 1]:t.offset[b - 1] + r[b - 1]])
          for b in (tup[3], tup[4], tup[5], tup[0], tup[1], tup[2])]
    e = np.zeros(2)
    lib.compute_en_(C.byref(C.c_double(f)), _pd(e), *[_pd(x) for x in ev], *_refs(td), None, None)
    nt = int(np.prod(td))
    d, s = np.empty(nt), np.empty(nt)
    _capi.check(lib.sdt_tile_download(_pd(d), _pd(s)))
    return e, d, s, calls


@pytest.mark.parametrize("occ,vir,osym,vsym", [
    ([3, 5], [4, 6, 5], None, None),
    ([4, 4, 2], [6, 6], None, None),
    ([3, 2, 3], [4, 5, 4, 3], [0, 1, 1], [1, 0, 1, 0]),
])
def test_tuples_through_tile_abi_match_oracle(lib, occ, vir, osym, vsym):
    t = ng.Tiling(occ, vir, occ_sym=osym, vir_sym=vsym).with_evl(8)
    P = orc.Problem(t, *ng.synth_inputs(t, 8))
    kl = P.task_list()
    e_tot, _, per_task, _ = P.ccsd_t()
    tiles = [P.tuple_tiles([int(x) for x in kl[q, :6]]) for q in range(len(kl))]
    # Tolerances scale with the problem, not the tuple: some tuples are exactly
    # zero by antisymmetry (three holes in a two-orbital tile) and come out
    # as +-1e-18 rounding on either side.
    sd = max(np.abs(rd).max() for _, rd in tiles)
    ss = max(np.abs(rs).max() for rs, _ in tiles)
    for q in range(len(kl)):
        tup = [int(x) for x in kl[q, :6]]
        e, d, s, _ = _drive_tuple(lib, P, t, tup)
        rs, rd = tiles[q]
        assert np.abs(d - rd.ravel(order="F")).max() <= 1e-13 * sd
        assert np.abs(s - rs.ravel(order="F")).max() <= 1e-13 * ss
        assert e[0] == pytest.approx(per_task[q, 0], rel=1e-12, abs=1e-13 * abs(e_tot))
        assert e[1] == pytest.approx(per_task[q, 1], rel=1e-12, abs=1e-13 * abs(e_tot))
    lib.dev_release_()
    assert _capi.last_error()[0] == 0


def test_tile_abi_rejects_mismatched_dims(lib):
    lib.dev_mem_d_(*_refs((2, 2, 2, 3, 3, 3)))
    a, b = np.ones(64), np.ones(64)
    lib.sd_t_d2_1_cuda_(*_refs((2, 2, 2, 3, 3, 4, 2)), None, _pd(a), _pd(b))
    code, msg = _capi.last_error()
    assert code == 1 and "do not match" in msg
    lib.dev_release_()


def test_memory_module_checks_live_blocks(lib):
    """finalizememmodule_ accepts a released tuple and flags a leaked one
    (memory.cu:164-171 asserts no live pointers)."""
    dims = _refs((2, 2, 2, 3, 3, 3))
    lib.initmemmodule_()
    lib.dev_mem_d_(*dims)
    lib.dev_mem_s_(*dims)
    lib.dev_release_()
    lib.finalizememmodule_()
    assert _capi.last_error()[0] == 0
    lib.initmemmodule_()
    lib.dev_mem_d_(*dims)
    lib.finalizememmodule_()
    code, msg = _capi.last_error()
    assert code == 4 and "live" in msg
    lib.dev_release_()
    lib.initmemmodule_()
