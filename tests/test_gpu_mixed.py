"""GPU tests of the mixed-precision (TF32 split) tensor-core path."""
import ctypes as C

import numpy as np
import pytest

from nwchem_gb300 import _capi
from nwchem_gb300.split import split_tf32, tf32

pytestmark = pytest.mark.gpu


def test_tf32_split_residual():
    """CPU check of the encoding: hi + lo carries x to ~2^-22."""
    x = np.random.default_rng(0).standard_normal(10000)
    hi, lo = split_tf32(x)
    assert np.array_equal(tf32(hi), hi) and np.array_equal(tf32(lo), lo)
    rel = np.abs(x - hi.astype(np.float64) - lo.astype(np.float64)) / np.abs(x)
    assert rel.max() < 2.0 ** -21


@pytest.mark.parametrize("K", [16, 96, 300])
def test_tcgen05_split_gemm(cuda_device, K):
    import torch
    rng = np.random.default_rng(K)
    A = rng.standard_normal((128, K))
    B = rng.standard_normal((256, K))
    ah, al = split_tf32(A)
    bh, bl = split_tf32(B)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda_device)
    t = [dev(x) for x in (ah, al, bh, bl)]
    D = torch.zeros((128, 256), dtype=torch.float32, device=cuda_device)
    torch.cuda.synchronize()
    lib = _capi.lib()
    lib.sdt_set_error_mode(1)
    rc = lib.sdt_tc_selftest(*[C.c_void_p(x.data_ptr()) for x in t], K, C.c_void_p(D.data_ptr()))
    _capi.check(rc, "sdt_tc_selftest")
    got = D.cpu().numpy().astype(np.float64)
    split = (ah.astype(np.float64) @ bh.T.astype(np.float64) + ah.astype(np.float64) @ bl.T.astype(np.float64)
             + al.astype(np.float64) @ bh.T.astype(np.float64))
    exact = A @ B.T
    scale = np.abs(exact).max()
    # FP32 round-to-nearest accumulation of 3K products: a random walk of
    # ~sqrt(3K) roundings of eps32 times the running sum
    tol = 2e-7 * np.sqrt(3 * K) * scale
    assert np.abs(got - split).max() <= tol
    assert np.abs(got - exact).max() <= tol
    # and no bias: the mean signed error is far below the largest one
    assert abs((got - split).mean()) <= 0.05 * np.abs(got - split).max()


MIXED_TILINGS = [
    ([6], [12], None, None),                       # one tile each, partial 8x4 boxes
    ([2, 4], [5, 3, 4], None, None),               # diagonal and mixed tuples
    ([3, 5, 2], [9, 6, 10, 3], None, None),
    ([8, 12], [16, 24], None, None),               # whole boxes
    ([3, 2, 3], [4, 5, 4, 3], [0, 1, 1], [1, 0, 1, 0]),   # irreps
]


@pytest.mark.parametrize("occ,vir,osym,vsym", MIXED_TILINGS)
def test_mixed_matches_fp64_and_oracle(cuda_device, occ, vir, osym, vsym):
    """TF32-split tensor-core form against the FP64 form and the oracle.
    Bound: 2e-6 relative on E[T], E(T) and each tuple's pair (FP32
    accumulation of the split products; the FP64 form agrees to ~1e-14)."""
    import nwchem_gb300 as ng
    from oracle import oracle as orc
    t = ng.Tiling(occ, vir, occ_sym=osym, vir_sym=vsym).with_evl(17)
    files = ng.synth_inputs(t, 17)
    kl = ng.task_list(t)
    e1, e2, pt, _ = orc.Problem(t, *files).ccsd_t()
    with ng.TriplesJob(t) as job:
        job.load(*files)
        d1, d2, dpt = job.run(kl, per_task=True)
        m1, m2, mpt = job.run(kl, per_task=True, precision=ng.PREC_MIXED_TF32)
        m1b, m2b = job.run(kl, precision=ng.PREC_MIXED_TF32)
    assert d1 == pytest.approx(e1, rel=1e-10) and d2 == pytest.approx(e2, rel=1e-10)
    assert m1 == pytest.approx(e1, rel=2e-6) and m2 == pytest.approx(e2, rel=2e-6)
    assert np.abs(mpt - pt).max() <= 2e-6 * max(abs(e1), abs(e2))
    assert (m1b, m2b) == (m1, m2)          # deterministic


@pytest.mark.parametrize("kseg", [0, 1, 3])
def test_mixed_segmented_drains(cuda_device, kseg):
    """Draining the accumulator in K segments gives the same energies (to the
    mixed form's bound) as one drain per term."""
    import nwchem_gb300 as ng
    t = ng.Tiling([3, 5, 2], [9, 6, 10, 3]).with_evl(5)
    files = ng.synth_inputs(t, 5)
    kl = ng.task_list(t)
    with ng.TriplesJob(t) as job:
        job.load(*files)
        f = job.run(kl)
        job.set_mixed_segment(kseg)
        m = job.run(kl, precision=ng.PREC_MIXED_TF32)
    assert m[0] == pytest.approx(f[0], rel=2e-6) and m[1] == pytest.approx(f[1], rel=2e-6)
