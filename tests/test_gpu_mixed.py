"""GPU tests of the mixed-precision (split-operand) tensor-core path:
TF32x3, BF16x3 and FP16x3 (power-of-two scaled)."""
import ctypes as C

import numpy as np
import pytest

from nwchem_gb300 import _capi
from nwchem_gb300.split import bf16_value, f16_value, split_bf16, split_f16, split_tf32, tf32

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


@pytest.mark.parametrize("bf16", [0, 1])
@pytest.mark.parametrize("K", [16, 96, 304])
def test_tcgen05_split_gemm16(cuda_device, bf16, K):
    """kind::f16 path: BF16 or FP16 split operands, FP32 accumulation."""
    import torch
    rng = np.random.default_rng(100 + K + bf16)
    A = rng.standard_normal((128, K))
    B = rng.standard_normal((256, K))
    split, value = (split_bf16, bf16_value) if bf16 else (split_f16, f16_value)
    ah, al = split(A)
    bh, bl = split(B)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int16)).to(cuda_device)
    t = [dev(x) for x in (ah, al, bh, bl)]
    D = torch.zeros((128, 256), dtype=torch.float32, device=cuda_device)
    torch.cuda.synchronize()
    lib = _capi.lib()
    lib.sdt_set_error_mode(1)
    rc = lib.sdt_tc_selftest16(*[C.c_void_p(x.data_ptr()) for x in t], K, bf16, C.c_void_p(D.data_ptr()))
    _capi.check(rc, "sdt_tc_selftest16")
    got = D.cpu().numpy().astype(np.float64)
    Ah, Al, Bh, Bl = (value(x) for x in (ah, al, bh, bl))
    want = Ah @ Bh.T + Ah @ Bl.T + Al @ Bh.T
    scale = np.abs(A @ B.T).max()
    tol = 2e-7 * np.sqrt(3 * K) * scale
    assert np.abs(got - want).max() <= tol
    assert np.abs(got - A @ B.T).max() <= (tol if not bf16 else 2.0 ** -15 * np.sqrt(K) * scale)


def test_energy_division_bound(cuda_device):
    """The epilogue's FP32 quotient X/D -- orbital energies shifted by the
    gap midpoint and rounded to FP32, D summed in FP32 (every hole term
    negative, every particle term positive, so no sum cancels), then
    __fdividef -- stays within 1e-6 of the FP64 quotient: at most ten FP32
    roundings relative to |D| (6e-7) plus 2 ulp for the division (1.2e-7)."""
    lib = _capi.lib()
    err = C.c_double()
    _capi.check(lib.sdt_check_division(1 << 22, 12345, C.byref(err)), "sdt_check_division")
    assert 0.0 < err.value < 1e-6, err.value


MIXED_TILINGS = [
    ([6], [12], None, None),                       # one tile each, partial 8x4 boxes
    ([2, 4], [5, 3, 4], None, None),               # diagonal and mixed tuples
    ([3, 5, 2], [9, 6, 10, 3], None, None),
    ([8, 12], [16, 24], None, None),               # whole boxes
    ([3, 2, 3], [4, 5, 4, 3], [0, 1, 1], [1, 0, 1, 0]),   # irreps
    ([1, 2, 3, 4, 5], [9, 7, 3, 1, 2], None, None),          # tiny and ragged tiles in every position
]


# Bound of each mixed form against the FP64 form, relative to |E|.
MIXED_BOUND = {"tf32": 2e-6, "fp16": 2e-6, "bf16": 2e-5}
PREC = {"tf32": 1, "bf16": 2, "fp16": 3}


@pytest.mark.parametrize("form", ["tf32", "fp16", "bf16"])
@pytest.mark.parametrize("occ,vir,osym,vsym", MIXED_TILINGS)
def test_mixed_matches_fp64_and_oracle(cuda_device, occ, vir, osym, vsym, form):
    """Split-operand tensor-core forms against the FP64 form and the oracle,
    E[T], E(T) and each tuple's pair, within MIXED_BOUND[form] of |E| (FP32
    accumulation of the split products; the FP64 form agrees to ~1e-14)."""
    import nwchem_gb300 as ng
    from oracle import oracle as orc
    t = ng.Tiling(occ, vir, occ_sym=osym, vir_sym=vsym).with_evl(17)
    files = ng.synth_inputs(t, 17)
    kl = ng.task_list(t)
    e1, e2, pt, _ = orc.Problem(t, *files).ccsd_t()
    bound = MIXED_BOUND[form]
    with ng.TriplesJob(t) as job:
        job.load(*files)
        d1, d2, dpt = job.run(kl, per_task=True)
        m1, m2, mpt = job.run(kl, per_task=True, precision=PREC[form])
        m1b, m2b = job.run(kl, precision=PREC[form])
    assert d1 == pytest.approx(e1, rel=1e-10) and d2 == pytest.approx(e2, rel=1e-10)
    assert m1 == pytest.approx(e1, rel=bound) and m2 == pytest.approx(e2, rel=bound)
    assert np.abs(mpt - pt).max() <= bound * max(abs(e1), abs(e2))
    assert (m1b, m2b) == (m1, m2)          # deterministic


@pytest.mark.parametrize("form,kseg", [("tf32", 0), ("tf32", 1), ("tf32", 3), ("fp16", 2), ("bf16", 5)])
def test_mixed_segmented_drains(cuda_device, form, kseg):
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
        m = job.run(kl, precision=PREC[form])
    b = MIXED_BOUND[form]
    assert m[0] == pytest.approx(f[0], rel=b) and m[1] == pytest.approx(f[1], rel=b)


def test_mixed_persistent_many_items(cuda_device):
    """More items than SMs: every CTA handles several sub-boxes in a row (the
    overlap of one item's energies with the next item's contractions), and a
    precision switch on the same job re-encodes the operands."""
    import nwchem_gb300 as ng
    t = ng.Tiling([8, 12], [24, 40]).with_evl(9)
    files = ng.synth_inputs(t, 9)
    kl = ng.task_list(t)
    with ng.TriplesJob(t) as job:
        job.load(*files)
        f = job.run(kl)
        for form in ("fp16", "tf32", "fp16"):
            m = job.run(kl, precision=PREC[form])
            b = MIXED_BOUND[form]
            assert m[0] == pytest.approx(f[0], rel=b) and m[1] == pytest.approx(f[1], rel=b)


@pytest.mark.parametrize("form", ["fp16", "tf32"])
def test_mixed_work_unit_shapes(cuda_device, form):
    """CTAs holding the finished sub-box in tensor memory give the same bits
    as CTAs holding it in registers."""
    import nwchem_gb300 as ng
    t = ng.Tiling([3, 5, 6], [9, 6, 10, 17]).with_evl(8)
    files = ng.synth_inputs(t, 8)
    kl = ng.task_list(t)
    with ng.TriplesJob(t) as job:
        job.load(*files)
        f = job.run(kl)
        a = job.run(kl, per_task=True, precision=PREC[form])
        job.set_mixed_shape(2)
        b = job.run(kl, per_task=True, precision=PREC[form])
    assert a[0] == b[0] and a[1] == b[1] and np.array_equal(a[2], b[2])
    bnd = MIXED_BOUND[form]
    assert b[0] == pytest.approx(f[0], rel=bnd) and b[1] == pytest.approx(f[1], rel=bnd)


def test_job_bytes_bound_holds_for_padded_holes(cuda_device):
    """The serving admission bound (sdt_job_bytes) covers what a job holds
    after a mixed run, for occupied tiles of 5 (the FP32 s1 copies pad the
    holes of each tile to a multiple of 4, 8 per tile here: 2.6x the dense
    vvoo block)."""
    import nwchem_gb300 as ng
    from nwchem_gb300 import serve
    t = ng.Tiling([5] * 8, [25] * 4).with_evl(5)
    files = ng.synth_inputs(t, 5)
    kl = ng.task_list(t)
    with ng.TriplesJob(t) as job:
        job.load(*files)
        f64 = job.device_bytes
        job.run(kl[:1], precision=PREC["fp16"])
        mixed = job.device_bytes
    assert 0 < f64 <= serve.job_bytes(t, ng.PREC_FP64)
    assert f64 < mixed <= serve.job_bytes(t, ng.PREC_MIXED_FP16)
