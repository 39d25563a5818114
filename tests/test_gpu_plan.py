"""GPU tests of plans: prepared tuple lists, CUDA-graph replay, per-tuple
work-unit shapes, and the autotuner's plans."""
import numpy as np
import pytest

import nwchem_gb300 as ng
from nwchem_gb300 import autotune

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def no_stray_error(cuda_device):
    """Every test leaves no recorded library error behind."""
    from nwchem_gb300 import _capi
    _capi.last_error()
    yield
    code, msg = _capi.last_error()
    assert code == 0, msg


@pytest.fixture(scope="module")
def sym_job(cuda_device):
    t = ng.Tiling([4, 8, 12, 8], [8, 16, 24, 16, 32], occ_sym=[0, 1, 2, 3], vir_sym=[1, 0, 3, 2, 0]).with_evl(4)
    files = ng.synth_inputs(t, 4)
    job = ng.TriplesJob(t)
    job.load(*files)
    yield t, job, ng.task_list(t)
    job.close()


@pytest.mark.parametrize("prec", [ng.PREC_FP64, ng.PREC_MIXED_FP16])
def test_plan_matches_job_run_and_graph_replays(sym_job, prec):
    t, job, kl = sym_job
    want = job.run(kl, per_task=True, precision=prec)
    job.set_timing(True)
    with ng.Plan(job, kl, prec) as p:
        a = p.run(per_task=True)
        p.capture()
        b = p.run(per_task=True)
        assert job.last_kernel_ms > 0          # replays time the kernels too
        c = p.run(per_task=True)
    for got in (a, b, c):
        assert got[0] == want[0] and got[1] == want[1] and np.array_equal(got[2], want[2])


def test_plan_per_tuple_shapes(sym_job):
    """Tuples split between the register-hold and the tensor-memory-hold
    shapes give each tuple's bits of the register-hold run, in the caller's
    order."""
    t, job, kl = sym_job
    shapes = np.array([[2, 1, 2][q % 3] for q in range(len(kl))], dtype=np.int32)
    with ng.Plan(job, kl, ng.PREC_MIXED_FP16) as p1, ng.Plan(job, kl, ng.PREC_MIXED_FP16, shapes) as p2:
        a = p1.run(per_task=True)
        p2.capture()
        b = p2.run(per_task=True)
    assert np.array_equal(a[2], b[2])
    assert b[0] == pytest.approx(a[0], rel=1e-14) and b[1] == pytest.approx(a[1], rel=1e-14)


def test_plan_detects_reencoded_operands(sym_job):
    t, job, kl = sym_job
    p = ng.Plan(job, kl[:5], ng.PREC_MIXED_FP16)
    job.run(kl[:5], precision=ng.PREC_MIXED_TF32)   # re-encodes the job's split operands
    with pytest.raises(ng.SdtError) as e:
        p.run()
    assert e.value.code == 4
    p.close()


def test_autotuned_plan(sym_job, tmp_path):
    t, job, kl = sym_job
    f = job.run(kl)
    tuner = autotune.Autotuner(job, forms=("fp16", "tf32"), sample=2, cache=tmp_path / "c.json")
    p, d = tuner.plan(kl)
    with p:
        e = p.run()
        e2 = p.run()
    assert d["form"] in ("fp16", "tf32") and set(d["shapes"].values()) <= {1, 2}
    assert e == e2
    assert e[0] == pytest.approx(f[0], rel=2e-6) and e[1] == pytest.approx(f[1], rel=2e-6)
