"""GPU tests of the serving loop: every served job's energies are the bits
of the same job run alone; jobs share the resident kernel's work queue
(continuous batching) and admitted jobs overlap; the byte budget holds; a
job larger than the budget is refused; the FP64 check is the FP64 form."""
import time

import numpy as np
import pytest

import nwchem_gb300 as ng
from nwchem_gb300 import serve

pytestmark = pytest.mark.gpu


def _alone(spec, files, prec):
    with ng.TriplesJob(spec.tiling) as job:
        job.load(*files)
        kl = ng.task_list(spec.tiling)
        return job.run(kl, precision=prec), job.run(kl)


def test_served_jobs_match_alone_and_overlap(cuda_device):
    specs = serve.job_stream(8, 200.0, 11, 8, 20)
    files = serve.prepare(specs)
    prec = ng.PREC_MIXED_FP16
    need = [serve.job_bytes(s.tiling, prec) for s in specs]
    budget = int(sum(sorted(need)[-3:]))              # room for about three jobs at a time
    with serve.Server(budget, slots=3, reserve=40, check_ctas=32) as srv:
        tickets = [srv.submit(s.tiling, f, prec, check_fp64=(s.id % 4 == 0)) for s, f in zip(specs, files)]
        srv.drain(600)
        st = [srv.status(t) for t in tickets]
        peak = srv.peak_bytes
    assert all(x["state"] == 2 for x in st), [x["msg"] for x in st]
    assert peak <= budget
    for spec, f, x in zip(specs, files, st):
        mixed, fp64 = _alone(spec, f, prec)
        assert x["energy"] == mixed                    # the same bits alone and in the mix
        if spec.id % 4 == 0:
            assert x["fp64"] == fp64
        assert x["energy"][1] == pytest.approx(fp64[1], rel=2e-6)
    iv = sorted((x["admitted"], x["finished"]) for x in st)
    assert any(iv[q + 1][0] < iv[q][1] for q in range(len(iv) - 1))   # some jobs ran together


def test_job_over_budget_is_refused(cuda_device):
    spec = serve.job_stream(1, 10.0, 3, 16, 16)[0]
    files = serve.prepare([spec])[0]
    with serve.Server(1 << 20, slots=1) as srv:
        tk = srv.submit(spec.tiling, files)
        srv.drain(60)
        x = srv.status(tk)
    assert x["state"] == -1 and x["rc"] == 3 and "budget" in x["msg"]


def test_fp64_check_waits_for_admissible_jobs(cuda_device):
    """A checked job delivers its energies first (state 3), the jobs queued
    behind it run next, and its FP64 check runs when none is waiting."""
    specs = serve.job_stream(3, 100.0, 5, 16, 16)  # jobs of some ms: all three are queued before the first ends
    files = serve.prepare(specs)
    prec = ng.PREC_MIXED_FP16
    with serve.Server(40 << 30, slots=1, reserve=40, check_ctas=32) as srv:
        tickets = [srv.submit(s.tiling, f, prec, check_fp64=(s.id == 0)) for s, f in zip(specs, files)]
        srv.drain(600)
        st = [srv.status(t) for t in tickets]
    assert all(x["state"] == 2 for x in st), [x["msg"] for x in st]
    assert st[0]["ran"] <= st[1]["admitted"] and st[2]["ran"] <= st[0]["finished"]
    mixed, fp64 = _alone(specs[0], files[0], prec)
    assert st[0]["energy"] == mixed and st[0]["fp64"] == fp64


def test_queue_jobs_share_one_resident_launch(cuda_device):
    """Jobs submitted back to back enter the shared work queue while the
    resident kernel runs: several jobs' items are taken and finished inside
    one launch, and each job's energies are the bits of the job run alone."""
    specs = serve.job_stream(4, 1000.0, 21, 10, 14)
    files = serve.prepare(specs)
    prec = ng.PREC_MIXED_FP16
    with serve.Server(40 << 30, slots=4, idle=0.5) as srv:
        tickets = [srv.submit(s.tiling, f, prec) for s, f in zip(specs, files)]
        srv.drain(600)
        st = [srv.status(t) for t in tickets]
        gens = [srv.launches(t) for t in tickets]
        stats = srv.queue_stats()
    assert all(x["state"] == 2 for x in st), [x["msg"] for x in st]
    assert stats["jobs"] == 4 and stats["in_queue"] == 0
    assert all(a > 0 and b > 0 for a, b in gens)
    # at least two jobs whose items were all taken and finished by the same launch
    same = [a for a, b in gens if a == b]
    assert len(same) >= 2 and max(same.count(g) for g in same) >= 2, (gens, stats)
    assert stats["max_in_queue"] >= 2
    for spec, f, x in zip(specs, files, st):
        mixed, fp64 = _alone(spec, f, prec)
        assert x["energy"] == mixed
        assert x["energy"][1] == pytest.approx(fp64[1], rel=2e-6)


def test_queue_kernel_leaves_when_idle_and_comes_back(cuda_device):
    """The resident kernel leaves after its idle time; a job submitted later
    starts a new launch and is served the same way."""
    specs = serve.job_stream(2, 10.0, 23, 8, 10)
    files = serve.prepare(specs)
    prec = ng.PREC_MIXED_FP16
    with serve.Server(40 << 30, slots=2, idle=0.02) as srv:
        t0 = srv.submit(specs[0].tiling, files[0], prec)
        srv.drain(600)
        time.sleep(0.3)                                  # well past the idle time: the kernel has left
        t1 = srv.submit(specs[1].tiling, files[1], prec)
        srv.drain(600)
        st = [srv.status(t0), srv.status(t1)]
        g0, g1 = srv.launches(t0), srv.launches(t1)
        stats = srv.queue_stats()
    assert all(x["state"] == 2 for x in st), [x["msg"] for x in st]
    assert stats["launches"] >= 2 and g1[0] > g0[1]
    for spec, f, x in zip(specs, files, st):
        assert x["energy"] == _alone(spec, f, prec)[0]


def test_queue_off_runs_each_job_alone(cuda_device):
    """With the shared queue turned off every job gets its own launches, and
    the energies are the same bits."""
    specs = serve.job_stream(3, 100.0, 25, 8, 12)
    files = serve.prepare(specs)
    prec = ng.PREC_MIXED_FP16
    with serve.Server(40 << 30, slots=2, queue=None) as srv:
        tickets = [srv.submit(s.tiling, f, prec) for s, f in zip(specs, files)]
        srv.drain(600)
        st = [srv.status(t) for t in tickets]
        stats = srv.queue_stats()
    assert stats["launches"] == 0 and stats["jobs"] == 0
    for spec, f, x in zip(specs, files, st):
        assert x["state"] == 2 and x["energy"] == _alone(spec, f, prec)[0]
