"""GPU parity of the batched path (sdt_job_*: device ingest of the TCE files
and the fused FP64 tuple kernel) against the oracle.

Tolerance: 1e-10 relative on E[T] and E(T), the bar for the FP64 form; the
observed agreement is ~1e-14 (FP64 with another summation order)."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import nwchem_gb300 as ng
from nwchem_gb300 import _capi
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "oracle_known_answers.json").read_text())
REL = 1e-10


@pytest.fixture(scope="module")
def gpu(cuda_device):
    _capi.lib().sdt_set_error_mode(1)
    return cuda_device


TILINGS = [
    ([6], [12], None, None),                       # one tile each, partial 4-boxes
    ([5], [9], None, None),
    ([2, 4], [5, 3, 4], None, None),               # diagonal and mixed tuples
    ([3, 5, 2], [4, 6, 4, 3], None, None),
    ([8, 12], [20, 24], None, None),               # multiples of 4
    ([3, 2, 3], [4, 5, 4, 3], [0, 1, 1], [1, 0, 1, 0]),   # irreps: filtered h7b/p7b
    ([4, 4, 4, 4], [8, 8, 8, 8], [0, 1, 2, 3], [3, 2, 1, 0]),
    ([1, 2, 3, 4, 5], [5, 4, 3, 2, 1], None, None),  # every tile size 1..5 in every position
]


@pytest.mark.parametrize("occ,vir,osym,vsym", TILINGS)
def test_fused_matches_oracle(gpu, occ, vir, osym, vsym):
    t = ng.Tiling(occ, vir, occ_sym=osym, vir_sym=vsym).with_evl(21)
    files = ng.synth_inputs(t, 21)
    P = orc.Problem(t, *files)
    kl = P.task_list()
    e1, e2, pt, _ = P.ccsd_t()
    with ng.TriplesJob(t) as job:
        job.load(*files)
        g1, g2, gpt = job.run(kl, per_task=True)
    assert g1 == pytest.approx(e1, rel=REL, abs=0)
    assert g2 == pytest.approx(e2, rel=REL, abs=0)
    tol = REL * max(abs(e1), abs(e2))
    assert np.abs(gpt - pt).max() <= tol


def test_fused_retiling_known_answer(gpu):
    """The GPU path reproduces the oracle's re-tiling known answers."""
    for g in GOLDEN["retiling"]:
        t = ng.Tiling(g["occ"], g["vir"]).with_evl(g["seed"])
        files = ng.synth_inputs(t, g["seed"])
        e1, e2 = ng.ccsd_t(t, *files)
        assert e1 == pytest.approx(g["E[T]"], rel=1e-12, abs=0)
        assert e2 == pytest.approx(g["E(T)"], rel=1e-12, abs=0)


def test_fused_workload0(gpu):
    """o=10, v=40 (seed 0): E[T], E(T), E[ST] against the oracle's values."""
    g = GOLDEN["configs"]["o10v40_seed0"]
    t = ng.config_tiling(0)
    files = ng.synth_inputs(t, 0)
    with ng.TriplesJob(t) as job:
        job.load(*files)
        e1, e2 = job.run(ng.task_list(t))
    assert e1 == pytest.approx(g["E[T]"], rel=REL, abs=0)
    assert e2 == pytest.approx(g["E(T)"], rel=REL, abs=0)
    assert (e2 - e1) == pytest.approx(g["E[ST]"], rel=1e-8, abs=0)


def _across_sizes(t, kl, rng, quantiles, extra=()):
    """Tuple indices at the given quantiles of the per-tuple FLOP count
    (seeded pick inside a narrow band around each), plus `extra`."""
    fl = np.array([ng.flops(t, kl[q:q + 1]) for q in range(len(kl))])
    order = np.argsort(fl, kind="stable")
    n = len(order)
    ids = []
    for qt in quantiles:
        lo, hi = int(qt * (n - 1)), min(n, int(qt * (n - 1)) + max(1, n // 50))
        ids.append(int(order[rng.integers(lo, hi)]))
    ids.extend(int(x) for x in extra)
    return np.unique(np.array(ids, dtype=np.int64)), fl


def _diagonal(k):
    return k[0] == k[1] or k[1] == k[2] or k[3] == k[4] or k[4] == k[5]


def test_fused_workload1_tuples_across_sizes(gpu):
    """o=40 (8/12/20), v=300 (11 tiles), seed 1: per-tuple energies of
    tuples drawn from every part of the size range (5 %, 25 %, 50 %, 75 %,
    95 % FLOP quantiles), the heaviest tuple of the 2860 (40x40x40x20x20x20,
    5.1e8 triples elements) and one tuple with no repeated tile, FP64 against
    the oracle at 1e-10 and each mixed form within its bound."""
    t = ng.config_tiling(1)
    files = ng.synth_inputs(t, 1)
    kl = ng.task_list(t)
    rng = np.random.default_rng(101)
    plain = [q for q in range(len(kl)) if not _diagonal(kl[q])]
    ids, fl = _across_sizes(t, kl, rng, (0.05, 0.25, 0.5, 0.75, 0.95), extra=(plain[len(plain) // 2],))
    ids = np.unique(np.append(ids, int(np.argmax(fl))))
    assert any(_diagonal(kl[q]) for q in ids) and any(not _diagonal(kl[q]) for q in ids)
    P = orc.Problem(t, *files)
    _, _, pt, _ = P.ccsd_t(kl, task_ids=ids)
    with ng.TriplesJob(t) as job:
        job.load(*files)
        _, _, gpt = job.run(kl[ids], per_task=True)
        mixed = {f: job.run(kl[ids], per_task=True, precision=p)[2] for f, p in (("tf32", 1), ("bf16", 2), ("fp16", 3))}
    assert np.allclose(gpt, pt, rtol=REL, atol=0)
    bound = {"tf32": 2e-5, "fp16": 2e-5, "bf16": 5e-5}   # per tuple: fewer elements than a whole job
    for f, m in mixed.items():
        assert np.all(np.abs(m - pt) <= bound[f] * np.abs(pt)), f


def test_fused_workload3_tuples_across_sizes(gpu):
    """Blocked spatial symmetry (8 irreps, the first 4096 tuples of its weight
    order, seed 3): per-tuple energies of the workload's own tuples at the
    10/30/50/70/90 % FLOP quantiles, FP64 against the oracle at 1e-10 and
    FP16x3 within its bound."""
    t = ng.config_tiling(3)
    files = ng.synth_inputs(t, 3)
    kl = ng.task_list(t)[:4096]
    ids, _ = _across_sizes(t, kl, np.random.default_rng(103), (0.1, 0.3, 0.5, 0.7, 0.9))
    P = orc.Problem(t, *files)
    _, _, pt, _ = P.ccsd_t(kl, task_ids=ids)
    with ng.TriplesJob(t) as job:
        job.load(*files)
        _, _, gpt = job.run(kl[ids], per_task=True)
        _, _, mpt = job.run(kl[ids], per_task=True, precision=ng.PREC_MIXED_FP16)
    assert np.allclose(gpt, pt, rtol=REL, atol=0)
    assert np.all(np.abs(mpt - pt) <= 2e-5 * np.abs(pt))


def test_fused_deterministic(gpu):
    t = ng.Tiling([3, 5, 2], [4, 6, 4, 3]).with_evl(2)
    files = ng.synth_inputs(t, 2)
    kl = ng.task_list(t)
    with ng.TriplesJob(t) as job:
        job.load(*files)
        a = job.run(kl, per_task=True)
        b = job.run(kl, per_task=True)
    assert a[0] == b[0] and a[1] == b[1] and np.array_equal(a[2], b[2])


def test_fused_capped_launches_same_bits(gpu):
    """Results do not depend on the launch width: capped persistent launches,
    with and without one CTA per SM, give the bits of the full launch."""
    t = ng.Tiling([3, 5, 2], [4, 6, 4, 3]).with_evl(2)
    files = ng.synth_inputs(t, 2)
    kl = ng.task_list(t)
    with ng.TriplesJob(t) as job:
        job.load(*files)
        ref = job.run(kl, per_task=True)
        for sms, excl in ((8, False), (8, True), (1, True)):
            job.set_max_ctas(sms, sm_exclusive=excl)
            e = job.run(kl, per_task=True)
            assert e[0] == ref[0] and e[1] == ref[1] and np.array_equal(e[2], ref[2]), (sms, excl)


def test_fused_subsets_add_up(gpu):
    """Energies are additive over tuple ranges (the sharding contract)."""
    t = ng.Tiling([3, 5, 2], [4, 6, 4, 3]).with_evl(2)
    files = ng.synth_inputs(t, 2)
    kl = ng.task_list(t)
    with ng.TriplesJob(t) as job:
        job.load(*files)
        e1, e2, pt = job.run(kl, per_task=True)
        h = len(kl) // 2
        x1, x2 = job.run(kl[:h])
        y1, y2 = job.run(kl[h:])
    assert x1 + y1 == pytest.approx(e1, rel=1e-13)
    assert x2 + y2 == pytest.approx(e2, rel=1e-13)


def test_fused_errors(gpu):
    t = ng.Tiling([3], [5]).with_evl(0)
    f1, f2, fv = ng.synth_inputs(t, 0)
    job = ng.TriplesJob(t)
    with pytest.raises(ng.SdtError) as e:
        job.run(ng.task_list(t))
    assert e.value.code == 4
    # drop the last V2 block from the hash: the load must name a missing block
    n = int(fv.hash[0])
    h = np.concatenate([[n - 1], fv.hash[1:n], fv.hash[n + 1:2 * n]]).astype(np.int64)
    with pytest.raises(ng.SdtError) as e:
        job.load(f1, f2, ng.TceFile(h, fv.data))
    assert e.value.code == 5
    job.load(f1, f2, fv)
    bad = ng.task_list(t).copy()
    bad[0, [0, 3]] = bad[0, [3, 0]]
    with pytest.raises(ng.SdtError) as e:
        job.run(bad)
    assert e.value.code == 1
    job.close()


def test_box_host_generates_same_inputs(gpu):
    """The GPU host (aarch64) produces byte-identical seeded inputs."""
    t = ng.config_tiling(0)
    dig = GOLDEN["synth_sha256"]
    for name, f in zip(("T1", "T2", "V2"), ng.synth_inputs(t, 0)):
        assert hashlib.sha256(f.data.tobytes()).hexdigest() == dig[f"o10v40_seed0_{name}"]["data"]
    assert hashlib.sha256(t.evl.tobytes()).hexdigest() == dig["o10v40_seed0_evl"]


def test_fused_reads_nwchem_layout_files(gpu, tmp_path):
    """T1/T2/V2 in NWChem's on-disk layout (every V2 block; the blocks the path
    never reads set to NaN) give the FP64 and mixed energies of the synthetic files."""
    from nwchem_gb300 import tcefile
    t = ng.Tiling([3, 2, 3], [4, 3, 5]).with_evl(23)
    files = ng.synth_inputs(t, 23)
    kinds = (ng.FILE_T1, ng.FILE_T2, ng.FILE_V2)
    read = []
    for kind, f in zip(kinds, files):
        p = tmp_path / f"f{kind}.bin"
        tcefile.write_tce_file(p, f, t, kind)
        if kind == ng.FILE_V2:
            h, nd = tcefile.tce_layout(t, kind)
            raw = np.fromfile(p, dtype=np.float64)
            n = int(h[0])
            for q in range(n):
                if f.lookup(int(h[1 + q])) < 0:
                    end = int(h[2 + n + q]) if q + 1 < n else nd
                    raw[int(h[1 + n + q]):end] = np.nan
            raw.tofile(p)
        read.append(tcefile.read_tce_file(p, t, kind, mmap=False))
    kl = ng.task_list(t)
    with ng.TriplesJob(t) as a, ng.TriplesJob(t) as b:
        a.load(*files)
        b.load(*read)
        for prec in (ng.PREC_FP64, ng.PREC_MIXED_TF32):
            assert a.run(kl, precision=prec) == b.run(kl, precision=prec)


def test_fused_checkpointed_run(gpu, tmp_path):
    """A restarted GPU run skips recorded ranges and returns the same bits."""
    from nwchem_gb300 import restart
    t = ng.Tiling([3, 5, 2], [4, 6, 4, 3]).with_evl(2)
    files = ng.synth_inputs(t, 2)
    kl = ng.task_list(t)
    with ng.TriplesJob(t) as job:
        job.load(*files)
        seen = []

        class Stop(RuntimeError):
            pass

        def runner(sub):
            seen.append(len(sub))
            if len(seen) == 4 and not hasattr(runner, "resumed"):
                raise Stop()
            return job.run(sub)

        ck = tmp_path / "c.jsonl"
        with pytest.raises(Stop):
            restart.CheckpointedRun(ck, kl, 9, runner).run()
        runner.resumed = True
        e = restart.CheckpointedRun(ck, kl, 9, runner).run()
        full = job.run(kl)
    assert e[0] == pytest.approx(full[0], rel=1e-13) and e[1] == pytest.approx(full[1], rel=1e-13)


def test_restricted_tiling_both_forms(gpu):
    """Restricted tilings (beta blocks read through their alpha twins, factor 2,
    tce_restricted.F and ccsd_t_dot.F:52-57): FP64 and mixed forms against the oracle."""
    t = ng.Tiling([3, 3], [4, 4], occ_spin=[1, 2], vir_spin=[1, 2], restricted=True,
                  alpha=[1, 1, 3, 3]).with_evl(6)
    files = ng.synth_inputs(t, 6)
    e1, e2, pt, _ = orc.Problem(t, *files).ccsd_t()
    kl = ng.task_list(t)
    with ng.TriplesJob(t) as job:
        job.load(*files)
        g1, g2, gpt = job.run(kl, per_task=True)
        m1, m2 = job.run(kl, precision=ng.PREC_MIXED_FP16)
    assert g1 == pytest.approx(e1, rel=REL, abs=0) and g2 == pytest.approx(e2, rel=REL, abs=0)
    assert np.abs(gpt - pt).max() <= REL * max(abs(e1), abs(e2))
    assert m1 == pytest.approx(e1, rel=2e-6) and m2 == pytest.approx(e2, rel=2e-6)


def test_per_tuple_output_writes_only_its_pairs(gpu):
    """Canary-padded outputs of a one-shot run and of a plan: exactly 2 * n
    doubles are written, and the energies out[2] only."""
    import ctypes as C
    t = ng.Tiling([3, 5, 2], [4, 6, 4, 3]).with_evl(2)
    files = ng.synth_inputs(t, 2)
    kl = np.ascontiguousarray(ng.task_list(t))
    n = len(kl)
    lib = _capi.lib()
    with ng.TriplesJob(t) as job:
        job.load(*files)
        ref = job.run(kl, per_task=True)
        for prec in (ng.PREC_FP64, ng.PREC_MIXED_FP16):
            pt = np.full(2 * n + 32, np.nan)
            e = np.full(2 + 8, np.nan)
            rc = lib.sdt_job_run(job._h, kl.ctypes.data_as(_capi.PI64), n, prec, e.ctypes.data_as(_capi.PD),
                                 pt.ctypes.data_as(_capi.PD), None)
            assert rc == 0
            assert np.all(np.isnan(pt[2 * n:])) and np.all(np.isnan(e[2:]))
            assert not np.any(np.isnan(pt[:2 * n])) and not np.any(np.isnan(e[:2]))
            if prec == ng.PREC_FP64:
                assert np.array_equal(pt[:2 * n].reshape(n, 2), ref[2]) and (e[0], e[1]) == ref[:2]
        with ng.Plan(job, kl, ng.PREC_FP64) as p:
            pt = np.full(2 * n + 32, np.nan)
            e = np.full(2 + 8, np.nan)
            assert lib.sdt_plan_run(p._h, None, e.ctypes.data_as(_capi.PD), pt.ctypes.data_as(_capi.PD)) == 0
            assert np.all(np.isnan(pt[2 * n:])) and np.all(np.isnan(e[2:]))
            assert np.array_equal(pt[:2 * n].reshape(n, 2), ref[2])


def test_fused_o64_shaped_tuple_slab(gpu):
    """A tuple of the o=64/v=512 workload's shape -- 64x64x64 particle and
    32x32x32 hole tiles, 8.6e9 triples elements, 2.1e6 sub-boxes -- with the
    contraction length cut to o + v = 256 (o=64 as 2x32, v=192 as 3x64, seed
    2).  The FP64 form's per-item energies over the slab p4 < 4, h1 < 4 (the
    first p4 box and h1 box) against the oracle's energy of that slab,
    evaluated as a tuple of the re-tiled orbital space, to 1e-10."""
    occ, vir = [32, 32], [64, 64, 64]
    t = ng.Tiling(occ, vir).with_evl(2)
    files = ng.synth_inputs(t, 2)
    kl = ng.task_list(t)
    row = next(k for k in kl if list(k[:6]) == [3, 4, 5, 1, 2, 2])
    with ng.TriplesJob(t) as job:
        job.load(*files)
        with ng.Plan(job, row[None, :]) as p:
            e = p.run()
            items = p.item_energies()
    nb = [16, 16, 16, 8, 8, 8]
    assert len(items) == int(np.prod(nb))
    idx = np.arange(len(items))
    box = []
    for n in reversed(nb):
        box.append(idx % n)
        idx //= n
    box = box[::-1]                                            # p4, p5, p6, h1, h2, h3 boxes
    slab = items[(box[0] == 0) & (box[3] == 0)].sum(axis=0)
    assert items.sum(axis=0)[1] == pytest.approx(e[1], rel=1e-12)
    occ2, vir2, new = orc.slab_retiling(occ, vir, [3, 4, 5, 1, 2, 2], 4, 4)
    t2 = ng.Tiling(occ2, vir2).with_evl(2)
    P2 = orc.Problem(t2, *ng.synth_inputs(t2, 2))
    kl2 = P2.task_list()
    q = next(i for i, k in enumerate(kl2) if list(k[:6]) == new)
    _, _, pt, _ = P2.ccsd_t(kl2, task_ids=np.array([q]))
    assert slab[0] == pytest.approx(pt[0, 0], rel=REL) and slab[1] == pytest.approx(pt[0, 1], rel=REL)
