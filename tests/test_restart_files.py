"""CPU tests: checkpoint/restart of a tuple-list evaluation, and reading TCE
files in NWChem's on-disk layout (the oracle stands in for the GPU runner)."""
import math

import numpy as np
import pytest

import nwchem_gb300 as ng
from nwchem_gb300 import restart, tcefile
from oracle import oracle as orc


class Interrupt(RuntimeError):
    pass


def _problem():
    t = ng.Tiling([3, 2, 3], [4, 3, 5]).with_evl(23)
    files = ng.synth_inputs(t, 23)
    return t, files, orc.Problem(t, *files)


def test_restart_resumes_and_matches_uninterrupted(tmp_path):
    t, files, P = _problem()
    kl = P.task_list()
    calls = []

    def runner(sub):
        calls.append(len(sub))
        e1, e2, _, _ = P.ccsd_t(sub)
        return e1, e2

    def failing_after(n):
        def r(sub):
            if len(calls) >= n:
                raise Interrupt()
            return runner(sub)
        return r

    ck = tmp_path / "ckpt.jsonl"
    with pytest.raises(Interrupt):
        restart.CheckpointedRun(ck, kl, 7, failing_after(3)).run()
    assert len(calls) == 3
    run = restart.CheckpointedRun(ck, kl, 7, runner)
    assert 0 < run.progress < 1
    e1, e2 = run.run()
    n_ranges = len(run.ranges)
    assert len(calls) == n_ranges           # the 3 finished ranges were not redone
    # identical to one uninterrupted run with the same ranges
    calls.clear()
    f1, f2 = restart.CheckpointedRun(tmp_path / "fresh.jsonl", kl, 7, runner).run()
    assert (e1, e2) == (f1, f2)
    _, _, pt, _ = P.ccsd_t()
    assert e1 == pytest.approx(math.fsum(pt[:, 0]), rel=1e-14)
    # a checkpoint of another tuple list is ignored
    other = restart.CheckpointedRun(ck, kl[:-1], 7, runner)
    assert other.progress == 0.0


def test_restart_tolerates_a_cut_line(tmp_path):
    t, files, P = _problem()
    kl = P.task_list()
    runner = lambda sub: P.ccsd_t(sub)[:2]
    ck = tmp_path / "c.jsonl"
    want = restart.CheckpointedRun(ck, kl, 11, runner).run()
    text = ck.read_text().splitlines()
    ck.write_text("\n".join(text[:-1]) + "\n" + text[-1][: len(text[-1]) // 2])
    assert restart.CheckpointedRun(ck, kl, 11, runner).run() == want


def test_tce_layout_matches_reference_enumeration():
    """T1/T2 layouts equal the synthetic files' (same loops as tce_t1/t2_offset);
    the V2 layout lists every allowed block, in key order."""
    t = ng.Tiling([2, 3], [3, 4]).with_evl(0)
    for kind in (ng.FILE_T1, ng.FILE_T2):
        h, nd = tcefile.tce_layout(t, kind)
        f = ng.synth_file(t, kind, 1)
        assert np.array_equal(h, f.hash) and nd == f.data.size
    h, nd = tcefile.tce_layout(t, ng.FILE_V2)
    n = int(h[0])
    N = t.noab + t.nvab
    assert n == sum(1 for g3 in range(1, N + 1) for g4 in range(g3, N + 1)
                    for g1 in range(1, N + 1) for g2 in range(g1, N + 1))
    assert (np.diff(h[1:n + 1]) > 0).all()


def test_full_layout_files_give_the_same_energies(tmp_path):
    """Files written in NWChem's full layout (every V2 block; the ones the path
    never reads filled with NaN) read back and give the same (T) energies."""
    t, files, P = _problem()
    e1, e2, _, _ = P.ccsd_t()
    paths = []
    for kind, f in zip((ng.FILE_T1, ng.FILE_T2, ng.FILE_V2), files):
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
        paths.append(p)
    read = [tcefile.read_tce_file(p, t, k) for p, k in zip(paths, (ng.FILE_T1, ng.FILE_T2, ng.FILE_V2))]
    assert read[2].data.size > files[2].data.size
    g1, g2, _, _ = orc.Problem(t, *read).ccsd_t()
    assert (g1, g2) == (e1, e2)
    with pytest.raises(ValueError):
        tcefile.read_tce_file(paths[0], t, ng.FILE_T2)
