"""CPU tests: the oracle against its known answers, and the host logic of
the library (tuple list, FLOP count, synthetic inputs) against the oracle."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import nwchem_gb300 as ng
from oracle import oracle as orc

GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "oracle_known_answers.json").read_text())


def _problem(occ, vir, seed, **kw):
    t = ng.Tiling(occ, vir, **kw).with_evl(seed)
    return t, orc.Problem(t, *ng.synth_inputs(t, seed))


def test_retiling_invariance_known_answer():
    """One orbital space, six tilings: the (T) energy must not move."""
    ref = GOLDEN["retiling"][0]
    for g in GOLDEN["retiling"]:
        _, P = _problem(g["occ"], g["vir"], g["seed"])
        e1, e2, _, kc = P.ccsd_t()
        assert len(kc) == g["tasks"]
        assert e1 == pytest.approx(g["E[T]"], rel=1e-13, abs=0)
        assert e2 == pytest.approx(g["E(T)"], rel=1e-13, abs=0)
        assert e1 == pytest.approx(ref["E[T]"], rel=1e-12, abs=0)
        assert e2 == pytest.approx(ref["E(T)"], rel=1e-12, abs=0)


def test_closed_form_known_answer():
    """The tiled driver + 27 kernels equal the dense spin-orbital closed form."""
    g = GOLDEN["closed_form"]
    _, P = _problem([g["o"]], [g["v"]], g["seed"])
    e1, e2, _, _ = P.ccsd_t()
    assert e1 == pytest.approx(g["E[T]"], rel=1e-12, abs=0)
    assert e2 == pytest.approx(g["E(T)"], rel=1e-12, abs=0)


def test_workload0_known_answer():
    g = GOLDEN["configs"]["o10v40_seed0"]
    t = ng.config_tiling(0)
    e1, e2, _, _ = orc.Problem(t, *ng.synth_inputs(t, 0)).ccsd_t()
    assert e1 == pytest.approx(g["E[T]"], rel=1e-13, abs=0)
    assert e2 == pytest.approx(g["E(T)"], rel=1e-13, abs=0)


def test_triples_antisymmetric():
    """With antisymmetric inputs the doubles tile is antisymmetric in a<->b, i<->j."""
    _, P = _problem([5], [7], 11)
    s, d = P.tuple_tiles([2, 2, 2, 1, 1, 1])          # Fortran (h3,h2,h1,p6,p5,p4)
    x = d.transpose(5, 4, 3, 2, 1, 0)                 # (a,b,c,i,j,k)
    y = s.transpose(5, 4, 3, 2, 1, 0)
    scale = np.abs(x).max()
    for perm in [(1, 0, 2, 3, 4, 5), (0, 2, 1, 3, 4, 5), (0, 1, 2, 4, 3, 5), (0, 1, 2, 3, 5, 4)]:
        assert np.abs(x + x.transpose(perm)).max() <= 1e-14 * scale
        assert np.abs(y + y.transpose(perm)).max() <= 1e-14 * np.abs(y).max()


@pytest.mark.parametrize("occ,vir,osym,vsym", [
    ([3, 5, 2], [4, 6, 4, 3], None, None),
    ([8, 12, 20], [20, 24, 24, 24, 24, 24, 30, 30, 30, 30, 40], None, None),
    ([2, 3, 2, 3], [4, 5, 4, 6, 5], [0, 1, 2, 3], [0, 1, 2, 3, 1]),
    ([4, 4], [6, 6, 8], [1, 1], [0, 1, 1]),
])
def test_task_list_matches_oracle(occ, vir, osym, vsym):
    """Same tuple set, same weight order, bit for bit (ccsd_t_neword)."""
    t = ng.Tiling(occ, vir, occ_sym=osym, vir_sym=vsym).with_evl(0)
    kl = ng.task_list(t)
    P = orc.Problem(t, *(ng.TceFile(np.zeros(1, np.int64), np.zeros(1)),) * 3)
    assert np.array_equal(kl, P.task_list())
    if osym is None:
        nv, no = len(vir), len(occ)
        assert len(kl) == (nv * (nv + 1) * (nv + 2) // 6) * (no * (no + 1) * (no + 2) // 6)


def test_kernel_call_counts():
    """Every sorted tuple fires 9 s1, 9 d1 per h7 tile and 9 d2 per p7 tile."""
    t, P = _problem([2, 3], [3, 2, 4], 1)
    _, _, _, kc = P.ccsd_t()
    assert (kc[:, 0] == 9).all()
    assert (kc[:, 1] == 9 * t.noab).all()
    assert (kc[:, 2] == 9 * t.nvab).all()


def test_symmetry_blocks_filtered():
    """With irreps, d1/d2 run only for spin/irrep-allowed h7b/p7b tiles."""
    t, P = _problem([2, 3, 2], [3, 2, 4, 3], 2, occ_sym=[0, 1, 1], vir_sym=[0, 1, 0, 1])
    e1, e2, _, kc = P.ccsd_t()
    assert np.isfinite(e1) and np.isfinite(e2)
    sym = lambda b: int(t.sym[b - 1])
    occ_tiles = range(1, t.noab + 1)
    vir_tiles = range(t.noab + 1, t.noab + t.nvab + 1)
    for row, calls in zip(P.task_list(), kc):
        a, b, c, i, j, k = (int(x) for x in row[:6])
        # s1 term (P,H) pairs, d1 (P,P',H) and d2 (P,H,H') triples, in kernel order
        s1 = [(a, i), (a, j), (a, k), (b, i), (b, j), (b, k), (c, i), (c, j), (c, k)]
        d1 = [(a, b, i), (a, b, j), (a, b, k), (b, c, i), (b, c, j), (b, c, k), (a, c, i), (a, c, j), (a, c, k)]
        d2 = [(a, i, j), (a, j, k), (a, i, k), (b, i, j), (b, j, k), (b, i, k), (c, i, j), (c, j, k), (c, i, k)]
        n_s1 = sum(sym(p) == sym(h) for p, h in s1)
        n_d1 = sum(sym(p) ^ sym(q) ^ sym(h) ^ sym(m) == 0 for p, q, h in d1 for m in occ_tiles)
        n_d2 = sum(sym(p) ^ sym(e) ^ sym(h) ^ sym(g) == 0 for p, h, g in d2 for e in vir_tiles)
        assert tuple(calls) == (n_s1, n_d1, n_d2)


def test_flops_match_survey_counts():
    """Algorithmic FLOPs sum Nt*18*(O+V+1) of workloads 0-2."""
    expect = {0: 5.875e10, 1: 9.430e14, 2: 4.282e16}
    for c, f in expect.items():
        t = ng.config_tiling(c)
        assert ng.flops(t, ng.task_list(t)) == pytest.approx(f, rel=5e-4)
    t = ng.config_tiling(1)
    assert len(ng.task_list(t)) == 2860
    assert len(ng.task_list(ng.config_tiling(2))) == 480


def test_synthetic_inputs_reproducible():
    """Seeded inputs are byte-identical to the committed digests."""
    t = ng.config_tiling(0)
    files = ng.synth_inputs(t, 0)
    dig = GOLDEN["synth_sha256"]
    for name, f in zip(("T1", "T2", "V2"), files):
        assert hashlib.sha256(f.hash.tobytes()).hexdigest() == dig[f"o10v40_seed0_{name}"]["hash"]
        assert hashlib.sha256(f.data.tobytes()).hexdigest() == dig[f"o10v40_seed0_{name}"]["data"]
    assert hashlib.sha256(t.evl.tobytes()).hexdigest() == dig["o10v40_seed0_evl"]


def test_synthetic_distributions():
    """T2 antisymmetric with sd ~0.02; energies inside the stated ranges."""
    t = ng.Tiling([10], [30]).with_evl(4)
    f1, f2, fv = ng.synth_inputs(t, 4)
    t2 = f2.data.reshape(30, 30, 10, 10)
    assert np.abs(t2 + t2.transpose(1, 0, 2, 3)).max() == 0.0
    assert np.abs(t2 + t2.transpose(0, 1, 3, 2)).max() == 0.0
    off = t2[np.triu_indices(30, 1)][:, np.triu_indices(10, 1)[0], np.triu_indices(10, 1)[1]]
    assert off.std() == pytest.approx(0.02, rel=0.05)
    assert f1.data.std() == pytest.approx(0.01, rel=0.1)
    assert (t.evl[:10] >= -1.5).all() and (t.evl[:10] < -0.4).all()
    assert (t.evl[10:] >= 0.2).all() and (t.evl[10:] < 2.5).all()


def test_restricted_mapping_reads_alpha_blocks():
    """Restricted tilings: beta-only blocks are read through their alpha twins,
    and the factor 2 applies (tce_restricted.F, ccsd_t_dot.F:52-57)."""
    occ, vir = [3, 3], [4, 4]
    t = ng.Tiling(occ, vir, occ_spin=[1, 2], vir_spin=[1, 2], restricted=True,
                  alpha=[1, 1, 3, 3]).with_evl(6)
    P = orc.Problem(t, *ng.synth_inputs(t, 6))
    e1, e2, _, kc = P.ccsd_t()
    assert np.isfinite(e1) and e1 < 0
    assert len(kc) == len(ng.task_list(t))


def test_oracle_workload_inputs_equal_the_library():
    """The checker-side generator (orc_synth.c), tilings, tuple lists and
    FLOP counts are byte for byte the library's, and the o=10/v=40 files
    match the committed digests: the CPU baseline runs on the same inputs
    without loading the product library."""
    import hashlib
    import json
    from pathlib import Path
    gold = json.loads((Path(__file__).resolve().parent / "golden" / "oracle_known_answers.json").read_text())
    for c in (0, 1, 3):
        a, b = orc.config_tiling(c), ng.config_tiling(c)
        assert np.array_equal(a.range, b.range) and np.array_equal(a.sym, b.sym)
        assert np.array_equal(a.evl, b.evl)
        fa = orc.synth_inputs(a, c)
        if c == 0:
            for name, f in zip(("T1", "T2", "V2"), fa):
                d = gold["synth_sha256"][f"o10v40_seed0_{name}"]
                assert hashlib.sha256(f.hash.tobytes()).hexdigest() == d["hash"]
                assert hashlib.sha256(f.data.tobytes()).hexdigest() == d["data"]
        if c != 1:   # o=40/v=300: 5.7 GB, compared through the tuple list only
            fb = ng.synth_inputs(b, c)
            for x, y in zip(fa, fb):
                assert np.array_equal(x.hash, y.hash) and np.array_equal(x.data, y.data)
        kl = orc.Problem(a, *fa).task_list()
        assert np.array_equal(kl, ng.task_list(b))
        assert orc.flops(a, kl) == ng.flops(b, kl)
    t = ng.Tiling([3, 2, 3], [4, 5, 4, 3], occ_sym=[0, 1, 1], vir_sym=[1, 0, 1, 0]).with_evl(5)
    o = orc.Tiling([3, 2, 3], [4, 5, 4, 3], [0, 1, 1], [1, 0, 1, 0], seed=5)
    for x, y in zip(orc.synth_inputs(o, 5), ng.synth_inputs(t, 5)):
        assert np.array_equal(x.hash, y.hash) and np.array_equal(x.data, y.data)


def test_slab_retiling_is_exact_on_the_oracle():
    """CPU check of the slab method the GPU test of the o=64-shaped tuple
    uses: the energy of the re-tiled tuple equals the slab p4 < 3, h1 < 2 of
    the original tuple, summed from the oracle's full triples tiles."""
    occ, vir = [6, 5], [7, 6, 8]
    t = ng.Tiling(occ, vir).with_evl(12)
    P = orc.Problem(t, *ng.synth_inputs(t, 12))
    tup = [3, 4, 5, 1, 2, 2]
    s, d = P.tuple_tiles(tup)                                  # (h3,h2,h1,p6,p5,p4)
    r, off = t.range, t.offset
    ev = [t.evl[off[b - 1]:off[b - 1] + r[b - 1]] for b in tup]   # p4,p5,p6,h1,h2,h3
    D = (ev[5][:, None, None, None, None, None] + ev[4][None, :, None, None, None, None]
         + ev[3][None, None, :, None, None, None] - ev[2][None, None, None, :, None, None]
         - ev[1][None, None, None, None, :, None] - ev[0][None, None, None, None, None, :])
    sl = (slice(None), slice(None), slice(0, 2), slice(None), slice(None), slice(0, 3))
    f = 0.5                                                    # h2 = h3 tile
    e1 = f * np.sum(d[sl] ** 2 / D[sl])
    e2 = f * np.sum(d[sl] * (d[sl] + s[sl]) / D[sl])
    occ2, vir2, new = orc.slab_retiling(occ, vir, tup, 3, 2)
    t2 = ng.Tiling(occ2, vir2).with_evl(12)
    P2 = orc.Problem(t2, *ng.synth_inputs(t2, 12))
    s2, d2 = P2.tuple_tiles(new)
    # the same elements; the contraction over the re-tiled virtual space is summed in other pieces
    assert np.allclose(d2, d[sl], rtol=0, atol=1e-14 * np.abs(d).max()) and np.array_equal(s2, s[sl])
    kl2 = P2.task_list()
    q = next(i for i, k in enumerate(kl2) if list(k[:6]) == new)
    _, _, pt, _ = P2.ccsd_t(kl2, task_ids=np.array([q]))
    assert pt[0, 0] == pytest.approx(e1, rel=1e-12) and pt[0, 1] == pytest.approx(e2, rel=1e-12)
