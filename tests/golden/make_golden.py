"""Regenerates tests/golden/oracle_known_answers.json.

Run from the repository root:  python tests/golden/make_golden.py

What is frozen here, and why it pins the oracle:
  * retiling: one orbital space (o=6, v=12, seed 5) under five tilings.  The
    (T) energy does not depend on the tiling; agreement across tilings pins the
    permutation tables, duplicate-row removal, multiplicity factors and the
    antisymmetry signs of the block fetches (ccsd_t_singles_l.F,
    offl_ccsd_t_doubles_l.F, tce_hashnsort.F, ccsd_t_dot.F).
  * closed_form: for o=5, v=9 (one tile each) the energies of the closed
    spin-orbital form E[T] = 1/36 sum X_d^2/D, E(T) = 1/36 sum X_d(X_d+X_s)/D,
    with X_d, X_s the 18 + 9 permuted products written out densely with numpy.
  * configs: E[T], E(T) of workload 0 (o=10, v=40, seed 0) from the oracle.
  * synth_sha256: digests of the seeded input files, so that any host
    (x86-64 or aarch64) can check it generates the same bytes.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import nwchem_gb300 as ng  # noqa: E402
from oracle import oracle as orc  # noqa: E402

OUT = Path(__file__).resolve().parent / "oracle_known_answers.json"

RETILINGS = [([6], [12]), ([2, 4], [5, 3, 4]), ([3, 3], [4, 4, 4]), ([1, 2, 3], [12]),
             ([6], [2, 2, 2, 2, 2, 2]), ([1, 1, 4], [7, 5])]


def closed_form(o: int, v: int, seed: int) -> dict:
    t = ng.Tiling([o], [v]).with_evl(seed)
    f1, f2, fv = ng.synth_inputs(t, seed)
    N = 2

    def blk(g3, g4, g1, g2, shape):
        off = fv.lookup(g2 - 1 + N * (g1 - 1 + N * (g4 - 1 + N * (g3 - 1))))
        return fv.data[off:off + int(np.prod(shape))].reshape(shape)

    t1 = f1.data.reshape(v, o)
    t2 = f2.data.reshape(v, v, o, o)
    V = blk(2, 2, 1, 2, (v, v, o, v))   # <p5 p6||h3 p7>
    w = blk(1, 2, 1, 1, (o, v, o, o))   # <h7 p6||h2 h3>
    u = blk(2, 2, 1, 1, (v, v, o, o))   # <p5 p6||h2 h3>
    es = np.einsum
    xd = (-es('abim,mcjk->abcijk', t2, w) + es('abjm,mcik->abcijk', t2, w) - es('abkm,mcij->abcijk', t2, w)
          - es('bcim,majk->abcijk', t2, w) + es('bcjm,maik->abcijk', t2, w) - es('bckm,maij->abcijk', t2, w)
          + es('acim,mbjk->abcijk', t2, w) - es('acjm,mbik->abcijk', t2, w) + es('ackm,mbij->abcijk', t2, w)
          - es('aeij,bcke->abcijk', t2, V) - es('aejk,bcie->abcijk', t2, V) + es('aeik,bcje->abcijk', t2, V)
          + es('beij,acke->abcijk', t2, V) + es('bejk,acie->abcijk', t2, V) - es('beik,acje->abcijk', t2, V)
          - es('ceij,abke->abcijk', t2, V) - es('cejk,abie->abcijk', t2, V) + es('ceik,abje->abcijk', t2, V))
    xs = (es('ai,bcjk->abcijk', t1, u) - es('aj,bcik->abcijk', t1, u) + es('ak,bcij->abcijk', t1, u)
          - es('bi,acjk->abcijk', t1, u) + es('bj,acik->abcijk', t1, u) - es('bk,acij->abcijk', t1, u)
          + es('ci,abjk->abcijk', t1, u) - es('cj,abik->abcijk', t1, u) + es('ck,abij->abcijk', t1, u))
    eo, ev = t.evl[:o], t.evl[o:]
    D = (eo[None, None, None, :, None, None] + eo[None, None, None, None, :, None]
         + eo[None, None, None, None, None, :] - ev[:, None, None, None, None, None]
         - ev[None, :, None, None, None, None] - ev[None, None, :, None, None, None])
    return {"o": o, "v": v, "seed": seed,
            "E[T]": float((xd * xd / D).sum() / 36.0),
            "E(T)": float((xd * (xd + xs) / D).sum() / 36.0)}


def main() -> None:
    out: dict = {"retiling": [], "closed_form": None, "configs": {}, "synth_sha256": {}}
    for occ, vir in RETILINGS:
        t = ng.Tiling(occ, vir).with_evl(5)
        e1, e2, _, kc = orc.Problem(t, *ng.synth_inputs(t, 5)).ccsd_t()
        out["retiling"].append({"occ": occ, "vir": vir, "seed": 5, "E[T]": e1, "E(T)": e2,
                                "tasks": int(len(kc))})
    out["closed_form"] = closed_form(5, 9, 3)
    t = ng.config_tiling(0)
    files = ng.synth_inputs(t, 0)
    e1, e2, _, _ = orc.Problem(t, *files).ccsd_t()
    out["configs"]["o10v40_seed0"] = {"E[T]": e1, "E(T)": e2, "E[ST]": e2 - e1}
    for name, f in zip(("T1", "T2", "V2"), files):
        out["synth_sha256"][f"o10v40_seed0_{name}"] = {
            "hash": hashlib.sha256(f.hash.tobytes()).hexdigest(),
            "data": hashlib.sha256(f.data.tobytes()).hexdigest()}
    out["synth_sha256"]["o10v40_seed0_evl"] = hashlib.sha256(t.evl.tobytes()).hexdigest()
    OUT.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
