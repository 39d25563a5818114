"""Regenerates tests/golden/reference_kernels.json from the reference's own code.

Run from the repository root; it needs the NWChem source tree (the
argument, else the NWCHEM_SRC environment variable, as oracle/f77_ref.py
takes it):

    python tests/golden/make_ref_golden.py [NWCHEM_SOURCE_TREE]

It builds oracle/_ref/libref_kernels.so with oracle/f77_ref.py -- a
statement-by-statement translation of src/tce/ccsd_t/ccsd_t_kernels_omp.F,
src/tce/ccsd_t/ccsd_t_dot.F, src/tce/ccsd_t/ccsd_t_neword.F and
src/tce/sort/tce_sort4.F / tce_sort2.F into C -- runs each of the 27 sd_t_*
kernels and ccsd_t_dot on seeded inputs, ccsd_t_6tasks / ccsd_t_neword on
the workloads' tilings (and spin-mixed, restricted and uniform ones), and
tce_sort_4 / tce_sort_2 for every index permutation, and records the sha256
of every output (kernels, tuple lists, sorts) and the energies
(ccsd_t_dot).  tests/test_reference_pin.py checks the oracle and the
library against these values on any machine, without the tree.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import f77_ref  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_kernels.json"
# (h3d, h2d, h1d, p6d, p5d, p4d, k7d): distinct dims catch index-order errors
DIMS = [(3, 2, 4, 5, 3, 2, 6), (4, 4, 4, 3, 3, 3, 5), (2, 3, 2, 4, 2, 3, 7)]
DOT_CASES = [  # (h1b,h2b,h3b,p4b,p5b,p6b, restricted): every multiplicity factor
    (1, 2, 3, 4, 5, 6, 0), (1, 1, 3, 4, 5, 5, 0), (2, 2, 2, 4, 4, 4, 0), (1, 2, 2, 5, 5, 6, 1), (1, 1, 1, 4, 6, 6, 1)]


def kernel_inputs(family: str, dims, seed: int):
    h3, h2, h1, p6, p5, p4, k7 = dims
    rng = np.random.default_rng(seed)
    nt = h3 * h2 * h1 * p6 * p5 * p4
    x = rng.standard_normal(nt)
    if family == "s1":
        a, b = rng.standard_normal(p4 * h1), rng.standard_normal(h3 * h2 * p6 * p5)
    elif family == "d1":
        a, b = rng.standard_normal(k7 * p4 * p5 * h1), rng.standard_normal(h3 * h2 * p6 * k7)
    else:
        a, b = rng.standard_normal(k7 * p4 * h1 * h2), rng.standard_normal(k7 * h3 * p6 * p5)
    return x, a, b


def dot_inputs(case, seed: int):
    rng = np.random.default_rng(seed)
    r = (3, 2, 4, 2, 3, 2)  # r_h1, r_h2, r_h3, r_p4, r_p5, r_p6
    nt = int(np.prod(r))
    s, d = rng.standard_normal(nt) * 0.01, rng.standard_normal(nt) * 0.05
    ev = [rng.uniform(-1.5, -0.4, r[0]), rng.uniform(-1.5, -0.4, r[1]), rng.uniform(-1.5, -0.4, r[2]),
          rng.uniform(0.2, 2.5, r[3]), rng.uniform(0.2, 2.5, r[4]), rng.uniform(0.2, 2.5, r[5])]
    return s, d, ev, r


# Tilings for the tuple list: (name, occ, vir, occ_spin, vir_spin, occ_sym, vir_sym, restricted)
TASK_TILINGS = [
    ("o40v300", [8, 12, 20], [20, 24, 24, 24, 24, 24, 30, 30, 30, 30, 40], None, None, None, None, 0),
    ("o64v512_uniform", [32, 32], [64] * 8, None, None, None, None, 0),
    ("spin_mixed", [3, 4, 3, 2], [6, 5, 7, 6, 4], [1, 2, 1, 2], [1, 2, 2, 1, 2], [0, 1, 0, 1], [1, 0, 0, 1, 1], 0),
    ("restricted", [3, 4, 3, 4], [6, 5, 6, 5], [1, 1, 2, 2], [1, 1, 2, 2], None, None, 1),
]


def task_tilings():
    """The tilings above plus the blocked-symmetry workload's (seed 3)."""
    out = list(TASK_TILINGS)
    rng = np.random.default_rng(3)
    occ = [int(x) for x in rng.choice([8, 12, 16, 24, 32], 8)]
    vir = [int(x) for x in rng.choice([16, 24, 32, 48, 64], 12)]
    out.append(("sym8", occ, vir, None, None, [q % 8 for q in range(8)], [q % 8 for q in range(12)], 0))
    return out


def tiling_arrays(rec):
    _, occ, vir, ospin, vspin, osym, vsym, restricted = rec
    n_o, n_v = len(occ), len(vir)
    rng = np.array(occ + vir, dtype=np.int64)
    spin = np.array(list(ospin or [1] * n_o) + list(vspin or [1] * n_v), dtype=np.int64)
    sym = np.array(list(osym or [0] * n_o) + list(vsym or [0] * n_v), dtype=np.int64)
    return rng, spin, sym, int(restricted)


def sort_input(dims, seed: int):
    return np.random.default_rng(seed).standard_normal(int(np.prod(dims)))


SORT4_DIMS = (2, 3, 4, 5)
SORT2_DIMS = (3, 5)


def main() -> None:
    lib = C.CDLL(str(f77_ref.build(Path(sys.argv[1]) if len(sys.argv) > 1 else f77_ref.DEFAULT_TREE)))
    i64 = lambda v: C.byref(C.c_int64(int(v)))
    pd = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    out = {"source": "translated from src/tce/ccsd_t/ccsd_t_kernels_omp.F and ccsd_t_dot.F by oracle/f77_ref.py",
           "kernels": [], "dot": []}
    for di, dims in enumerate(DIMS):
        for family in ("s1", "d1", "d2"):
            for k in range(1, 10):
                seed = 1000 * di + 100 * ("s1", "d1", "d2").index(family) + k
                x, a, b = kernel_inputs(family, dims, seed)
                fd = dims[:6] if family == "s1" else dims
                getattr(lib, f"sd_t_{family}_{k}_")(*[i64(v) for v in fd], pd(x), pd(a), pd(b))
                out["kernels"].append({"family": family, "k": k, "dims": list(dims), "seed": seed,
                                       "sha256": hashlib.sha256(x.tobytes()).hexdigest(), "sum": float(x.sum())})
    for ci, case in enumerate(DOT_CASES):
        s, d, ev, r = dot_inputs(case, 7000 + ci)
        e1, e2 = C.c_double(0.0), C.c_double(0.0)
        h1b, h2b, h3b, p4b, p5b, p6b, restricted = case
        lib.ccsd_t_dot_(pd(s), pd(d), i64(restricted), i64(h1b), i64(h2b), i64(h3b), i64(p4b), i64(p5b), i64(p6b),
                        *[pd(e) for e in ev], *[i64(x) for x in r], C.byref(e1), C.byref(e2))
        out["dot"].append({"case": list(case), "seed": 7000 + ci, "E[T]": e1.value, "E(T)": e2.value})
    out["source"] += ", ccsd_t_neword.F, tce_sort4.F and tce_sort2.F"
    out["tasks"] = []
    lib.ccsd_t_6tasks_.restype = C.c_int64
    p64 = lambda a: a.ctypes.data_as(C.POINTER(C.c_int64))
    for rec in task_tilings():
        rng, spin, sym, restricted = tiling_arrays(rec)
        noab, nvab = len(rec[1]), len(rec[2])
        n = lib.ccsd_t_6tasks_(i64(restricted), i64(noab), i64(nvab), p64(spin), p64(sym))
        kaux = np.zeros(7 * max(n, 1), dtype=np.int64)
        klist = np.zeros(7 * max(n, 1), dtype=np.int64)
        thresh = C.c_int64(0)
        lib.ccsd_t_neword_(i64(n), i64(0), C.byref(thresh), i64(restricted), i64(noab), i64(nvab), p64(spin),
                           p64(sym), p64(rng), p64(kaux), p64(klist))
        out["tasks"].append({"name": rec[0], "occ": rec[1], "vir": rec[2], "occ_spin": rec[3], "vir_spin": rec[4],
                             "occ_sym": rec[5], "vir_sym": rec[6], "restricted": rec[7], "n": int(n),
                             "sha256": hashlib.sha256(klist[:7 * n].tobytes()).hexdigest(),
                             "first": klist[:7].tolist()})
    out["sort4"] = []
    import itertools
    for pi, perm in enumerate(itertools.permutations((1, 2, 3, 4))):
        x = sort_input(SORT4_DIMS, 8000 + pi)
        y = np.zeros_like(x)
        factor = C.c_double(-1.0 if pi % 2 else 1.0)
        lib.tce_sort_4_(pd(x), pd(y), *[i64(v) for v in SORT4_DIMS], *[i64(v) for v in perm], C.byref(factor))
        out["sort4"].append({"perm": list(perm), "seed": 8000 + pi, "factor": factor.value,
                             "sha256": hashlib.sha256(y.tobytes()).hexdigest()})
    out["sort2"] = []
    for pi, perm in enumerate(((1, 2), (2, 1))):
        x = sort_input(SORT2_DIMS, 8100 + pi)
        y = np.zeros_like(x)
        factor = C.c_double(-1.0)
        lib.tce_sort_2_(pd(x), pd(y), *[i64(v) for v in SORT2_DIMS], *[i64(v) for v in perm], C.byref(factor))
        out["sort2"].append({"perm": list(perm), "seed": 8100 + pi, "factor": -1.0,
                             "sha256": hashlib.sha256(y.tobytes()).hexdigest()})
    OUT.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {OUT}: {len(out['kernels'])} kernels, {len(out['dot'])} dot cases, {len(out['tasks'])} tuple "
          f"lists, {len(out['sort4']) + len(out['sort2'])} sorts")


if __name__ == "__main__":
    main()
