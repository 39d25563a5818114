"""Regenerates tests/golden/reference_kernels.json from the reference's own code.

Run from the repository root; it needs the NWChem source tree (the
argument, else the NWCHEM_SRC environment variable, as oracle/f77_ref.py
takes it):

    python tests/golden/make_ref_golden.py [NWCHEM_SOURCE_TREE]

It builds oracle/_ref/libref_kernels.so with oracle/f77_ref.py -- a
statement-by-statement translation of src/tce/ccsd_t/ccsd_t_kernels_omp.F
and src/tce/ccsd_t/ccsd_t_dot.F into C -- runs each of the 27 sd_t_* kernels
and ccsd_t_dot on seeded inputs, and records the sha256 of every output
(the kernels) and the energies (ccsd_t_dot).  tests/test_reference_pin.py
checks the oracle against these values on any machine, without the tree.
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
    OUT.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {OUT}: {len(out['kernels'])} kernels, {len(out['dot'])} dot cases")


if __name__ == "__main__":
    main()
