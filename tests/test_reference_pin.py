"""CPU: the oracle against outputs of the reference's own code.

tests/golden/reference_kernels.json holds digests of the 27 sd_t_* kernels
and energies of ccsd_t_dot, produced by the reference's Fortran translated
statement by statement into C (oracle/f77_ref.py, tests/golden/make_ref_golden.py).
The oracle's restated kernels must reproduce every output bit for bit; its
energy sum (compensated, where the reference's OpenMP reduction order is
unspecified) to 1e-14 relative."""
import ctypes as C
import hashlib
import json
import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as orc

GOLD = json.loads((Path(__file__).resolve().parent / "golden" / "reference_kernels.json").read_text())
sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
from make_ref_golden import dot_inputs, kernel_inputs  # noqa: E402


@pytest.mark.parametrize("rec", GOLD["kernels"], ids=lambda r: f"{r['family']}_{r['k']}_{'x'.join(map(str, r['dims']))}")
def test_oracle_kernel_bitwise_equals_reference(rec):
    x, a, b = kernel_inputs(rec["family"], rec["dims"], rec["seed"])
    fd = rec["dims"][:6] if rec["family"] == "s1" else rec["dims"]
    orc.kernel(rec["family"], rec["k"], fd, x, a, b)
    assert hashlib.sha256(x.tobytes()).hexdigest() == rec["sha256"]


@pytest.mark.parametrize("rec", GOLD["dot"], ids=lambda r: "_".join(map(str, r["case"])))
def test_oracle_dot_equals_reference(rec):
    s, d, ev, r = dot_inputs(tuple(rec["case"]), rec["seed"])
    h1b, h2b, h3b, p4b, p5b, p6b, restricted = rec["case"]
    e1, e2 = C.c_double(0.0), C.c_double(0.0)
    lib = orc.lib()
    lib.orc_ccsd_t_dot.restype = None
    pd = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    lib.orc_ccsd_t_dot(pd(s), pd(d), C.c_int64(restricted), C.c_int64(h1b), C.c_int64(h2b), C.c_int64(h3b),
                       C.c_int64(p4b), C.c_int64(p5b), C.c_int64(p6b), *[pd(e) for e in ev],
                       *[C.c_int64(x) for x in r], C.byref(e1), C.byref(e2))
    assert e1.value == pytest.approx(rec["E[T]"], rel=1e-14, abs=0)
    assert e2.value == pytest.approx(rec["E(T)"], rel=1e-14, abs=0)
