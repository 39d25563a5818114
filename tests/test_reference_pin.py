"""CPU: the oracle against outputs of the reference's own code.

tests/golden/reference_kernels.json holds digests of the 27 sd_t_* kernels
and energies of ccsd_t_dot, produced by the reference's Fortran translated
statement by statement into C (oracle/f77_ref.py, tests/golden/make_ref_golden.py),
and the tuple lists of ccsd_t_neword.F and the block permutations of
tce_sort4.F / tce_sort2.F translated the same way.
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


def _tiling(rec):
    import nwchem_gb300 as ng
    alpha = None
    if rec["restricted"]:   # beta tiles map onto the alpha tiles of the same length, in order
        spins = rec["occ_spin"] + rec["vir_spin"]
        n_o = len(rec["occ"])
        alpha = []
        for b, sp in enumerate(spins):
            lo, hi = (0, n_o) if b < n_o else (n_o, len(spins))
            alpha.append(b + 1 if sp == 1 else [q for q in range(lo, hi) if spins[q] == 1][
                [q for q in range(lo, hi) if spins[q] == 2].index(b)] + 1)
    return ng.Tiling(rec["occ"], rec["vir"], occ_spin=rec["occ_spin"], vir_spin=rec["vir_spin"],
                     occ_sym=rec["occ_sym"], vir_sym=rec["vir_sym"], restricted=bool(rec["restricted"]), alpha=alpha)


@pytest.mark.parametrize("rec", GOLD["tasks"], ids=lambda r: r["name"])
def test_tuple_list_equals_reference(rec):
    """The tuple set and weight order of ccsd_t_6tasks / ccsd_t_neword
    (translated from the reference), bit for bit: the oracle's restatement
    and the library's host code (sdt_tasks_list)."""
    import nwchem_gb300 as ng
    t = _tiling(rec)
    nofile = type("F", (), {"hash": np.zeros(1, dtype=np.int64), "data": np.zeros(1)})()
    kl_orc = orc.Problem(t, nofile, nofile, nofile).task_list()
    kl_lib = ng.task_list(t)
    assert len(kl_orc) == rec["n"] and len(kl_lib) == rec["n"]
    for kl in (kl_orc, kl_lib):
        assert hashlib.sha256(np.ascontiguousarray(kl, dtype=np.int64).tobytes()).hexdigest() == rec["sha256"]


@pytest.mark.parametrize("rec", GOLD["sort4"], ids=lambda r: "".join(map(str, r["perm"])))
def test_sort4_equals_reference(rec):
    from make_ref_golden import SORT4_DIMS, sort_input
    x = sort_input(SORT4_DIMS, rec["seed"])
    y = np.zeros_like(x)
    pd = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    orc.lib().orc_tce_sort_4(pd(x), pd(y), *SORT4_DIMS, *rec["perm"], rec["factor"])
    assert hashlib.sha256(y.tobytes()).hexdigest() == rec["sha256"]


@pytest.mark.parametrize("rec", GOLD["sort2"], ids=lambda r: "".join(map(str, r["perm"])))
def test_sort2_equals_reference(rec):
    from make_ref_golden import SORT2_DIMS, sort_input
    x = sort_input(SORT2_DIMS, rec["seed"])
    y = np.zeros_like(x)
    pd = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    orc.lib().orc_tce_sort_2(pd(x), pd(y), *SORT2_DIMS, *rec["perm"], rec["factor"])
    assert hashlib.sha256(y.tobytes()).hexdigest() == rec["sha256"]
