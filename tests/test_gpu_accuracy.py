"""GPU: the mixed forms' absolute energy error at molecular magnitude.

The synthetic workloads have |E(T)| of tens to millions of Eh (random
amplitudes, not converged CCSD ones), so their absolute errors say nothing
about a 1 µEh target.  Here the same generator's inputs are multiplied by a
scale s chosen so that |E(T)| is 0.05 Eh (both energies scale by s**4), and
each split form must stay within 1 µEh of the oracle (o=10/v=40, where the
oracle takes a second) or of the FP64 form (a long-K case; the FP64 form is
held to 1e-10 of the oracle by the other tests), for E[T], E(T) and
E[ST] = E(T) - E[T]."""
import json
from pathlib import Path

import numpy as np
import pytest

import nwchem_gb300 as ng
from nwchem_gb300 import _capi
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "oracle_known_answers.json").read_text())
UEH = 1e-6          # the bound: 1 microhartree
FORMS = {"tf32": ng.PREC_MIXED_TF32, "bf16": ng.PREC_MIXED_BF16, "fp16": ng.PREC_MIXED_FP16}


def _errors(m, ref):
    return abs(m[0] - ref[0]), abs(m[1] - ref[1]), abs((m[1] - m[0]) - (ref[1] - ref[0]))


def test_molecular_scale_o10v40_against_oracle(cuda_device):
    """o=10, v=40, seed 0, inputs scaled to |E(T)| = 0.05 Eh: the oracle,
    the FP64 form and the three split forms."""
    _capi.lib().sdt_set_error_mode(1)
    t = ng.config_tiling(0)
    s = ng.molecular_scale(GOLDEN["configs"]["o10v40_seed0"]["E(T)"])
    files = ng.synth_inputs(t, 0, scale=s)
    o1, o2, _, _ = orc.Problem(t, *files).ccsd_t()
    assert 0.04 < abs(o2) < 0.06
    kl = ng.task_list(t)
    with ng.TriplesJob(t) as job:
        job.load(*files)
        f = job.run(kl)
        mixed = {name: job.run(kl, precision=p) for name, p in FORMS.items()}
    assert f[0] == pytest.approx(o1, rel=1e-10) and f[1] == pytest.approx(o2, rel=1e-10)
    for name, m in mixed.items():
        assert max(_errors(m, (o1, o2))) <= UEH, (name, _errors(m, (o1, o2)))


def test_molecular_scale_long_k_against_fp64(cuda_device):
    """o=32 (16,16), v=320 (20 tiles of 16), seed 6: K = o + v = 352 as in
    the o=40/v=300 workload, 48 tuples spread over the weight order, inputs
    scaled to |E(T)| = 0.05 Eh over those tuples; each split form against
    the FP64 form, plain and with segmented drains."""
    _capi.lib().sdt_set_error_mode(1)
    t = ng.Tiling([16, 16], [16] * 20).with_evl(6)
    kl_all = ng.task_list(t)
    kl = kl_all[np.linspace(0, len(kl_all) - 1, 48).round().astype(np.int64)]
    with ng.TriplesJob(t) as job:
        job.load(*ng.synth_inputs(t, 6))
        e_nat = job.run(kl)
    s = ng.molecular_scale(e_nat[1])
    with ng.TriplesJob(t) as job:
        job.load(*ng.synth_inputs(t, 6, scale=s))
        f = job.run(kl)
        assert 0.04 < abs(f[1]) < 0.06
        assert f[1] == pytest.approx(e_nat[1] * s ** 4, rel=1e-12)
        for kseg in (0, 4):
            job.set_mixed_segment(kseg)
            for name, p in FORMS.items():
                m = job.run(kl, precision=p)
                assert max(_errors(m, f)) <= UEH, (name, kseg, _errors(m, f))
