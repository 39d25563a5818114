"""CPU tests of the autotuner's host logic (classes, choices, cache) with an
injected timing function in place of GPU runs."""
from types import SimpleNamespace

import numpy as np

import nwchem_gb300 as ng
from nwchem_gb300 import autotune


def _setup():
    t = ng.Tiling([4, 8, 12], [8, 16, 24, 32], occ_sym=[0, 1, 0], vir_sym=[1, 0, 1, 0]).with_evl(3)
    return t, ng.task_list(t)


def test_classes_partition_the_list():
    t, kl = _setup()
    tuner = autotune.Autotuner(SimpleNamespace(tiling=t), measure=lambda *a: 1.0)
    cl = tuner.classes(kl)
    idx = np.sort(np.concatenate(list(cl.values())))
    assert np.array_equal(idx, np.arange(len(kl)))
    for c, ids in cl.items():
        assert all(autotune.size_class(t, kl[q]) == c for q in ids)


def test_choices_are_the_cheapest_and_cached(tmp_path):
    t, kl = _setup()
    calls = []

    def fake(sub, precision, shape):
        calls.append((len(sub), precision, shape))
        # fp16 fastest; the tensor-memory hold shape pays off only for the biggest class
        base = {ng.PREC_MIXED_FP16: 1.0, ng.PREC_MIXED_BF16: 1.1, ng.PREC_MIXED_TF32: 2.0}[precision]
        big = max(autotune.size_class(t, k) for k in sub) == max(autotune.size_class(t, k) for k in kl)
        return ng.flops(t, sub) * base * (0.9 if (shape == 2 and big) else 1.0)

    cache = tmp_path / "tune.json"
    tuner = autotune.Autotuner(SimpleNamespace(tiling=t), cache=cache, measure=fake, sample=3)
    d = tuner.tune(kl)
    assert d["form"] == "fp16"
    top = max(tuner.classes(kl))
    assert all(v == (2 if c == top else 1) for c, v in d["shapes"].items())
    assert cache.exists() and calls
    shapes = tuner.shapes(kl, d)
    assert shapes.shape == (len(kl),) and set(shapes.tolist()) <= {1, 2}
    # a second tuner reuses the cache without timing anything
    calls.clear()
    again = autotune.Autotuner(SimpleNamespace(tiling=t), cache=cache, measure=fake).tune(kl)
    assert again == d and not calls


def test_forms_restrict_the_split_choice():
    t, kl = _setup()
    fake = lambda sub, prec, shape: {ng.PREC_MIXED_BF16: 1.0}.get(prec, 5.0)
    d = autotune.Autotuner(SimpleNamespace(tiling=t), forms=("tf32", "fp16"), measure=fake).tune(kl)
    assert d["form"] in ("tf32", "fp16")
