"""CPU check of the numerical argument behind the mixed form's FP32 energy
denominators: with the orbital energies shifted by the midpoint of the
occupied-virtual gap, every hole term of D = (e_i + e_j + e_k) - (e_a + e_b
+ e_c) is negative and every particle term positive, so the FP32 sums (in
the kernel's order) do not cancel and D keeps a relative error of a few
FP32 roundings.  Emulated with numpy float32 on the library's own seeded
orbital energies; the device quotient itself is checked on the GPU
(test_gpu_mixed.test_energy_division_bound)."""
import numpy as np
import pytest

import nwchem_gb300 as ng


@pytest.mark.parametrize("occ,vir,seed", [([8, 12, 20], [20, 24, 24, 30, 40], 1), ([32, 32], [64] * 4, 2),
                                          ([10], [40], 0)])
def test_shifted_fp32_denominators(occ, vir, seed):
    t = ng.Tiling(occ, vir).with_evl(seed)
    o, v = t.nocc, t.nvir
    eo, ev = t.evl[:o], t.evl[o:o + v]
    assert eo.max() < ev.min()                       # a gap: the generator's ranges
    mu = 0.5 * (eo.max() + ev.min())
    fo, fv = (eo - mu).astype(np.float32), (ev - mu).astype(np.float32)
    assert np.all(fo < 0) and np.all(fv > 0)
    rng = np.random.default_rng(seed)
    n = 200_000
    i, j, k = (rng.integers(0, o, n) for _ in range(3))
    a, b, c = (rng.integers(0, v, n) for _ in range(3))
    d32 = ((fo[i] + fo[j]) + fo[k]) - ((fv[a] + fv[b]) + fv[c])      # the energy warps' order
    d64 = (eo[i] + eo[j] + eo[k]) - (ev[a] + ev[b] + ev[c])
    rel = np.abs(d32.astype(np.float64) - d64) / np.abs(d64)
    # six conversions and five additions, each within half an FP32 ulp of a value no larger than |D|
    assert rel.max() < 11 * 2.0 ** -24, rel.max()
