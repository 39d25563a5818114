"""Orbital tilings in the TCE convention and the synthetic workloads.

Tiles are numbered 1..noab (occupied) then noab+1..noab+nvab (virtual), each
with a length (range), a spin label (1 alpha, 2 beta) and an irrep (0..7),
as src/tce/include/tce.fh:14-21 and src/tce/tce_tile.F:1238-1335 set them.
offset[b] is the position of tile b's first orbital in evl_sorted (occupied
orbitals first, then virtual).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _capi


@dataclass
class Tiling:
    occ: list[int]
    vir: list[int]
    occ_spin: list[int] | None = None
    vir_spin: list[int] | None = None
    occ_sym: list[int] | None = None
    vir_sym: list[int] | None = None
    restricted: bool = False
    alpha: list[int] | None = None
    evl: np.ndarray | None = None
    name: str = "custom"
    _keep: list = field(default_factory=list, repr=False)

    def __post_init__(self):
        self.occ = [int(x) for x in self.occ]
        self.vir = [int(x) for x in self.vir]
        n_o, n_v = len(self.occ), len(self.vir)
        self.occ_spin = list(self.occ_spin or [1] * n_o)
        self.vir_spin = list(self.vir_spin or [1] * n_v)
        self.occ_sym = list(self.occ_sym or [0] * n_o)
        self.vir_sym = list(self.vir_sym or [0] * n_v)
        if min(self.occ + self.vir) < 1:
            raise ValueError("tile lengths must be positive")
        self.range = np.array(self.occ + self.vir, dtype=np.int64)
        self.spin = np.array(self.occ_spin + self.vir_spin, dtype=np.int64)
        self.sym = np.array(self.occ_sym + self.vir_sym, dtype=np.int64)
        self.offset = np.concatenate([[0], np.cumsum(self.range)[:-1]]).astype(np.int64)
        self.alpha_arr = None if self.alpha is None else np.array(self.alpha, dtype=np.int64)
        if self.restricted and self.alpha_arr is None:
            raise ValueError("a restricted tiling needs the beta->alpha tile map")
        if self.evl is None:
            self.evl = np.zeros(self.nocc + self.nvir)
        self.evl = np.ascontiguousarray(self.evl, dtype=np.float64)

    @property
    def noab(self) -> int:
        return len(self.occ)

    @property
    def nvab(self) -> int:
        return len(self.vir)

    @property
    def nocc(self) -> int:
        return int(sum(self.occ))

    @property
    def nvir(self) -> int:
        return int(sum(self.vir))

    def with_evl(self, seed: int) -> "Tiling":
        """Sets seeded orbital energies (occupied U[-1.5,-0.4], virtual U[0.2,2.5])."""
        evl = np.empty(self.nocc + self.nvir)
        _capi.check(_capi.lib().sdt_synth_evl(self.nocc, self.nvir, seed,
                                              evl.ctypes.data_as(_capi.PD)), "sdt_synth_evl")
        self.evl = evl
        return self

    def struct(self) -> _capi.SdtTiling:
        """The sdt_tiling view of this tiling (arrays stay owned by self)."""
        p64 = lambda a: a.ctypes.data_as(_capi.PI64)
        s = _capi.SdtTiling(self.noab, self.nvab, p64(self.range), p64(self.spin), p64(self.sym),
                            p64(self.offset),
                            p64(self.alpha_arr) if self.alpha_arr is not None else C.cast(None, _capi.PI64),
                            self.evl.ctypes.data_as(_capi.PD), 1 if self.restricted else 0)
        self._keep = [s]
        return s


def config_tiling(config: int, seed: int | None = None) -> Tiling:
    """Tilings of the benchmark workloads (spin-orbital, unrestricted, no symmetry).

    0: o=10, v=40, one tile each (seed 0)
    1: o=40 as 8/12/20, v=300 as 20,24x5,30x4,40 (seed 1)
    2: o=64 as 2x32, v=512 as 8x64 (seed 2)
    3: blocked spatial symmetry: 8 occupied tiles (irreps 0..7) with lengths
       drawn from {8,12,16,24,32} and 12 virtual tiles (irreps 0..7,0..3)
       from {16,24,32,48,64}, drawn by numpy's PCG64 with seed 3; the
       workload is the first 4096 tuples of the weight order (seed 3)
    """
    if config == 0:
        t = Tiling([10], [40], name="o10v40")
    elif config == 1:
        t = Tiling([8, 12, 20], [20, 24, 24, 24, 24, 24, 30, 30, 30, 30, 40], name="o40v300")
    elif config == 2:
        t = Tiling([32, 32], [64] * 8, name="o64v512")
    elif config == 3:
        rng = np.random.default_rng(3)
        occ = [int(x) for x in rng.choice([8, 12, 16, 24, 32], 8)]
        vir = [int(x) for x in rng.choice([16, 24, 32, 48, 64], 12)]
        t = Tiling(occ, vir, occ_sym=[q % 8 for q in range(8)], vir_sym=[q % 8 for q in range(12)],
                   name="sym8_o%dv%d" % (sum(occ), sum(vir)))
    else:
        raise ValueError(f"no tiling for workload {config}")
    return t.with_evl(config if seed is None else seed)


def random_tiling(rng: np.random.Generator, nocc_tiles: int, nvir_tiles: int, occ_sizes, vir_sizes,
                  nsym: int = 1, seed: int = 0) -> Tiling:
    """A tiling with tile lengths drawn from the given sets and irreps 0..nsym-1."""
    occ = [int(rng.choice(occ_sizes)) for _ in range(nocc_tiles)]
    vir = [int(rng.choice(vir_sizes)) for _ in range(nvir_tiles)]
    osym = [int(x) for x in rng.integers(0, nsym, nocc_tiles)]
    vsym = [int(x) for x in rng.integers(0, nsym, nvir_tiles)]
    return Tiling(occ, vir, occ_sym=osym, vir_sym=vsym, name="random").with_evl(seed)
