"""Autotuner of the mixed form's launch choices (no reference counterpart).

The reference schedules tuples by weight only (ccsd_t_neword.F); on GB300
the batched path also chooses, per job, which split encoding runs the d1/d2
contractions (TF32x3, BF16x3 or scaled FP16x3, among the forms the caller's
accuracy allows) and, per size class of tuples, the kernel's work-unit
shape: one 8x8x8x4x4x4 sub-box per CTA with the finished sub-box held in
registers (two tensor-memory accumulators), or the same with it held in
tensor memory (one accumulator, free registers for the FP64 energy work).

A size class is the pair (log2 of the tuple's virtual sub-box count,
log2 of its occupied sub-box count), rounded.  For each class the tuner
times every candidate on up to `sample` tuples of the class (evenly spaced
in the list) and keeps the one with the least time per algorithmic FLOP.
Decisions can be cached in a JSON file keyed by the tiling.  The timing
function is injectable (measure(klist, precision, shape) -> seconds), which
is how the host logic is tested without a GPU.
"""
from __future__ import annotations

import hashlib
import json
import math
from pathlib import Path
from typing import Callable

import numpy as np

from .tiling import Tiling
from .triples import PREC_MIXED_BF16, PREC_MIXED_FP16, PREC_MIXED_TF32, Plan, TriplesJob, flops

FORMS = {"tf32": PREC_MIXED_TF32, "bf16": PREC_MIXED_BF16, "fp16": PREC_MIXED_FP16}
SHAPES = (1, 2)  # work-unit shapes: the finished sub-box kept in registers, or in TMEM

Measure = Callable[[np.ndarray, int, int], float]


def size_class(tiling: Tiling, k) -> str:
    r = tiling.range
    nv = 1
    for d in range(3):
        nv *= -(-int(r[k[d] - 1]) // 8)
    no = 1
    for d in range(3, 6):
        no *= -(-int(r[k[d] - 1]) // 4)
    return f"v{round(math.log2(nv))}o{round(math.log2(no))}"


def tiling_key(tiling: Tiling) -> str:
    h = hashlib.sha256()
    for a in (tiling.range, tiling.spin, tiling.sym):
        h.update(np.ascontiguousarray(a, dtype=np.int64).tobytes())
    return h.hexdigest()[:16]


class Autotuner:
    def __init__(self, job: TriplesJob, forms=("fp16", "bf16", "tf32"), sample: int = 4,
                 cache: str | Path | None = None, measure: Measure | None = None):
        unknown = [f for f in forms if f not in FORMS]
        if unknown or not forms:
            raise ValueError(f"forms must be a non-empty subset of {sorted(FORMS)}")
        self.job = job
        self.tiling = job.tiling
        self.forms = tuple(forms)
        self.sample = int(sample)
        self.cache = Path(cache) if cache else None
        self.measure = measure or self._measure_gpu
        self.log: list[dict] = []

    # -- measurement ---------------------------------------------------------
    def _measure_gpu(self, klist: np.ndarray, precision: int, shape: int) -> float:
        self.job.set_timing(True)
        with Plan(self.job, klist, precision, np.full(len(klist), shape, dtype=np.int32)) as p:
            p.run()
            p.run()
        return self.job.last_kernel_ms / 1e3

    def _cost(self, klist: np.ndarray, precision: int, shape: int) -> float:
        sec = self.measure(klist, precision, shape)
        per = sec / max(flops(self.tiling, klist), 1.0)
        self.log.append({"tuples": int(len(klist)), "precision": precision, "shape": shape, "s_per_flop": per})
        return per

    # -- classes ---------------------------------------------------------------
    def classes(self, klist: np.ndarray) -> dict[str, np.ndarray]:
        out: dict[str, list[int]] = {}
        for q, k in enumerate(np.asarray(klist)):
            out.setdefault(size_class(self.tiling, k), []).append(q)
        return {c: np.array(v, dtype=np.int64) for c, v in sorted(out.items())}

    def _pick(self, klist: np.ndarray, idx: np.ndarray) -> np.ndarray:
        m = min(self.sample, len(idx))
        return klist[idx[np.linspace(0, len(idx) - 1, m).round().astype(np.int64)]]

    # -- cache -----------------------------------------------------------------
    def _load(self) -> dict:
        if self.cache and self.cache.exists():
            try:
                return json.loads(self.cache.read_text()).get(tiling_key(self.tiling), {})
            except (OSError, ValueError):
                return {}
        return {}

    def _store(self, entry: dict) -> None:
        if not self.cache:
            return
        try:
            allc = json.loads(self.cache.read_text()) if self.cache.exists() else {}
        except (OSError, ValueError):
            allc = {}
        allc[tiling_key(self.tiling)] = entry
        self.cache.parent.mkdir(parents=True, exist_ok=True)
        self.cache.write_text(json.dumps(allc, indent=1, sort_keys=True))

    # -- decisions -------------------------------------------------------------
    def tune(self, klist: np.ndarray) -> dict:
        """{'form': name, 'shapes': {class: shape}} for this tuple list."""
        klist = np.ascontiguousarray(klist, dtype=np.int64).reshape(-1, 7)
        cached = self._load()
        classes = self.classes(klist)
        if cached.get("form") in self.forms and all(c in cached.get("shapes", {}) for c in classes):
            return cached
        # split encoding: on a sample of the class holding the most FLOPs
        weight = {c: flops(self.tiling, klist[idx]) for c, idx in classes.items()}
        main = max(weight, key=weight.get)
        probe = self._pick(klist, classes[main])
        form = min(self.forms, key=lambda f: self._cost(probe, FORMS[f], 1))
        shapes = {}
        for c, idx in classes.items():
            s = self._pick(klist, idx)
            shapes[c] = min(SHAPES, key=lambda n: self._cost(s, FORMS[form], n))
        entry = {"form": form, "shapes": shapes}
        self._store(entry)
        return entry

    def shapes(self, klist: np.ndarray, decision: dict) -> np.ndarray:
        return np.array([decision["shapes"][size_class(self.tiling, k)] for k in klist], dtype=np.int32)

    def plan(self, klist: np.ndarray, capture: bool = True, stream=None) -> tuple[Plan, dict]:
        """A plan of the whole list with the tuned choices (CUDA graph captured)."""
        klist = np.ascontiguousarray(klist, dtype=np.int64).reshape(-1, 7)
        d = self.tune(klist)
        p = Plan(self.job, klist, FORMS[d["form"]], self.shapes(klist, d))
        if capture:
            p.capture(stream)
        return p, d
