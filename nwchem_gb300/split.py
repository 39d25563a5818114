"""Host-side TF32 split of FP64 values (the mixed form's operand encoding).

hi = tf32(x), lo = tf32(x - hi), each rounded to nearest with ties away
from zero (the device's cvt.rna.tf32.f32) and kept in an fp32 container.
"""
from __future__ import annotations

import numpy as np


def tf32(x: np.ndarray) -> np.ndarray:
    """Round fp32 values to TF32 (10 explicit mantissa bits), ties away from zero."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((b + np.uint32(0x1000)) & np.uint32(0xFFFFE000)).astype(np.uint32)
    return r.view(np.float32)


def split_tf32(x: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    x = np.asarray(x, dtype=np.float64)
    hi = tf32(x.astype(np.float32))
    lo = tf32((x - hi.astype(np.float64)).astype(np.float32))
    return hi, lo
