"""Host-side split of FP64 values into two narrower values (the mixed
form's operand encodings), for tests and for checking the device encoders.

TF32: hi = tf32(x), lo = tf32(x - hi), rounded to nearest with ties away
from zero (the device's cvt.rna.tf32.f32), kept in fp32 containers.
BF16 / FP16: hi = round(x), lo = round(x - hi), round to nearest even,
returned as raw 16-bit patterns together with their values.
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


def bf16_bits(x: np.ndarray) -> np.ndarray:
    """bf16 patterns of fp32 values, round to nearest even (finite inputs)."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = (b + np.uint64(0x7FFF) + ((b >> np.uint64(16)) & np.uint64(1))) >> np.uint64(16)
    return r.astype(np.uint16)


def bf16_value(bits: np.ndarray) -> np.ndarray:
    return (np.asarray(bits, dtype=np.uint32) << np.uint32(16)).view(np.float32).astype(np.float64)


def split_bf16(x: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(hi, lo) bf16 bit patterns of x."""
    x = np.asarray(x, dtype=np.float64)
    hi = bf16_bits(x.astype(np.float32))
    lo = bf16_bits((x - bf16_value(hi)).astype(np.float32))
    return hi, lo


def split_f16(x: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(hi, lo) fp16 bit patterns of x (the caller scales x into fp16 range)."""
    x = np.asarray(x, dtype=np.float64)
    hi = x.astype(np.float32).astype(np.float16)
    lo = (x - hi.astype(np.float64)).astype(np.float32).astype(np.float16)
    return hi.view(np.uint16), lo.view(np.uint16)


def f16_value(bits: np.ndarray) -> np.ndarray:
    return np.asarray(bits, dtype=np.uint16).view(np.float16).astype(np.float64)
