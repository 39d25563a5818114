"""Host-side mirror of NWChem's (T) entry point for the triples tile path.

ccsd_t(tiling, t1, t2, v2) plays the role of the reference's
ccsd_t(d_t1,k_t1_offset,d_t2,k_t2_offset,d_v2,k_v2_offset,energy1,energy2,
size_t1) (src/tce/ccsd_t/ccsd_t.F:19-20): the three TCE files go in, E[T]
(energy1, the "CCSD[T] correction") and E(T) (energy2, the "CCSD(T)
correction") come out.  E[ST] = E(T) - E[T].

TceFile holds one TCE file in host memory: the tce_hash table (hash[0] = n,
keys ascending in hash[1..n], block offsets in hash[n+1..2n]) and the block
data, each block row-major in its key order.
"""
from __future__ import annotations

import ctypes as C
import weakref
from dataclasses import dataclass

import numpy as np

from . import _capi
from .tiling import Tiling

FILE_T1, FILE_T2, FILE_V2 = 0, 1, 2
PREC_FP64 = 0
PREC_MIXED_TF32 = 1   # TF32x3: hi*hi + hi*lo + lo*hi of TF32 pairs
PREC_MIXED_BF16 = 2   # BF16x3
PREC_MIXED_FP16 = 3   # FP16x3 with power-of-two operand scaling
PREC_MIXED = (PREC_MIXED_TF32, PREC_MIXED_BF16, PREC_MIXED_FP16)


@dataclass
class TceFile:
    hash: np.ndarray
    data: np.ndarray

    def struct(self) -> _capi.SdtFile:
        return _capi.SdtFile(self.hash.ctypes.data_as(_capi.PI64), self.data.ctypes.data_as(_capi.PD),
                             int(self.data.size))

    @property
    def nbytes(self) -> int:
        return int(self.data.nbytes + self.hash.nbytes)

    def lookup(self, key: int) -> int:
        """Block offset of key (tce_hash), or -1."""
        n = int(self.hash[0])
        keys = self.hash[1:n + 1]
        i = int(np.searchsorted(keys, key))
        if i < n and keys[i] == key:
            return int(self.hash[n + 1 + i])
        return -1


def synth_file(tiling: Tiling, kind: int, seed: int, pinned: bool = False, scale: float = 1.0) -> TceFile:
    """Seeded synthetic TCE file (T1, T2 or V2 with its vvov, ovoo and vvoo
    blocks), every element multiplied by `scale` (amplitudes and integrals
    scaled by s scale both energies by s**4)."""
    lib = _capi.lib()
    ts = tiling.struct()
    nb, nd = C.c_int64(), C.c_int64()
    _capi.check(lib.sdt_synth_file(C.byref(ts), kind, seed, C.byref(nb), C.byref(nd), None, None),
                "sdt_synth_file")
    h = np.empty(2 * nb.value + 1, dtype=np.int64)
    if pinned:
        import torch
        d = torch.empty(max(nd.value, 1), dtype=torch.float64, pin_memory=True).numpy()[:nd.value]
    else:
        d = np.empty(nd.value, dtype=np.float64)
    _capi.check(lib.sdt_synth_file(C.byref(ts), kind, seed, C.byref(nb), C.byref(nd),
                                   h.ctypes.data_as(_capi.PI64), d.ctypes.data_as(_capi.PD)),
                "sdt_synth_file")
    if scale != 1.0:
        d *= scale
    return TceFile(h, d)


def synth_inputs(tiling: Tiling, seed: int, pinned: bool = False,
                 scale: float = 1.0) -> tuple[TceFile, TceFile, TceFile]:
    """The seeded T1, T2 and V2 files; `scale` multiplies every element (the
    energies scale by scale**4, which brings the synthetic E(T) of many Eh
    to the tens of mEh of a molecule)."""
    return tuple(synth_file(tiling, k, seed, pinned, scale) for k in (FILE_T1, FILE_T2, FILE_V2))


def molecular_scale(e_t: float, target: float = 0.05) -> float:
    """The input scale that maps a synthetic E(T) of e_t Eh to |E(T)| = target."""
    return (target / abs(e_t)) ** 0.25 if e_t else 1.0


def task_list(tiling: Tiling) -> np.ndarray:
    """(n, 7) tuple list in the reference's weight order (ccsd_t_neword)."""
    lib = _capi.lib()
    ts = tiling.struct()
    n = lib.sdt_tasks_count(C.byref(ts))
    if n < 0:
        _capi.check(-n, "sdt_tasks_count")
    kl = np.empty((max(n, 1), 7), dtype=np.int64)
    _capi.check(lib.sdt_tasks_list(C.byref(ts), n, kl.ctypes.data_as(_capi.PI64)), "sdt_tasks_list")
    return kl[:n]


def flops(tiling: Tiling, klist: np.ndarray) -> float:
    """Algorithmic FLOPs: sum over tuples of Nt*18*(O_allowed+V_allowed+1)."""
    kl = np.ascontiguousarray(klist, dtype=np.int64)
    ts = tiling.struct()
    return float(_capi.lib().sdt_tasks_flops(C.byref(ts), kl.ctypes.data_as(_capi.PI64), len(kl)))


def _stream_ptr(stream) -> C.c_void_p:
    if stream is None:
        return C.c_void_p(None)
    if hasattr(stream, "cuda_stream"):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


class TriplesJob:
    """One (T) problem resident on the GPU (T1/T2/V2 and orbital energies)."""

    def __init__(self, tiling: Tiling):
        self.tiling = tiling
        self._lib = _capi.lib()
        self._ts = tiling.struct()
        h = C.c_void_p()
        _capi.check(self._lib.sdt_job_create(C.byref(self._ts), C.byref(h)), "sdt_job_create")
        self._h = h
        self._plans = weakref.WeakSet()

    def load(self, t1: TceFile, t2: TceFile, v2: TceFile, stream=None) -> None:
        s = [t1.struct(), t2.struct(), v2.struct()]
        _capi.check(self._lib.sdt_job_load(self._h, C.byref(s[0]), C.byref(s[1]), C.byref(s[2]),
                                           _stream_ptr(stream)), "sdt_job_load")

    def run(self, klist: np.ndarray, per_task: bool = False, stream=None, precision: int = PREC_FP64):
        kl = np.ascontiguousarray(klist, dtype=np.int64).reshape(-1, 7)
        e = np.zeros(2)
        pt = np.zeros((len(kl), 2)) if per_task else None
        _capi.check(self._lib.sdt_job_run(self._h, kl.ctypes.data_as(_capi.PI64), len(kl), precision,
                                          e.ctypes.data_as(_capi.PD),
                                          pt.ctypes.data_as(_capi.PD) if per_task else None,
                                          _stream_ptr(stream)), "sdt_job_run")
        return (float(e[0]), float(e[1]), pt) if per_task else (float(e[0]), float(e[1]))

    def set_timing(self, on: bool = True) -> None:
        """Bracket the fused launches of each run with CUDA events."""
        _capi.check(self._lib.sdt_job_set_timing(self._h, 1 if on else 0), "sdt_job_set_timing")

    def set_mixed_segment(self, chunks: int) -> None:
        """Mixed form: drain the tensor-core accumulator every `chunks` K chunks
        (8 TF32 or 16 BF16/FP16 values each; 0: once per contraction term)."""
        _capi.check(self._lib.sdt_job_set_mixed_segment(self._h, int(chunks)), "sdt_job_set_mixed_segment")

    def set_max_ctas(self, sms: int, sm_exclusive: bool = False) -> None:
        """Cap the persistent launches at `sms` SMs' worth of CTAs (0: all);
        with sm_exclusive the FP64 launches take one CTA per SM, so a capped
        launch occupies exactly `sms` SMs."""
        _capi.check(self._lib.sdt_job_set_max_ctas(self._h, int(sms)), "sdt_job_set_max_ctas")
        _capi.check(self._lib.sdt_job_set_sm_exclusive(self._h, 1 if sm_exclusive else 0), "sdt_job_set_sm_exclusive")

    def set_mixed_shape(self, shape: int) -> None:
        """Mixed form: work-unit shape 1 (default; the finished sub-box in
        registers) or 2 (the finished sub-box in tensor memory)."""
        _capi.check(self._lib.sdt_job_set_mixed_shape(self._h, int(shape)), "sdt_job_set_mixed_shape")

    @property
    def last_kernel_ms(self) -> float:
        return float(self._lib.sdt_job_last_kernel_ms(self._h))

    @property
    def device_bytes(self) -> int:
        return int(self._lib.sdt_job_device_bytes(self._h))

    def close(self) -> None:
        if self._h:
            for p in list(self._plans):  # plans are bound to the job: free them first
                p.close()
            self._lib.sdt_job_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ccsd_t(tiling: Tiling, t1: TceFile, t2: TceFile, v2: TceFile) -> tuple[float, float]:
    """(energy1, energy2) = (E[T], E(T)) for the whole tuple list (ccsd_t.F:19-297)."""
    lib = _capi.lib()
    ts = tiling.struct()
    s = [t1.struct(), t2.struct(), v2.struct()]
    e1, e2 = C.c_double(), C.c_double()
    _capi.check(lib.sdt_ccsd_t(C.byref(ts), C.byref(s[0]), C.byref(s[1]), C.byref(s[2]),
                               C.byref(e1), C.byref(e2)), "sdt_ccsd_t")
    return e1.value, e2.value


class Plan:
    """A prepared evaluation of a tuple list on a job (sdt_plan_*): host
    indexing and uploads happen once; run() replays the captured CUDA graph
    when capture() was called, else launches.  shapes (one per tuple, 1 or
    2) picks the mixed kernel's work-unit shape per tuple."""

    def __init__(self, job: TriplesJob, klist: np.ndarray, precision: int = PREC_FP64, shapes=None):
        self.job = job
        self._lib = job._lib
        self.klist = np.ascontiguousarray(klist, dtype=np.int64).reshape(-1, 7)
        self.shapes = None if shapes is None else np.ascontiguousarray(shapes, dtype=np.int32)
        if self.shapes is not None and len(self.shapes) != len(self.klist):
            raise ValueError("one work-unit shape per tuple")
        h = C.c_void_p()
        _capi.check(self._lib.sdt_plan_create(
            job._h, self.klist.ctypes.data_as(_capi.PI64), len(self.klist), int(precision),
            None if self.shapes is None else self.shapes.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(h)),
            "sdt_plan_create")
        self._h = h
        self.precision = int(precision)
        job._plans.add(self)

    @property
    def items(self) -> int:
        return int(self._lib.sdt_plan_items(self._h))

    def item_energies(self) -> np.ndarray:
        """(items, 2) per-item (E[T], E(T)) pairs of the last run."""
        out = np.zeros((self.items, 2))
        _capi.check(self._lib.sdt_plan_item_energies(self._h, out.ctypes.data_as(_capi.PD), self.items),
                    "sdt_plan_item_energies")
        return out

    def capture(self, stream=None) -> None:
        _capi.check(self._lib.sdt_plan_capture(self._h, _stream_ptr(stream)), "sdt_plan_capture")

    def launch(self, stream=None) -> None:
        _capi.check(self._lib.sdt_plan_launch(self._h, _stream_ptr(stream)), "sdt_plan_launch")

    def run(self, stream=None, per_task: bool = False):
        e = np.zeros(2)
        pt = np.zeros((len(self.klist), 2)) if per_task else None
        _capi.check(self._lib.sdt_plan_run(self._h, _stream_ptr(stream), e.ctypes.data_as(_capi.PD),
                                           pt.ctypes.data_as(_capi.PD) if per_task else None), "sdt_plan_run")
        return (float(e[0]), float(e[1]), pt) if per_task else (float(e[0]), float(e[1]))

    def close(self) -> None:
        if self._h:
            self._lib.sdt_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
