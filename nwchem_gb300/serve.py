"""Serving of independent (T) jobs (no reference counterpart): the host side
of sdt_server_* plus the synthetic job stream of the serving workload.

Server keeps each submitted job's tiling and files alive until the job has
finished.  job_stream() draws the workload's jobs: Poisson arrivals at
`rate` jobs/s; per job o ~ U{omin..omax}, v = round(o * U[5,8]); occupied
tiles drawn from {8,12,16,24,32} and virtual tiles from {16,24,32,48,64}
(the last tile of each space trimmed to the total), irreps drawn from
0..nsym-1 (default 1: no spatial symmetry, so every job has tuples);
orbital energies and T1/T2/V2 seeded with the job id.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _capi
from .tiling import Tiling
from .triples import PREC_MIXED_FP16, TceFile, synth_inputs

OCC_SIZES = (8, 12, 16, 24, 32)
VIR_SIZES = (16, 24, 32, 48, 64)


def job_bytes(tiling: Tiling, precision: int) -> int:
    return int(_capi.lib().sdt_job_bytes(C.byref(tiling.struct()), precision))


def simulate(arrival, nbytes, service, budget: int, slots: int):
    """The server's admission policy on the host: (start, end) per job."""
    a = np.ascontiguousarray(arrival, dtype=np.float64)
    b = np.ascontiguousarray(nbytes, dtype=np.int64)
    s = np.ascontiguousarray(service, dtype=np.float64)
    start, end = np.zeros(len(a)), np.zeros(len(a))
    _capi.check(_capi.lib().sdt_admission_simulate(len(a), a.ctypes.data_as(_capi.PD), b.ctypes.data_as(_capi.PI64),
                                                   s.ctypes.data_as(_capi.PD), int(budget), int(slots),
                                                   start.ctypes.data_as(_capi.PD), end.ctypes.data_as(_capi.PD)),
                "sdt_admission_simulate")
    return start, end


def simulate_checks(arrival, nbytes, service, check_service, budget: int, slots: int):
    """The server's policy with deferred FP64 checks on the host: (start,
    ready, done) per job; check_service < 0 means no check."""
    a = np.ascontiguousarray(arrival, dtype=np.float64)
    b = np.ascontiguousarray(nbytes, dtype=np.int64)
    s = np.ascontiguousarray(service, dtype=np.float64)
    c = np.ascontiguousarray(check_service, dtype=np.float64)
    start, ready, done = np.zeros(len(a)), np.zeros(len(a)), np.zeros(len(a))
    P = _capi.PD
    _capi.check(_capi.lib().sdt_serving_simulate(len(a), a.ctypes.data_as(P), b.ctypes.data_as(_capi.PI64),
                                                 s.ctypes.data_as(P), c.ctypes.data_as(P), int(budget), int(slots),
                                                 start.ctypes.data_as(P), ready.ctypes.data_as(P),
                                                 done.ctypes.data_as(P)), "sdt_serving_simulate")
    return start, ready, done


def _split(total: int, sizes, rng) -> list[int]:
    out, left = [], total
    while left > 0:
        x = int(rng.choice(sizes))
        out.append(min(x, left))
        left -= out[-1]
    return out


@dataclass
class JobSpec:
    id: int
    arrival: float
    tiling: Tiling


def job_stream(n: int, rate: float, seed: int, omin: int = 8, omax: int = 80, nsym: int = 1,
               vmin_factor: float = 5.0, vmax_factor: float = 8.0) -> list[JobSpec]:
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for q in range(n):
        t += float(rng.exponential(1.0 / rate))
        o = int(rng.integers(omin, omax + 1))
        v = int(round(o * rng.uniform(vmin_factor, vmax_factor)))
        occ, vir = _split(o, OCC_SIZES, rng), _split(v, VIR_SIZES, rng)
        osym = [int(x) for x in rng.integers(0, nsym, len(occ))]
        vsym = [int(x) for x in rng.integers(0, nsym, len(vir))]
        til = Tiling(occ, vir, occ_sym=osym, vir_sym=vsym, name=f"job{q}").with_evl(q)
        out.append(JobSpec(q, t, til))
    return out


@dataclass
class _Held:
    tiling: Tiling
    files: tuple
    structs: list = field(default_factory=list)


class Server:
    """sdt_server_*: admission against an HBM budget, `slots` jobs in
    flight.  queue: the precision whose jobs go through the shared device
    work queue drained by one resident kernel (continuous batching; None
    turns it off and every job gets its own launches), with work-unit
    `shape`, `reserve` SMs kept free for loading other jobs and `idle` s
    of waiting for work before the kernel leaves."""

    def __init__(self, budget_bytes: int, slots: int = 4, max_ctas: int = 0, check_ctas: int | None = None,
                 queue: int | None = PREC_MIXED_FP16, shape: int = 1, reserve: int = 16, idle: float = 0.2):
        self._lib = _capi.lib()
        h = C.c_void_p()
        _capi.check(self._lib.sdt_server_create(int(budget_bytes), int(slots), int(max_ctas), C.byref(h)),
                    "sdt_server_create")
        self._h = h
        _capi.check(self._lib.sdt_server_set_queue(h, int(queue or 0), int(shape), int(reserve), float(idle)),
                    "sdt_server_set_queue")
        if check_ctas is not None:
            _capi.check(self._lib.sdt_server_set_check_ctas(h, int(check_ctas)), "sdt_server_set_check_ctas")
        self._held: dict[int, _Held] = {}

    def submit(self, tiling: Tiling, files: tuple[TceFile, TceFile, TceFile], precision: int = PREC_MIXED_FP16,
               check_fp64: bool = False) -> int:
        ts = tiling.struct()
        fs = [f.struct() for f in files]
        tk = C.c_int64()
        _capi.check(self._lib.sdt_server_submit(self._h, C.byref(ts), C.byref(fs[0]), C.byref(fs[1]),
                                                C.byref(fs[2]), int(precision), 1 if check_fp64 else 0,
                                                C.byref(tk)), "sdt_server_submit")
        self._held[tk.value] = _Held(tiling, tuple(files), [ts] + fs)
        return tk.value

    def status(self, ticket: int) -> dict:
        st = C.c_int()
        e, f, tm = np.zeros(2), np.zeros(2), np.zeros(5)
        buf = C.create_string_buffer(512)
        rc = self._lib.sdt_server_status(self._h, int(ticket), C.byref(st), e.ctypes.data_as(_capi.PD),
                                         f.ctypes.data_as(_capi.PD), tm.ctypes.data_as(_capi.PD), buf, 512)
        if st.value in (2, -1):
            self._held.pop(ticket, None)
        return {"state": st.value, "rc": rc, "energy": (float(e[0]), float(e[1])), "fp64": (float(f[0]), float(f[1])),
                "submitted": float(tm[0]), "admitted": float(tm[1]), "loaded": float(tm[2]),
                "ran": float(tm[3]), "finished": float(tm[4]),
                "msg": buf.value.decode(errors="replace")}

    def cancel(self, ticket: int) -> None:
        """Cancel a job that is still queued (raises SdtError if it was admitted)."""
        _capi.check(self._lib.sdt_server_cancel(self._h, int(ticket)), "sdt_server_cancel")

    def drain(self, timeout: float = 3600.0) -> None:
        _capi.check(self._lib.sdt_server_drain(self._h, float(timeout)), "sdt_server_drain")

    @property
    def peak_bytes(self) -> int:
        return int(self._lib.sdt_server_peak_bytes(self._h))

    def queue_stats(self) -> dict:
        st = np.zeros(4, dtype=np.int64)
        _capi.check(self._lib.sdt_server_queue_stats(self._h, st.ctypes.data_as(_capi.PI64)), "sdt_server_queue_stats")
        return {"launches": int(st[0]), "jobs": int(st[1]), "max_in_queue": int(st[2]), "in_queue": int(st[3])}

    def launches(self, ticket: int) -> tuple[int, int]:
        """(launch that took the job's first item, launch that finished its last)."""
        a, b = C.c_int(), C.c_int()
        _capi.check(self._lib.sdt_server_job_launches(self._h, int(ticket), C.byref(a), C.byref(b)),
                    "sdt_server_job_launches")
        return a.value, b.value

    def close(self) -> None:
        if self._h:
            self._lib.sdt_server_destroy(self._h)
            self._h = C.c_void_p()
            self._held.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def prepare(specs: list[JobSpec]) -> list[tuple]:
    """The seeded T1/T2/V2 files of each job (seed = job id)."""
    return [synth_inputs(s.tiling, s.id) for s in specs]
