#!/usr/bin/env python3
"""Throughput of the (T) triples tile path on GB300.

Workload: the tiled FP64 drop-in problem o=40 (tiles 8/12/20), v=300 (tiles
20,24x5,30x4,40), seeded synthetic T1/T2/V2 (seed 1).  Its weight-ordered
tuple list (2860 tuples, 9.43e14 algorithmic FLOPs) is cut into 256 strided
slices; one step evaluates one slice (about 11 tuples, ~3.7e12 FLOPs) -- all
27 tile kernels per tuple and the energy sum.  Steps rotate through slices.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--extras all|none|o64,serve,mol]

value: algorithmic TFLOP/s with the inputs resident in HBM (CUDA events on
the launching stream, max over ranks).  e2e: the same metric through the
public API with the TCE files copied from pinned host memory and the
energies read back every step (two jobs double-buffer the inputs, so step
s+1's copies and ingest overlap step s's kernels).

--impl reference times the CPU restatement of the reference's (T) kernels
and drivers (the oracle, oracle/) on all host cores, without loading the
product library: per step a seeded uniform sample of 2 tuples of that
step's slice (the same slice the GPU step evaluates), the same config.  The
GPU line reports its own FP64 throughput on exactly those sampled tuples
too ("same_sample"), and its cpu_baseline times the oracle on them.

The default run also reports (--extras): the mixed forms on the same steps
with absolute errors; the o=64/v=512 workload (FP64 on one seeded tuple,
each mixed form on 48 tuples, segmented drains); a molecular-magnitude case
(the o=40/v=300 inputs scaled so one step's |E(T)| is 0.05 Eh); and a
serving stream through the shared work queue.  On one GB300 the default
run takes about ten minutes: the 20 timed FP64 steps ~85 s, the o=64/v=512
FP64 tuple ~82 s, the serving stream's two deferred FP64 checks ~2 min.
Multi-GPU: each rank takes its own slices (weak scaling, no collective on
the data path); energies are summed on the host.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_SLICES = 256
SEED = 1
CPU_TUPLES = 2            # tuples of each step's slice the reference arm evaluates
WORKLOAD = ("o40v300 tiled FP64 drop-in: o=40 as 8/12/20, v=300 as 20,24x5,30x4,40, seed 1; "
            "step = one of 256 strided slices of the 2860-tuple weight-ordered list")
METRIC = "(T) TFLOP/s"
CONFIG = {"workload": WORKLOAD, "form": "fp64"}
# DRAM bytes per algorithmic FLOP of fused_fp64_kernel: ncu dram__bytes_read.sum +
# dram__bytes_write.sum (327.9 MB + 26.2 MB) over one launch on 2 tuples of the
# o=40/v=114 case (2.587e11 FLOPs)
FP64_DRAM_BYTES_PER_FLOP = (327.9e6 + 26.2e6) / 2.587e11
MIXED_FORMS = (("tf32", 1), ("bf16", 2), ("fp16", 3))
MIXED_NOTE = {"tf32": "TF32x3: TF32 hi/lo pairs, kind::tf32", "bf16": "BF16x3: bf16 hi/lo pairs, kind::f16",
              "fp16": "FP16x3: fp16 hi/lo pairs of power-of-two scaled operands, kind::f16",
              "all": "FP32 accumulation in TMEM; s1 products, denominator and quotient FP32 "
                     "(orbital energies shifted to the gap midpoint); energy sums FP64"}
MOLECULAR_EH = 0.05       # |E(T)| of a mid-sized molecule, for the absolute-error bound


def _slices(n_tasks: int) -> list[np.ndarray]:
    return [np.arange(s, n_tasks, N_SLICES) for s in range(N_SLICES)]


def ref_sample(slice_ids: np.ndarray, step: int, flops_of=None, cap: float | None = None) -> np.ndarray:
    """The reference arm's tuples for a step: a seeded uniform draw of
    CPU_TUPLES tuples of the step's slice (all sizes equally likely).  cap
    (tests only) restricts the draw to tuples of at most that many FLOPs."""
    ids = np.asarray(slice_ids)
    if cap is not None:
        ids = np.array([i for i in ids if flops_of(int(i)) <= cap] or [min(ids, key=lambda i: flops_of(int(i)))])
    rng = np.random.default_rng(7919 + step)
    k = min(CPU_TUPLES, len(ids))
    return np.sort(rng.choice(ids, k, replace=False)).astype(np.int64)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while active."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.proc, self.path = index, None, None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[3:7]):
                if val.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _oracle_workload():
    """The o=40/v=300 workload on the checker side (no product library)."""
    from oracle import oracle as orc
    t = orc.config_tiling(1)
    files = orc.synth_inputs(t, SEED)
    P = orc.Problem(t, *files)
    return orc, t, files, P, P.task_list()


def reference_arm(args) -> None:
    ws, rank, _ = _dist()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    orc, t, files, P, kl = _oracle_workload()
    sl = _slices(len(kl))
    cap = float(os.environ["SDT_CPU_FLOP_CAP"]) if "SDT_CPU_FLOP_CAP" in os.environ else None
    flops_of = lambda i: orc.flops(t, kl[i:i + 1])
    times, flops = [], []
    for s in range(args.warmup + args.steps):
        ids = ref_sample(sl[s % N_SLICES], s, flops_of, cap)
        t0 = time.perf_counter()
        P.ccsd_t(kl, task_ids=ids)
        dt = time.perf_counter() - t0
        if s >= args.warmup:
            times.append(dt)
            flops.append(orc.flops(t, kl[ids]))
    value = sum(flops) / sum(times) / 1e12
    sample = (f"per step {CPU_TUPLES} tuples drawn uniformly (seed 7919+step) from the step's slice; "
              f"{sum(flops):.3e} FLOPs in {sum(times):.1f} s; C/OpenMP restatement of ccsd_t_kernels_omp.F + drivers")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded; distributions of the o=40/v=300 workload)", "config": dict(CONFIG),
            "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _measured_bf16() -> tuple[float, str]:
    path = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(path.read_text())["bf16_tflops"]), "MEASURED_PEAKS.json bf16_tflops (burst)"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback 1.9 PFLOP/s bf16 (no MEASURED_PEAKS.json)"


def _errors(m, f) -> dict:
    """Errors of a mixed (E[T], E(T)) against the FP64 pair: absolute (Eh)
    and relative for E[T], E(T) and E[ST] = E(T) - E[T]; the absolute error
    of E(T) at molecular magnitude (|E(T)| = 0.05 Eh, same relative error)."""
    est_m, est_f = m[1] - m[0], f[1] - f[0]
    rel_t = abs(m[1] - f[1]) / abs(f[1]) if f[1] else None
    return {"abs_Eh": {"E[T]": abs(m[0] - f[0]), "E(T)": abs(m[1] - f[1]), "E[ST]": abs(est_m - est_f)},
            "rel": {"E[T]": abs(m[0] - f[0]) / abs(f[0]) if f[0] else None, "E(T)": rel_t,
                    "E[ST]": abs(est_m - est_f) / abs(est_f) if est_f else None},
            "E(T)_at_0.05Eh_uEh": rel_t * MOLECULAR_EH * 1e6 if rel_t is not None else None}


def extra_reference_gpu(ng, t, files, kl, samples, job) -> dict:
    """NWChem's own CUDA tile path (sd_t_total.cu, built for sm_103a) on the
    reference arm's sampled tuples: per tuple the reference driver logic on
    the host (fetch, sort) and the reference's sd_t_*_cuda_ kernels and
    compute_en_ on the GPU; wall time per tuple, and each tuple's energies
    against this library's FP64 form."""
    from oracle import oracle as orc
    from oracle import ref_cuda
    if not ref_cuda.staged():
        return {"unavailable": "the reference CUDA sources were not staged into oracle/_ref/cuda/ with the build"}
    try:
        t0 = time.perf_counter()
        runner = ref_cuda.TileRunner()
        build_s = time.perf_counter() - t0
    except (OSError, RuntimeError) as e:
        return {"unavailable": f"reference CUDA build failed: {str(e)[-300:]}"}
    P = orc.Problem(t, *files)
    ids = np.concatenate(list(samples))
    runner.tuple_energy(P, [int(x) for x in kl[ids[0], :6]])          # warm-up (pool, module load)
    wall, fl, rel = 0.0, 0.0, 0.0
    ours_pt = job.run(kl[ids], per_task=True)[2]
    for q, i in enumerate(ids):
        tup = [int(x) for x in kl[i, :6]]
        t0 = time.perf_counter()
        e = runner.tuple_energy(P, tup)
        wall += time.perf_counter() - t0
        fl += ng.flops(t, kl[i:i + 1])
        rel = max(rel, float(np.max(np.abs(e - ours_pt[q]) / np.abs(ours_pt[q]))))
    runner.close()
    return {"value": fl / wall / 1e12, "unit": "TFLOP/s", "tuples": int(len(ids)), "flops": fl, "wall_s": wall,
            "build_s": build_s, "max_rel_diff_vs_this_fp64_per_tuple": rel,
            "what": "src/tce/ccsd_t/sd_t_total.cu + memory.cu (FP64 SIMT kernels) compiled with nvcc for sm_103a, "
                    "driven per tuple like ccsd_t_gpu.F: host fetch/sort of every sub-block, H2D copy, kernel, "
                    "compute_en_; the oracle's host driver stands in for the Fortran driver"}


def extra_molecular(ng, t, kl, ids, e_nat) -> dict:
    """One step of the o=40/v=300 workload with every input scaled so that
    the step's |E(T)| is 0.05 Eh: FP64 and each mixed form, absolute errors."""
    s = ng.molecular_scale(e_nat[1], MOLECULAR_EH)
    out = {"case": "o40v300 step 0 slice, inputs x %.6g so |E(T)| = %.3g Eh" % (s, MOLECULAR_EH)}
    with ng.TriplesJob(t) as job:
        job.load(*ng.synth_inputs(t, SEED, scale=s))
        f = job.run(kl[ids])
        out["fp64_E"] = list(f)
        out["fp64_vs_scaled_natural_rel"] = abs(f[1] - e_nat[1] * s ** 4) / abs(f[1])
        for form, prec in MIXED_FORMS:
            m = job.run(kl[ids], precision=prec)
            err = _errors(m, f)
            out[form] = {"E": list(m), "abs_uEh": {k: v * 1e6 for k, v in err["abs_Eh"].items()}}
    return out


def extra_o64v512(ng, stream, bf16) -> dict:
    """o=64 (2x32), v=512 (8x64), seed 2: FP64 on one seeded tuple (8.6e9
    triples elements, 8.9e13 FLOPs), each mixed form on 48 strided tuples of
    the 480 (that tuple among them) with its error against the FP64 tuple,
    and FP16x3 with segmented drains."""
    t = ng.config_tiling(2)
    kl = ng.task_list(t)
    batch = kl[np.arange(0, len(kl), 10)]
    pick = int(np.random.default_rng(2).integers(len(batch)))
    one = batch[pick:pick + 1]
    fl_one, fl_batch = ng.flops(t, one), ng.flops(t, batch)
    t0 = time.perf_counter()
    files = ng.synth_inputs(t, 2)
    out = {"workload": "o64v512: o=64 as 2x32, v=512 as 8x64, seed 2", "fp64_tuple": [int(x) for x in one[0, :6]],
           "batch_tuples": int(len(batch)), "batch_flops": fl_batch, "input_generation_s": time.perf_counter() - t0}
    peak = None
    with ng.TriplesJob(t) as job:
        t0 = time.perf_counter()
        job.load(*files, stream=stream)
        stream.synchronize()
        out["load_s"] = time.perf_counter() - t0
        del files
        job.set_timing(True)
        f = job.run(one, stream=stream)
        fp64_tf = fl_one / job.last_kernel_ms / 1e9
        peak = ng.lib().sdt_probe_fp64_tflops(200)
        out["fp64"] = {"E": list(f), "tflops": fp64_tf, "kernel_s": job.last_kernel_ms / 1e3, "peak": peak,
                       "frac_of_fp64_peak": fp64_tf / peak if peak > 0 else None}
        for form, prec in MIXED_FORMS:
            job.run(one, stream=stream, precision=prec)           # encodes the split operands
            e1, e2, pt = job.run(batch, stream=stream, precision=prec, per_task=True)
            tf = fl_batch / job.last_kernel_ms / 1e9
            ceiling = bf16[0] / (6.0 if form == "tf32" else 3.0)
            out[form] = {"tflops": tf, "kernel_s": job.last_kernel_ms / 1e3, "speedup_vs_fp64": tf / fp64_tf,
                         "frac_of_bf16_peak": tf / bf16[0], "frac_of_split_ceiling": tf / ceiling,
                         "errors_vs_fp64_tuple": _errors(tuple(pt[pick]), f)}
        seg = {}
        job.run(one, stream=stream, precision=3)
        for kseg in (8, 4, 2):
            job.set_mixed_segment(kseg)
            e1, e2, pt = job.run(batch, stream=stream, precision=3, per_task=True)
            seg[str(kseg)] = {"tflops": fl_batch / job.last_kernel_ms / 1e9,
                              "rel_err_E(T)": _errors(tuple(pt[pick]), f)["rel"]["E(T)"]}
        job.set_mixed_segment(0)
        seg["0"] = {"tflops": out["fp16"]["tflops"], "rel_err_E(T)": out["fp16"]["errors_vs_fp64_tuple"]["rel"]["E(T)"]}
        out["fp16_segmented_drains"] = seg
        out["device_bytes"] = job.device_bytes
    out["bf16_peak"] = bf16[0]
    return out


def serve_stream(ng, jobs: int, rate: float, omin: int, omax: int, slots: int, check_every: int,
                 max_ctas: int = 0, queue: bool = True, reserve: int = 16) -> dict:
    """Serving stream: Poisson arrivals at `rate` jobs/s, o ~ U{omin..omax},
    v = round(o * U[5,8]), tiles from {8..32} / {16..64} (no irreps), inputs
    seeded with the job id; FIFO admission against a 150 GB HBM budget with
    `slots` jobs in flight; the mixed form (FP16x3) on every job through the
    shared work queue drained by the resident kernel (or, queue off, one
    launch per job), the FP64 form as a check on every check_every-th job.
    Inputs are generated before the stream starts; a job's latency runs from
    its arrival (submission) to its energies; the phase times split it into
    queueing, loading (tables, copies, ingest, encoding, plan) and computing
    (queue wait, kernels, sums)."""
    from nwchem_gb300 import serve
    specs = serve.job_stream(jobs, rate, 4, omin, omax)
    t0 = time.perf_counter()
    files = serve.prepare(specs)
    gen_s = time.perf_counter() - t0
    prec = ng.PREC_MIXED_FP16
    budget = 150 * 10**9
    check = [check_every > 0 and s.id % check_every == 0 for s in specs]
    with serve.Server(budget, slots=slots, max_ctas=max_ctas, queue=prec if queue else None,
                      reserve=reserve) as srv:
        w = srv.submit(specs[0].tiling, files[0], prec)       # warm-up job, not counted
        srv.drain(600)
        srv.status(w)
        t_start = time.perf_counter()
        tickets = []
        for s, f, c in zip(specs, files, check):
            delay = s.arrival - (time.perf_counter() - t_start)
            if delay > 0:
                time.sleep(delay)
            tickets.append(srv.submit(s.tiling, f, prec, check_fp64=c))
        srv.drain(3600)
        st = [srv.status(t) for t in tickets]
        gens = [srv.launches(t) for t in tickets]
        qs = srv.queue_stats()
        peak = srv.peak_bytes
    ok = [x for x in st if x["state"] == 2]
    lat = np.array([x["ran"] - x["submitted"] for x in ok])      # arrival to energies
    phase = {k: np.array([x[b] - x[a] for x in ok]) for k, a, b in (
        ("queue", "submitted", "admitted"), ("load", "admitted", "loaded"), ("compute", "loaded", "ran"),
        ("service", "admitted", "ran"))}
    span = max(x["ran"] for x in ok) - min(x["submitted"] for x in ok)
    t_first = min(x["submitted"] for x in ok)
    checks_done = [x["finished"] - t_first for x, c in zip(st, check) if c and x["state"] == 2]
    flops = sum(ng.flops(s.tiling, ng.task_list(s.tiling)) for s, x in zip(specs, st) if x["state"] == 2)
    chk = [x for x, c in zip(st, check) if c and x["state"] == 2]
    errs = [abs(x["energy"][1] - x["fp64"][1]) / abs(x["fp64"][1]) for x in chk if x["fp64"][1] != 0.0]
    aerr = [abs(x["energy"][1] - x["fp64"][1]) for x in chk]
    worst = int(np.argmax([x["ran"] - x["submitted"] if x["state"] == 2 else -1 for x in st]))
    wx = st[worst]
    worst_job = {"id": specs[worst].id, "o": specs[worst].tiling.nocc, "v": specs[worst].tiling.nvir,
                 "checked": bool(check[worst]), "launches": list(gens[worst]),
                 **{k: wx[b] - wx[a] for k, a, b in (("queue", "submitted", "admitted"), ("load", "admitted", "loaded"),
                                                     ("compute", "loaded", "ran"))}}
    shared = {}
    for a, b in gens:
        if a > 0 and a == b:
            shared[a] = shared.get(a, 0) + 1
    return {
        "workload": f"serving: {jobs} jobs, Poisson {rate:g} jobs/s, o ~ U{{{omin}..{omax}}}, "
                    f"v = round(o*U[5,8]), tiles {{8..32}}/{{16..64}}, seed = job id",
        "continuous_batching": queue, "slots": slots, "reserve_sms": reserve if queue else None,
        "budget_bytes": budget, "peak_admitted_bytes": peak,
        "jobs_done": len(ok), "jobs_failed": len(st) - len(ok),
        "jobs_per_s": len(ok) / span, "span_s": span, "p50_latency_s": float(np.percentile(lat, 50)),
        "p99_latency_s": float(np.percentile(lat, 99)), "mean_latency_s": float(lat.mean()),
        "offered_jobs_per_s": len(specs) / specs[-1].arrival,
        "phase_p50_s": {k: float(np.percentile(v, 50)) for k, v in phase.items()},
        "phase_p99_s": {k: float(np.percentile(v, 99)) for k, v in phase.items()},
        "tflops": flops / span / 1e12, "fp64_checked": len(chk), "fp64_checks_done_at_s": checks_done,
        "queue": {**qs, "most_jobs_finished_in_one_launch": max(shared.values()) if shared else 0},
        "slowest_job": worst_job,
        "max_rel_err_E(T)_vs_fp64": max(errs) if errs else None,
        "max_abs_err_E(T)_vs_fp64_Eh": max(aerr) if aerr else None,
        "input_generation_s": gen_s}


def ours(args) -> None:  # noqa: C901
    import torch
    import torch.distributed as dist

    import nwchem_gb300 as ng
    from nwchem_gb300 import _capi

    ws, rank, local = _dist()
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _capi.lib()
    lib.sdt_set_error_mode(1)
    extras = set() if args.extras == "none" else (
        {"o64", "serve", "mol", "refgpu"} if args.extras == "all" else set(args.extras.split(",")))
    if ws > 1:
        extras = set()

    t = ng.config_tiling(1)
    kl = ng.task_list(t)
    sl = _slices(len(kl))
    files = ng.synth_inputs(t, SEED, pinned=True)
    in_bytes = sum(f.nbytes for f in files)
    nstep = args.warmup + args.steps
    step_ids = [sl[(s * ws + rank) % N_SLICES] for s in range(nstep)]
    step_flops = [ng.flops(t, kl[ids]) for ids in step_ids]

    stream = torch.cuda.Stream(device=dev)
    job = ng.TriplesJob(t)
    job.load(*files, stream=stream)
    job.set_timing(True)
    dev_bytes = job.device_bytes

    def barrier():
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    def max_sum(x: float, y: float) -> tuple[float, float]:
        if ws == 1:
            return x, y
        tt = torch.tensor([x, y], dtype=torch.float64, device=dev)
        mx = tt.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        dist.all_reduce(tt, op=dist.ReduceOp.SUM)
        return float(mx[0]), float(tt[1])

    energies = []
    for s in range(args.warmup):
        job.run(kl[step_ids[s]], stream=stream)
    peak = lib.sdt_probe_fp64_tflops(200)

    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    launches0 = lib.sdt_launch_count()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    kern_ms = []
    ev0.record(stream)
    for s in range(args.warmup, nstep):
        e = job.run(kl[step_ids[s]], stream=stream)
        kern_ms.append(job.last_kernel_ms)
        energies.append(e)
    ev1.record(stream)
    barrier()
    launches = lib.sdt_launch_count() - launches0
    clocks = sampler.stop()
    my_flops = sum(step_flops[args.warmup:])
    elapsed, total_flops = max_sum(ev0.elapsed_time(ev1) / 1e3, my_flops)
    value = total_flops / elapsed / 1e12
    kern_avg_s = sum(kern_ms) / len(kern_ms) / 1e3
    achieved = (my_flops / args.steps) / kern_avg_s / 1e12

    # End to end through the public API: pinned-host TCE files -> device,
    # ingest, run, energies back, every step.  Two jobs on two streams
    # double-buffer the inputs: while one job runs step s, a host thread
    # loads step s+1's files into the other (the copies overlap the
    # contraction kernel; the first step's load is not hidden).
    e2e_steps = min(args.steps, 5)
    job2 = ng.TriplesJob(t)
    jobs, streams = (job, job2), (stream, torch.cuda.Stream(device=dev))
    load_s = []

    def load(k):
        tl = time.perf_counter()
        jobs[k].load(*files, stream=streams[k])      # returns once the ingest is done
        load_s.append(time.perf_counter() - tl)

    barrier()
    t0 = time.perf_counter()
    e2e_flops = 0.0
    load(0)
    for s in range(e2e_steps):
        ids = step_ids[args.warmup + s]
        nxt = None
        if s + 1 < e2e_steps:
            nxt = threading.Thread(target=load, args=((s + 1) % 2,))
            nxt.start()
        jobs[s % 2].run(kl[ids], stream=streams[s % 2])
        if nxt is not None:
            nxt.join()
        e2e_flops += step_flops[args.warmup + s]
    barrier()
    e2e_t, e2e_flops = max_sum(time.perf_counter() - t0, e2e_flops)
    job2.close()
    e2e = e2e_flops / e2e_t / 1e12

    # The reference arm's sampled tuples of every step, on the GPU (FP64).
    samp = [ref_sample(sl[s % N_SLICES], s) for s in range(nstep)] if rank == 0 else []
    same = None
    if rank == 0:
        ms, fl = 0.0, 0.0
        for s in range(args.warmup, nstep):
            job.run(kl[samp[s]], stream=stream)
            ms += job.last_kernel_ms
            fl += ng.flops(t, kl[samp[s]])
        same = {"value": fl / ms / 1e9, "unit": "TFLOP/s", "tuples": int(sum(len(samp[s]) for s in range(args.warmup, nstep))),
                "flops": fl, "note": "FP64 kernel time on the tuples the reference arm samples (the same steps)"}

    # Mixed forms (split products on the tensor cores) on the same steps.
    bf16 = _measured_bf16()
    mixed = {}
    for form, prec in MIXED_FORMS:
        job.run(kl[step_ids[0]], stream=stream, precision=prec)   # builds the split operands
        barrier()
        ev0.record(stream)
        mixed_e, mixed_ms = [], []
        for s in range(args.warmup, nstep):
            mixed_e.append(job.run(kl[step_ids[s]], stream=stream, precision=prec))
            mixed_ms.append(job.last_kernel_ms)
        ev1.record(stream)
        barrier()
        mixed_t, _ = max_sum(ev0.elapsed_time(ev1) / 1e3, 0.0)
        mv = total_flops / mixed_t / 1e12
        ach = (my_flops / args.steps) / (sum(mixed_ms) / len(mixed_ms) / 1e3) / 1e12
        per_step = [_errors(m, f) for m, f in zip(mixed_e, energies)]
        total = _errors((sum(m[0] for m in mixed_e), sum(m[1] for m in mixed_e)),
                        (sum(f[0] for f in energies), sum(f[1] for f in energies)))
        ceiling = bf16[0] / (6.0 if form == "tf32" else 3.0)
        mixed[form] = {
            "value": mv, "unit": "TFLOP/s", "speedup_vs_fp64": mv / value,
            "errors_all_steps": total,
            "max_rel_err_E(T)_per_step": max(e["rel"]["E(T)"] for e in per_step),
            "max_abs_err_E(T)_per_step_Eh": max(e["abs_Eh"]["E(T)"] for e in per_step),
            "roofline": {"bound": "tensor", "achieved": ach, "peak": bf16[0], "unit": "TFLOP/s",
                         "frac": ach / bf16[0], "peak_source": bf16[1], "split_ceiling": ceiling,
                         "frac_of_split_ceiling": ach / ceiling},
        }

    cpu = None
    extra = {}
    if rank == 0 and "refgpu" in extras:
        extra["reference_gpu"] = extra_reference_gpu(ng, t, files, kl, samp[args.warmup:args.warmup + 3], job)
    job.close()
    if rank == 0 and ws == 1 and not args.no_cpu:
        from oracle import oracle as orc
        cores = os.cpu_count() or 1
        P = orc.Problem(t, *files)
        ids = np.concatenate([samp[args.warmup + s] for s in range(min(2, args.steps))])
        t0 = time.perf_counter()
        P.ccsd_t(kl, task_ids=ids)
        dt = time.perf_counter() - t0
        f = ng.flops(t, kl[ids])
        cpu = {"value": f / dt / 1e12, "unit": "TFLOP/s", "cores": cores, "kind": "port",
               "sample": f"the reference arm's sampled tuples of the first {min(2, args.steps)} timed steps "
                         f"({len(ids)} tuples, {f:.3e} FLOPs, {dt:.1f} s); C/OpenMP restatement of "
                         "ccsd_t_kernels_omp.F + drivers"}
        del P

    if rank == 0 and "mol" in extras:
        extra["molecular_scale"] = extra_molecular(ng, t, kl, step_ids[args.warmup], energies[0])
    files = None                       # the o=64/v=512 inputs need the host memory
    if rank == 0 and "o64" in extras:
        extra["o64v512"] = extra_o64v512(ng, stream, bf16)
    if rank == 0 and "serve" in extras:
        extra["serving"] = serve_stream(ng, args.jobs, args.rate, args.omin, args.omax, args.slots,
                                        args.check_every)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded; distributions of the o=40/v=300 workload)",
            "config": dict(CONFIG),
            "workload_detail": {"tuples_per_step": float(np.mean([len(x) for x in step_ids[args.warmup:]])),
                                "flops_per_step": my_flops / args.steps,
                                "cache": f"inputs larger than L2 ({dev_bytes / 1e9:.1f} GB resident operands)",
                                "E[T]_E(T)_last_step": list(energies[-1])},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak if peak > 0 else None,
                         "traffic": FP64_DRAM_BYTES_PER_FLOP * my_flops / args.steps,
                         "traffic_note": "dram read+write bytes per launch, scaled by FLOPs from the ncu capture "
                                         "of the 2-tuple o40v114 case (354 MB for 2.587e11 FLOPs; operands stay "
                                         "L2-resident, so traffic grows with the work, not with reuse)",
                         "peak_source": "measured in-run: FP64 mma.sync m8n8k4 probe (no FP64 entry in "
                                        "MEASURED_PEAKS.json)",
                         "kernel": "fused_fp64_kernel"},
            "cpu_baseline": cpu,
            "same_sample": same,
            "e2e": {"value": e2e, "unit": "TFLOP/s", "h2d_bytes_per_step": int(in_bytes),
                    "d2h_bytes_per_step": 16, "steps": e2e_steps, "load_s": [round(x, 4) for x in load_s],
                    "overlap": "step s+1's files copied and ingested into a second job on its own stream "
                               "while step s runs"},
            "gpu_launches": int(launches),
            "clocks": clocks,
            "mixed": {
                "forms": MIXED_NOTE, "kernel": "split_fused_kernel", **mixed,
                "note": "algorithmic FLOPs counted once; each product is three MMAs (hi*hi+hi*lo+lo*hi) and "
                        "TF32 runs at half the BF16 rate, so the split ceilings are peak/3 (BF16, FP16) "
                        "and peak/6 (TF32); errors against the FP64 form on the same steps"},
            **extra,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def profile_case(args) -> None:  # noqa: C901
    """Small case for ncu, one warm-up launch then one launch of the fused
    kernel on `--tuples` tuples: --case o40v114 (under 1 GB on the device,
    operands still larger than L2): o=40 as 8/12/20, v=114 as 20,24,30,40,
    seed 1, tuples from the middle of the weight-ordered list; --case o64v128
    (about 4 GB): o=64 as 2x32, v=128 as 2x64, seed 2, the first tuples."""
    import torch

    import nwchem_gb300 as ng
    torch.cuda.set_device(0)
    if args.case == "sym8s":
        # blocked symmetry, small: o=48 as 6x8 (irreps 0..5), v=128 as 8x16 (irreps 0..7), seed 3
        t = ng.Tiling([8] * 6, [16] * 8, occ_sym=list(range(6)), vir_sym=list(range(8)), name="sym8s").with_evl(3)
        files = ng.synth_inputs(t, 3)
        kl = ng.task_list(t)
        sel = kl[:args.tuples]
    elif args.case == "o64v128":
        # whole 8x8x8x4x4x4 sub-boxes, as in the o=64/v=512 workload
        t = ng.Tiling([32, 32], [64, 64], name="o64v128").with_evl(2)
        files = ng.synth_inputs(t, 2)
        kl = ng.task_list(t)
        sel = kl[:args.tuples]
    else:
        t = ng.Tiling([8, 12, 20], [20, 24, 30, 40], name="o40v114").with_evl(SEED)
        kl = ng.task_list(t)
        files = ng.synth_inputs(t, SEED)
        mid = len(kl) // 2
        sel = kl[mid:mid + args.tuples]
    with ng.TriplesJob(t) as job:
        job.load(*files)
        job.set_timing(True)
        job.set_mixed_shape(args.shape)
        prec = dict(MIXED_FORMS).get(args.mixed, ng.PREC_FP64)
        job.run(sel, precision=prec)
        e = job.run(sel, precision=prec)
        print(json.dumps({"profile_case": args.case, "form": args.mixed or "fp64", "shape": args.shape,
                          "tuples": int(len(sel)),
                          "flops": ng.flops(t, sel),
                          "kernel_ms": job.last_kernel_ms, "device_bytes": job.device_bytes,
                          "tflops": ng.flops(t, sel) / job.last_kernel_ms / 1e9, "energies": list(e)}),
              flush=True)


def workload_o10v40(args) -> None:
    """o=10, v=40, one tile each, seed 0 (one tuple, 5.875e10 FLOPs): the FP64
    form and each mixed form on the GPU (kernel time, average of 5 runs after
    a warm-up), the oracle on all host cores over the whole problem, and each
    result against the oracle's energies, at natural and molecular scale."""
    import torch

    import nwchem_gb300 as ng
    from oracle import oracle as orc
    torch.cuda.set_device(0)
    t = ng.config_tiling(0)
    kl = ng.task_list(t)
    fl = ng.flops(t, kl)
    out = {"workload": "o10v40: o=10, v=40, one tile each, seed 0", "tuples": int(len(kl)), "flops": fl}
    o_nat = None
    for label, scale in (("natural", 1.0), ("molecular", None)):
        if scale is None:
            scale = ng.molecular_scale(o_nat[1], MOLECULAR_EH)
        files = ng.synth_inputs(t, 0, scale=scale)
        t0 = time.perf_counter()
        o1, o2, _, _ = orc.Problem(t, *files).ccsd_t()
        cpu_s = time.perf_counter() - t0
        o_nat = o_nat or (o1, o2)
        res = {"scale": scale, "oracle": {"E": [o1, o2], "s": cpu_s, "tflops": fl / cpu_s / 1e12,
                                          "cores": os.cpu_count()}}
        with ng.TriplesJob(t) as job:
            job.load(*files)
            job.set_timing(True)
            for form, prec in [("fp64", ng.PREC_FP64)] + list(MIXED_FORMS):
                e = job.run(kl, precision=prec)
                ms = []
                for _ in range(5):
                    e = job.run(kl, precision=prec)
                    ms.append(job.last_kernel_ms)
                res[form] = {"E": list(e), "kernel_ms": float(np.mean(ms)), "tflops": fl / np.mean(ms) / 1e9,
                             "errors_vs_oracle": _errors(e, (o1, o2))}
        out[label] = res
    print(json.dumps(out), flush=True)


def workload_o64v512(args) -> None:
    import torch

    import nwchem_gb300 as ng
    torch.cuda.set_device(0)
    print(json.dumps(extra_o64v512(ng, torch.cuda.Stream(), _measured_bf16())), flush=True)


def workload_sym8(args) -> None:
    """Blocked spatial symmetry (8 irreps; o=148 as 8 tiles of 8-32, v=336 as
    12 tiles of 16-64, seed 3): the first 4096 tuples of the weight order in
    one plan -- the autotuner's split form and per-size-class work-unit
    shapes, one persistent launch per shape drawing from a device queue,
    captured as a CUDA graph and replayed; the FP64 form on the whole list
    (--fp64-all, ~15 min) or on a seeded sample of 16 tuples, for the error."""
    import torch

    import nwchem_gb300 as ng
    from nwchem_gb300 import autotune
    torch.cuda.set_device(0)
    t = ng.config_tiling(3)
    kl = ng.task_list(t)[:4096]
    t0 = time.perf_counter()
    files = ng.synth_inputs(t, 3)
    gen_s = time.perf_counter() - t0
    samp = np.arange(len(kl)) if args.fp64_all else np.sort(np.random.default_rng(0).choice(len(kl), 16, replace=False))
    stream = torch.cuda.Stream()
    fl_all, fl_s = ng.flops(t, kl), ng.flops(t, kl[samp])
    out = {"workload": f"{t.name}: 8 irreps, occupied tiles {t.occ}, virtual tiles {t.vir}, seed 3, "
                       f"first 4096 of {len(ng.task_list(t))} tuples", "flops": fl_all}
    with ng.TriplesJob(t) as job:
        t0 = time.perf_counter()
        job.load(*files, stream=stream)
        stream.synchronize()
        out["load_s"] = time.perf_counter() - t0
        job.set_timing(True)
        f = job.run(kl[samp], stream=stream, per_task=True)
        out["fp64"] = {"tuples": int(len(samp)), "tflops": fl_s / job.last_kernel_ms / 1e9,
                       "kernel_s": job.last_kernel_ms / 1e3, "E": list(f[:2])}
        t0 = time.perf_counter()
        tuner = autotune.Autotuner(job, forms=("fp16", "tf32"), sample=4)
        plan, d = tuner.plan(kl, capture=True, stream=stream)
        out["autotune"] = {"s": time.perf_counter() - t0, "form": d["form"], "shapes": d["shapes"],
                           "classes": len(d["shapes"])}
        with plan:
            plan.run(stream=stream)                      # warm-up replay
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            reps = max(1, min(args.steps, 3))
            for _ in range(reps):
                e = plan.run(stream=stream)
            ev1.record(stream)
            stream.synchronize()
            g_s = ev0.elapsed_time(ev1) / 1e3 / reps
            out["mixed_graph"] = {"form": d["form"], "tflops": fl_all / g_s / 1e12, "s_per_run": g_s, "E": list(e),
                                  "items": plan.items}
        for form, prec in (("fp16", 3), ("tf32", 1)):
            m = job.run(kl[samp], stream=stream, per_task=True, precision=prec)
            out[f"{form}_errors_vs_fp64"] = _errors(m[:2], f[:2])
            tf = fl_s / job.last_kernel_ms / 1e9
            out[f"{form}_tflops_on_fp64_tuples"] = tf
        t0 = time.perf_counter()
        job.run(kl, stream=stream, precision=autotune.FORMS[d["form"]])   # one-shot path (plan built and freed)
        out["mixed_one_shot_s"] = time.perf_counter() - t0
        out["device_bytes"] = job.device_bytes
    out["input_generation_s"] = gen_s
    print(json.dumps(out), flush=True)


def workload_serve(args) -> None:
    import torch

    import nwchem_gb300 as ng
    torch.cuda.set_device(0)
    print(json.dumps(serve_stream(ng, args.jobs, args.rate, args.omin, args.omax, args.slots, args.check_every,
                                  args.max_ctas, queue=not args.no_queue, reserve=args.reserve)), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--extras", default="all", help="all, none, or a comma list of o64,serve,mol")
    ap.add_argument("--profile", action="store_true", help="small single-launch case for ncu")
    ap.add_argument("--tuples", type=int, default=2, help="tuples in the --profile case")
    ap.add_argument("--workload", default="o40v300", choices=["o40v300", "o10v40", "o64v512", "sym8", "serve"])
    ap.add_argument("--fp64-all", action="store_true", help="sym8: the FP64 form on all 4096 tuples")
    ap.add_argument("--jobs", type=int, default=200, help="serve: jobs in the stream")
    ap.add_argument("--rate", type=float, default=50.0, help="serve: Poisson arrival rate (jobs/s)")
    ap.add_argument("--omin", type=int, default=8, help="serve: smallest occupied size")
    ap.add_argument("--omax", type=int, default=16, help="serve: largest occupied size")
    ap.add_argument("--slots", type=int, default=8, help="serve: jobs in flight")
    ap.add_argument("--check-every", type=int, default=100, help="serve: FP64 check on every n-th job (0: none)")
    ap.add_argument("--max-ctas", type=int, default=0, help="serve, queue off: CTA cap per job launch (0: all SMs)")
    ap.add_argument("--no-queue", action="store_true", help="serve: one launch per job instead of the shared queue")
    ap.add_argument("--reserve", type=int, default=16, help="serve: SMs the resident kernel leaves free")
    ap.add_argument("--case", default="o40v114", choices=["o40v114", "o64v128", "sym8s"], help="--profile case")
    ap.add_argument("--shape", type=int, default=1, choices=[1, 2], help="mixed work-unit shape")
    ap.add_argument("--mixed", default="", choices=["", "tf32", "bf16", "fp16"],
                    help="--profile case in a mixed form")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.impl == "reference" and args.workload == "o40v300" and not args.profile:
        reference_arm(args)            # the oracle only: the product library is not loaded
        return
    import nwchem_gb300.build as b
    b.build()
    if args.workload == "o10v40":
        workload_o10v40(args)
    elif args.workload == "o64v512":
        workload_o64v512(args)
    elif args.workload == "sym8":
        workload_sym8(args)
    elif args.workload == "serve":
        workload_serve(args)
    elif args.profile:
        profile_case(args)
    else:
        ours(args)


if __name__ == "__main__":
    main()
