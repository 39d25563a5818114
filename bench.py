#!/usr/bin/env python3
"""Throughput of the (T) triples tile path on GB300.

Workload: the tiled FP64 drop-in problem o=40 (tiles 8/12/20), v=300 (tiles
20,24x5,30x4,40), seeded synthetic T1/T2/V2 (seed 1).  Its weight-ordered
tuple list (2860 tuples, 9.43e14 algorithmic FLOPs) is cut into 128 strided
slices; one step evaluates one slice (about 22 tuples, ~7e12 FLOPs) -- all
27 tile kernels per tuple and the energy sum.  Steps rotate through slices.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value: algorithmic TFLOP/s with the inputs resident in HBM (CUDA events on
the launching stream, max over ranks).  e2e: the same metric through the
public API with the TCE files copied from pinned host memory and the
energies read back every step.  --impl reference times the CPU restatement
of the reference's (T) kernels and drivers (the oracle) on the host cores.
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

N_SLICES = 128
SEED = 1
WORKLOAD = ("o40v300 tiled FP64 drop-in: o=40 as 8/12/20, v=300 as 20,24x5,30x4,40, seed 1; "
            "step = one of 128 strided slices of the 2860-tuple weight-ordered list")
METRIC = "(T) TFLOP/s"


def _slices(n_tasks: int) -> list[np.ndarray]:
    return [np.arange(s, n_tasks, N_SLICES) for s in range(N_SLICES)]


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


def cpu_sample(tiling, files, klist, slice_ids, target_flops: float):
    """Tuples of a slice (smallest first) until target_flops, for the CPU leg."""
    import nwchem_gb300 as ng
    fl = np.array([ng.flops(tiling, klist[i:i + 1]) for i in slice_ids])
    order = np.argsort(fl)
    chosen, acc = [], 0.0
    for k in order:
        if acc >= target_flops:
            break
        chosen.append(int(slice_ids[k]))
        acc += fl[k]
    return np.array(sorted(chosen), dtype=np.int64), acc


def run_cpu(tiling, files, klist, ids) -> float:
    from oracle import oracle as orc
    P = orc.Problem(tiling, *files)
    t0 = time.perf_counter()
    P.ccsd_t(klist, task_ids=ids)
    return time.perf_counter() - t0


def reference_arm(args) -> None:
    ws, rank, _ = _dist()
    if rank != 0:
        return
    import nwchem_gb300 as ng
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    t = ng.config_tiling(1)
    files = ng.synth_inputs(t, SEED)
    kl = ng.task_list(t)
    sl = _slices(len(kl))
    target = float(os.environ.get("SDT_CPU_STEP_FLOPS", "1.5e11"))
    times, flops = [], []
    for s in range(args.warmup + args.steps):
        ids, f = cpu_sample(t, files, kl, sl[s % N_SLICES], target)
        dt = run_cpu(t, files, kl, ids)
        if s >= args.warmup:
            times.append(dt)
            flops.append(f)
    value = sum(flops) / sum(times) / 1e12
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "form": "fp64"},
            "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                             "sample": f"per step the smallest tuples of that step's slice up to {target:.1e} "
                                       f"FLOPs; C/OpenMP restatement of ccsd_t_kernels_omp.F + drivers"},
            "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def ours(args) -> None:
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

    t = ng.config_tiling(1)
    kl = ng.task_list(t)
    sl = _slices(len(kl))
    files = ng.synth_inputs(t, SEED, pinned=True)
    in_bytes = sum(f.nbytes for f in files)
    step_ids = [sl[(s * ws + rank) % N_SLICES] for s in range(args.warmup + args.steps)]
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
    for s in range(args.warmup, args.warmup + args.steps):
        e = job.run(kl[step_ids[s]], stream=stream)
        kern_ms.append(job.last_kernel_ms)
        energies.append(e)
    ev1.record(stream)
    barrier()
    launches = lib.sdt_launch_count() - launches0
    clocks = sampler.stop()
    elapsed = ev0.elapsed_time(ev1) / 1e3
    my_flops = sum(step_flops[args.warmup:])
    if ws > 1:
        tt = torch.tensor([elapsed, my_flops], dtype=torch.float64, device=dev)
        mx = tt.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        dist.all_reduce(tt, op=dist.ReduceOp.SUM)
        elapsed, total_flops = float(mx[0]), float(tt[1])
    else:
        total_flops = my_flops
    value = total_flops / elapsed / 1e12

    # End to end through the public API: pinned-host TCE files -> device,
    # ingest, run, energies back, every step.
    e2e_steps = min(args.steps, 2)
    barrier()
    t0 = time.perf_counter()
    e2e_flops = 0.0
    for s in range(e2e_steps):
        ids = step_ids[args.warmup + s]
        job.load(*files, stream=stream)
        job.run(kl[ids], stream=stream)
        e2e_flops += step_flops[args.warmup + s]
    barrier()
    e2e_t = time.perf_counter() - t0
    if ws > 1:
        tt = torch.tensor([e2e_t, e2e_flops], dtype=torch.float64, device=dev)
        mx = tt.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        dist.all_reduce(tt, op=dist.ReduceOp.SUM)
        e2e_t, e2e_flops = float(mx[0]), float(tt[1])
    e2e = e2e_flops / e2e_t / 1e12

    kern_avg_s = sum(kern_ms) / len(kern_ms) / 1e3
    achieved = (my_flops / args.steps) / kern_avg_s / 1e12
    job.close()

    if rank == 0:
        cpu = None
        if ws == 1 and not args.no_cpu:
            cores = os.cpu_count() or 1
            ids, f = cpu_sample(t, files, kl, step_ids[args.warmup], float(os.environ.get("SDT_CPU_FLOPS", "3e11")))
            dt = run_cpu(t, files, kl, ids)
            cpu = {"value": f / dt / 1e12, "unit": "TFLOP/s", "cores": cores, "kind": "port",
                   "sample": f"{len(ids)} smallest tuples of one step slice ({f:.3e} FLOPs, {dt:.1f} s); "
                             "C/OpenMP restatement of ccsd_t_kernels_omp.F + drivers"}
        line = {
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded; distributions of the o=40/v=300 workload)",
            "config": {"workload": WORKLOAD, "form": "fp64", "tuples_per_step": int(np.mean([len(x) for x in step_ids])),
                       "flops_per_step": my_flops / args.steps,
                       "cache": f"inputs larger than L2 ({dev_bytes / 1e9:.1f} GB resident operands)",
                       "E[T]_E(T)_last_step": list(energies[-1])},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak if peak > 0 else None, "traffic": None,
                         "peak_source": "measured in-run: FP64 mma.sync m8n8k4 probe (no FP64 entry in "
                                        "MEASURED_PEAKS.json)",
                         "kernel": "fused_fp64_kernel"},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e, "unit": "TFLOP/s", "h2d_bytes_per_step": int(in_bytes),
                    "d2h_bytes_per_step": 16, "steps": e2e_steps},
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def profile_case(args) -> None:
    """Small case for ncu (under 1 GB on the device, operands still larger
    than L2): o=40 as 8/12/20, v=114 as 20,24,30,40, seed 1; the fused
    kernel on `--tuples` tuples from the middle of the weight-ordered list,
    one warm-up launch then one launch."""
    import torch

    import nwchem_gb300 as ng
    torch.cuda.set_device(0)
    t = ng.Tiling([8, 12, 20], [20, 24, 30, 40], name="o40v114").with_evl(SEED)
    kl = ng.task_list(t)
    files = ng.synth_inputs(t, SEED)
    mid = len(kl) // 2
    sel = kl[mid:mid + args.tuples]
    with ng.TriplesJob(t) as job:
        job.load(*files)
        job.set_timing(True)
        job.run(sel)
        e = job.run(sel)
        print(json.dumps({"profile_case": True, "tuples": int(len(sel)), "flops": ng.flops(t, sel),
                          "kernel_ms": job.last_kernel_ms, "device_bytes": job.device_bytes,
                          "tflops": ng.flops(t, sel) / job.last_kernel_ms / 1e9, "energies": list(e)}),
              flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--profile", action="store_true", help="small single-launch case for ncu")
    ap.add_argument("--tuples", type=int, default=2, help="tuples in the --profile case")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    import nwchem_gb300.build as b
    b.build()
    if args.profile:
        profile_case(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        ours(args)


if __name__ == "__main__":
    main()
