"""Multi-rank path on CPU: two gloo ranks each evaluate their round-robin
share of the tuples (with the oracle standing in for the per-GPU work) and
combine per-tuple energies; the result must equal the single-rank total bit
for bit, and a rank that fails is reported on the host, not hung."""
import math
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import nwchem_gb300 as ng
from nwchem_gb300 import shard
from oracle import oracle as orc

OCC, VIR, SEED = [3, 2, 3], [4, 3, 5], 13


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out, fail_rank):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    os.environ["OMP_NUM_THREADS"] = "1"
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = ng.Tiling(OCC, VIR).with_evl(SEED)
        P = orc.Problem(t, *ng.synth_inputs(t, SEED))
        kl = P.task_list()
        ids = shard.rank_tasks(len(kl), world, rank)
        status = 0
        try:
            if rank == fail_rank:
                raise RuntimeError("injected failure on this rank")
            _, _, pt, _ = P.ccsd_t(kl, task_ids=ids)
        except RuntimeError:
            status, pt = 1, np.zeros((0, 2))
        # every rank learns of a failed rank on the host before combining
        st = [None] * world
        dist.all_gather_object(st, status)
        if any(st):
            out[rank] = ("failed", st)
            return
        out[rank] = ("ok", shard.allreduce_energies(pt))
    finally:
        dist.destroy_process_group()


def _run(world, fail_rank=-1):
    mgr = mp.get_context("spawn").Manager()   # no fork of this (threaded) process
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), out, fail_rank), nprocs=world, join=True)
    return dict(out)


def test_two_ranks_equal_single_rank_bit_for_bit():
    t = ng.Tiling(OCC, VIR).with_evl(SEED)
    P = orc.Problem(t, *ng.synth_inputs(t, SEED))
    _, _, pt, _ = P.ccsd_t()
    want = (math.fsum(pt[:, 0]), math.fsum(pt[:, 1]))
    res = _run(2)
    assert res[0][0] == "ok" and res[1][0] == "ok"
    assert res[0][1] == want and res[1][1] == want


def test_failed_rank_is_reported_to_all_ranks():
    res = _run(2, fail_rank=1)
    assert res[0] == ("failed", [0, 1]) and res[1] == ("failed", [0, 1])


def test_rank_tasks_partition():
    parts = [shard.rank_tasks(11, 3, r) for r in range(3)]
    assert sorted(np.concatenate(parts).tolist()) == list(range(11))
    with pytest.raises(ValueError):
        shard.rank_tasks(5, 2, 2)
