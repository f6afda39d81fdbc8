"""Multi-rank path of the batched workload on CPU (gloo, world size 2): the
ranks' shares of the instances are disjoint, cover the batch, and are
balanced by estimated work; the slowest-rank time is taken with a MAX
all-reduce, as bench.py does on GPUs."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from poromec_gb300 import meshgen


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, edges, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    share = meshgen.partition_instances(edges, world)[rank]
    n = torch.tensor([len(share)])
    gathered = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(gathered, n)
    idx = torch.zeros(len(edges), dtype=torch.int64)
    idx[share] = rank + 1
    dist.all_reduce(idx)  # each instance claimed by exactly one rank -> values 1..world
    t = torch.tensor([float(rank + 1)])
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        out.put((idx.tolist(), [int(g) for g in gathered], float(t)))
    dist.destroy_process_group()


def test_partition_two_ranks_gloo():
    edges = [p["n"] for p in meshgen.batch_instances(ninst=12, nmin=8, nmax=32, seed=4242)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, edges, q)) for r in range(2)]
    for p in procs:
        p.start()
    idx, counts, tmax = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(set(idx)) == [1, 2] and sum(counts) == len(edges)
    assert tmax == 2.0
    w = [sum(e ** 3 for e, r in zip(edges, idx) if r == k) for k in (1, 2)]
    assert max(w) <= 1.5 * min(w)


def test_partition_single_rank_is_everything():
    assert meshgen.partition_instances([8, 9, 10], 1) == [[0, 1, 2]]
