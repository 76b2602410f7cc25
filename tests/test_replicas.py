"""Replicas across ranks (CPU, gloo, world size 2): disjoint sample ranges
and the timing reductions bench.py uses (max of times, sum of rays)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from rustracer_gb300 import replicas


def test_sample_ranges_disjoint_and_complete():
    world, spp, steps = 4, 8, 3
    got = sorted(replicas.sample_range(r, world, k, spp) for r in range(world) for k in range(steps))
    assert got[0][0] == 0 and got[-1][1] == world * spp * steps
    assert all(a[1] == b[0] for a, b in zip(got, got[1:]))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    times, counts = replicas.combine([1.0 + rank, 10.0 * (rank + 1)], [100.0 * (rank + 1)])
    out[rank] = (times, counts)
    dist.destroy_process_group()


def test_combine_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        times, counts = out[r]
        assert times == [2.0, 20.0] and counts == [300.0]


def test_combine_single_rank():
    assert replicas.combine([1.5], [7.0]) == ([1.5], [7.0])
