"""Multi-rank host logic on CPU: two gloo ranks shard a probe set (every probe
exactly once), time their shares, and agree on the whole-job throughput."""
import os
import socket

import pytest

from althea_gb300 import dist

torch = pytest.importorskip("torch")


def test_shard_partitions():
    n, world = 257, 4
    got = sorted(i for r in range(world) for i in dist.shard(n, r, world))
    assert got == list(range(n))
    with pytest.raises(ValueError):
        dist.shard(4, 2, 2)
    assert dist.job_throughput([10, 10], [2.0, 4.0]) == 5.0


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, sizes, out):
    import torch.distributed as tdist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    mine = dist.shard(len(sizes), rank, world)
    work = float(sum(sizes[i] for i in mine))       # stand-in for bake time
    units = float(len(mine))
    slowest = dist.allreduce_max(work)
    total = dist.allreduce_sum(units)
    out[rank] = (mine, slowest, total, total / slowest)
    tdist.destroy_process_group()


def test_two_gloo_ranks_agree_on_job_throughput():
    import torch.multiprocessing as mp
    world = 2
    sizes = [256, 512, 1024, 2048, 256, 512, 1024]
    mgr = mp.get_context("spawn").Manager()  # no fork of a process that runs threads
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), sizes, out), nprocs=world, join=True)
    r0, r1 = out[0], out[1]
    assert sorted(r0[0] + r1[0]) == list(range(len(sizes)))
    assert r0[1] == r1[1] == max(sum(sizes[i] for i in r0[0]), sum(sizes[i] for i in r1[0]))
    assert r0[2] == r1[2] == len(sizes)
    assert r0[3] == r1[3] == pytest.approx(len(sizes) / r0[1])
