"""CPU test of the multi-rank (replicas only) bench path with gloo, world size 2.

Each rank gets disjoint Philox keys; the reported value is the summed work of
all ranks over the slowest rank's time; nothing else crosses ranks."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    seeds = bench.replica_seeds(rank, bench.NTEMP)
    every = [None] * world
    dist.all_gather_object(every, seeds)
    tmax, work = bench.combine_ranks(1.0 + rank, 1000.0 * (rank + 1), dist, "cpu")
    line = bench.multi_line(work, tmax, world, 10, 3, 50, 10)
    out.put((rank, every, tmax, work, line))
    dist.destroy_process_group()


def test_two_ranks_gloo():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = [q.get(timeout=120) for _ in range(2)]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    got.sort()
    (_, every, tmax, work, line) = got[0]
    assert not set(every[0]) & set(every[1])
    assert tmax == 2.0 and work == 3000.0
    assert line["value"] == 1500.0 and line["n_gpus"] == 2 and line["scaling"] == "weak"
    assert got[1][2] == 2.0 and got[1][3] == 3000.0
