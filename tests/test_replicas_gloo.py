"""The multi-GPU form of the benchmark is replicas only: every rank runs the same step on its own
GPU with no data exchange, and the ranks meet only on the host (a barrier around the timed region
and the maximum of the ranks' times). This checks that host logic with two gloo ranks on the CPU.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    w, r, local = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(w)
    t = bench.max_over_ranks(0.25 + rank, w)
    # the reference arm does its work on rank 0 only; the other ranks return at once
    args = type("A", (), dict(steps=1, warmup=0))()
    if rank != 0:
        bench.run_reference(args, w, r, local)
    bench.barrier(w)
    import torch.distributed as dist
    dist.destroy_process_group()
    out.put((rank, t))


def test_two_gloo_ranks_share_the_maximum_time():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=10) for _ in range(world))
    assert res == {0: 1.25, 1: 1.25}
