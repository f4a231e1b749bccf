"""The multi-rank bookkeeping of the benchmark (one process per GPU, replicas
only): barrier and max-over-ranks, run as two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    bench.barrier(torch)
    got = bench.max_over_ranks(torch, [1.0 + rank, 10.0 - rank, 0.5 * rank], torch.device("cpu"))
    out.put((rank, got))
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0] == res[1] == [2.0, 10.0, 0.5]


def test_max_over_ranks_single_process_is_identity():
    torch = pytest.importorskip("torch")
    import bench
    assert bench.max_over_ranks(torch, [3, 1.5], torch.device("cpu")) == [3.0, 1.5]
    bench.barrier(torch)  # no process group: a no-op
