"""The bench's multi-GPU form is independent replicas (the path has no
exchange step).  Its host logic -- max-over-ranks timing and the barrier --
is checked here with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MDG_BENCH_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench

    w, r, _ = bench.dist_setup()
    bench.barrier(w)
    m = bench.reduce_max(1.5 + r, w)
    q.put((r, w, m))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_reduce_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2, 2.5), (1, 2, 2.5)]
