"""The multi-process path of bench.py on the CPU: with world size 2 (gloo),
the barrier and the max-over-ranks reduction of the step time that make
the whole-job number; each rank is an independent replica (no collective on
the data path)."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    d, w, r, lr = bench.dist_init()
    assert (w, r, lr) == (world, rank, rank)
    bench.barrier(d)
    got = bench.allreduce_max(d, 10.0 + rank)
    q.put((rank, got))
    d.destroy_process_group()


def test_world_size_two_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res == {0: 11.0, 1: 11.0}
