"""bench.py's multi-rank helpers on the CPU: two gloo ranks take the max of
their timings and meet at the barrier (the N > 1 path of the bench uses the
same calls over NCCL), and the JSON contract helpers need no GPU."""

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        q.put((rank, bench.aggregate_seconds(0.5 + rank, world, device="cpu")))
        bench.barrier(world)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got == {0: 1.5, 1: 1.5}


def test_single_rank_helpers_and_bytes():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.aggregate_seconds(0.25, 1) == 0.25
    bench.barrier(1)
    # algorithmic bytes of the 2048^2 -> 1536^2 apply quoted in the bench line
    assert bench.apply_bytes(64, 2048 * 2048, 1536 * 1536, 12786465) == 1798887696
    assert bench.dist_env() == (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
                                int(os.environ.get("LOCAL_RANK", "0")))
