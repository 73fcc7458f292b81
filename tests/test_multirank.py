"""bench.py's replica path on CPU: two gloo ranks, max-over-ranks timing and
the whole-job rate (the SpMV does not shard: --gpus N runs N replicas)."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    import bench
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        w, r, _ = bench.dist_setup()
        bench.barrier(w)
        local_ms = 10.0 + 5.0 * r  # rank 1 is slower
        rate, ms = bench.replica_rate(1_000_000, local_ms, w)
        q.put((r, w, rate, ms))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, w, rate, ms in out:
        assert w == 2 and ms == pytest.approx(15.0)
        assert rate == pytest.approx(2 * 1_000_000 / 0.015)


def test_single_rank_rate():
    import bench
    rate, ms = bench.replica_rate(500, 2.0, 1)
    assert ms == 2.0 and rate == pytest.approx(500 / 0.002)
