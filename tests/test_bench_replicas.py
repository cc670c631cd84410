"""bench.py with N > 1: replicas on separate GPUs, timed by the slowest rank (host logic, gloo on CPU).

Each rank runs an independent replica of the request (the path has no data exchange between requests); the
job's value is all ranks' pixels over the slowest rank's time, and the reference arm runs on rank 0 only.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, lr = bench.dist_env()
    local_ms = [12.5, 20.0][rank]
    slow = bench.slowest_rank_ms(local_ms)
    value = bench.replica_mpix(1920 * 1080, slow, w)
    dist.barrier()
    ref = bench.run_reference(type("A", (), {"warmup": 0, "steps": 1})(), bench.PLAIN_LARGE) if rank == 1 else None
    dist.destroy_process_group()
    out.put((rank, r, w, lr, slow, value, ref))


def test_replicas_report_the_slowest_rank():
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(k, 2, port, q)) for k in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, r, w, lr, slow, value, ref in res:
        assert (r, w, lr) == (rank, 2, rank)
        assert slow == 20.0  # both ranks see the slowest rank's time
        assert value == pytest.approx(2 * 1920 * 1080 / 20e-3 / 1e6)
    assert res[1][6] is None  # the reference arm does no work off rank 0


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.slowest_rank_ms(7.0) == 7.0
    assert bench.replica_mpix(1000, 1.0, 1) == pytest.approx(1.0)
