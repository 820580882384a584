"""bench.py's multi-rank host logic with two gloo ranks on the CPU (each GPU
runs an independent replica; ranks meet only at the timing barriers and the
max-over-ranks reduction): the barrier, the reduction, the whole-job replica
throughput, and the reference arm's rank-0-only rule."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        bench.rank_barrier()
        worst = bench.max_over_ranks(1.5 + rank)  # rank r took 1.5 + r seconds
        mpx = bench.replica_mpx(8 * bench.OW * bench.OH, worst, world)
        ref = bench.run_reference(None, rank) if rank != 0 else "skipped"
        bench.rank_barrier()
        q.put((rank, worst, mpx, ref))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    import bench
    for rank, worst, mpx, ref in res:
        assert worst == 2.5  # the slowest rank's time, on every rank
        assert mpx == pytest.approx(2 * 8 * bench.OW * bench.OH / 2.5 / 1e6)
    assert res[1][3] is None  # the reference arm: rank 1 does no work


def test_single_process_helpers():
    import bench
    bench.rank_barrier()  # no process group: nothing to wait for
    assert bench.max_over_ranks(3.25) == 3.25
    assert bench.replica_mpx(1e6, 0.5, 1) == pytest.approx(2.0)
