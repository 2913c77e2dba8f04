"""bench.py's multi-rank host logic on CPU: two gloo ranks, one process each
as torchrun launches them.  Every rank runs the whole workload (replicas, no
collective on the data path), so the only exchange is the job time.  Each
rank must get the slowest rank's time, and the job rate must count both ranks'
audio over it.  The reference arm's non-zero ranks return without work."""
import argparse
import os
import socket

import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        t_rank = 0.25 + 0.5 * rank  # rank 1 is the slower one
        t_max = bench.max_over_ranks(t_rank, world)
        rate = bench.job_rate(2.0, 3, world, t_max)
        ref = "n/a"
        if rank != 0:
            args = argparse.Namespace(workload="jnd_sweep", steps=1, warmup=3)
            ref = bench.run_reference(args, rank, world)
        q.put((rank, t_max, rate, ref))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_share_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get() for _ in range(2))
    for rank, t_max, rate, ref in got:
        assert t_max == 0.75
        assert abs(rate - 2.0 * 3 * 2 / 0.75) < 1e-12
        if rank == 1:
            assert ref is None


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(1.5, 1) == 1.5
    assert bench.job_rate(28.9, 5, 1, 1.25) == 28.9 * 5 / 1.25
