"""bench.py's N-rank path (replicas, one process per GPU) on CPU: two gloo ranks
agree on the max-over-ranks step time and read their rank from the launcher's
environment."""
import os

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        r, w, local = bench.rank_info()
        t = bench.max_over_ranks(0.1 * (r + 1), w, device='cpu')
        dist.barrier()
        q.put((r, w, local, t))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_share_the_max_step_time():
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = 29650 + os.getpid() % 200
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[0] for g in got] == [0, 1] and all(g[1] == 2 for g in got)
    assert [g[2] for g in got] == [0, 1]
    assert all(abs(g[3] - 0.2) < 1e-15 for g in got)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(0.25, 1) == 0.25
