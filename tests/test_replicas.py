"""The N>1 bench path is replicas only: each rank solves its own case (its own seed),
there is no data-path collective, and the job time is the slowest rank's.  These
tests run that host logic as two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    try:
        import torch
        import torch.distributed as dist
        import bench
        dist.init_process_group("gloo", rank=rank, world_size=ws)
        env = bench.dist_env()
        t_local = 0.5 + rank                     # rank 1 is the slower one
        t_max = bench.max_over_ranks(t_local, ws, torch.device("cpu"))
        seeds = [None] * ws
        dist.all_gather_object(seeds, bench.replica_seed(rank))
        rate = bench.job_rate(ws, 20, t_max)
        # the reference arm runs on rank 0 alone; the other ranks leave without work
        if rank != 0:
            class _Args:
                steps, warmup, gpus = 1, 0, ws
            bench.run_reference(_Args())
        dist.barrier()
        dist.destroy_process_group()
        q.put((rank, env, t_max, seeds, rate, None))
    except Exception as e:  # reported to the parent
        q.put((rank, None, None, None, None, repr(e)))


def test_two_replica_ranks_gloo():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in procs:
        r, env, t_max, seeds, rate, err = q.get(timeout=180)
        out[r] = (env, t_max, seeds, rate, err)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        env, t_max, seeds, rate, err = out[r]
        assert err is None, err
        assert env == (2, r, r)
        assert t_max == 1.5                       # max over ranks, the same on both
        assert len(set(seeds)) == 2               # independent cases per replica
        assert rate == pytest.approx(2 * 20 / 1.5)


def test_single_rank_helpers():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, 1, None) == 3.25
    assert bench.job_rate(1, 10, 2.0) == 5.0
    assert bench.replica_seed(0) != bench.replica_seed(1)
