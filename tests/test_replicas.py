"""Host logic of the multi-process replica run, on CPU with the gloo backend
(world size 2): per-rank seeds differ, the job time is the slowest rank's, and
a rank that fails before the timed region is reported to the others by the
process group instead of leaving them waiting."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from rvgp_gb300 import replicas


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, times, out_q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, lr = replicas.world()
    dist.barrier()
    t = replicas.max_over_ranks(times[rank])
    seeds = [None] * world
    dist.all_gather_object(seeds, replicas.replica_seed(7, r))
    dist.barrier()
    out_q.put((r, w, lr, t, seeds, replicas.job_throughput(t, w)))
    dist.destroy_process_group()


def test_max_over_ranks_and_seeds_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    world, port = 2, _free_port()
    times = [0.25, 0.5]
    procs = [ctx.Process(target=_worker, args=(r, world, port, times, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, w, lr, t, seeds, thr) in enumerate(res):
        assert (rank, w, lr) == (r, world, r)
        assert t == pytest.approx(0.5)  # the slowest rank's time
        assert len(set(seeds)) == world  # every replica has its own inputs
        assert thr == pytest.approx(world / 0.5)


def _failing_worker(rank, world, port, out_q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    from datetime import timedelta
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=timedelta(seconds=5))
    if rank == 1:
        dist.destroy_process_group()
        raise SystemExit(3)  # a rank that leaves between steps, before the timed region
    try:
        replicas.max_over_ranks(1.0)
        out_q.put("no error")
    except Exception as e:  # the survivor learns of it from the collective, within its timeout
        out_q.put(type(e).__name__)


def test_rank_failure_surfaces_as_error_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    world, port = 2, _free_port()
    procs = [ctx.Process(target=_failing_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    msg = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
    assert msg != "no error"
    assert procs[1].exitcode == 3


def test_single_process_is_identity():
    assert replicas.max_over_ranks(1.25) == 1.25
    assert replicas.job_throughput(0.5, 1) == 2.0
