"""Several GPUs = independent problems sharded across ranks (no data-path
collective).  The host-side logic runs here as world_size-2 gloo process
groups on the CPU: the shard assignment, and the whole-job rate (sum of the
ranks' units over the slowest rank's time)."""
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

# the spawned ranks import this module afresh: load the package here too
sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import __graft_entry__  # noqa: E402

__graft_entry__.load_package()
from pdesolver_gb300 import problems, replicas  # noqa: E402


def test_shard_balances_and_covers():
    work = [5.0, 1.0, 4.0, 4.0, 2.0, 2.0, 1.0, 9.0]
    parts = replicas.shard(work, 3)
    assert sorted(i for p in parts for i in p) == list(range(len(work)))
    loads = [sum(work[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(work)
    assert replicas.shard(work, 3) == parts            # deterministic
    assert replicas.shard(work, 1) == [list(range(len(work)))]
    with pytest.raises(ValueError):
        replicas.shard(work, 0)


def test_shard_of_the_batched_workload():
    """the 96 problems of the batched workload split over 2 and 8 ranks by
    their element-block work, each rank within one problem of the mean."""
    specs = problems.config4_specs()
    work = [2 * s["n"] ** 2 * ((3, 7, 12, 18)[s["p"] - 1] * 4) ** 2 for s in specs]
    for world in (2, 8):
        parts = replicas.shard(work, world)
        loads = [sum(work[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(work)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, work, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = replicas.shard(work, world)[rank]
        units = len(mine)
        seconds = 1.0 + rank                       # rank 1 is the slow one
        rate, total, tmax = replicas.job_rate(units, seconds, dist)
        out[rank] = (mine, rate, total, tmax)
    finally:
        dist.destroy_process_group()


def test_job_rate_over_two_gloo_ranks():
    work = [3.0, 1.0, 2.0, 2.0, 5.0]
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(2, _free_port(), work, out), nprocs=2, join=True)
        res = dict(out)
    parts = replicas.shard(work, 2)
    assert [res[r][0] for r in (0, 1)] == parts
    for r in (0, 1):
        _, rate, total, tmax = res[r]
        assert total == len(work) and tmax == 2.0
        assert rate == pytest.approx(len(work) / 2.0)
