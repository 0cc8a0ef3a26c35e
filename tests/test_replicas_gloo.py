"""Replica bookkeeping of multi-GPU runs, exercised with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from femflow_gb300 import replicas as R


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w = R.world()
        share = R.shard(256, r, w)
        units = sum(1000 + i for i in share)      # particles of this rank's scenes
        secs = 1.0 + r                            # rank 1 is the slow one
        R.barrier()
        out[rank] = (list(share), R.max_over_ranks(secs), R.sum_over_ranks(units), R.job_throughput(units, secs))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    shares = [out[r][0] for r in range(world)]
    assert sorted(shares[0] + shares[1]) == list(range(256))  # every scene exactly once
    total = sum(1000 + i for i in range(256))
    for r in range(world):
        _, tmax, usum, thr = out[r]
        assert tmax == 2.0 and usum == total
        assert thr == pytest.approx(total / 2.0)


@pytest.mark.parametrize("n,w", [(256, 3), (5, 8), (0, 2), (7, 1)])
def test_shard_covers_everything_once(n, w):
    got = [i for r in range(w) for i in R.shard(n, r, w)]
    assert got == list(range(n))
    sizes = [len(R.shard(n, r, w)) for r in range(w)]
    assert max(sizes) - min(sizes) <= 1


def test_single_process_defaults():
    assert R.max_over_ranks(3.5) == 3.5 and R.sum_over_ranks(2.0) == 2.0
    assert R.job_throughput(10.0, 2.0) == 5.0
