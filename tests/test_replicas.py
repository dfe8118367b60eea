"""The multi-GPU path of the bench is replicas (the sweep does not shard across GPUs here):
every rank runs the whole workload, the job's time is the slowest rank's, and the value is
world x the per-rank cell-updates over that time. This checks the reduction with two gloo
ranks on the CPU."""
import os

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks([12.5, 17.0][rank], dist, "cpu")
    out[rank] = (t, bench.replica_value(world, 1e9, t))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = 29000 + os.getpid() % 1000
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs)
        for r in range(2):
            t, v = out[r]
            assert t == 17.0
            assert v == pytest.approx(2 * 1e9 / 17e-3 / 1e9)
