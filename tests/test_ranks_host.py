"""The multi-GPU layout on CPU: bench.py runs one replica per rank (the path shards by
ray; no collective on the data path). Two gloo ranks check the pieces the replicas
share: each rank's workload is its own seeded ray batch, the job time is the slowest
rank's, and the whole-job throughput counts every rank's rays."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = [12.0, 15.0][rank]
        t_ms = bench.max_over_ranks(local_ms, dist, device="cpu")
        value = bench.whole_job_mrays(world, 1 << 24, 5, t_ms * 5 * 1e-3)
        o, d = bench.rank_rays(rank, 4096)
        out[rank] = (t_ms, value, float(o[:16].sum()), float(d[:16].sum()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_rank_and_count_every_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = 29500 + os.getpid() % 1000
        procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    (t0, v0, o0, d0), (t1, v1, o1, d1) = res[0], res[1]
    assert t0 == t1 == 15.0
    assert v0 == v1 == pytest.approx(2 * (1 << 24) / 15e-3 / 1e6)
    assert (o0, d0) != (o1, d1)  # the replicas trace different batches


def test_single_process_is_its_own_maximum():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, None) == 3.5
    assert bench.whole_job_mrays(1, 1000, 2, 1e-3) == pytest.approx(2.0)
