"""bench.py's whole-job figure over replica ranks (max of the timed
milliseconds, sum of the units), with two gloo ranks on the CPU."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    ms, value = bench.aggregate_ranks(10.0 + 5.0 * rank, 1000 * (rank + 1), dist, "cpu")
    slowest = bench.max_over_ranks([1.0 + rank, 3.0 - rank], dist, "cpu")
    out[rank] = (ms, value, slowest)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replica_ranks_aggregate():
    port = 29500 + os.getpid() % 2000
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    for r in (0, 1):
        ms, value, slowest = res[r]
        assert ms == 15.0                               # the slowest rank
        assert abs(value - 3000 / 15e-3) < 1e-6 * value  # all ranks' units in that time
        assert slowest == [2.0, 3.0]                    # end-to-end times: each the slowest rank's
