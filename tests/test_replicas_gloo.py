"""The multi-process path of bench.py on the CPU: two ranks over gloo (the
transform does not shard across GPUs here, so N GPUs run N replicas). Each
rank reports its own step time; the job time is the max over ranks and the
job's throughput is the sum of the replicas' bytes over that time."""
import os
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ws, r, local = bench._dist()
    assert (ws, r, local) == (world, rank, rank)
    bench._barrier(ws)
    my_ms = 1.0 + rank  # rank 1 is the slower replica
    ms = bench._allreduce_max(my_ms, ws)
    value = bench.replica_value(2**30, ms, ws)
    out[rank] = (ms, value)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_replicas_take_max_time_and_sum_bytes(world):
    import random
    port = random.randint(20000, 40000)
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(world, port, out), nprocs=world, join=True,
                       start_method="spawn")
    assert sorted(out.keys()) == list(range(world))
    for r in range(world):
        ms, value = out[r]
        assert ms == float(world)  # max over ranks
        assert abs(value - 2**30 * world / (world * 1e-3) / 1e9) < 1e-9
