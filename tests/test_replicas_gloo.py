"""The multi-GPU path of the plain step is 'replicas only' (a single grid does
not shard): every rank advances its own scene and the job's throughput is
ranks x cells x steps / slowest rank. Covered here with two gloo ranks on CPU,
each running an oracle replica."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle
    import bench
    f = oracle.OracleFluid(34, 0.1, 4, 1e-3, 1e-3)
    f.fill_obstacle(5, 5, 9 + rank, 12)
    secs = f.run(2, np.full((2, 1), 17, np.uint32), np.full((2, 1), 17, np.uint32),
                 np.ones((2, 1), np.float32), np.zeros((2, 1), np.float32),
                 np.zeros((2, 1), np.float32), timed=True)
    local = secs + 0.25 * rank  # make the ranks' times differ

    def reduce_max(x):
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    value, t = bench.replicas_value(local, 2, world, reduce_max)
    out[rank] = (value, t, local, float(f.field("density").sum()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas_aggregate_on_the_slowest_rank():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world,
                       start_method="spawn")
    v0, t0, l0, d0 = out[0]
    v1, t1, l1, d1 = out[1]
    assert t0 == t1 == pytest.approx(max(l0, l1))
    import bench
    assert v0 == v1 == pytest.approx(world * bench.N * bench.N * 2 / max(l0, l1))
    assert d0 != d1  # the replicas are independent scenes
