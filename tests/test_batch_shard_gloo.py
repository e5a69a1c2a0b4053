"""The batched form's multi-GPU split: scenes are partitioned over ranks by
work (size^2 x sweeps, greedy largest first) with no data shared and no
collective on the data path; the job's throughput is all ranks' cells over
the slowest rank's frame time. Covered with two gloo ranks on CPU: each rank
computes the split on its own, the parts cover the 4096-scene workload
exactly once with under 5 % load imbalance, and the aggregate uses the
slowest rank."""
import os
import socket

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
    import bench
    from equilibrium_gb300.batch import partition_scenes
    cfgs, _ = bench.batch_workload()
    parts, loads = partition_scenes(cfgs, world)
    mine = parts[rank]
    cells = float(sum((cfgs[q][0] - 2) ** 2 for q in mine))
    ms = 10.0 + 5.0 * rank  # the ranks' frame times differ

    def red(x, op):
        t = torch.tensor([x], dtype=torch.float64)
        dist.all_reduce(t, op=op)
        return float(t.item())

    total = red(cells, dist.ReduceOp.SUM)
    slowest = red(ms, dist.ReduceOp.MAX)
    out[rank] = (mine, loads, total, slowest, cells)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_scene_split_covers_the_batch_once_and_balances():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world,
                       start_method="spawn")
    import bench
    cfgs, _ = bench.batch_workload()
    m0, loads0, total0, slow0, c0 = out[0]
    m1, loads1, total1, slow1, c1 = out[1]
    assert loads0 == loads1  # both ranks computed the same split
    assert sorted(list(m0) + list(m1)) == list(range(len(cfgs)))
    assert not set(m0) & set(m1)
    assert max(loads0) / (sum(loads0) / world) - 1.0 < 0.05
    assert total0 == total1 == c0 + c1 == sum((c[0] - 2) ** 2 for c in cfgs)
    assert slow0 == slow1 == pytest.approx(15.0)
