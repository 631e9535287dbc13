"""Multi-GPU is replicas only (the sweep does not shard): the bench's whole-job
timing is the maximum over ranks and the value sums the replicas' work. Checked
here with two gloo ranks on the CPU."""

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = [120.0, 250.0][rank]
    m = bench.max_over_ranks(ms, "cpu")
    out[rank] = m
    out[2 + rank] = bench.replica_value(world, 127, 5, m)
    dist.destroy_process_group()


def test_max_over_ranks_and_replica_value():
    world = 2
    out = torch.zeros(4, dtype=torch.float64).share_memory_()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    assert out[0].item() == out[1].item() == 250.0
    assert out[2].item() == out[3].item() == pytest.approx(2 * 127 * 5 / 0.25)
