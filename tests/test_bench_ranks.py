"""The multi-replica bench path on CPU: two gloo ranks combine their timings
(max over ranks, units of all ranks), as `bench.py --gpus 2` does over NCCL."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _worker(rank, world, port, times, out):
    import torch
    import torch.distributed as dist
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    import bench
    t_max, value = bench.combine_ranks(times[rank], 1000.0, world, torch.device('cpu'))
    out[rank] = (t_max, value)
    dist.destroy_process_group()


def test_combine_ranks_two_gloo_ranks():
    world = 2
    times = [0.5, 0.8]
    mgr = mp.Manager()
    out = mgr.dict()
    port = _free_port()
    mp.start_processes(_worker, args=(world, port, times, out), nprocs=world, join=True, start_method='spawn')
    for r in range(world):
        t_max, value = out[r]
        assert t_max == pytest.approx(0.8)
        assert value == pytest.approx(1000.0 * world / 0.8)


def test_combine_ranks_single():
    import bench
    assert bench.combine_ranks(0.25, 100.0, 1, None) == (0.25, 400.0)
