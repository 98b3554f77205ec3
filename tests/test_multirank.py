"""The replica path of bench.py on CPU: two gloo ranks, each times its own work, and every
rank ends with the maximum (the whole-job time) - the reduction the GPU run uses over NCCL."""
import os
import socket

import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks([10.0 + rank, 3.0 * rank], dist, device='cpu')
    out[rank] = t
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max_time():
    mgr = mp.Manager()
    out = mgr.dict()
    port = _free_port()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0] == out[1] == [11.0, 3.0]
