"""bench.py's N-GPU path without GPUs: two gloo ranks reduce their timings
the way the replicas do (slowest rank's time, all ranks' work)."""
import os
import socket
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 100.0 + 50.0 * rank           # rank 1 is the slow one
    rays = 1e6 * (rank + 1)
    res = bench.reduce_over_ranks(ms, rays, ms / 1e3 * 1.1, rays * 0.5)
    out[rank] = res
    dist.barrier()
    dist.destroy_process_group()


def test_replica_reduction_two_ranks():
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(2, port, out), nprocs=2, start_method="spawn")
    for r in range(2):
        ms, rays, e2e_s, e2e_rays = out[r]
        assert ms == 150.0 and rays == 3e6
        assert abs(e2e_s - 0.165) < 1e-12 and e2e_rays == 1.5e6
