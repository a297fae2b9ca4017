"""Multi-rank path of bench.py on CPU (gloo, world size 2).

The stream+collide path has no cross-GPU exchange: N ranks run N independent
replicas and the whole-job rate is all ranks' node updates over the slowest
rank's time.  This checks that reduction with two gloo ranks.
"""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms_local = 10.0 + 5.0 * rank  # rank 1 is the slow one
    ms, value = bench.aggregate(ms_local, nodes=1000, steps=20, world=world, dist=dist)
    dist.barrier()
    out[rank] = (ms, value)
    dist.destroy_process_group()


def test_replicas_rate_uses_slowest_rank():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        ms, value = res[rank]
        assert ms == 15.0
        assert value == pytest.approx(1000 * 20 * world / 0.015 / 1e6)
