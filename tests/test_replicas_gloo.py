"""bench.py's multi-process (replica) logic with world_size 2 over gloo, on CPU.

Each rank times its own replica; the reported time is the max over ranks and
the throughput counts all ranks' points (weak scaling). No GPU involved.
"""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, results):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    w, r, local = bench.dist_env()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(w)
    elapsed = 100.0 + 50.0 * rank  # rank 1 is the slow one
    m = bench.max_over_ranks(elapsed, w)
    results[rank] = m
    dist.destroy_process_group()


@pytest.mark.timeout(120) if hasattr(pytest.mark, "timeout") else (lambda f: f)
def test_max_over_ranks_world2():
    world = 2
    port = _free_port()
    manager = mp.Manager()
    results = manager.dict()
    mp.spawn(_worker, args=(world, port, results), nprocs=world, join=True)
    assert results[0] == results[1] == 150.0


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    bench.barrier(1)
