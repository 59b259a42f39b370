"""The multi-process path of bench.py (N replicas under torchrun, one per GPU: samples are independent, so
every rank runs its own batch and no collective touches the data path) on CPU with gloo, world size 2: the
reported step time is the slowest rank's."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        out[rank] = bench.reduce_max(1.5 + rank, dist)
    finally:
        dist.destroy_process_group()


def test_step_time_is_the_slowest_replica():
    world = 2
    with mp.Manager() as manager:
        out = manager.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        assert dict(out) == {0: 2.5, 1: 2.5}
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_max(3.25, None) == 3.25


if __name__ == "__main__":  # pragma: no cover
    pytest.main([__file__])
