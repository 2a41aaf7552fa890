"""The multi-GPU path is replicas only (one scene does not shard): each rank
steps its own copy and the job's time is the slowest rank's. The aggregation
bench.py uses, run as two gloo ranks on CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench

    seconds = [2.0, 3.5][rank]  # rank 1 is the slow one
    slow = bench.slowest_rank(seconds, ws, device="cpu")
    out[rank] = (slow, bench.replica_rate(600, ws, slow))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_slowest_rank():
    ws = 2
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.start_processes(_rank, args=(ws, _free_port(), out), nprocs=ws, start_method="spawn", join=True)
    assert out[0] == out[1] == (3.5, 2 * 600 / 3.5)


def test_single_rank_needs_no_collective():
    import bench

    assert bench.slowest_rank(1.25, 1) == 1.25
    assert bench.replica_rate(600, 1, 1.25) == 480.0
