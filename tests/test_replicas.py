"""The benchmark's N > 1 path: independent replicas, whole-job rate = all
ranks' cell-updates over the slowest rank's time (world size 2, gloo)."""
import os
import socket


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seconds = [2.0, 3.0][rank]  # the slower rank sets the job time
        out[rank] = bench.replica_rate(seconds, 1000, world, device="cpu")
    finally:
        dist.destroy_process_group()


def test_replica_rate_is_total_work_over_the_slowest_rank():
    import torch.multiprocessing as mp
    with mp.get_context("spawn").Manager() as m:  # no fork of a threaded process
        out = m.dict()
        mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
        assert dict(out) == {0: (2000 / 3.0, 3.0), 1: (2000 / 3.0, 3.0)}


def test_single_replica_needs_no_process_group():
    import bench
    assert bench.replica_rate(2.0, 1000, 1) == (500.0, 2.0)
