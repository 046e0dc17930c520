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


def test_quoted_ncu_figures_parse():
    """The bench line quotes two figures from committed ncu summaries: the
    headline kernel's DRAM bytes per launch and the algorithmic flop count."""
    import bench
    traffic = bench._profile_value("stage_kernel_fp64_droplet_1024x512.md", "dram_bytes_per_launch")
    flops = bench._profile_value("flop_count_droplet_1024x512.md", "algorithmic_flops_per_cell_update")
    assert traffic is not None and 1e7 < traffic < 1e9
    assert flops is not None and 1e3 < flops < 1e4
