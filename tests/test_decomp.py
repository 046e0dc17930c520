"""Domain decomposition: the reference's split of the cells, neighbour maps
with periodic wrap-around, halo strips, the rank-to-rank exchange over gloo
(world size 2, on the host), and subdomains on one GPU that reproduce the
undecomposed run bit for bit."""
import os
import socket

import numpy as np
import pytest

from microfc_gb300 import cases, decomp, preprocess


def test_split_follows_the_reference_rule():
    c = cases.sod_1d(m=100, steps=2)  # 101 cells
    x_cb, _, _, _ = preprocess.generate(c)
    subs = decomp.decompose(c, x_cb, px=3)
    assert [s.case.m + 1 for s in subs] == [34, 34, 33]  # (m+1)//3, the first (m+1)%3 get one more
    assert [s.start[0] for s in subs] == [0, 34, 68]
    assert [s.neighbors for s in subs] == [{(0, 1): 1}, {(0, 0): 0, (0, 1): 2}, {(0, 0): 1}]
    assert subs[0].case.bc_x == (-3, 1) and subs[1].case.bc_x == (0, 2) and subs[2].case.bc_x == (1, -3)
    for s in subs:  # each subdomain's cell boundaries are the global ones
        assert np.array_equal(s.x_cb, x_cb[s.start[0]:s.start[0] + s.case.m + 2])


def test_periodic_boundaries_wrap_to_the_far_subdomain():
    c = cases.sod_1d(m=99, steps=2).replace(bc_x=(-1, -1))
    x_cb, _, _, _ = preprocess.generate(c)
    subs = decomp.decompose(c, x_cb, px=2)
    assert subs[0].neighbors == {(0, 0): 1, (0, 1): 1} and subs[1].neighbors == {(0, 0): 0, (0, 1): 0}
    one = decomp.decompose(c, x_cb, px=1)
    assert one[0].neighbors == {} and one[0].case.bc_x == (-1, -1)


def test_2d_grid_of_subdomains_and_halo_strips():
    c = cases.shock_droplet_2d(nx=128, ny=64, steps=2)
    x_cb, y_cb, _, q = preprocess.generate(c)
    subs = decomp.decompose(c, x_cb, y_cb, px=2, py=2)
    assert [s.coords for s in subs] == [(0, 0, 0), (1, 0, 0), (0, 1, 0), (1, 1, 0)]
    assert subs[0].neighbors == {(0, 1): 1, (1, 1): 2}
    assert subs[3].neighbors == {(0, 0): 2, (1, 0): 1}
    H = 3
    for s in subs:
        local = q[s.window()]
        for (d, side), peer in s.neighbors.items():
            strip = decomp.halo_strip(s, local, d, side, H)
            # what the neighbour reads as its ghost cell at depth k on its opposite side
            o = subs[peer]
            for k in range(H):
                if d == 0:
                    gx = o.start[0] - 1 - k if side == 1 else o.start[0] + o.case.m + 1 + k
                    ref = q[:, 0, o.start[1]:o.start[1] + o.case.n + 1, gx]
                    assert np.array_equal(strip[:, 0, :, k], ref)
                else:
                    gy = o.start[1] - 1 - k if side == 1 else o.start[1] + o.case.n + 1 + k
                    ref = q[:, 0, gy, o.start[0]:o.start[0] + o.case.m + 1]
                    assert np.array_equal(strip[:, 0, k, :], ref)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _exchange_worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        c = cases.sod_1d(m=99, steps=2).replace(bc_x=(-1, -1))
        x_cb, _, _, q = preprocess.generate(c)
        q = q + np.arange(q.size, dtype=np.float64).reshape(q.shape) * 1e-3  # distinct values everywhere
        s = decomp.decompose(c, x_cb, px=world)[rank]
        local = q[s.window()]
        strips = {k: torch.from_numpy(decomp.halo_strip(s, local, k[0], k[1], 3)) for k in s.neighbors}
        got = decomp.exchange(s, strips)
        ok = True
        for (d, side), t in got.items():
            # the strip arriving on my side `side` is the neighbour's strip of its opposite side
            peer = decomp.decompose(c, x_cb, px=world)[s.neighbors[(d, side)]]
            ref = decomp.halo_strip(peer, q[peer.window()], d, 1 - side, 3)
            ok &= np.array_equal(t.numpy(), ref)
        out[rank] = bool(ok)
    finally:
        dist.destroy_process_group()


def test_rank_to_rank_exchange_over_gloo():
    import torch.multiprocessing as mp
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:  # no fork of a threaded process
        out = m.dict()
        mp.spawn(_exchange_worker, args=(2, port, out), nprocs=2, join=True)
        assert dict(out) == {0: True, 1: True}


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["sod", "sod_periodic", "droplet_2x2", "droplet_split_4x1"])
def test_subdomains_on_one_gpu_reproduce_the_whole_domain(kind):
    from microfc_gb300 import Simulation
    if kind.startswith("sod"):
        c = cases.sod_1d(m=199, steps=20, dt=2e-4)
        if kind == "sod_periodic":
            c = c.replace(bc_x=(-1, -1))
        px, py = 3, 1
    else:
        prec = "split" if "split" in kind else "fp64"
        c = cases.shock_droplet_2d(nx=128, ny=64, steps=20, precision=prec)
        px, py = (2, 2) if "2x2" in kind else (4, 1)
    x_cb, y_cb, _, q = preprocess.generate(c)
    with Simulation(c, x_cb, y_cb, q_cons=q) as sim:
        sim.run(0, 20)
        ref = sim.download()
    with decomp.MultiDomain(c, x_cb, y_cb, q_cons=q, px=px, py=py) as md:
        md.run(0, 20)
        got = md.download()
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_3d_subdomains_reproduce_the_whole_domain(prec):
    from microfc_gb300 import Simulation
    c = cases.shock_bubble_3d(N=52, steps=5, precision=prec).replace(m=53, n=51, p=52)
    x_cb, y_cb, z_cb, q = preprocess.generate(c)
    with Simulation(c, x_cb, y_cb, z_cb, q_cons=q) as sim:
        sim.run(0, 5)
        ref = sim.download()
    with decomp.MultiDomain(c, x_cb, y_cb, q_cons=q, px=2, py=1, pz=2, z_cb=z_cb) as md:
        md.run(0, 5)
        got = md.download()
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))


def test_3d_split_and_strips():
    c = cases.shock_bubble_3d(N=52, steps=2, precision="fp64").replace(m=53, n=51, p=52)
    x_cb, y_cb, z_cb, q = preprocess.generate(c)
    subs = decomp.decompose(c, x_cb, y_cb, px=2, py=2, pz=2, z_cb=z_cb)
    assert len(subs) == 8 and subs[7].coords == (1, 1, 1) and subs[7].start == (27, 26, 27)
    assert subs[0].neighbors == {(0, 1): 1, (1, 1): 2, (2, 1): 4}
    s, o = subs[0], subs[4]  # z neighbours
    strip = decomp.halo_strip(s, q[s.window()], 2, 1, 3)
    assert strip.shape == (c.sys_size, 3, s.case.n + 1, s.case.m + 1)
    for k in range(3):
        assert np.array_equal(strip[:, k], q[:, o.start[2] - 1 - k, :s.case.n + 1, :s.case.m + 1])


@pytest.mark.gpu
def test_processor_boundary_context_refuses_the_fused_step():
    from microfc_gb300 import Simulation
    from microfc_gb300._lib import MfcError
    c = cases.sod_1d(m=99, steps=2)
    x_cb, _, _, q = preprocess.generate(c)
    s = decomp.decompose(c, x_cb, px=2)[0]
    with Simulation(s.case, s.x_cb, q_cons=np.ascontiguousarray(q[s.window()]), check=False) as sim:
        with pytest.raises(MfcError, match="mfc_gpu_rk_stage"):
            sim.tvd_rk(0)
