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
                    assert strip.shape[3] == o.case.m + 3  # widened by the two x ghost cells
                    assert np.array_equal(strip[:, 0, k, 1:-1], ref)


def test_2d_y_strips_forward_the_diagonal_cells():
    """The first and last columns of a 2-D y strip are the sender's x ghost
    cells: across an x processor boundary the diagonal neighbour's cells (what
    the receiver's viscous corner gradients read), elsewhere the x boundary
    condition's ghost value."""
    c = cases.shock_droplet_2d(nx=128, ny=64, steps=2).replace(bc_x=(-2, -3))
    x_cb, y_cb, _, q = preprocess.generate(c)
    q = q + np.arange(q.size, dtype=np.float64).reshape(q.shape) * 1e-3  # distinct values everywhere
    subs = decomp.decompose(c, x_cb, y_cb, px=2, py=2)
    H = 3
    for s in subs:
        sx, sy = s.start[0], s.start[1]
        rows = slice(sy, sy + s.case.n + 1)
        left = q[:, 0, rows, sx - 1] if (0, 0) in s.neighbors else None
        right = q[:, 0, rows, sx + s.case.m + 1] if (0, 1) in s.neighbors else None
        for (d, side), peer in s.neighbors.items():
            if d != 1:
                continue
            strip = decomp.halo_strip(s, q[s.window()], 1, side, H, x_ghosts=(left, right))
            for k in range(H):
                gy = sy + k if side == 0 else sy + s.case.n - k
                if left is not None:
                    assert np.array_equal(strip[:, 0, k, 0], q[:, 0, gy, sx - 1])
                else:  # symmetry: the mirrored edge cell with the x-momentum flipped
                    want = q[:, 0, gy, sx].copy()
                    want[c.num_fluids] *= -1
                    assert np.array_equal(strip[:, 0, k, 0], want)
                if right is not None:
                    assert np.array_equal(strip[:, 0, k, -1], q[:, 0, gy, sx + s.case.m + 1])
                else:  # extrapolation: the edge cell
                    assert np.array_equal(strip[:, 0, k, -1], q[:, 0, gy, sx + s.case.m])


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
@pytest.mark.parametrize("kind", ["sod", "sod_periodic", "droplet_2x2", "droplet_split_4x1", "droplet_gated_2x2",
                                  "droplet_gated_periodic_3x2"])
def test_subdomains_on_one_gpu_reproduce_the_whole_domain(kind):
    """Gated cases included: the decisions a step's first stage stores at
    the ghost positions beside a processor boundary come from the halo, so
    the later stages read what the undecomposed run reads there."""
    from microfc_gb300 import Simulation, gate
    params = None
    if kind.startswith("sod"):
        c = cases.sod_1d(m=199, steps=20, dt=2e-4)
        if kind == "sod_periodic":
            c = c.replace(bc_x=(-1, -1))
        px, py = 3, 1
    else:
        prec = "split" if "split" in kind else "gated" if "gated" in kind else "fp64"
        c = cases.shock_droplet_2d(nx=128, ny=64, steps=20, precision=prec)
        if "periodic" in kind:
            c = c.replace(bc_x=(-1, -1), bc_y=(-1, -1))
        px, py = (2, 2) if "2x2" in kind else (3, 2) if "3x2" in kind else (4, 1)
        params = gate.load() if prec == "gated" else None
    x_cb, y_cb, _, q = preprocess.generate(c)
    with Simulation(c, x_cb, y_cb, q_cons=q) as sim:
        if params is not None:
            sim.set_gate(params)
        sim.run(0, 20)
        ref = sim.download()
    with decomp.MultiDomain(c, x_cb, y_cb, q_cons=q, px=px, py=py) as md:
        if params is not None:
            md.set_gate(params)
        md.run(0, 20)
        got = md.download()
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))


def _viscous_case(kind):
    """A viscous case and its process grid.  "dyadic" grids have cell
    boundaries k * 2^-j, so every cell centre and centre spacing is exact."""
    if kind.startswith("sod"):
        c = cases.sod_1d(m=255, steps=20, dt=5e-5).replace(re_shear=(50.0, 80.0), re_bulk=(30.0, 0.0))
        x_cb, _, _, q = preprocess.generate(c)
        return c, x_cb, None, q, 3, 1
    prec = kind.split("_")[-1]
    c = cases.shock_droplet_2d(nx=128, ny=64, steps=20, precision=prec)
    c = c.replace(re_shear=(1.0 / 1e-1, 1.0 / 2e-3), re_bulk=(0.0, 1.0 / 5e-3))
    if "periodic" in kind:
        c = c.replace(bc_x=(-1, -1), bc_y=(-1, -1))
    x_cb, y_cb, _, q = preprocess.generate(c)
    if "dyadic" in kind:  # same number of cells, spacing 2^-13 instead of 0.02/128
        x_cb = np.arange(-1, c.m + 1, dtype=np.float64) * 2.0 ** -13
        y_cb = np.arange(-1, c.n + 1, dtype=np.float64) * 2.0 ** -13
    return c, x_cb, y_cb, q, int(kind[0]), int(kind[2])


def _whole_and_split(c, x_cb, y_cb, q, px, py):
    from microfc_gb300 import Simulation
    assert c.viscous
    with Simulation(c, x_cb, y_cb, q_cons=q) as sim:
        sim.run(0, 20)
        ref = sim.download()
    with decomp.MultiDomain(c, x_cb, y_cb, q_cons=q, px=px, py=py) as md:
        md.run(0, 20)
        got = md.download()
    return got, ref


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["2x2_dyadic_fp64", "3x2_dyadic_split", "4x1_dyadic_fp64", "sod3_fp64",
                                  "2x2_periodic_dyadic_fp64"])
def test_viscous_subdomains_reproduce_the_whole_domain(kind):
    """Viscous terms across processor boundaries, including the corner cells
    of the cross derivatives that come from the diagonal neighbours: bit for
    bit where the cell centres are exact (dyadic grids; the 1-D Sod grid has
    256 cells on [0, 1])."""
    got, ref = _whole_and_split(*_viscous_case(kind))
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))


@pytest.mark.gpu
def test_viscous_subdomains_on_a_general_grid():
    """On a general grid a subdomain builds its ghost cell centre from the
    neighbour's width, x_cc(-1) = x_cc(0) - (dx(0) + dx(-1))/2, as the
    reference's s_populate_grid_variables_buffers does after the width
    exchange; the undecomposed run takes the interior centre x_cb + dx/2.
    The two centre spacings differ in the last bit, so the viscous gradients
    next to a processor boundary do too: the runs agree to round-off."""
    from conftest import rel_l1
    got, ref = _whole_and_split(*_viscous_case("4x1_fp64"))
    err = rel_l1(got, ref)
    assert err.max() <= 1e-10, err
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
