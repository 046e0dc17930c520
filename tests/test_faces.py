"""Standalone s_weno and s_hllc_riemann_solver (mfc_gpu_weno, mfc_gpu_riemann).

The oracle restates both routines over the face window (cells -1 .. s+1 of
the sweep direction, interior cells across it).  On the CPU the oracle's face
values and fluxes are checked to reassemble its own s_compute_rhs bit for bit
(so the window, the argument swap of m_rhs.fpp:545-556 and the bc -4 states
are the ones the RHS uses); on the GPU the two entry points are compared with
the oracle bit for bit (plain FP64, the fused path's arithmetic).
"""
import ctypes

import numpy as np
import pytest

from microfc_gb300 import Simulation, _lib, cases, preprocess

CASES = {
    "droplet": lambda: cases.shock_droplet_2d(nx=64, ny=40, steps=2),
    "droplet-bc-riemann": lambda: cases.shock_droplet_2d(nx=48, ny=40, steps=2).replace(bc_x=(-4, -4), bc_y=(-2, -4)),
    "droplet-periodic-weno3": lambda: cases.shock_droplet_2d(nx=48, ny=40, steps=2).replace(bc_x=(-1, -1),
                                                                                           weno_order=3),
    "sod": lambda: cases.sod_1d(m=199, steps=2, dt=1e-4),
    "sod-weno1": lambda: cases.sod_1d(m=99, steps=2, dt=1e-4).replace(weno_order=1, bc_x=(-2, -4)),
    "bubble3d": lambda: cases.shock_bubble_3d(N=32, steps=2, precision="fp64"),
}


def _axis(case, d):
    return 3 - d


def _assemble_rhs(case, o, x_cb, y_cb, z_cb, q):
    """flux divergence + alpha*div(u) of m_rhs.fpp:564-654 from the oracle's
    standalone WENO and Riemann solves, in the oracle's operation order."""
    S, nf = case.sys_size, case.num_fluids
    ab = case.adv_idx
    rhs = np.zeros(case.shape)
    for d, cb in enumerate((x_cb, y_cb, z_cb)[:case.num_dims]):
        vl, vr = o.weno(d)
        flux, src = o.riemann(d, vr, vl)
        ax = _axis(case, d)
        s1 = flux.shape[ax] - 1
        lo = [slice(None)] * 4
        hi = [slice(None)] * 4
        lo[ax], hi[ax] = slice(0, s1), slice(1, s1 + 1)
        shp = [1, 1, 1, 1]
        shp[ax] = s1
        inv = (1.0 / (cb[1:] - cb[:-1])).reshape(shp)
        df = flux[tuple(lo)] - flux[tuple(hi)]
        rhs = inv * df if d == 0 else rhs + inv * df
        ds = src[tuple(hi[1:])] - src[tuple(lo[1:])]
        for f in range(nf):
            rhs[ab + f] = rhs[ab + f] + inv[0] * q[ab + f] * ds
    return rhs


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_faces_reassemble_its_rhs(oracle_lib, name):
    case = CASES[name]()
    x_cb, y_cb, z_cb, q = preprocess.generate(case)
    o = oracle_lib.Oracle(case, x_cb, y_cb, z_cb)
    o.set_state(q)
    rhs_ref, _ = o.compute_rhs()
    rhs = _assemble_rhs(case, o, x_cb, y_cb, z_cb, q)
    assert np.array_equal(rhs, rhs_ref), np.abs(rhs - rhs_ref).max()


def test_entry_points_refuse_null_arguments():
    L = _lib.load()
    buf = (ctypes.c_double * 8)()
    assert L.mfc_gpu_weno(None, 0, buf, buf) == _lib.MFC_ERR_INVALID
    assert L.mfc_gpu_riemann(None, 0, buf, buf, buf, buf) == _lib.MFC_ERR_INVALID


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_weno_and_riemann_match_the_oracle_bitwise(oracle_lib, name):
    case = CASES[name]()
    x_cb, y_cb, z_cb, q = preprocess.generate(case)
    o = oracle_lib.Oracle(case, x_cb, y_cb, z_cb)
    o.set_state(q)
    with Simulation(case, x_cb, y_cb, z_cb, q_cons=q) as sim:
        for d in range(case.num_dims):
            vl, vr = sim.s_weno(d)
            rl, rr = o.weno(d)
            assert np.array_equal(vl, rl) and np.array_equal(vr, rr), f"dir {d}: WENO values differ"
            # the reference's argument order: qL_prim_rs = vR, qR_prim_rs = vL
            flux, src = sim.s_hllc_riemann_solver(d, vr, vl)
            rflux, rsrc = o.riemann(d, vr, vl)
            assert np.array_equal(flux, rflux), f"dir {d}: fluxes differ"
            assert np.array_equal(src, rsrc), f"dir {d}: interface velocities differ"


@pytest.mark.gpu
def test_faces_refuse_split_precision_and_bad_directions():
    case = cases.shock_droplet_2d(nx=64, ny=32, steps=2, precision="split")
    with Simulation(case) as sim:
        with pytest.raises(_lib.MfcError):
            sim.s_weno(0)
    with Simulation(case.replace(precision="fp64")) as sim:
        with pytest.raises(_lib.MfcError):
            sim.s_weno(2)
