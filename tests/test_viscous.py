"""Viscous terms on the GPU against the oracle: bit for bit in FP64 (1-D
and 2-D, several boundary conditions), within tolerance in split
precision; switching the viscosity off restores the inviscid kernels."""
import numpy as np
import pytest

from conftest import rel_l1
from microfc_gb300 import cases, preprocess

pytestmark = pytest.mark.gpu


def _shear_wave(nx=64, ny=25, re=100.0, bulk=0.0, steps=40, dt=2e-3, precision="fp64"):
    from test_oracle_pins import _shear_wave as sw
    c, x_cb, y_cb, q, _ = sw(nx, ny, re, 0.01, bulk, steps, dt)
    return c.replace(precision=precision), x_cb, y_cb, q


def _viscous_droplet(bc=(-3, -3), precision="fp64", steps=20):
    c = cases.shock_droplet_2d(nx=96, ny=48, steps=steps, precision=precision)
    # water (fluid 1) and air (fluid 2), Re = 1 / mu in the case's units, raised
    # so that the viscous terms are visible within a few steps on this grid
    return c.replace(bc_x=bc, bc_y=bc, re_shear=(1.0 / 1e-1, 1.0 / 2e-3), re_bulk=(0.0, 1.0 / 5e-3))


def _gpu_and_oracle(oracle_lib, case, x_cb, y_cb, q, steps):
    from microfc_gb300 import Simulation
    with Simulation(case, x_cb, y_cb, q_cons=q) as sim:
        sim.run(0, steps)
        got = sim.download()
    o = oracle_lib.Oracle(case.replace(precision="fp64"), x_cb, y_cb)
    o.set_state(q)
    o.run(0, steps, case.dt)
    return got, o.get_state()


WRF = pytest.mark.parametrize("wrf", [False, True], ids=["fd_gradients", "weno_Re_flux"])


@WRF
def test_shear_wave_matches_oracle_bitwise(oracle_lib, wrf):
    c, x_cb, y_cb, q = _shear_wave(re=100.0, bulk=40.0)
    c = c.replace(weno_re_flux=wrf)
    got, ref = _gpu_and_oracle(oracle_lib, c, x_cb, y_cb, q, c.t_step_stop)
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))


@WRF
@pytest.mark.parametrize("bc", [(-3, -3), (-2, -2), (-1, -1), (-4, -4), (-2, -3)])
def test_viscous_droplet_matches_oracle_bitwise(oracle_lib, bc, wrf):
    c = _viscous_droplet(bc).replace(weno_re_flux=wrf)
    x_cb, y_cb, _, q = preprocess.generate(c)
    got, ref = _gpu_and_oracle(oracle_lib, c, x_cb, y_cb, q, c.t_step_stop)
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), rel_l1(got, ref)


@WRF
def test_viscous_sod_1d_matches_oracle_bitwise(oracle_lib, wrf):
    c = cases.sod_1d(m=199, steps=40, dt=1e-4).replace(re_shear=(50.0, 80.0), re_bulk=(30.0, 0.0),
                                                        weno_re_flux=wrf)
    x_cb, _, _, q = preprocess.generate(c)
    got, ref = _gpu_and_oracle(oracle_lib, c, x_cb, None, q, c.t_step_stop)
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))


def test_viscosity_changes_the_result_and_can_be_switched_off(oracle_lib):
    from microfc_gb300 import Simulation
    c = _viscous_droplet()
    x_cb, y_cb, _, q = preprocess.generate(c)
    inv = c.replace(re_shear=(), re_bulk=())
    with Simulation(inv, x_cb, y_cb, q_cons=q) as sim:
        sim.run(0, c.t_step_stop)
        q_inv = sim.download()
    with Simulation(c, x_cb, y_cb, q_cons=q) as sim:
        sim.set_viscosity((0.0, 0.0), (0.0, 0.0))
        sim.run(0, c.t_step_stop)
        assert np.array_equal(sim.download(), q_inv)
    with Simulation(c, x_cb, y_cb, q_cons=q) as sim:
        sim.run(0, c.t_step_stop)
        assert rel_l1(sim.download(), q_inv)[c.mom_idx] > 1e-8


@WRF
def test_split_precision_viscous_error_bounded(oracle_lib, wrf):
    c = _viscous_droplet(precision="split").replace(weno_re_flux=wrf)
    x_cb, y_cb, _, q = preprocess.generate(c)
    got, ref = _gpu_and_oracle(oracle_lib, c, x_cb, y_cb, q, c.t_step_stop)
    err = rel_l1(got, ref)
    assert err[[0, 1, c.adv_idx, c.adv_idx + 1]].max() <= 1e-3, err


def test_gated_viscous_error_bounded_and_the_viscous_terms_act(oracle_lib):
    """The learned gate with the viscous terms: within the gated form's bar
    (density and volume-fraction L1 <= 1e-3) of the FP64 oracle, and
    different from the inviscid gated run."""
    from microfc_gb300 import Simulation, gate
    params = gate.load()
    c = _viscous_droplet(precision="gated")
    x_cb, y_cb, _, q = preprocess.generate(c)
    out = {}
    for name, case in (("viscous", c), ("inviscid", c.replace(re_shear=(), re_bulk=()))):
        with Simulation(case, x_cb, y_cb, q_cons=q) as sim:
            sim.set_gate(params)
            sim.run(0, c.t_step_stop)
            assert sim.status() == 0
            out[name] = sim.download()
    o = oracle_lib.Oracle(c.replace(precision="fp64"), x_cb, y_cb)
    o.set_state(q)
    o.run(0, c.t_step_stop, c.dt)
    err = rel_l1(out["viscous"], o.get_state())
    assert err[[0, 1, c.adv_idx, c.adv_idx + 1]].max() <= 1e-3, err
    assert rel_l1(out["viscous"], out["inviscid"])[c.mom_idx] > 1e-8


def test_viscous_refusals():
    from microfc_gb300 import Simulation
    from microfc_gb300._lib import MfcError
    b = cases.shock_bubble_3d(N=28, steps=2, precision="fp64")
    with Simulation(b) as sim:
        with pytest.raises(MfcError, match="1-D and 2-D"):
            sim.set_viscosity((10.0, 10.0))


def test_weno_re_flux_changes_the_result_and_refusals(oracle_lib):
    """The two gradient discretisations give different results; the WENO
    gradients need a viscous context."""
    from microfc_gb300 import Simulation
    from microfc_gb300._lib import MfcError
    c = _viscous_droplet(steps=10)
    x_cb, y_cb, _, q = preprocess.generate(c)
    out = []
    for wrf in (False, True):
        with Simulation(c.replace(weno_re_flux=wrf), x_cb, y_cb, q_cons=q) as sim:
            sim.run(0, 10)
            out.append(sim.download())
            if wrf:
                assert sim.launches == 10 * 3 * (1 + 4)  # four preparation kernels per stage
    assert rel_l1(out[1], out[0])[c.mom_idx] > 1e-10
    with Simulation(cases.shock_droplet_2d(nx=96, ny=48, steps=2), x_cb, y_cb, q_cons=q) as sim:
        with pytest.raises(MfcError, match="viscous context"):
            sim.set_viscous_gradients(True)
