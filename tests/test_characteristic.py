"""WENO of the characteristic fields (mfc_gpu_set_reconstruction,
MFC_RECON_CHARACTERISTIC; case key char_decomp).

The reference reconstructs the primitive variables only
(src/simulation/m_weno.fpp:470-536), so the characteristic projection has no
reference output to match: the oracle restates it (Solver::weno with
char_decomp, pinned by tests/test_oracle_pins.py against the exact Sod
solution and a moving material interface) and the GPU path is required to be
bit-identical to the oracle, as the primitive FP64 path is.
"""
import numpy as np
import pytest

from conftest import rel_l1
from microfc_gb300 import Simulation, _lib, cases, preprocess

CASES = {
    "sod-weno5": lambda: cases.sod_1d(m=299, steps=200, dt=1e-4),
    "sod-weno3-rk2": lambda: cases.sod_1d(m=199, steps=100, dt=1e-4).replace(weno_order=3, time_stepper=2),
    "droplet": lambda: cases.shock_droplet_2d(nx=96, ny=64, steps=40),
    "droplet-bc-mix": lambda: cases.shock_droplet_2d(nx=64, ny=48, steps=30).replace(bc_x=(-2, -4), bc_y=(-1, -1)),
    "droplet-weno3": lambda: cases.shock_droplet_2d(nx=64, ny=48, steps=30).replace(weno_order=3),
    "bubble3d": lambda: cases.shock_bubble_3d(N=32, steps=10, precision="fp64"),
    "bubble3d-bc-mix": lambda: cases.shock_bubble_3d(N=28, steps=8, precision="fp64").replace(
        bc_y=(-2, -4), bc_z=(-1, -1)),
}


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_characteristic_weno_matches_the_oracle_bitwise(oracle_lib, name):
    case = CASES[name]().replace(char_decomp=True)
    x_cb, y_cb, z_cb, q = preprocess.generate(case)
    o = oracle_lib.Oracle(case, x_cb, y_cb, z_cb)
    o.set_state(q)
    dref = o.run(0, case.t_step_stop, case.dt)
    ref = o.get_state()
    with Simulation(case, x_cb, y_cb, z_cb, q_cons=q) as sim:
        dgot = sim.run(0, case.t_step_stop)
        assert sim.status() == 0
        got = sim.download()
    assert dgot == dref
    assert np.all(np.isfinite(got))
    assert rel_l1(got, ref).max() <= 1e-10
    assert np.count_nonzero(got != ref) == 0, f"{np.count_nonzero(got != ref)} values differ"
    # and it is a different reconstruction from the primitive one
    o2 = oracle_lib.Oracle(case.replace(char_decomp=False), x_cb, y_cb, z_cb)
    o2.set_state(q)
    o2.run(0, case.t_step_stop, case.dt)
    assert np.count_nonzero(o2.get_state() != ref) > 0


@pytest.mark.gpu
def test_characteristic_tile_variants_agree_and_switching_back_restores_primitive(oracle_lib):
    case = cases.shock_droplet_2d(nx=80, ny=48, steps=10)
    x_cb, y_cb, _, q = preprocess.generate(case)
    outs = []
    with Simulation(case, x_cb, y_cb, q_cons=q) as sim:
        sim.set_reconstruction("characteristic")
        v = 0
        while True:
            try:
                sim.select_variant(v)
            except _lib.MfcError:
                break
            sim.upload(q)
            sim.run(0, 10)
            outs.append(sim.download())
            v += 1
        sim.set_reconstruction("primitive")
        sim.upload(q)
        sim.run(0, 10)
        prim = sim.download()
    assert len(outs) >= 2
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])
    ref = oracle_lib.Oracle(case, x_cb, y_cb)
    ref.set_state(q)
    ref.run(0, 10, case.dt)
    assert np.array_equal(prim, ref.get_state())


@pytest.mark.gpu
def test_characteristic_refusals():
    split = cases.shock_droplet_2d(nx=64, ny=32, steps=2, precision="split")
    with Simulation(split) as sim:
        with pytest.raises(_lib.MfcError):
            sim.set_reconstruction("characteristic")
    visc = cases.shock_droplet_2d(nx=64, ny=32, steps=2).replace(re_shear=(100.0, 100.0))
    with Simulation(visc) as sim:
        with pytest.raises(_lib.MfcError):
            sim.set_reconstruction("characteristic")


def test_case_check_refuses_unsupported_characteristic_configurations():
    cases.shock_bubble_3d(N=32, steps=2, precision="fp64").replace(char_decomp=True).check()  # 3-D is taken
    with pytest.raises(ValueError):
        cases.shock_droplet_2d(nx=64, ny=32, steps=2, precision="split").replace(char_decomp=True).check()
    with pytest.raises(ValueError):
        cases.sod_1d(m=99, steps=2, dt=1e-4).replace(weno_order=1, char_decomp=True).check()
