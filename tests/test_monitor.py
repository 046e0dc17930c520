"""The fused ICFL monitor (the reference's run-time information) and the
CFL-driven time step built on it."""
import numpy as np
import pytest

from microfc_gb300 import Simulation, cases, preprocess
from microfc_gb300._lib import MfcError

pytestmark = pytest.mark.gpu


def icfl_numpy(case, q, dt, cbs):
    """ICFL of m_data_output.fpp:197-242 evaluated on a state."""
    prim = preprocess.to_primitive(case, q)
    nf = case.num_fluids
    rho = sum(prim[f] for f in range(nf))
    gam = sum(prim[case.adv_idx + f] * case.gammas[f] for f in range(nf))
    pinf = sum(prim[case.adv_idx + f] * case.pi_infs[f] for f in range(nf))
    c = np.sqrt(((gam + 1.0) * prim[case.E_idx] + pinf) / (gam * rho))
    rate = np.zeros_like(c)
    for d in range(case.num_dims):
        w = np.diff(np.asarray(cbs[d]))
        shp = [1, 1, 1]
        shp[2 - d] = -1
        rate = np.maximum(rate, (np.abs(prim[case.mom_idx + d]) + c) / w.reshape(shp))
    return dt * rate.max()


@pytest.mark.parametrize("nd", [1, 2, 3])
def test_icfl_matches_the_reference_formula(nd):
    if nd == 1:
        c = cases.sod_1d(m=199, steps=5, dt=1e-4)
    elif nd == 2:
        c = cases.shock_droplet_2d(nx=128, ny=64, steps=5)
    else:
        c = cases.shock_bubble_3d(N=28, steps=5, precision="fp64").replace(m=27, n=25, p=26)
    x, y, z, q = preprocess.generate(c)
    with Simulation(c, x, y, z, q_cons=q) as sim:
        sim.set_monitor(True)
        for step in range(3):
            sim.icfl(reset=True)
            sim.tvd_rk(step)
            got = sim.icfl()
            ref = icfl_numpy(c, sim.download(), c.dt, (x, y, z))
            assert got == pytest.approx(ref, rel=1e-12)


def test_monitor_changes_no_result():
    c = cases.shock_droplet_2d(nx=96, ny=48, steps=6)
    x, y, _, q = preprocess.generate(c)
    out = []
    for on in (False, True):
        with Simulation(c, x, y, q_cons=q) as sim:
            sim.set_monitor(on)
            sim.run(0, 6)
            out.append(sim.download())
    assert np.array_equal(out[0], out[1])


def test_run_fails_like_the_reference_when_icfl_exceeds_one():
    c = cases.shock_droplet_2d(nx=96, ny=48, steps=1, cfl=1.2)
    with Simulation(c) as sim:
        sim.set_monitor(True)
        with pytest.raises(MfcError, match="ICFL is greater than 1.0"):
            sim.run(0, 1)


def test_cfl_driven_steps_run_at_the_requested_cfl():
    c = cases.shock_droplet_2d(nx=128, ny=64, steps=40, cfl=0.1)
    x, y, _, q = preprocess.generate(c)
    with Simulation(c, x, y, q_cons=q) as sim:
        dt, t = sim.run_cfl(20, cfl=0.3, dt=c.dt)
        assert t > 0 and dt > c.dt  # started at CFL 0.1
        final = sim.download()
    assert icfl_numpy(c, final, dt, (x, y)) == pytest.approx(0.3, rel=1e-9)


@pytest.mark.parametrize("nd", [1, 2, 3])
def test_monitor_flags_a_non_physical_pressure(nd):
    """The stability monitor sets MFC_FLAG_NEG_PRESSURE when a cell's squared
    sound speed is not positive: here the energy of a block of water cells
    is zeroed, which puts their pressure below the stiffened gas's limit
    (-gamma pi_inf; an ideal gas's pressure goes to zero or below); the same
    case without the change leaves the status clear."""
    from microfc_gb300._lib import MFC_FLAG_NEG_PRESSURE
    if nd == 1:
        c = cases.sod_1d(m=199, steps=1, dt=1e-4)
        water = (slice(None), slice(None), slice(90, 110))
    elif nd == 2:
        c = cases.shock_droplet_2d(nx=96, ny=48, steps=1)
        water = (slice(None), slice(20, 28), slice(34, 42))  # inside the droplet
    else:
        c = cases.shock_bubble_3d(N=28, steps=1, precision="fp64").replace(m=27, n=25, p=26)
        water = (slice(8, 18), slice(8, 18), slice(8, 18))  # around the bubble (both gases ideal)
    x, y, z, q = preprocess.generate(c)
    for broken in (False, True):
        qq = q.copy()
        if broken:
            qq[(c.E_idx,) + water] = 0.0
        with Simulation(c, x, y, z, q_cons=qq) as sim:
            sim.set_monitor(True)
            sim.tvd_rk(0)
            flags = sim.status(clear=True)
        assert bool(flags & MFC_FLAG_NEG_PRESSURE) == broken, (nd, broken, flags)
