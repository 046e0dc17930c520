"""Parity of the CUDA path (through the C ABI) with the oracle.

The bar, from the plain FP64 contract: relative L1 <= 1e-10 in every
conserved field after the stated number of steps.  The split-precision path
is checked against the FP64 oracle at <= 1e-3 in density and volume fraction.
"""
import numpy as np
import pytest

from conftest import rel_l1
from microfc_gb300 import Simulation, cases, preprocess

pytestmark = pytest.mark.gpu

TOL_FP64 = 1e-10
TOL_SPLIT = 1e-3


def _oracle_run(oracle_lib, case, x_cb, y_cb, q, steps):
    o = oracle_lib.Oracle(case, x_cb, y_cb)
    o.set_state(q)
    dt = o.run(0, steps, case.dt)
    return o.get_state(), dt


def _gpu_run(case, x_cb, y_cb, q, steps):
    with Simulation(case, x_cb, y_cb, q_cons=q) as sim:
        dt = sim.run(0, steps)
        assert sim.status() == 0
        return sim.download(), dt


def _check(case, got, ref, tol, bitwise=True):
    """Per-field relative L1 within tol; the plain FP64 path follows the
    reference's operation order without FMA contraction, so it is also
    required to be bit-identical to the oracle."""
    err = rel_l1(got, ref)
    assert np.all(np.isfinite(got))
    assert err.max() <= tol, f"{case.name}: per-field rel L1 {err}"
    if bitwise:
        ndiff = int(np.count_nonzero(got != ref))
        assert ndiff == 0, f"{case.name}: {ndiff} values differ from the oracle (rel L1 {err})"
    return err


@pytest.mark.parametrize("weno_order", [5, 3, 1])
@pytest.mark.parametrize("time_stepper", [3, 2, 1])
def test_sod_1d_matches_oracle(oracle_lib, weno_order, time_stepper):
    case = cases.sod_1d(m=399, steps=100, dt=1e-4).replace(weno_order=weno_order, time_stepper=time_stepper)
    x_cb, _, _, q = preprocess.generate(case)
    ref, dref = _oracle_run(oracle_lib, case, x_cb, None, q, 100)
    got, dgot = _gpu_run(case, x_cb, None, q, 100)
    assert dgot == dref
    _check(case, got, ref, TOL_FP64)


def test_sod_1d_config_size_100_steps(oracle_lib):
    case = cases.sod_1d()  # 1000 cells, dt 5e-5
    x_cb, _, _, q = preprocess.generate(case)
    ref, _ = _oracle_run(oracle_lib, case, x_cb, None, q, 100)
    got, _ = _gpu_run(case, x_cb, None, q, 100)
    _check(case, got, ref, TOL_FP64)


@pytest.mark.parametrize("nx,ny", [(64, 32), (100, 60)])
def test_droplet_2d_small_matches_oracle(oracle_lib, nx, ny):
    case = cases.shock_droplet_2d(nx=nx, ny=ny, steps=50)
    x_cb, y_cb, _, q = preprocess.generate(case)
    ref, _ = _oracle_run(oracle_lib, case, x_cb, y_cb, q, 50)
    got, _ = _gpu_run(case, x_cb, y_cb, q, 50)
    _check(case, got, ref, TOL_FP64)


@pytest.mark.parametrize("bc", [(-1, -1), (-2, -2), (-4, -4), (-2, -3)])
def test_droplet_2d_boundary_conditions(oracle_lib, bc):
    case = cases.shock_droplet_2d(nx=48, ny=32, steps=30).replace(bc_x=bc, bc_y=bc)
    x_cb, y_cb, _, q = preprocess.generate(case)
    ref, _ = _oracle_run(oracle_lib, case, x_cb, y_cb, q, 30)
    got, _ = _gpu_run(case, x_cb, y_cb, q, 30)
    _check(case, got, ref, TOL_FP64)


def test_compute_rhs_matches_oracle(oracle_lib):
    case = cases.shock_droplet_2d(nx=64, ny=48, steps=10)
    x_cb, y_cb, _, q = preprocess.generate(case)
    o = oracle_lib.Oracle(case, x_cb, y_cb)
    o.set_state(q)
    o.run(0, 5, case.dt)  # develop some structure first
    q5 = o.get_state()
    rref, pref = o.compute_rhs(0)
    with Simulation(case, x_cb, y_cb, q_cons=q5) as sim:
        rhs, prim = sim.s_compute_rhs()
    assert np.array_equal(prim, pref)
    assert np.array_equal(rhs, rref)


@pytest.mark.parametrize("name", ["sod_1d_200_weno5_rk3", "sod_1d_200_weno3_rk2", "droplet_2d_48x32_weno5_rk3",
                                  "droplet_2d_40x40_periodic", "droplet_2d_40x32_symmetry_riemann",
                                  "viscous_droplet_2d_40x32_weno_re_flux"])
def test_matches_golden_fixture(name):
    """The CUDA path reproduces the committed oracle fixtures bit for bit."""
    import os
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "golden"))
    import make_golden
    g = np.load(os.path.join(here, "golden", name + ".npz"))
    case = make_golden.GOLDEN[name][0]()
    y_cb = g["y_cb"] if case.n > 0 else None
    got, dt_final = _gpu_run(case, g["x_cb"], y_cb, g["q0"], int(g["steps"]))
    assert dt_final == float(g["dt_final"])
    _check(case, got, g["q"], TOL_FP64)


@pytest.mark.slow
def test_droplet_2d_full_size_100_steps(oracle_lib):
    """The headline configuration (1024x512) after 100 steps."""
    case = cases.shock_droplet_2d()
    x_cb, y_cb, _, q = preprocess.generate(case)
    ref, _ = _oracle_run(oracle_lib, case, x_cb, y_cb, q, 100)
    got, _ = _gpu_run(case, x_cb, y_cb, q, 100)
    err = _check(case, got, ref, TOL_FP64)
    print("per-field rel L1 after 100 steps:", err)


def test_split_precision_error_bounded(oracle_lib):
    case = cases.shock_droplet_2d(nx=256, ny=128, steps=100)
    x_cb, y_cb, _, q = preprocess.generate(case)
    ref, _ = _oracle_run(oracle_lib, case, x_cb, y_cb, q, 100)
    got, _ = _gpu_run(case.replace(precision="split"), x_cb, y_cb, q, 100)
    err = rel_l1(got, ref)
    assert not np.array_equal(got, ref)  # the split path really ran in FP32
    nf = case.num_fluids
    dens_alpha = list(range(nf)) + [case.adv_idx + f for f in range(nf)]
    assert np.all(np.isfinite(got))
    assert err[dens_alpha].max() <= TOL_SPLIT, err
    print("split precision per-field rel L1:", err)


def _stretch(cb, amp):
    """A smooth, monotone non-uniform grid with the same end points."""
    a, b = cb[0], cb[-1]
    s = (cb - a) / (b - a)
    return a + (b - a) * (s + amp / (2 * np.pi) * np.sin(2 * np.pi * s))


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_stretched_grid_matches_oracle(oracle_lib, prec):
    """Grid-dependent WENO coefficients (s_compute_weno_coefficients on a
    non-uniform grid): every cell has its own coefficient record."""
    case = cases.shock_droplet_2d(nx=96, ny=64, steps=30)
    x_cb, y_cb, _, q = preprocess.generate(case)
    x_cb, y_cb = _stretch(x_cb, 0.15), _stretch(y_cb, 0.1)
    assert np.ptp(np.diff(x_cb)) > 0.2 * np.diff(x_cb).mean()
    ref, _ = _oracle_run(oracle_lib, case, x_cb, y_cb, q, 30)
    with Simulation(case.replace(precision=prec), x_cb, y_cb, q_cons=q) as sim:
        assert sim.set_uniform_coefficients(True) == 0  # no shared record on this grid
        sim.run(0, 30)
        assert sim.status() == 0
        got = sim.download()
    if prec == "fp64":
        _check(case, got, ref, TOL_FP64)
    else:
        err = rel_l1(got, ref)
        nf = case.num_fluids
        dens_alpha = list(range(nf)) + [case.adv_idx + f for f in range(nf)]
        assert np.all(np.isfinite(got)) and err[dens_alpha].max() <= TOL_SPLIT, err


def test_pre_process_stretched_grid_runs_like_the_oracle(oracle_lib):
    """A case file's stretch_x/stretch_y (m_grid.f90:72-90): the device
    initial condition on the context's stretched cell boundaries, then 10
    plain FP64 steps, against the oracle on the host pre_process's grid and
    state."""
    import dataclasses
    case = cases.shock_droplet_2d(nx=96, ny=64, steps=10).replace(
        stretch_x=(12.0, 0.006, 0.010, 1), stretch_y=(12.0, 0.004, 0.006, 1))
    # the map stretches the domain to about [0, 0.04] x [0, 0.018]: the
    # background patch covers it
    bg = dataclasses.replace(case.patches[0], centroid=(0.025, 0.0125, 0.0), length=(0.05, 0.025, 0.0))
    case = case.replace(patches=[bg] + list(case.patches[1:]), dt=1.8e-8)  # CFL 0.3 on the finest cells
    case.check()
    x_cb, y_cb, _, q = preprocess.generate(case)
    ref, _ = _oracle_run(oracle_lib, case, x_cb, y_cb, q, 10)
    with Simulation(case, ic="device") as sim:
        q_dev = sim.download()
        scale = np.abs(q).reshape(q.shape[0], -1).max(axis=1)[:, None, None, None]
        assert np.all(np.abs(q_dev - q) <= 2e-15 * scale)  # tanh of the smoothed droplet
    with Simulation(case, x_cb, y_cb, q_cons=q) as sim:
        sim.run(0, 10)
        assert sim.status() == 0
        got = sim.download()
    _check(case, got, ref, TOL_FP64)


def _bubble(nx, ny, nz, steps, **kw):
    c = cases.shock_bubble_3d(N=max(nx, ny, nz), steps=steps, precision="fp64")
    c = c.replace(m=nx - 1, n=ny - 1, p=nz - 1, **kw)
    return c


@pytest.mark.parametrize("bc", [(-3, -3), (-1, -1), (-2, -4)])
def test_bubble_3d_matches_oracle(oracle_lib, bc):
    """3-D (the z-extension): directional sweeps vs the oracle, bit for bit."""
    case = _bubble(32, 28, 26, 8, bc_x=bc, bc_y=bc, bc_z=bc)
    x_cb, y_cb, z_cb, q = preprocess.generate(case)
    o = oracle_lib.Oracle(case, x_cb, y_cb, z_cb)
    o.set_state(q)
    o.run(0, 8, case.dt)
    ref = o.get_state()
    with Simulation(case, x_cb, y_cb, z_cb, q_cons=q) as sim:
        sim.run(0, 8)
        got = sim.download()
        assert sim.launches == 3 * 3 * 8
    _check(case, got, ref, TOL_FP64)


def test_bubble_3d_compute_rhs_matches_oracle(oracle_lib):
    case = _bubble(28, 26, 30, 4)
    x_cb, y_cb, z_cb, q = preprocess.generate(case)
    o = oracle_lib.Oracle(case, x_cb, y_cb, z_cb)
    o.set_state(q)
    o.run(0, 3, case.dt)
    q3 = o.get_state()
    rref, pref = o.compute_rhs(0)
    with Simulation(case, x_cb, y_cb, z_cb, q_cons=q3) as sim:
        rhs, prim = sim.s_compute_rhs()
    assert np.array_equal(prim, pref)
    assert np.array_equal(rhs, rref)


@pytest.mark.parametrize("bc", [(-3, -3), (-2, -4)])
def test_bubble_3d_split_precision_error_bounded(oracle_lib, bc):
    """Split 3-D sweeps against the FP64 oracle; (-2, -4) puts reflecting
    walls at the start of every direction (the y and z sweeps negate the
    stored normal velocity of the mirrored cells)."""
    case = _bubble(48, 40, 40, 20, bc_x=bc, bc_y=bc, bc_z=bc)
    x_cb, y_cb, z_cb, q = preprocess.generate(case)
    o = oracle_lib.Oracle(case, x_cb, y_cb, z_cb)
    o.set_state(q)
    o.run(0, 20, case.dt)
    ref = o.get_state()
    with Simulation(case.replace(precision="split"), x_cb, y_cb, z_cb, q_cons=q) as sim:
        sim.run(0, 20)
        got = sim.download()
    err = rel_l1(got, ref)
    dens_alpha = [0, 1, case.adv_idx, case.adv_idx + 1]
    assert np.all(np.isfinite(got)) and not np.array_equal(got, ref)
    assert err[dens_alpha].max() <= TOL_SPLIT, err


@pytest.mark.parametrize("prec", ["fp64", "split"])
def test_status_flags_nan_and_clear(prec):
    """A NaN planted in the uploaded state is flagged by the stage kernel and
    reported as an error by the run loop (the reference aborts on NaN)."""
    from microfc_gb300._lib import MfcError, MFC_FLAG_NAN
    case = cases.sod_1d(m=99, steps=2, dt=1e-4).replace(precision=prec)
    x_cb, _, _, q = preprocess.generate(case)
    q[0, 0, 0, 50] = np.nan
    with Simulation(case, x_cb, q_cons=q) as sim:
        with pytest.raises(MfcError):
            sim.run(0, 2)
        assert sim.status(clear=True) & MFC_FLAG_NAN
        assert sim.status() == 0


def test_launch_count_is_stages_times_steps():
    case = cases.sod_1d(m=99, steps=7, dt=1e-4)
    x_cb, _, _, q = preprocess.generate(case)
    with Simulation(case, x_cb, q_cons=q) as sim:
        sim.run(0, 7)
        assert sim.launches == 3 * 7


@pytest.mark.slow
@pytest.mark.parametrize("precision", ["fp64", "split", "gated"])
def test_full_size_periodic_box_conserves_mass_momentum_energy(precision):
    """A size-independent property at the headline size: the droplet at
    1024x512 in a periodic box, 100 steps on the GPU.  The partial
    densities, momenta and energy are conserved (fluxes telescope), to FP64
    round-off in the plain path and to the round-off of the FP32 increments
    on the split and gated paths; the volume fractions carry a
    non-conservative source and are not summed."""
    from microfc_gb300 import Simulation, gate
    import os
    if precision == "gated" and not os.path.exists(gate.WEIGHTS_FILE):
        pytest.skip("no trained gate parameters")
    case = cases.shock_droplet_2d().replace(bc_x=(-1, -1), bc_y=(-1, -1), precision=precision)
    with Simulation(case, ic="device") as sim:
        if precision == "gated":
            sim.set_gate(gate.load())
        q0 = sim.download()
        sim.run(0, 100)
        assert sim.status() == 0
        q1 = sim.download()
    tol = 1e-13 if precision == "fp64" else 1e-9
    mom = slice(case.mom_idx, case.mom_idx + case.num_dims)
    # a momentum component that is round-off noise (rho v before the shock
    # reaches the droplet) is measured against the momentum's own scale
    mom_scale = np.abs(q0[mom]).sum() + np.abs(q1[mom]).sum()
    for v in range(case.E_idx + 1):
        s0, s1 = q0[v].sum(), q1[v].sum()
        scale = mom_scale if case.mom_idx <= v < case.E_idx else np.abs(q0[v]).sum() + np.abs(q1[v]).sum()
        assert abs(s1 - s0) <= tol * scale, (precision, v, s0, s1, abs(s1 - s0) / scale)
    assert not np.array_equal(q0, q1)


@pytest.mark.slow
@pytest.mark.parametrize("precision,n", [("split", 256), ("fp64", 128)])
def test_3d_periodic_box_conserves_mass_momentum_energy(precision, n):
    """The same property on the 3-D sweeps at the config-3 size (split,
    256^3) and at 128^3 in plain FP64, 10 steps in a periodic box."""
    from microfc_gb300 import Simulation
    case = cases.shock_bubble_3d(N=n, precision=precision).replace(bc_x=(-1, -1), bc_y=(-1, -1), bc_z=(-1, -1))
    with Simulation(case, ic="device") as sim:
        q0 = sim.download()
        sim.run(0, 10)
        assert sim.status() == 0
        q1 = sim.download()
    tol = 1e-13 if precision == "fp64" else 1e-9
    mom = slice(case.mom_idx, case.mom_idx + case.num_dims)
    mom_scale = np.abs(q0[mom]).sum() + np.abs(q1[mom]).sum()
    for v in range(case.E_idx + 1):
        s0, s1 = q0[v].sum(), q1[v].sum()
        scale = mom_scale if case.mom_idx <= v < case.E_idx else np.abs(q0[v]).sum() + np.abs(q1[v]).sum()
        assert abs(s1 - s0) <= tol * scale, (precision, v, s0, s1, abs(s1 - s0) / scale)
    assert not np.array_equal(q0, q1)


@pytest.mark.slow
@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_state_beyond_2_31_elements_conserves(precision):
    """A maximum-size case: the droplet at 24576x12800 (315 M cells, 2.2e9
    values per register -- element offsets beyond 2^31 -- 17.6 GB per
    register, ~71 GB on the device), periodic, 2 steps: the kernels' 64-bit
    addressing keeps the partial densities, momenta and energy conserved.
    The sums are taken one variable at a time (2.5 GB on the host)."""
    from microfc_gb300 import Simulation
    # dt of the 1024x512 grid scaled with the finer spacing (y); the host
    # pre_process that would pick it is skipped: the initial condition is
    # made on the device
    case = cases.shock_droplet_2d(nx=24576, ny=12800, steps=2, dt=4.0e-9 * 512 / 12800).replace(
        bc_x=(-1, -1), bc_y=(-1, -1), precision=precision)
    assert case.sys_size * case.cells > 2 ** 31
    nx, ny = case.m + 1, case.n + 1
    buf = np.empty((ny, nx))

    def sums():
        out = []
        for v in range(case.E_idx + 1):
            sim.download_var(v, buf, nx)
            out.append((buf.sum(), np.abs(buf).sum()))
        # the far corner of the last variable, updated by the last tiles
        sim.download_var(case.sys_size - 1, buf, nx)
        return out, buf[-4:, -4:].copy()

    with Simulation(case, ic="device") as sim:
        s0, c0 = sums()
        sim.run(0, 2)
        assert sim.status() == 0
        s1, c1 = sums()
    tol = 1e-13 if precision == "fp64" else 1e-9
    mom = range(case.mom_idx, case.E_idx)
    mom_scale = sum(s0[v][1] + s1[v][1] for v in mom)
    for v in range(case.E_idx + 1):
        scale = mom_scale if v in mom else s0[v][1] + s1[v][1]
        assert abs(s1[v][0] - s0[v][0]) <= tol * scale, (precision, v, s0[v], s1[v])
    assert np.all(np.isfinite(c1))


@pytest.mark.slow
def test_3d_state_beyond_2_31_elements_conserves():
    """The same on the 3-D sweeps: the bubble at 648^3 in split precision
    (272 M cells, 2.2e9 values per register, 17.4 GB each; ~105 GB on the
    device with the sweeps' work area, whose primitive segment reaches 4.4e9
    values), periodic, 2 steps."""
    from microfc_gb300 import Simulation
    N = 648
    # dt of the 128^3 grid at CFL 0.3, scaled with the spacing
    case = cases.shock_bubble_3d(N=N, steps=2, precision="split", dt=6.7374e-4 * 128 / N).replace(
        bc_x=(-1, -1), bc_y=(-1, -1), bc_z=(-1, -1))
    assert case.sys_size * case.cells > 2 ** 31
    buf = np.empty((N, N, N))

    def sums():
        out = []
        for v in range(case.E_idx + 1):
            sim.download_var(v, buf, N, N * N)
            out.append((buf.sum(), np.abs(buf).sum()))
        return out

    with Simulation(case, ic="device") as sim:
        s0 = sums()
        sim.run(0, 2)
        assert sim.status() == 0
        s1 = sums()
    mom = range(case.mom_idx, case.E_idx)
    mom_scale = sum(s0[v][1] + s1[v][1] for v in mom)
    for v in range(case.E_idx + 1):
        scale = mom_scale if v in mom else s0[v][1] + s1[v][1]
        assert abs(s1[v][0] - s0[v][0]) <= 1e-9 * scale, (v, s0[v], s1[v])
    assert s1 != s0
