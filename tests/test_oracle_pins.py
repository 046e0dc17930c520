"""Known-answer and invariant tests that pin the oracle.

The reference ships no tests, golden vectors or fixtures, and it cannot be
built here (Fortran), so the oracle is pinned by physics and numerics:
the exact Sod solution, the WENO5 order of accuracy, discrete conservation,
pressure/velocity equilibrium across a material interface, mirror symmetry,
and agreement of the two pre_process restatements.
"""
import numpy as np
import pytest

import exact_riemann
from microfc_gb300 import Case, Patch, cases, preprocess


def _run(oracle_lib, case, steps=None):
    x_cb, y_cb, z_cb, q = preprocess.generate(case)
    o = oracle_lib.Oracle(case, x_cb, y_cb, z_cb)
    o.set_state(q)
    o.run(0, case.t_step_stop if steps is None else steps, case.dt)
    return x_cb, y_cb, q, o.get_state()


def _sod_error(oracle_lib, m, char_decomp=False):
    t_end = 0.1
    dt = 2e-4 * 400 / (m + 1)
    steps = int(round(t_end / dt))
    case = cases.sod_1d(m=m, steps=steps, dt=dt).replace(char_decomp=char_decomp)
    x_cb, _, _, q = _run(oracle_lib, case)
    prim = preprocess.to_primitive(case, q)
    rho = q[0, 0, 0] + q[1, 0, 0]
    xc = 0.5 * (x_cb[1:] + x_cb[:-1])
    ex = exact_riemann.sample(xc, t_end, 0.5, (1.0, 0.0, 1.0), (0.125, 0.0, 0.1), 1.4)
    dx = 1.0 / (m + 1)
    return (np.abs(rho - ex[0]).sum() * dx, np.abs(prim[case.E_idx, 0, 0] - ex[2]).sum() * dx,
            np.abs(prim[case.mom_idx, 0, 0] - ex[1]).sum() * dx)


def test_sod_matches_exact_solution_and_converges(oracle_lib):
    e200 = _sod_error(oracle_lib, 199)
    e400 = _sod_error(oracle_lib, 399)
    # shock-capturing schemes converge at first order in L1 across discontinuities
    assert e400[0] < 2e-3 and e400[1] < 1.5e-3 and e400[2] < 4e-3, e400
    assert e400[0] < 0.75 * e200[0] and e400[1] < 0.75 * e200[1], (e200, e400)


def test_characteristic_weno_matches_exact_sod_solution_and_converges(oracle_lib):
    """WENO of the characteristic fields (no reference counterpart): the same
    known answer as the primitive reconstruction, at least as close to it."""
    e200 = _sod_error(oracle_lib, 199, char_decomp=True)
    e400 = _sod_error(oracle_lib, 399, char_decomp=True)
    prim = _sod_error(oracle_lib, 399)
    assert e400[0] < 2e-3 and e400[1] < 1.5e-3 and e400[2] < 4e-3, e400
    assert e400[0] < 0.75 * e200[0] and e400[1] < 0.75 * e200[1], (e200, e400)
    assert e400[0] <= 1.1 * prim[0] and e400[1] <= 1.1 * prim[1], (e400, prim)


def _moving_interface(**kw):
    gw, piw = cases.stiffened(6.12, 3.43e8)
    ga, pia = cases.stiffened(1.4)
    left = Patch(geometry=1, centroid=(0.25, 0, 0), length=(0.5, 0, 0), alpha_rho=(1000.0 * 0.999, 1.2 * 1e-3),
                 alpha=(0.999, 1e-3), vel=(50.0, 0, 0), pres=1e5)
    right = Patch(geometry=1, centroid=(0.75, 0, 0), length=(0.5, 0, 0), alpha_rho=(1000.0 * 1e-3, 1.2 * 0.999),
                  alpha=(1e-3, 0.999), vel=(50.0, 0, 0), pres=1e5)
    return Case(m=99, x_domain=(0.0, 1.0), dt=1e-5, t_step_stop=50, t_step_save=50, num_fluids=2,
                time_stepper=3, weno_order=5, weno_eps=1e-16, bc_x=(-3, -3), gammas=(gw, ga),
                pi_infs=(piw, pia), patches=[left, right], **kw)


def test_characteristic_weno_keeps_a_material_interface_in_equilibrium(oracle_lib):
    """A water/air interface moving with uniform p and u stays in equilibrium
    with the characteristic projection too, although its fields mix p, u and
    the partial densities."""
    case = _moving_interface(char_decomp=True)
    _, _, _, q = _run(oracle_lib, case)
    prim = preprocess.to_primitive(case, q)
    assert np.isfinite(q).all()
    assert np.abs(prim[case.mom_idx] / 50.0 - 1.0).max() < 1e-9
    assert np.abs(prim[case.E_idx] / 1e5 - 1.0).max() < 1e-6


def _smooth_case(m, weno_order, steps, dt):
    """Density wave advected at u=1 through a periodic box; p, u uniform."""
    g, pi = cases.stiffened(1.4)
    return Case(m=m, x_domain=(0.0, 1.0), dt=dt, t_step_stop=steps, t_step_save=steps, num_fluids=1,
                time_stepper=3, weno_order=weno_order, weno_eps=1e-16, bc_x=(-1, -1), gammas=(g,),
                pi_infs=(pi,), patches=[Patch(geometry=1, centroid=(0.5, 0, 0), length=(1.0, 0, 0),
                                              alpha_rho=(1.0,), alpha=(1.0,), vel=(1.0, 0, 0), pres=1.0)])


def _advect_error(oracle_lib, m):
    case = _smooth_case(m, 5, steps=0, dt=1.0)
    t_end = 0.1
    dx = 1.0 / (m + 1)
    # dt ~ dx^(5/3) keeps the RK3 error (dt^3) below WENO5's (dx^5)
    steps = int(round(t_end / (0.2 * dx * (32.0 * dx) ** (2.0 / 3.0))))
    dt = t_end / steps
    case = case.replace(dt=dt, t_step_stop=steps, t_step_save=steps)
    x_cb, _, _, q = preprocess.generate(case)
    # replace the density with a smooth wave (cell averages of 1 + 0.2 sin(2 pi x))
    a, b = x_cb[:-1], x_cb[1:]
    avg = 1.0 + 0.2 * (np.cos(2 * np.pi * a) - np.cos(2 * np.pi * b)) / (2 * np.pi * (b - a))
    gam = case.gammas[0]
    q[0, 0, 0] = avg
    q[1, 0, 0] = avg * 1.0
    q[2, 0, 0] = gam * 1.0 + 0.5 * avg
    o = oracle_lib.Oracle(case, x_cb)
    o.set_state(q)
    o.run(0, steps, dt)
    s = o.get_state()
    a2, b2 = a - t_end, b - t_end
    exact = 1.0 + 0.2 * (np.cos(2 * np.pi * a2) - np.cos(2 * np.pi * b2)) / (2 * np.pi * (b2 - a2))
    return np.abs(s[0, 0, 0] - exact).mean()


def test_weno5_is_high_order_on_smooth_flow(oracle_lib):
    e1 = _advect_error(oracle_lib, 31)
    e2 = _advect_error(oracle_lib, 63)
    order = np.log2(e1 / e2)
    assert order > 4.5, (e1, e2, order)


@pytest.mark.parametrize("nd", [1, 2, 3])
def test_periodic_box_conserves_mass_momentum_energy(oracle_lib, nd):
    if nd == 1:
        case = cases.sod_1d(m=99, steps=40, dt=2e-4).replace(bc_x=(-1, -1))
    elif nd == 2:
        case = cases.shock_droplet_2d(nx=40, ny=32, steps=30).replace(bc_x=(-1, -1), bc_y=(-1, -1))
    else:
        case = cases.shock_bubble_3d(N=28, steps=8, precision="fp64").replace(
            m=27, n=25, p=26, bc_x=(-1, -1), bc_y=(-1, -1), bc_z=(-1, -1))
    x_cb, y_cb, q0, q1 = _run(oracle_lib, case)
    for v in range(case.E_idx + 1):  # partial densities, momenta, energy are conserved
        s0, s1 = q0[v].sum(), q1[v].sum()
        scale = np.abs(q0[v]).sum() + np.abs(q1[v]).sum()
        assert abs(s1 - s0) <= 1e-12 * scale, (v, s0, s1)


def test_material_interface_keeps_pressure_and_velocity_uniform(oracle_lib):
    """A water/air interface moving with uniform p and u: the 5-equation
    model with HLLC and the alpha*div(u) term keeps p and u uniform."""
    gw, piw = cases.stiffened(6.12, 3.43e8)
    ga, pia = cases.stiffened(1.4)
    left = Patch(geometry=1, centroid=(0.25, 0, 0), length=(0.5, 0, 0), alpha_rho=(1000.0 * 0.999, 1.2 * 1e-3),
                 alpha=(0.999, 1e-3), vel=(50.0, 0, 0), pres=1e5)
    right = Patch(geometry=1, centroid=(0.75, 0, 0), length=(0.5, 0, 0), alpha_rho=(1000.0 * 1e-3, 1.2 * 0.999),
                  alpha=(1e-3, 0.999), vel=(50.0, 0, 0), pres=1e5)
    case = Case(m=99, x_domain=(0.0, 1.0), dt=1e-5, t_step_stop=50, t_step_save=50, num_fluids=2,
                time_stepper=3, weno_order=5, weno_eps=1e-16, bc_x=(-3, -3), gammas=(gw, ga),
                pi_infs=(piw, pia), patches=[left, right])
    _, _, _, q = _run(oracle_lib, case)
    prim = preprocess.to_primitive(case, q)
    assert np.abs(prim[case.mom_idx] / 50.0 - 1.0).max() < 1e-9
    assert np.abs(prim[case.E_idx] / 1e5 - 1.0).max() < 1e-6


def test_droplet_is_mirror_symmetric_about_the_midplane(oracle_lib):
    case = cases.shock_droplet_2d(nx=64, ny=32, steps=40)
    _, _, _, q = _run(oracle_lib, case)
    mirrored = q[:, :, ::-1, :].copy()
    mirrored[case.mom_idx + 1] *= -1.0
    scale = np.abs(q).reshape(q.shape[0], -1).max(axis=1)
    diff = np.abs(q - mirrored).reshape(q.shape[0], -1).max(axis=1)
    # mirrored cells see their stencils in reverse order (left- and right-face
    # coefficient sets, different summation order), so symmetry holds to
    # amplified round-off only
    assert np.all(diff <= 1e-8 * scale), diff / scale


@pytest.mark.parametrize("builder", [
    lambda: cases.sod_1d(m=199, steps=10, dt=1e-4),
    lambda: cases.shock_droplet_2d(nx=80, ny=40, steps=10),
    lambda: cases.shock_droplet_2d(nx=64, ny=64, steps=10, mach=2.0, radius=3e-3),
])
def test_preprocess_matches_oracle_restatement(oracle_lib, builder):
    case = builder()
    x_cb, y_cb, _, q = preprocess.generate(case)
    ox, oy, _, oq = oracle_lib.generate_ic(case)
    assert np.array_equal(x_cb, ox)
    if case.n > 0:
        assert np.array_equal(y_cb, oy)
    scale = np.abs(q).reshape(q.shape[0], -1).max(axis=1)[:, None, None, None]
    assert np.all(np.abs(q - oq) <= 1e-14 * scale)


def test_time_loop_trims_the_last_dt_like_the_cpu_build(oracle_lib):
    case = cases.sod_1d(m=49, steps=7, dt=0.1)
    x_cb, _, _, q = preprocess.generate(case)
    o = oracle_lib.Oracle(case, x_cb)
    o.set_state(q)
    dt_final = o.run(0, 7, 0.1)
    # replay p_main.fpp:196-318 in Python
    dt, mytime, t_step, final = 0.1, 0.0, 0, 7 * 0.1
    while True:
        mytime += dt
        if t_step == 7:
            break
        if mytime + dt >= final:
            dt = final - mytime
        t_step += 1
    assert dt_final == dt


def _shear_wave(nx=64, ny=25, re=100.0, amp=0.01, bulk=0.0, steps=250, dt=2e-3):
    """Periodic box, rho = p = 1 (gamma 1.4), v = amp sin(2 pi x): a viscous
    shear wave that decays as exp(-(2 pi)^2 t / (Re rho)) (tau = grad u / Re)."""
    g, pi = cases.stiffened(1.4)
    box = Patch(geometry=3, centroid=(0.5, 0.5 * ny / nx, 0), length=(1.0, ny / nx, 0),
                alpha_rho=(1.0,), alpha=(1.0,), vel=(0.0, 0.0, 0), pres=1.0)
    c = Case(m=nx - 1, n=ny - 1, x_domain=(0.0, 1.0), y_domain=(0.0, ny / nx), dt=dt, t_step_stop=steps,
             t_step_save=steps, num_fluids=1, time_stepper=3, weno_order=5, weno_eps=1e-16, bc_x=(-1, -1),
             bc_y=(-1, -1), gammas=(g,), pi_infs=(pi,), re_shear=(re,), re_bulk=(bulk,), patches=[box],
             name="shear_wave")
    x_cb, y_cb, _, q = preprocess.generate(c)
    xc = 0.5 * (x_cb[1:] + x_cb[:-1])
    v = amp * np.sin(2 * np.pi * xc)
    q[c.mom_idx + 1, 0] = v[None, :] * q[0, 0]               # rho v
    q[c.E_idx, 0] = q[c.E_idx, 0] + 0.5 * q[0, 0] * v[None, :] ** 2
    return c, x_cb, y_cb, q, xc


@pytest.mark.parametrize("weno_re_flux", [False, True], ids=["fd_gradients", "weno_gradients"])
def test_viscous_shear_wave_decays_at_the_kinematic_viscosity(oracle_lib, weno_re_flux):
    """Both gradient discretisations of the viscous stresses: the default
    finite differences and weno_Re_flux's WENO-reconstructed gradients."""
    c, x_cb, y_cb, q, xc = _shear_wave()
    c = c.replace(weno_re_flux=weno_re_flux)
    o = oracle_lib.Oracle(c, x_cb, y_cb)
    o.set_state(q)
    o.run(0, c.t_step_stop, c.dt)
    out = o.get_state()
    v = out[c.mom_idx + 1, 0] / out[0, 0]
    amp = 2 * np.mean(v * np.sin(2 * np.pi * xc)[None, :])
    t = c.t_step_stop * c.dt
    expect = 0.01 * np.exp(-(2 * np.pi) ** 2 * t / 100.0)
    assert amp == pytest.approx(expect, rel=5e-3), (amp, expect, 0.01)
    # only viscous heating (second order in the amplitude) drives any x-motion
    assert np.abs(out[c.mom_idx, 0]).max() < 1e-6
    # inviscid, the wave keeps its amplitude up to WENO dissipation
    ci = c.replace(re_shear=(0.0,))
    oi = oracle_lib.Oracle(ci, x_cb, y_cb)
    oi.set_state(q)
    oi.run(0, ci.t_step_stop, ci.dt)
    vi = oi.get_state()[c.mom_idx + 1, 0] / oi.get_state()[0, 0]
    assert 2 * np.mean(vi * np.sin(2 * np.pi * xc)[None, :]) == pytest.approx(0.01, rel=2e-3)


def test_bulk_viscosity_damps_an_acoustic_wave(oracle_lib):
    """1-D: u = amp sin(2 pi x) launches sound waves; bulk viscosity (tau =
    div u / Re_2) removes kinetic energy that the inviscid run keeps."""
    c2, x_cb, y_cb, q, xc = _shear_wave()
    ke = []
    for bulk in (0.0, 50.0):
        g, pi = cases.stiffened(1.4)
        box = Patch(geometry=1, centroid=(0.5, 0, 0), length=(1.0, 0, 0), alpha_rho=(1.0,), alpha=(1.0,),
                    vel=(0.0, 0, 0), pres=1.0)
        c = Case(m=99, x_domain=(0.0, 1.0), dt=1e-3, t_step_stop=200, t_step_save=200, num_fluids=1,
                 time_stepper=3, weno_order=5, weno_eps=1e-16, bc_x=(-1, -1), gammas=(g,), pi_infs=(pi,),
                 re_bulk=(bulk,), patches=[box])
        xb, _, _, q1 = preprocess.generate(c)
        xcc = 0.5 * (xb[1:] + xb[:-1])
        u = 0.01 * np.sin(2 * np.pi * xcc)
        q1[c.mom_idx, 0, 0] = u * q1[0, 0, 0]
        q1[c.E_idx, 0, 0] = q1[c.E_idx, 0, 0] + 0.5 * q1[0, 0, 0] * u ** 2
        o = oracle_lib.Oracle(c, xb)
        o.set_state(q1)
        o.run(0, c.t_step_stop, c.dt)
        s = o.get_state()
        ke.append(float(np.sum(0.5 * s[c.mom_idx, 0, 0] ** 2 / s[0, 0, 0])))
    assert ke[1] < 0.95 * ke[0], ke
