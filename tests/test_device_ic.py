"""The device initial-condition generator (pre_process on the GPU) against
the host pre_process and the oracle's restatement."""
import numpy as np
import pytest

from microfc_gb300 import cases, preprocess
from microfc_gb300.case import Case, Patch


def _mixed_case():
    """Line segments and an unsmoothed circle that alters only one patch."""
    g, pi = cases.stiffened(1.4)
    gw, piw = cases.stiffened(6.12, 3.43e8)
    bg = Patch(geometry=3, centroid=(0.5, 0.25, 0), length=(1.0, 0.5, 0),
               alpha_rho=(0.0, 1.0), alpha=(0.0, 1.0), vel=(0.1, -0.2, 0), pres=1.0)
    strip = Patch(geometry=3, centroid=(0.2, 0.25, 0), length=(0.2, 0.5, 0), alter_patch=(1,),
                  alpha_rho=(0.0, 2.0), alpha=(0.0, 1.0), vel=(0.5, 0.0, 0), pres=3.0)
    drop = Patch(geometry=2, centroid=(0.55, 0.2, 0), radius=0.12, alter_patch=(2,),
                 alpha_rho=(1000.0, 0.0), alpha=(1.0, 0.0), vel=(0.0, 0.0, 0), pres=1.0)
    drop2 = Patch(geometry=2, centroid=(0.2, 0.3, 0), radius=0.08, smoothen=True, smooth_patch_id=2,
                  smooth_coeff=0.8, alter_patch=(2,),
                  alpha_rho=(900.0, 0.0), alpha=(1.0, 0.0), vel=(0.0, 0.3, 0), pres=2.0)
    return Case(m=95, n=47, x_domain=(0.0, 1.0), y_domain=(0.0, 0.5), dt=1e-5, t_step_stop=2, t_step_save=2,
                num_fluids=2, time_stepper=3, weno_order=5, weno_eps=1e-16, bc_x=(-3, -3), bc_y=(-3, -3),
                gammas=(gw, g), pi_infs=(piw, pi), patches=[bg, strip, drop, drop2], name="mixed")


def _gallery_case():
    """Every 2-D patch geometry of the reference: a background rectangle,
    a smoothed sweep line and ellipse, an isentropic-vortex disc, a
    varcircle annulus and a 2-D analytical patch (pressure bump)."""
    g, pi = cases.stiffened(1.4)
    gw, piw = cases.stiffened(6.12, 3.43e8)
    air = dict(alpha_rho=(0.0, 1.2), alpha=(0.0, 1.0))
    water = dict(alpha_rho=(1000.0, 0.0), alpha=(1.0, 0.0))
    bg = Patch(geometry=3, centroid=(0.5, 0.25, 0), length=(1.0, 0.5, 0), vel=(0.1, 0.0, 0), pres=1e5, **air)
    sweep = Patch(geometry=4, centroid=(0.7, 0.25, 0), normal=(1.0, 0.5, 0), smoothen=True, smooth_patch_id=1,
                  smooth_coeff=0.5, alter_patch=(1,), vel=(0.4, -0.1, 0), pres=2e5,
                  alpha_rho=(0.0, 2.0), alpha=(0.0, 1.0))
    ell = Patch(geometry=5, centroid=(0.3, 0.25, 0), radii=(0.12, 0.06, 0), smoothen=True, smooth_patch_id=1,
                smooth_coeff=0.8, alter_patch=(1,), vel=(0.0, 0.0, 0), pres=1e5, **water)
    vortex = Patch(geometry=6, centroid=(0.3, 0.1, 0), radius=0.05, alter_patch=(1, 3),
                   vel=(0.0, 0.2, 0), pres=1.5e5, **water)
    ring = Patch(geometry=18, centroid=(0.8, 0.38, 0), radius=0.08, epsilon=0.03, alter_patch=(1, 2),
                 vel=(0.0, 0.0, 0), pres=3e5, **water)
    bump = Patch(geometry=7, centroid=(0.55, 0.25, 0), length=(0.12, 0.1, 0), alter_patch=(1, 2, 3),
                 vel=(0.0, 0.0, 0), pres=1e5, **air)
    return Case(m=99, n=49, x_domain=(0.0, 1.0), y_domain=(0.0, 0.5), dt=1e-7, t_step_stop=2, t_step_save=2,
                num_fluids=2, time_stepper=3, weno_order=5, weno_eps=1e-16, bc_x=(-3, -3), bc_y=(-3, -3),
                gammas=(gw, g), pi_infs=(piw, pi), patches=[bg, sweep, ell, vortex, ring, bump], name="gallery")


def _analytical_1d_case():
    """The reference's 1-D analytical patch (pressure bump) over a line segment."""
    g, pi = cases.stiffened(1.4)
    line = Patch(geometry=1, centroid=(0.5, 0, 0), length=(1.0, 0, 0), alpha_rho=(1.0,), alpha=(1.0,),
                 vel=(0.0,), pres=1.0)
    bump = Patch(geometry=15, centroid=(0.5, 0, 0), length=(0.5, 0, 0), alter_patch=(1,), alpha_rho=(1.0,),
                 alpha=(1.0,), vel=(0.2,), pres=1.0)
    return Case(m=199, x_domain=(0.0, 1.0), dt=1e-4, t_step_stop=2, t_step_save=2, num_fluids=1,
                time_stepper=3, weno_order=5, weno_eps=1e-16, bc_x=(-3, -3), gammas=(g,), pi_infs=(pi,),
                patches=[line, bump], name="analytical1d")


def _stretched_gallery_case():
    """The gallery on a grid stretched in x and y (m_grid.f90:72-90): fine
    in the middle band of each direction, coarse towards the ends."""
    return _gallery_case().replace(stretch_x=(10.0, 0.35, 0.65, 1), stretch_y=(10.0, 0.15, 0.35, 2),
                                   name="gallery_stretched")


def test_stretched_grid_follows_the_hyperbolic_map():
    c = _stretched_gallery_case()
    c.check()
    x_cb, y_cb, _ = preprocess.grid(c)
    assert x_cb[0] == 0.0 and np.all(np.diff(x_cb) > 0) and np.all(np.diff(y_cb) > 0)
    w = np.diff(x_cb)
    # finest cells in the band between x_a and x_b, coarser towards both ends
    assert 0.25 < x_cb[np.argmin(w)] < 0.75 and w[0] > 2 * w.min() and w[-1] > 2 * w.min()
    # one pass of the map at a few boundaries, in scalar arithmetic
    import math
    a, xa, xb = 10.0, 0.35, 0.65
    for i in (0, 17, 50, 100):
        u = i / 100.0
        f = u / a * (a + math.log(math.cosh(a * (u - xa))) + math.log(math.cosh(a * (u - xb)))
                     - 2.0 * math.log(math.cosh(a * (xb - xa) / 2.0)))
        assert math.isclose(x_cb[i], f, rel_tol=1e-14, abs_tol=1e-300)
    _, _, _, q = preprocess.generate(c)
    assert np.all(np.isfinite(q))


@pytest.mark.parametrize("change,msg", [
    (dict(stretch_x=(10.0, 0.6, 0.4, 1)), "stretch_x, x_a and x_b"),
    (dict(stretch_x=(10.0, 0.35, 0.65, 0)), "loops_x"),
    (dict(stretch_y=(-1e6, 0.15, 0.35, 1)), "stretch_y and a_y"),
    (dict(stretch_x=(-10.0, 0.35, 0.65, 1), x_domain=(-1.0, 1.0)), "x_domain%beg"),
])
def test_stretch_check_rejects_like_the_reference(change, msg):
    c = _gallery_case().replace(**change)
    with pytest.raises(ValueError, match=msg):
        c.check()
    with pytest.raises(ValueError, match="n and stretch_y"):
        _analytical_1d_case().replace(stretch_y=(10.0, 0.1, 0.2, 1)).check()


def test_stretch_keys_of_a_case_file():
    from microfc_gb300.case import Case as C
    d = {"m": 49, "n": 0, "dt": 1e-4, "t_step_stop": 2, "t_step_save": 2, "num_fluids": 1,
         "fluid_pp(1)%gamma": 2.5, "fluid_pp(1)%pi_inf": 0.0, "stretch_x": "T", "a_x": 4.0, "x_a": 0.3,
         "x_b": 0.7, "loops_x": 2, "patch_icpp(1)%geometry": 1, "patch_icpp(1)%x_centroid": 0.5,
         "patch_icpp(1)%length_x": 1.0, "patch_icpp(1)%pres": 1.0, "patch_icpp(1)%alpha_rho(1)": 1.0,
         "patch_icpp(1)%alpha(1)": 1.0, "patch_icpp(1)%normal(1)": 0.5, "patch_icpp(1)%radii(2)": 0.25,
         "patch_icpp(1)%epsilon": 0.125}
    c = C.from_dict(d)
    assert c.stretch_x == (4.0, 0.3, 0.7, 2) and c.stretch_y == ()
    pt = c.patches[0]
    assert pt.normal == (0.5, 0.0, 0.0) and pt.radii == (0.0, 0.25, 0.0) and pt.epsilon == 0.125


def test_every_geometry_covers_cells():
    """Each patch of the gallery owns cells of its own after all patches are
    laid (the smoothed ones where eta rounds to 1), and the analytical
    patches raise the pressure by the bump, most at their centroid."""
    c = _gallery_case()
    _, _, _, q = preprocess.generate(c)
    prim = preprocess.to_primitive(c, q)
    E = c.E_idx
    p = prim[E][0]
    assert p.max() > 3e5 * 0.99 and np.isclose(p.max(), 3e5)  # the ring
    # the 2-D analytical patch multiplies its pressure by 1 + 0.2 exp(-s^2/0.01)
    x_cb, y_cb, _ = preprocess.grid(c)
    i0 = np.searchsorted(x_cb, 0.55) - 1
    j0 = np.searchsorted(y_cb, 0.25) - 1
    s2 = (x_cb[i0 + 1] - 0.55) ** 2 + (y_cb[j0 + 1] - 0.25) ** 2
    assert np.isclose(p[j0, i0], 1e5 * (1 + 0.2 * np.exp(-s2 / 0.01)), rtol=1e-14)
    c1 = _analytical_1d_case()
    _, _, _, q1 = preprocess.generate(c1)
    p1 = preprocess.to_primitive(c1, q1)[c1.E_idx][0, 0]
    assert p1[:50].max() == 1.0 and p1[100] > 1.19 and np.argmax(p1) in (98, 99)


@pytest.mark.parametrize("builder", [_gallery_case, _analytical_1d_case, _stretched_gallery_case],
                         ids=["gallery2d", "analytical1d", "stretched"])
def test_preprocess_geometries_match_the_oracle(builder):
    import oracle
    c = builder()
    x_cb, y_cb, _, q = preprocess.generate(c)
    ox, oy, _, q_or = oracle.generate_ic(c)
    # log and cosh of the stretching: numpy's and the C library's may differ in the last bit
    assert np.allclose(x_cb, ox, rtol=4e-16, atol=0) and (y_cb is None or np.allclose(y_cb, oy, rtol=4e-16, atol=0))
    scale = np.abs(q).reshape(q.shape[0], -1).max(axis=1)[:, None, None, None]
    # on the stretched grid the last-bit differences of the cell centres are
    # amplified by the smoothed interfaces' slope (smooth_coeff/dx ~ 100)
    tol = 1e-13 if c.stretch_x else 2e-15
    assert np.all(np.abs(q - q_or) <= tol * scale)
    assert (q == q_or).mean() > 0.95


@pytest.mark.parametrize("patch,msg", [
    (Patch(geometry=4, centroid=(0.5, 0.2, 0), normal=(0.0, 0.0, 0)), "normal is zero"),
    (Patch(geometry=5, centroid=(0.5, 0.2, 0), radii=(0.1, 0.0, 0)), "semi-axes"),
    (Patch(geometry=8, centroid=(0.5, 0.2, 0), radius=0.1), "geometry 8"),
    (Patch(geometry=11, centroid=(0.5, 0.2, 0)), "geometry 11"),
])
def test_preprocess_refuses_bad_patches(patch, msg):
    c = _gallery_case()
    bad = c.replace(patches=[c.patches[0], patch.__class__(**{**patch.__dict__, "alter_patch": (1,),
                                                              "alpha_rho": (1.0, 0.0), "alpha": (1.0, 0.0)})])
    with pytest.raises(ValueError, match=msg):
        preprocess.generate(bad)


def test_device_patch_records_follow_the_case():
    c = _mixed_case()
    arr, dom = preprocess.device_patches(c)
    assert len(arr) == 4 and list(dom[:4]) == [0.0, 1.0, 0.0, 0.5]
    assert [arr[i].smooth_patch_id for i in range(4)] == [1, 2, 3, 2]
    assert [list(arr[i].alter_patch)[:4] for i in range(4)] == [[1, 0, 0, 0], [1, 1, 0, 0], [1, 0, 1, 0],
                                                                 [1, 0, 1, 0]]
    assert arr[3].smoothen == 1 and arr[2].smoothen == 0


def _cases():
    return [
        ("sod", cases.sod_1d(m=199, steps=2)),
        ("mixed", _mixed_case()),
        ("droplet", cases.shock_droplet_2d(nx=128, ny=64, steps=2)),
        ("bubble", cases.shock_bubble_3d(N=28, steps=2, precision="fp64")),
        ("gallery", _gallery_case()),
        ("analytical1d", _analytical_1d_case()),
        ("stretched", _stretched_gallery_case()),
    ]


@pytest.mark.gpu
@pytest.mark.parametrize("name,case", _cases(), ids=[n for n, _ in _cases()])
def test_device_initial_condition_matches_host_pre_process(name, case):
    from microfc_gb300 import Simulation
    _, _, _, q_host = preprocess.generate(case)
    with Simulation(case, ic="device") as sim:
        q_dev = sim.download()
        assert sim.launches == 1
    # tanh (smoothed patches) and exp (analytical patches) come from the
    # device's and the host's own libraries
    smoothed = any(p.smoothen or p.geometry in (7, 15) for p in case.patches)
    if not smoothed:
        assert np.array_equal(q_dev.view(np.uint64), q_host.view(np.uint64))
    else:
        # tanh of the smoothed interface may differ from the host libm in the last bit
        scale = np.abs(q_host).reshape(q_host.shape[0], -1).max(axis=1)
        err = np.abs(q_dev - q_host).reshape(q_host.shape[0], -1).max(axis=1)
        assert (err <= 2e-15 * scale + 1e-300).all(), err / scale
        same = (q_dev == q_host).mean()
        assert same > 0.9, same


@pytest.mark.gpu
@pytest.mark.parametrize("builder", [_mixed_case, _gallery_case, _analytical_1d_case, _stretched_gallery_case],
                         ids=["mixed", "gallery2d", "analytical1d", "stretched"])
def test_device_initial_condition_matches_the_oracle(builder):
    import oracle
    from microfc_gb300 import Simulation
    case = builder()
    _, _, _, q_or = oracle.generate_ic(case)
    with Simulation(case, ic="device") as sim:
        q_dev = sim.download()
    err = np.abs(q_dev - q_or).max(axis=(1, 2, 3)) / np.abs(q_or).max(axis=(1, 2, 3))
    assert (err <= 2e-15).all(), err


@pytest.mark.gpu
def test_device_initial_condition_then_steps_like_the_host_one():
    from microfc_gb300 import Simulation
    case = cases.sod_1d(m=199, steps=20)
    out = []
    for ic in ("host", "device"):
        with Simulation(case, ic=ic) as sim:
            sim.run(0, 20)
            out.append(sim.download())
    assert np.array_equal(out[0], out[1])


@pytest.mark.gpu
def test_ensemble_device_initial_condition():
    from microfc_gb300.ensemble import Ensemble, random_droplet_cases
    cl = random_droplet_cases(count=4, seed=3, steps=2, precision="fp64", sizes=(64, 128))
    with Ensemble(cl, ic="device") as ens:
        for i, c in enumerate(cl):
            _, _, _, q = preprocess.generate(c)
            d = ens.download(i)
            scale = np.abs(q).reshape(q.shape[0], -1).max(axis=1)
            err = np.abs(d - q).reshape(q.shape[0], -1).max(axis=1)
            assert (err <= 2e-15 * scale).all()


@pytest.mark.gpu
def test_device_initial_condition_rejects_bad_patches():
    from microfc_gb300 import Simulation
    from microfc_gb300._lib import MfcError
    case = cases.sod_1d(m=99, steps=2)
    bad = case.replace(patches=[Patch(geometry=2, centroid=(0.5, 0, 0), radius=0.1, alpha_rho=(1.0, 0.0),
                                      alpha=(1.0, 0.0), vel=(0.0, 0, 0), pres=1.0)])
    with Simulation(case) as sim:
        with pytest.raises(MfcError, match="geometry"):
            sim.generate_ic(bad)
    # 2-D: the device refuses what the host pre_process refuses
    g2 = _gallery_case()
    with Simulation(g2) as sim:
        for patch, msg in ((Patch(geometry=5, centroid=(0.5, 0.2, 0), radii=(0.1, 0.0, 0)), "semi-axes"),
                           (Patch(geometry=4, centroid=(0.5, 0.2, 0)), "normal is zero"),
                           (Patch(geometry=9, centroid=(0.5, 0.2, 0), length=(0.1, 0.1, 0.1)), "geometry")):
            p = Patch(**{**patch.__dict__, "alter_patch": (1,), "alpha_rho": (1.0, 0.0), "alpha": (1.0, 0.0)})
            with pytest.raises(MfcError, match=msg):
                sim.generate_ic(g2.replace(patches=[g2.patches[0], p]))
        sim.generate_ic(g2)  # the context still takes a valid set
