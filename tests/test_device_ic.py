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
    ]


@pytest.mark.gpu
@pytest.mark.parametrize("name,case", _cases(), ids=[n for n, _ in _cases()])
def test_device_initial_condition_matches_host_pre_process(name, case):
    from microfc_gb300 import Simulation
    _, _, _, q_host = preprocess.generate(case)
    with Simulation(case, ic="device") as sim:
        q_dev = sim.download()
        assert sim.launches == 1
    smoothed = any(p.smoothen for p in case.patches)
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
def test_device_initial_condition_matches_the_oracle():
    import oracle
    from microfc_gb300 import Simulation
    case = _mixed_case()
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
