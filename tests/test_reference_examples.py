"""The reference's own example cases, end to end.

tests/golden/reference_cases/<example>.json is the case dictionary that
examples/<example>/case.py of the reference prints (written by
tests/golden/make_reference_cases.py from the reference's scripts): the
1-D Sod, Kapila and vacuum shock tubes, the 2-D advection, shear-layer,
shock-bubble, shock-droplet and viscous cases.  They pin the case-file
handling against inputs the reference itself produces, and they run the
hot path on the reference's own physics, grids, boundary conditions and
time steps rather than on cases written here.

CPU: every fixture parses (Case.from_dict), passes the input checks
(m_checker), carries the dictionary's values (the viscous example's
weno_Re_flux = T included: its viscous stresses take WENO-reconstructed
velocity gradients), and the Python initial
condition equals the oracle's C restatement of pre_process bit for bit (to
the last bit of tanh where a patch is smoothed).

GPU: each example runs through the p_main loop (mfc_gpu_run, last-step dt
trim included) and is compared bit for bit with the oracle stepped the same
way: the examples whose complete run costs the oracle a few seconds run to
their own t_step_stop (Sod 1000 steps, vacuum 15000, Kapila 6025, advection
1000, viscous 10, shock-droplet 10 on its 5001 x 741 grid); the shear layer
(400000 steps) and the shock-bubble (38487) run their first 300 steps.  The
split-precision path is run on the same examples for 100 steps against the
same FP64 oracle at the split contract's bar: relative L1 <= 1e-3 in the
partial densities and volume fractions, and at the same bar in the energy
and in the momentum measured as a vector.  The Sod example also runs
through the driver command (pre_process, saves, data files) as a user
would run it.
"""
import glob
import json
import os

import numpy as np
import pytest

from conftest import rel_l1
from microfc_gb300 import Case, Simulation, preprocess

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = os.path.join(HERE, "golden", "reference_cases")
NAMES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(FIXTURES, "*.json")))
TOL_SPLIT = 1e-3

# steps of the GPU-vs-oracle run: None = the example's own t_step_stop
FULL_RUN = {"1D_sodshocktube": None, "1D_vacuum": None, "1D_kapilashocktube": None, "2D_advection": None,
            "2D_viscous": None, "2D_shockdroplet": None, "2D_shearlayer": 300, "2D_shockbubble": 300}


def _load(name):
    with open(os.path.join(FIXTURES, name + ".json")) as f:
        return json.load(f)


def _case(name) -> Case:
    return Case.from_dict(_load(name))


def _grids(case, x_cb, y_cb, z_cb):
    return x_cb, (y_cb if case.n > 0 else None), (z_cb if case.p > 0 else None)


def _assert_same_initial_condition(case, q, q_ref):
    """Bit for bit, except where a smoothed patch (tanh) or an analytical one
    (exp) takes a transcendental from a different library: numpy's, the C
    library's and the device's may differ in the last bit."""
    if not any(p.smoothen or p.geometry in (7, 15) for p in case.patches):
        assert np.array_equal(q.view(np.uint64), q_ref.view(np.uint64))
        return
    scale = np.abs(q_ref).reshape(q_ref.shape[0], -1).max(axis=1)
    err = np.abs(q - q_ref).reshape(q_ref.shape[0], -1).max(axis=1)
    assert (err <= 2e-15 * scale).all(), err / scale
    assert (q == q_ref).mean() > 0.95


def test_every_reference_example_is_present():
    assert NAMES == ["1D_kapilashocktube", "1D_sodshocktube", "1D_vacuum", "2D_advection", "2D_shearlayer",
                     "2D_shockbubble", "2D_shockdroplet", "2D_viscous"]
    assert set(FULL_RUN) == set(NAMES)


@pytest.mark.parametrize("name", NAMES)
def test_reference_example_parses_checks_and_keeps_its_values(name):
    d = _load(name)
    c = Case.from_dict(d)
    c.check()
    assert c.weno_re_flux == (d.get("weno_Re_flux") == "T")
    nf = int(d["num_fluids"])
    assert (c.m, c.n, c.p) == (d["m"], d["n"], d.get("p", 0))
    assert c.num_fluids == nf and c.weno_order == d["weno_order"] and c.time_stepper == d["time_stepper"]
    assert c.dt == d["dt"] and c.weno_eps == d["weno_eps"]
    assert (c.t_step_start, c.t_step_stop, c.t_step_save) == (d["t_step_start"], d["t_step_stop"], d["t_step_save"])
    assert c.bc_x == (d["bc_x%beg"], d["bc_x%end"])
    if c.n > 0:
        assert c.bc_y == (d["bc_y%beg"], d["bc_y%end"])
        assert c.y_domain == (d["y_domain%beg"], d["y_domain%end"])
    assert c.x_domain == (d["x_domain%beg"], d["x_domain%end"])
    for i in range(nf):
        assert c.gammas[i] == d[f"fluid_pp({i + 1})%gamma"]
        assert c.pi_infs[i] == d[f"fluid_pp({i + 1})%pi_inf"]
        assert c.re_shear[i] == d.get(f"fluid_pp({i + 1})%Re(1)", 0.0)
        assert c.re_bulk[i] == d.get(f"fluid_pp({i + 1})%Re(2)", 0.0)
    assert c.viscous == any(k.startswith("fluid_pp(") and "%Re(" in k for k in d)
    assert len(c.patches) == d["num_patches"]
    for i, p in enumerate(c.patches, start=1):
        assert p.geometry == d[f"patch_icpp({i})%geometry"]
        assert p.pres == d[f"patch_icpp({i})%pres"]
        for f in range(nf):
            assert p.alpha_rho[f] == d[f"patch_icpp({i})%alpha_rho({f + 1})"]
            assert p.alpha[f] == d[f"patch_icpp({i})%alpha({f + 1})"]
        for a in range(1 + (c.n > 0)):
            assert p.vel[a] == d[f"patch_icpp({i})%vel({a + 1})"]
        assert p.alter_patch == tuple(sorted(
            int(k[len(f"patch_icpp({i})%alter_patch("):-1]) for k, v in d.items()
            if k.startswith(f"patch_icpp({i})%alter_patch(") and v == "T"))


@pytest.mark.parametrize("name", NAMES)
def test_reference_example_initial_condition_matches_the_oracle_restatement(name, oracle_lib):
    c = _case(name)
    x, y, z, q = preprocess.generate(c)
    ox, oy, oz, oq = oracle_lib.generate_ic(c)
    assert np.array_equal(x, ox)
    if c.n > 0:
        assert np.array_equal(y, oy)
    _assert_same_initial_condition(c, q, oq)
    assert np.isfinite(q).all()


def _oracle_run(oracle_lib, c, grids, q, stop):
    o = oracle_lib.Oracle(c, *grids)
    o.set_state(q)
    dt = o.run(c.t_step_start, stop, c.dt)
    return o.get_state(), dt


@pytest.mark.gpu
@pytest.mark.parametrize("name", [pytest.param(n, marks=pytest.mark.slow) if n == "2D_shockdroplet" else n
                                  for n in NAMES])
def test_reference_example_runs_bitwise_like_the_oracle(name, oracle_lib):
    c = _case(name)
    stop = FULL_RUN[name] or c.t_step_stop
    x, y, z, q = preprocess.generate(c)
    grids = _grids(c, x, y, z)
    with Simulation(c, *grids, q_cons=q) as sim:
        dt = sim.run(c.t_step_start, stop)
        assert sim.status() == 0
        got = sim.download()
    ref, dt_ref = _oracle_run(oracle_lib, c, grids, q, stop)
    assert dt == dt_ref
    assert np.isfinite(got).all()
    assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), rel_l1(got, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in NAMES if n != "2D_shockdroplet"])
def test_reference_example_split_precision_within_the_contract(name, oracle_lib):
    c = _case(name).replace(precision="split")
    stop = c.t_step_start + 100
    x, y, z, q = preprocess.generate(c)
    grids = _grids(c, x, y, z)
    with Simulation(c, *grids, q_cons=q) as sim:
        sim.run(c.t_step_start, stop)
        assert sim.status() == 0
        got = sim.download()
    ref, _ = _oracle_run(oracle_lib, c.replace(precision="fp64"), grids, q, stop)
    err = rel_l1(got, ref)
    nf, nd = c.num_fluids, c.num_dims
    mom = slice(c.mom_idx, c.mom_idx + nd)
    mom_err = np.abs(got[mom] - ref[mom]).sum() / np.abs(ref[mom]).sum()
    print(name, "split vs FP64 oracle, per-field rel L1:", err.tolist(), "momentum vector:", mom_err)
    assert np.isfinite(got).all()
    # the contract's fields: partial densities and volume fractions
    assert err[:nf].max() <= TOL_SPLIT and err[c.adv_idx:c.adv_idx + nf].max() <= TOL_SPLIT, err
    # and the rest at the same bar: the energy, and the momentum as a vector
    # (a component that starts at zero, the y-momentum of the shear layer and
    # of the viscous case, is round-off-sized against its own scale)
    assert err[c.E_idx] <= TOL_SPLIT and mom_err <= TOL_SPLIT, (err, mom_err)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_reference_example_device_initial_condition_matches_the_host(name):
    c = _case(name)
    x, y, z, q = preprocess.generate(c)
    with Simulation(c, *_grids(c, x, y, z), ic="device") as sim:
        got = sim.download()
    _assert_same_initial_condition(c, got, q)


@pytest.mark.gpu
def test_reference_example_through_the_driver_command(tmp_path, oracle_lib, capsys):
    """The reference's Sod example as a user runs it: its case dictionary
    into `python -m microfc_gb300.driver` (pre_process, then the p_main loop
    with its saves every t_step_save steps and the D/ text files); the data
    file of the last save equals the oracle's state bit for bit."""
    from microfc_gb300 import driver, io
    name = "1D_sodshocktube"
    c = _case(name)
    driver.main([os.path.join(FIXTURES, name + ".json"), "--dir", str(tmp_path)])
    res = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert res["saved"] == list(range(c.t_step_save, c.t_step_stop + 1, c.t_step_save))
    assert (tmp_path / "D" / f"cons.1.00.{c.t_step_stop:06d}.dat").exists()
    _, _, _, q = io.read_data_files(str(tmp_path), c.t_step_stop, c)
    x, y, z, q0 = preprocess.generate(c)
    ref, _ = _oracle_run(oracle_lib, c, _grids(c, x, y, z), q0, c.t_step_stop)
    assert np.array_equal(q.view(np.uint64), ref.view(np.uint64))
