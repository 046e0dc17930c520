"""The opt-in contracted FP64 variant (MFC_PREC_FP64_FMA, 2-D WENO5).

Its kernels are the bit-faithful FP64 kernels compiled with multiply-add
contraction, so they round differently from the contraction-off oracle the
plain path is pinned to, as a default-flag CPU build of the reference does.
The test measures that distance at the configuration-2 size and length
(1024 x 512, 100 steps) against both oracle builds: within the FP64 bar
(relative L1 <= 1e-10) in every conserved field but the y-momentum, which is
round-off noise at that time (see tests/test_reference_flags.py), and not
bit-identical (the contraction took place).
"""
import numpy as np
import pytest

from conftest import rel_l1
from microfc_gb300 import Simulation, cases, preprocess

TOL_FP64 = 1e-10


def _names(case):
    nf, nd = case.num_fluids, case.num_dims
    return ([f"alpha_rho{i + 1}" for i in range(nf)] + ["mom_x", "mom_y", "mom_z"][:nd] + ["E"]
            + [f"alpha{i + 1}" for i in range(nf)])


@pytest.mark.gpu
def test_contracted_variant_small_case_close_to_the_oracle(oracle_lib):
    case = cases.shock_droplet_2d(nx=128, ny=64, steps=50)
    x_cb, y_cb, _, q = preprocess.generate(case)
    with Simulation(case.replace(precision="fp64_fma"), x_cb, y_cb, q_cons=q) as sim:
        sim.run(0, 50)
        assert sim.status() == 0
        got = sim.download()
    o = oracle_lib.Oracle(case, x_cb, y_cb)
    o.set_state(q)
    o.run(0, 50, case.dt)
    ref = o.get_state()
    err = rel_l1(got, ref)
    others = [i for i in range(case.sys_size) if i != case.mom_idx + 1]
    assert np.all(np.isfinite(got))
    assert err[others].max() <= TOL_FP64, err
    assert np.count_nonzero(got != ref) > 0


@pytest.mark.gpu
@pytest.mark.slow
def test_contracted_variant_full_size_against_both_oracle_builds(oracle_lib):
    case = cases.shock_droplet_2d(nx=1024, ny=512, steps=100)
    x_cb, y_cb, _, q = preprocess.generate(case)
    with Simulation(case.replace(precision="fp64_fma"), x_cb, y_cb, q_cons=q) as sim:
        sim.tune(3)
        sim.run(0, 100)
        assert sim.status() == 0
        got = sim.download()
    others = [i for i in range(case.sys_size) if i != case.mom_idx + 1]
    for build in ("exact", "native"):
        o = oracle_lib.Oracle(case, x_cb, y_cb, build=build)
        o.set_state(q)
        o.run(0, 100, case.dt)
        ref = o.get_state()
        err = rel_l1(got, ref)
        print(f"contracted FP64 vs {build} oracle, per-field rel L1:", dict(zip(_names(case), err.tolist())))
        assert err[others].max() <= TOL_FP64, (build, err)
        # the round-off field against the momentum's scale
        mom_y = case.mom_idx + 1
        dv = np.abs(got[mom_y] - ref[mom_y]).sum() / np.abs(ref[case.mom_idx]).sum()
        print(f"  sum|d(rho v)| / sum|rho u| = {dv:.3e}")
        assert dv <= TOL_FP64
