"""FP64 parity against a CPU build with the reference's Release flags.

The reference's CPU build is gfortran -O3 -march/-mcpu=native with the
compiler's default floating-point contraction (fused multiply-adds wherever
the target has them).  The parity oracle is built with contraction off so
that it gives the same bits on every host, and the plain FP64 GPU path is
bit-identical to it.  Here the same oracle sources are built with the
Release flags (oracle/Makefile, ``libmfc_oracle_native.so``) and the GPU
path is compared with that build on the shock-droplet at 1024 x 512 after
100 steps, the size and length of the FP64 contract (relative L1 <= 1e-10 per
conserved field).

What the comparison shows: the partial densities, the volume fractions, the
total energy and the x-momentum agree to <= 1e-10.  The y-momentum does not:
after 100 steps the shock has not reached the droplet and the y-momentum is
round-off noise of order 1e-9 of the x-momentum, so any change of rounding --
here the contraction of a multiply and an add into one FMA -- changes it by
a relative amount of order one.  The test asserts the bar on every field but
the y-momentum and prints that field's figure, asserts the y-momentum's
difference against the momentum scale (sum |rho v - rho v_ref| / sum |rho u|)
at the same bar, and checks that the two CPU builds really differ (so that
the comparison is not vacuous).
"""
import numpy as np
import pytest

from conftest import rel_l1
from microfc_gb300 import Simulation, cases, preprocess

TOL_FP64 = 1e-10


@pytest.mark.gpu
@pytest.mark.slow
def test_droplet_full_size_against_release_flag_build(oracle_lib):
    case = cases.shock_droplet_2d(nx=1024, ny=512, steps=100)
    x_cb, y_cb, _, q = preprocess.generate(case)
    with Simulation(case, x_cb, y_cb, q_cons=q) as sim:
        dgot = sim.run(0, 100)
        assert sim.status() == 0
        got = sim.download()
    native = oracle_lib.Oracle(case, x_cb, y_cb, build="native")
    native.set_state(q)
    dref = native.run(0, 100, case.dt)
    ref = native.get_state()
    exact = oracle_lib.Oracle(case, x_cb, y_cb, build="exact")
    exact.set_state(q)
    exact.run(0, 100, case.dt)
    ref_exact = exact.get_state()

    assert dgot == dref
    assert np.all(np.isfinite(got))
    err = rel_l1(got, ref)
    nf, nd = case.num_fluids, case.num_dims
    names = ([f"alpha_rho{i + 1}" for i in range(nf)] + ["mom_x", "mom_y", "mom_z"][:nd] + ["E"]
             + [f"alpha{i + 1}" for i in range(nf)])
    print("GPU FP64 vs Release-flag CPU build, per-field rel L1:", dict(zip(names, err.tolist())))
    print("GPU FP64 vs contraction-off oracle, values that differ:", int(np.count_nonzero(got != ref_exact)))
    mom_y = case.mom_idx + 1
    others = [i for i in range(case.sys_size) if i != mom_y]
    assert err[others].max() <= TOL_FP64, err
    # the y-momentum's difference measured against the momentum's own scale
    # (sum |rho u|): round-off, far inside the bar
    scale = np.abs(ref[case.mom_idx]).sum()
    dv = np.abs(got[mom_y] - ref[mom_y]).sum() / scale
    print(f"sum|d(rho v)| / sum|rho u| = {dv:.3e}; max|rho v| / max|rho u| = "
          f"{np.abs(ref[mom_y]).max() / np.abs(ref[case.mom_idx]).max():.3e}")
    assert dv <= TOL_FP64
    # the two CPU builds round differently (contraction happened), and the GPU
    # path is the contraction-off one bit for bit
    assert np.count_nonzero(ref != ref_exact) > 0
    assert np.array_equal(got, ref_exact)
