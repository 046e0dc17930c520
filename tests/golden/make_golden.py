"""Generates the golden fixtures in this directory from the oracle.

The reference has no golden vectors and cannot be built here, so these
fixtures freeze the oracle's own outputs on small cases.  They pin the oracle
against regressions and across host architectures (x86-64 here, aarch64 on
the GPU hosts; the oracle is built without FMA contraction), and the GPU
parity tests compare the CUDA path against them directly.

Run from the repository root:  python tests/golden/make_golden.py [name ...]
(no names: every fixture).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from microfc_gb300 import cases, preprocess  # noqa: E402

# name -> (case builder, steps)
GOLDEN = {
    "sod_1d_200_weno5_rk3": (lambda: cases.sod_1d(m=199, steps=60, dt=2e-4), 60),
    "sod_1d_200_weno3_rk2": (lambda: cases.sod_1d(m=199, steps=60, dt=2e-4).replace(weno_order=3, time_stepper=2), 60),
    "droplet_2d_48x32_weno5_rk3": (lambda: cases.shock_droplet_2d(nx=48, ny=32, steps=25), 25),
    "droplet_2d_40x40_periodic": (lambda: cases.shock_droplet_2d(nx=40, ny=40, steps=20).replace(
        bc_x=(-1, -1), bc_y=(-1, -1)), 20),
    "droplet_2d_40x32_symmetry_riemann": (lambda: cases.shock_droplet_2d(nx=40, ny=32, steps=20).replace(
        bc_x=(-4, -3), bc_y=(-2, -2)), 20),
    # viscous terms with WENO velocity gradients (weno_Re_flux = T)
    "viscous_droplet_2d_40x32_weno_re_flux": (lambda: cases.shock_droplet_2d(nx=40, ny=32, steps=15).replace(
        re_shear=(10.0, 500.0), re_bulk=(0.0, 200.0), weno_re_flux=True), 15),
}


def compute(name):
    builder, steps = GOLDEN[name]
    case = builder()
    x_cb, y_cb, _, q0 = preprocess.generate(case)
    o = oracle.Oracle(case, x_cb, y_cb)
    o.set_state(q0)
    dt_final = o.run(0, steps, case.dt)
    return case, x_cb, y_cb, q0, o.get_state(), steps, dt_final


def main(names):
    for name in names or GOLDEN:
        case, x_cb, y_cb, q0, q1, steps, dt_final = compute(name)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), q0=q0, q=q1, x_cb=x_cb,
                            y_cb=y_cb if y_cb is not None else np.zeros(0), steps=steps, dt=case.dt,
                            dt_final=dt_final)
        print(name, q1.shape, steps)


if __name__ == "__main__":
    main(sys.argv[1:])
