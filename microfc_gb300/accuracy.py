"""Error of the reduced-precision forms against the plain FP64 path.

The split form (FP32 WENO and HLLC, FP64 state, RK update and pressure
recovery) and the gated form (split plus the learned WENO gate) are run
beside the plain FP64 path from the same initial state, and the per-field
relative L1 error sum|q - q_fp64| / sum|q_fp64| of the conserved variables
is reported.  The plain FP64 path reproduces the CPU oracle bit for bit
(tests/test_gpu_parity.py), so at sizes where the CPU oracle would run for
hours the FP64 GPU result stands in for it.

    python -m microfc_gb300.accuracy --config bubble3d   # 256^3 air/helium shock-bubble, 500 steps, split
    python -m microfc_gb300.accuracy --config droplet2d  # 2048x1024 shock-droplet, 2000 steps, split and gated
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import cases, preprocess
from .solver import Simulation


def rel_l1(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Per-field relative L1 error over the first axis (absolute where b is 0)."""
    a = a.reshape(a.shape[0], -1)
    b = b.reshape(b.shape[0], -1)
    num = np.abs(a - b).sum(axis=1)
    den = np.abs(b).sum(axis=1)
    return np.where(den > 0, num / np.where(den > 0, den, 1.0), num)


def field_names(case) -> list[str]:
    nf, nd = case.num_fluids, case.num_dims
    return ([f"alpha_rho{f + 1}" for f in range(nf)] + [f"mom_{'xyz'[d]}" for d in range(nd)] + ["E"]
            + [f"alpha{f + 1}" for f in range(nf)])


def run(case, precision: str, steps: int, q0, grid, gate_params=None, device: int = 0):
    """(final state, seconds) of `steps` time steps in the given precision."""
    import torch
    c = case.replace(precision=precision)
    with Simulation(c, *grid, q_cons=q0, device=device) as sim:
        if gate_params is not None:
            sim.set_gate(gate_params)
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        sim.run(0, steps)
        torch.cuda.synchronize(device)
        dt = time.perf_counter() - t0
        if sim.status() != 0:
            raise RuntimeError(f"{precision} run flagged a non-finite state")
        return sim.download(), dt


def compare(case, steps: int, modes, device: int = 0) -> dict:
    x, y, z, q0 = preprocess.generate(case)
    grid = (x, y, z)
    ref, t_ref = run(case, "fp64", steps, q0, grid, device=device)
    names = field_names(case)
    out = {"case": case.name, "cells": int(case.cells), "steps": steps,
           "fp64_seconds": t_ref, "fp64_cell_updates_per_s": case.cells * steps / t_ref, "modes": {}}
    for prec, params in modes:
        q, t = run(case, prec, steps, q0, grid, params, device)
        err = rel_l1(q, ref)
        out["modes"][prec] = {"rel_l1": dict(zip(names, map(float, err))), "seconds": t,
                              "cell_updates_per_s": case.cells * steps / t,
                              "max_rel_l1_density_and_volume_fraction": float(max(
                                  err[i] for i, n in enumerate(names) if n.startswith("alpha")))}
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--config", choices=["bubble3d", "droplet2d"], required=True)
    ap.add_argument("--n", type=int, default=None, help="cells per direction (bubble3d) or in x (droplet2d)")
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--out", default=None, help="write the JSON result here too")
    a = ap.parse_args(argv)
    if a.config == "bubble3d":
        n = a.n or 256
        steps = a.steps or 500
        case = cases.shock_bubble_3d(N=n, steps=steps, precision="fp64")
        modes = [("split", None)]
    else:
        from . import gate
        n = a.n or 2048
        steps = a.steps or 2000
        case = cases.shock_droplet_2d(nx=n, ny=n // 2, steps=steps)
        modes = [("split", None), ("gated", gate.load())]
    res = compare(case, steps, modes)
    res["config"] = a.config
    text = json.dumps(res, indent=1)
    print(text)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text + "\n")


if __name__ == "__main__":
    main()
