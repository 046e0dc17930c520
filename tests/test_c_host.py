"""The C ABI exercised the way MicroFC's Fortran host would exercise it.

tests/c_host/p_main_host.c is a plain C program, compiled with gcc against
include/mfc_gpu.h and linked to libmfc_gpu.so, that issues the call sequence
of the reference's p_main (src/simulation/p_main.fpp:186-193, 196-318):
mfc_gpu_init (with mfc_gpu_set_viscosity and, for weno_Re_flux,
mfc_gpu_set_viscous_gradients in viscous cases), one mfc_gpu_upload per
variable from ghost-padded
sf(-b:m+b, -b:n+b) arrays with the leading dimension m + 2b + 1, one
mfc_gpu_tvd_rk per time step with the last-step dt trim, and at every save
step mfc_gpu_status (the NaN scan) and one mfc_gpu_download per variable
back into the padded arrays.  It is the same sequence the Fortran bridge
(microfc_gb300/fortran/m_gpu_bridge.f90) issues.

The ghost layers of the host arrays are filled with NaN: the library must
neither read them (boundary conditions are applied on the device) nor write
them (downloads fill the interior only).  The saved states are compared bit
for bit with the oracle stepped through the same loop.
"""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from microfc_gb300 import Case, build as gbuild, cases, preprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_host", "p_main_host.c")


def _compile(tmp_path):
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    lib = gbuild.build()
    exe = str(tmp_path / "p_main_host")
    libdir = os.path.dirname(lib)
    cmd = [gcc, "-O2", "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
           "-L", libdir, "-lmfc_gpu", f"-Wl,-rpath,{libdir}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_host_compiles_and_links_against_the_header_and_library(tmp_path):
    """Every entry point p_main's sequence needs resolves in libmfc_gpu.so."""
    exe = _compile(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


def _write_input(path, case, x_cb, y_cb, q, t_step_start, t_step_stop, t_step_save):
    b = case.buff_size
    nf = case.num_fluids
    hdr = np.array([case.m, case.n, nf, case.weno_order, case.time_stepper, case.bc_x[0], case.bc_x[1],
                    case.bc_y[0], case.bc_y[1], t_step_start, t_step_stop, t_step_save, int(case.viscous),
                    int(case.weno_re_flux)], dtype=np.int32)
    nxp = case.m + 2 * b + 1
    nyp = case.n + 2 * b + 1 if case.n > 0 else 1
    pad = np.full((case.sys_size, nyp, nxp), np.nan)
    oy = b if case.n > 0 else 0
    pad[:, oy:oy + case.n + 1, b:b + case.m + 1] = q[:, 0]
    with open(path, "wb") as f:
        f.write(hdr.tobytes())
        f.write(np.array([case.weno_eps, case.dt], dtype=np.float64).tobytes())
        f.write(np.asarray(case.gammas[:nf], dtype=np.float64).tobytes())
        f.write(np.asarray(case.pi_infs[:nf], dtype=np.float64).tobytes())
        if case.viscous:
            f.write(np.asarray(case.re_shear[:nf], dtype=np.float64).tobytes())
            f.write(np.asarray(case.re_bulk[:nf], dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(x_cb, dtype=np.float64).tobytes())
        if case.n > 0:
            f.write(np.ascontiguousarray(y_cb, dtype=np.float64).tobytes())
        f.write(pad.tobytes())
    return pad.shape, oy, b


def _reference_example(name):
    """One of the reference's example cases (tests/golden/reference_cases)."""
    with open(os.path.join(ROOT, "tests", "golden", "reference_cases", name + ".json")) as f:
        return Case.from_dict(json.load(f))


def _oracle_saves(oracle_lib, case, x_cb, y_cb, q, t_step_start, t_step_stop, t_step_save):
    """The oracle stepped through p_main's loop; states at the save steps."""
    o = oracle_lib.Oracle(case, x_cb, y_cb)
    o.set_state(q)
    dt = case.dt
    t_step = t_step_start
    mytime = 0.0 if t_step == 0 else t_step * dt
    finaltime = t_step_stop * dt
    saves = []
    while True:
        mytime = mytime + dt
        o.tvd_rk(dt, t_step == t_step_stop)
        if t_step == t_step_stop:
            break
        if (mytime + dt) >= finaltime:
            dt = finaltime - mytime
        t_step += 1
        if (t_step - t_step_start) % t_step_save == 0 or t_step == t_step_stop:
            saves.append((t_step, o.get_state()))
    return saves, dt


@pytest.mark.gpu
@pytest.mark.parametrize("builder", [
    lambda: cases.shock_droplet_2d(nx=96, ny=48, steps=12),
    lambda: cases.shock_droplet_2d(nx=64, ny=40, steps=12).replace(bc_x=(-2, -4), bc_y=(-1, -1)),
    lambda: cases.sod_1d(m=299, steps=12, dt=1e-4),
    lambda: _reference_example("2D_viscous"),
], ids=["droplet", "droplet-bc-mix", "sod", "viscous-example-weno_Re_flux"])
def test_c_host_runs_p_main_sequence_bitwise_like_the_oracle(tmp_path, oracle_lib, builder):
    exe = _compile(tmp_path)
    case = builder()
    x_cb, y_cb, _, q = preprocess.generate(case)
    start, stop, save = 0, 12, 5
    inp, outp = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    shape, oy, b = _write_input(inp, case, x_cb, y_cb, q, start, stop, save)
    r = subprocess.run([exe, inp, outp], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr

    ref, dt_ref = _oracle_saves(oracle_lib, case, x_cb, y_cb, q, start, stop, save)
    raw = open(outp, "rb").read()
    per = int(np.prod(shape)) * 8
    off = 0
    for t_ref, state in ref:
        t_step = int(np.frombuffer(raw, dtype=np.int32, count=1, offset=off)[0])
        off += 4
        pad = np.frombuffer(raw, dtype=np.float64, count=per // 8, offset=off).reshape(shape)
        off += per
        assert t_step == t_ref
        interior = pad[:, oy:oy + case.n + 1, b:b + case.m + 1]
        assert np.array_equal(interior, state[:, 0]), f"t_step {t_step}: differs from the oracle"
        ghost = pad.copy()
        ghost[:, oy:oy + case.n + 1, b:b + case.m + 1] = np.nan
        assert np.isnan(ghost).all(), "a download wrote into the ghost layers"
    dt_got = float(np.frombuffer(raw, dtype=np.float64, count=1, offset=off)[0])
    assert off + 8 == len(raw)
    assert dt_got == dt_ref
    assert [t for t, _ in ref] == [5, 10, 12]
