"""pre_process / simulation executables around the hot path: the reference's
save cadence, data files and D/ text files, restart from t_step_start, and
asynchronous snapshots that overlap with the time steps."""
import os

import numpy as np
import pytest

from microfc_gb300 import cases, io, preprocess


def test_text_files_follow_the_fortran_layout(tmp_path):
    c = cases.sod_1d(m=9, steps=2)
    x_cb, _, _, q = preprocess.generate(c)
    files = io.write_text_files(str(tmp_path), 7, c, q, x_cb)
    names = sorted(os.path.basename(f) for f in files)
    assert names[0] == "cons.1.00.000007.dat" and len(names) == 2 * c.sys_size
    lines = open(tmp_path / "D" / "cons.1.00.000007.dat").read().split("\n")
    assert len(lines) == c.m + 2 and lines[-1] == ""
    assert all(len(s) == 80 for s in lines[:-1])
    # cell j is labelled with x_cb(j), its right boundary
    assert float(lines[0][:40]) == pytest.approx(x_cb[1], abs=1e-14)
    assert float(lines[0][40:]) == pytest.approx(q[0].ravel()[0], abs=1e-14)
    # 1-D primitive pressure from the stiffened-gas energy
    p = open(tmp_path / "D" / f"prim.{c.E_idx + 1}.00.000007.dat").read().split("\n")
    assert float(p[0][40:]) == pytest.approx(1.0, abs=1e-13) and float(p[-2][40:]) == pytest.approx(0.1, abs=1e-13)

    c2 = cases.shock_droplet_2d(nx=8, ny=4, steps=2)
    x_cb, y_cb, _, q = preprocess.generate(c2)
    io.write_text_files(str(tmp_path), 3, c2, q, x_cb, y_cb)
    text = open(tmp_path / "D" / "cons.1.00.000003.dat").read()
    blocks = text.split("\n\n")
    assert len(blocks) == c2.m + 2 and blocks[-1] == ""  # one block per j, each closed by an empty line
    first = blocks[0].split("\n")
    assert len(first) == c2.n + 1 and all(len(s) == 120 for s in first)
    assert float(first[1][40:80]) == pytest.approx(y_cb[2], abs=1e-14)
    assert io._fortran_f(1e30, 40, 14) == "*" * 40 and io._fortran_f(float("nan"), 40, 14).strip() == "NaN"


@pytest.mark.gpu
def test_simulate_saves_like_p_main_and_restarts(tmp_path):
    from microfc_gb300 import Simulation, driver
    c = cases.sod_1d(m=199, steps=20, dt=2e-4).replace(t_step_save=5)
    d = str(tmp_path)
    driver.pre_process(c, d)
    res = driver.simulate(c, d)
    assert res["saved"] == [5, 10, 15, 20]
    assert os.path.exists(os.path.join(d, "D", "cons.1.00.000020.dat"))
    _, _, _, q20 = io.read_data_files(d, 20, c)
    with Simulation(c) as sim:
        sim.run(0, 20)
        ref = sim.download()
    assert np.array_equal(q20, ref)
    # restart from the files of step 10 (m_start_up reads p_all/p0/<t_step_start>/)
    c2 = c.replace(t_step_start=10)
    d2 = str(tmp_path / "restart")
    os.makedirs(os.path.join(d2, "p_all", "p0"))
    os.symlink(os.path.join(d, "p_all", "p0", "10"), os.path.join(d2, "p_all", "p0", "10"))
    res2 = driver.simulate(c2, d2, text_files=False)
    assert res2["saved"] == [15, 20]
    _, _, _, r20 = io.read_data_files(d2, 20, c2)
    _, _, _, q10 = io.read_data_files(d, 10, c)
    with Simulation(c2, q_cons=q10) as sim:
        sim.run(10, 20)
        assert np.array_equal(r20, sim.download())
    # the restarted time differs from the accumulated one only in the rounding of the trimmed last dt
    assert np.abs(r20 - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.gpu
def test_snapshot_is_taken_in_stream_order_and_overlaps_later_steps():
    from microfc_gb300 import Simulation
    c = cases.shock_droplet_2d(nx=128, ny=64, steps=30)
    with Simulation(c) as sim:
        for t in range(5):
            sim.tvd_rk(t)
        sim.snapshot(0)
        for t in range(5, 10):  # issued while the copy is in flight
            sim.tvd_rk(t)
        sim.snapshot(1)
        snap5 = sim.snapshot_wait(0).copy()
        snap10 = sim.snapshot_wait(1).copy()
        final = sim.download()
    with Simulation(c) as sim:
        for t in range(5):
            sim.tvd_rk(t)
        ref5 = sim.download()
    assert np.array_equal(snap5, ref5)
    assert np.array_equal(snap10, final)
