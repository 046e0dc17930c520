"""The reference's two executables around the hot path, on the GPU state.

``pre_process(case, case_dir)`` writes the initial condition where the
simulation reads it (p_all/p0/0/, src/pre_process/m_data_output.fpp);
``simulate(case, case_dir)`` is p_main (src/simulation/p_main.fpp:77-318):
it reads p_all/p0/<t_step_start>/ (m_start_up.fpp:298-390, which is also how
a run restarts), advances t_step_start .. t_step_stop with the dt trim of the
CPU build, and every t_step_save steps checks the state for NaN and writes
p_all/p0/<t_step>/ plus the D/ text files (p_main.fpp:291-315,
m_data_output.fpp:316-462).

Unlike the reference, whose "!$acc update host" stalls the time loop at
every save, the state is snapshot on the device and copied to pinned host
memory on a second stream while the next steps run; a writer thread turns
finished snapshots into files.
"""
from __future__ import annotations

import argparse
import json
import os
import threading
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import io, preprocess
from .case import Case
from .solver import Simulation

# runs of at least this many steps autotune the tile variant first (about
# three launches of each variant: a few steps' worth of time)
TUNE_MIN_STEPS = 200


def pre_process(case: Case, case_dir: str, ic: str = "host") -> str:
    """Initial condition into p_all/p0/0/ (the pre_process executable's output)."""
    if ic == "device":
        with Simulation(case, ic="device") as sim:
            q = sim.download()
        x_cb, y_cb, z_cb = preprocess.grid(case)
    else:
        x_cb, y_cb, z_cb, q = preprocess.generate(case)
    return io.write_data_files(case_dir, 0, case, q, x_cb, y_cb, z_cb)


def simulate(case: Case, case_dir: str, text_files: bool = True, device: int = 0, monitor: bool = False,
             on_save=None) -> dict:
    """p_main on the GPU; returns timing and the saved steps."""
    case.check()
    x_cb, y_cb, z_cb, q0 = io.read_data_files(case_dir, case.t_step_start, case)
    saved = []
    errors = []
    lock = threading.Lock()
    t0 = time.perf_counter()
    with Simulation(case, x_cb, y_cb, z_cb, q_cons=q0, device=device, check=False) as sim, \
            ThreadPoolExecutor(max_workers=1) as writer:
        if monitor:
            sim.set_monitor(True)
        if case.t_step_stop - case.t_step_start >= TUNE_MIN_STEPS:
            sim.tune(3)  # the fastest tile variant; every variant gives the same bits
        pending = [None, None]

        def write(t_step, slot):
            try:
                q = sim.snapshot_wait(slot)
                if np.isnan(q).any():  # p_main.fpp:298-304
                    bad = np.argwhere(np.isnan(q))[0]
                    raise FloatingPointError(f"NaN at {tuple(int(v) for v in bad)} of step {t_step}: Error")
                io.write_data_files(case_dir, t_step, case, q, x_cb, y_cb, z_cb)
                if text_files:
                    io.write_text_files(case_dir, t_step, case, q, x_cb, y_cb)
                if on_save is not None:
                    on_save(t_step, q)
                with lock:
                    saved.append(t_step)
            except BaseException as e:  # reported after the loop
                with lock:
                    errors.append(e)

        dt = case.dt
        t_step = case.t_step_start
        mytime = 0.0 if t_step == 0 else t_step * dt
        finaltime = case.t_step_stop * dt
        slot = 0
        while True:
            mytime = mytime + dt
            sim.tvd_rk(t_step, dt)
            if t_step == case.t_step_stop:
                break
            if (mytime + dt) >= finaltime:
                dt = finaltime - mytime
            t_step = t_step + 1
            if (t_step - case.t_step_start) % case.t_step_save == 0 or t_step == case.t_step_stop:
                if pending[slot] is not None:
                    pending[slot].result()  # the writer is done with this slot
                sim.snapshot(slot)
                pending[slot] = writer.submit(write, t_step, slot)
                slot ^= 1
            if errors:
                break
        for f in pending:
            if f is not None:
                f.result()
        status = sim.status()
        icfl = sim.icfl() if monitor else None
    elapsed = time.perf_counter() - t0
    if errors:
        raise errors[0]
    if status:
        raise FloatingPointError("NaN or Inf in the conservative state")
    return {"steps": case.t_step_stop - case.t_step_start, "saved": sorted(saved), "seconds": elapsed,
            "final_dt": dt, "icfl_max": icfl}


def main(argv=None):
    ap = argparse.ArgumentParser(description="pre_process + simulation of a case dictionary (JSON)")
    ap.add_argument("case_json", help="JSON object with the reference's case-file keys")
    ap.add_argument("--dir", default=".", help="case directory (p_all/ and D/ go here)")
    ap.add_argument("--no-pre-process", action="store_true", help="restart from existing p_all files")
    ap.add_argument("--no-text", action="store_true", help="skip the D/ text files")
    a = ap.parse_args(argv)
    with open(a.case_json) as f:
        case = Case.from_dict(json.load(f))
    os.makedirs(a.dir, exist_ok=True)
    if not a.no_pre_process:
        pre_process(case, a.dir)
    print(json.dumps(simulate(case, a.dir, text_files=not a.no_text)))


if __name__ == "__main__":
    main()
