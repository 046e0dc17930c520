"""Benchmark of the MicroFC hot path on GB300.

Workload: 2-D air shock (Mach 1.47) on a water droplet, 1024 x 512 cells,
2 fluids (7 equations), WENO5-JS + HLLC + TVD-RK3, plain FP64.  One "step" is
one full time step (3 fused RK-stage launches).  Metric: cell-updates/s =
interior cells x steps / seconds.

* value   -- device-resident state, CUDA-event time of each step on the
             library's stream; L2 is flushed (256 MiB write) between steps.
* e2e     -- the same through the public API with host buffers: every step
             uploads the state from pinned host memory, advances one step and
             downloads the state (all inside the timed region).
* roofline     -- the slower-of roofline of the stage kernel: algorithmic
                  flops per launch (counted by the oracle) / the launch's
                  CUDA-event duration against the FP64 (split precision:
                  FP32) FMA peak measured in-process, with the HBM figure
                  (algorithmic 448 B per cell-update against the measured
                  copy bandwidth) beside it; "bound" names whichever of the
                  two the kernel is closer to.
* cpu_baseline -- the oracle (C++ restatement of the reference's CPU code)
                  built with the reference's Release flags (-O3, -march /
                  -mcpu=native, default FMA contraction), OpenMP over the host
                  cores, on the full 1024 x 512 grid.

``--impl reference`` times that CPU implementation alone and prints the
reference arm's line.  Under torchrun (N > 1) every rank runs an independent
replica (the path has no exchange on a one-GPU-per-box deployment); value is
the sum over ranks with the max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

NX, NY = 1024, 512
BYTES_PER_CELL_UPDATE = 448  # 8 * S doubles, S = 7 (fused RK3 compulsory traffic)
WORKLOAD = "2D shock-droplet 1024x512, 2 fluids, WENO5-JS + HLLC + TVD-RK3, plain FP64"
METRIC = "cell-updates/s (2D shock-droplet 1024x512, plain FP64)"


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _profile_value(name: str, key: str):
    """A figure from a committed ncu summary under profiles/ (``key: value``)."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        with open(path) as f:
            for line in f:
                if line.strip().startswith(key + ":"):
                    return float(line.split(":", 1)[1].split()[0])
    except (OSError, ValueError):
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int, period_ms: int = 50):
        self.index = index
        self.period_ms = period_ms
        self.samples = []
        self._proc = None
        self._t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        # one nvidia-smi process streaming a line every period_ms
        try:
            self._proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                           "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            for line in self._proc.stdout:
                if line.strip():
                    self.samples.append([v.strip() for v in line.split(",")])
        except Exception:
            pass

    def __enter__(self):
        self._t.start()
        time.sleep(0.1)  # the first line is out before the timed region starts
        return self

    def __exit__(self, *exc):
        if self._proc is not None:
            self._proc.terminate()  # the process this sampler started
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[2 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_rate(seconds: float, units_per_rank: int, ws: int, device: str = "cuda"):
    """Whole-job rate of N independent replicas: every rank processed
    units_per_rank cell-updates; the job took as long as its slowest rank.
    Returns (units of all ranks / max seconds, max seconds)."""
    if ws > 1:
        import torch
        import torch.distributed as dist
        tt = torch.tensor([seconds], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        seconds = float(tt.item())
    return ws * units_per_rank / seconds, seconds


CPU_FLAGS = "g++ -O3 -march/-mcpu=native, default FMA contraction (the reference's Release flags), OpenMP"


def _cpu_oracle():
    """The oracle's Release-flag build on the full workload, all host cores."""
    import oracle
    from microfc_gb300 import cases, preprocess
    case = cases.shock_droplet_2d(nx=NX, ny=NY)
    x_cb, y_cb, _, q = preprocess.generate(case)
    o = oracle.Oracle(case, x_cb, y_cb, threads=os.cpu_count() or 1, build="native")
    o.set_state(q)
    return o, case, oracle.lib("native").mfo_get_threads()


def cpu_baseline(min_seconds: float = 10.0, max_steps: int = 400):
    """Full RK3 steps of the 1024 x 512 workload on the host cores until
    min_seconds of CPU work have run (at least 3 steps)."""
    o, case, cores = _cpu_oracle()
    o.tvd_rk(case.dt)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps and (steps < 3 or time.perf_counter() - t0 < min_seconds):
        o.tvd_rk(case.dt)
        steps += 1
    t = time.perf_counter() - t0
    return {"value": case.cells * steps / t, "unit": "cell-updates/s", "cores": cores, "kind": "port",
            "flags": CPU_FLAGS, "same_config": True,
            "sample": f"{steps} full RK3 time steps of the {NX}x{NY} workload (C++ restatement of the "
                      f"reference's CPU code, OpenMP over {cores} threads)"}


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    o, case, cores = _cpu_oracle()
    for _ in range(args.warmup):
        o.tvd_rk(case.dt)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.tvd_rk(case.dt)
    t = time.perf_counter() - t0
    v = case.cells * args.steps / t
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "cell-updates/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "cells": case.cells, "sample": f"the full {NX}x{NY} grid every step",
                   "l2": "n/a (CPU)", "flags": CPU_FLAGS},
        "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": cores, "kind": "port", "flags": CPU_FLAGS,
                         "same_config": True,
                         "sample": f"{args.steps} RK3 steps of the full {NX}x{NY} workload; the reference "
                                   "(Fortran + Fypp) cannot be built here, so its C++ restatement (the oracle) "
                                   "runs, built with the reference's Release flags"},
        "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _time_steps(sim, stream, flush, steps, warmup, dt):
    """CUDA-event time (s) of `steps` time steps of a Simulation, L2 flushed between steps."""
    import torch
    for _ in range(warmup):
        sim.tvd_rk(0, dt)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with torch.cuda.stream(stream):
        for i in range(steps):
            flush.fill_(float(i))
            ev[i][0].record(stream)
            sim.tvd_rk(0, dt)
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev) / 1e3


def other_modes(args, case, x_cb, y_cb, q0, flush, fp64_rate):
    """Split precision, split + learned gate (the gated FP32 form) on the same
    workload, the 3-D shock-bubble of config 3 in split precision against
    plain FP64, and the 64-case ensemble of config 5 against 64 sequential
    plain FP64 runs.  Accuracy of these modes against FP64 is asserted by
    tests/test_gpu_parity.py, tests/test_gate.py and tests/test_ensemble.py."""
    import numpy as np
    import torch
    from microfc_gb300 import Simulation, _lib, gate
    from microfc_gb300.ensemble import Ensemble, random_droplet_cases
    out = {}
    params = gate.load() if os.path.exists(gate.WEIGHTS_FILE) else None
    modes = [("split", None)] + ([("gated", params)] if params is not None else [])
    for prec, p in modes:
        with Simulation(case.replace(precision=prec), x_cb, y_cb, q_cons=q0) as s:
            if p is not None:
                s.set_gate(p)
            variant, _ = s.tune(5)
            s.select_variant(variant)
            tma = bool(s.variant_features(variant) & _lib.MFC_VARIANT_TMA)
            st = torch.cuda.ExternalStream(s.stream)
            t = _time_steps(s, st, flush, args.steps, args.warmup, case.dt)
            rate = case.cells * args.steps / t
            out[prec] = {"value": rate, "unit": "cell-updates/s", "ms_per_step": 1e3 * t / args.steps,
                         "vs_plain_fp64": rate / fp64_rate, "tile_variant": variant, "tma_staging": tma}
    if params is None:
        out["gated"] = {"unavailable": "no trained gate parameters (python -m microfc_gb300.gate)"}
    # the opt-in contracted FP64 variant: rate, its FP64 roofline fraction,
    # and its distance from the plain (bit-faithful) path after 100 steps
    flops = _profile_value("flop_count_droplet_1024x512.md", "algorithmic_flops_per_cell_update")
    fp64_peak, _ = _lib.measure_peaks(torch.cuda.current_device())
    with Simulation(case.replace(precision="fp64_fma"), x_cb, y_cb, q_cons=q0) as s:
        variant, _ = s.tune(5)
        s.select_variant(variant)
        st = torch.cuda.ExternalStream(s.stream)
        t = _time_steps(s, st, flush, args.steps, args.warmup, case.dt)
        rate = case.cells * args.steps / t
        s.upload(q0)
        s.run(0, 100)
        q_fma = s.download()
    with Simulation(case, x_cb, y_cb, q_cons=q0) as s:
        s.run(0, 100)
        q_plain = s.download()
    a, b = q_fma.reshape(q_fma.shape[0], -1), q_plain.reshape(q_plain.shape[0], -1)
    l1 = (np.abs(a - b).sum(axis=1) / np.abs(b).sum(axis=1)).tolist()
    out["fp64_fma"] = {"value": rate, "unit": "cell-updates/s", "ms_per_step": 1e3 * t / args.steps,
                       "vs_plain_fp64": rate / fp64_rate, "tile_variant": variant,
                       "roofline": {"bound": "fp64", "achieved": flops * rate / 1e12 if flops else None,
                                    "peak": fp64_peak, "unit": "TFLOP/s",
                                    "frac": flops * rate / 1e12 / fp64_peak if flops else None},
                       "rel_l1_vs_plain_fp64_100_steps": l1}
    # WENO of the characteristic fields (FP64, bit-identical to the oracle's
    # restatement): its rate on the same workload
    with Simulation(case.replace(char_decomp=True), x_cb, y_cb, q_cons=q0) as s:
        variant, _ = s.tune(5)
        s.select_variant(variant)
        st = torch.cuda.ExternalStream(s.stream)
        t = _time_steps(s, st, flush, args.steps, args.warmup, case.dt)
        rate = case.cells * args.steps / t
    out["fp64_characteristic"] = {"value": rate, "unit": "cell-updates/s", "ms_per_step": 1e3 * t / args.steps,
                                  "vs_plain_fp64": rate / fp64_rate, "tile_variant": variant}
    # the viscous terms (m_viscous.fpp) on the same workload: water and air
    # with shear and bulk Reynolds numbers (1/mu in the case's units), plain
    # FP64 (bit-identical to the oracle) and split precision, with
    # finite-difference and with WENO (weno_Re_flux) velocity gradients
    visc = {"workload": "2D shock-droplet 1024x512 with viscous terms (Re shear 10 / 500, bulk 0 / 200)",
            "unit": "cell-updates/s"}
    vcase = case.replace(re_shear=(1.0 / 1e-1, 1.0 / 2e-3), re_bulk=(0.0, 1.0 / 5e-3))
    for precv, wrf in (("fp64", False), ("split", False), ("fp64", True), ("split", True)):
        key = precv + ("_weno_Re_flux" if wrf else "")
        with Simulation(vcase.replace(precision=precv, weno_re_flux=wrf), x_cb, y_cb, q_cons=q0) as s:
            variant, _ = s.tune(5)
            s.select_variant(variant)
            st = torch.cuda.ExternalStream(s.stream)
            t = _time_steps(s, st, flush, args.steps, args.warmup, case.dt)
            visc[key] = case.cells * args.steps / t
            visc[key + "_vs_inviscid"] = visc[key] / (fp64_rate if precv == "fp64" else out["split"]["value"])
    out["viscous"] = visc
    # config 4's grid: the droplet at 2048 x 1024 (7 equations, 117 MB per
    # register), gated against split and plain FP64 on the same case; the
    # device initial condition avoids a host pre_process of 2 M cells
    from microfc_gb300 import cases
    c4 = cases.shock_droplet_2d(nx=2048, ny=1024)
    r4, v4 = {}, {}
    for prec4, n4 in (("fp64", 4), ("split", 20)) + ((("gated", 20),) if params is not None else ()):
        with Simulation(c4.replace(precision=prec4), ic="device") as s:
            if prec4 == "gated":
                s.set_gate(params)
            v4[prec4], _ = s.tune(3)
            s.select_variant(v4[prec4])
            st = torch.cuda.ExternalStream(s.stream)
            r4[prec4] = c4.cells * n4 / _time_steps(s, st, flush, n4, 3, c4.dt)
    out["config4_2048x1024"] = {
        "workload": "2D shock-droplet 2048x1024, 2 fluids, WENO5-JS + HLLC + TVD-RK3",
        "unit": "cell-updates/s", "plain_fp64": r4["fp64"], "split": r4["split"],
        "tile_variants": v4, "timing": "CUDA events per step on the library's stream, L2 flushed between steps"}
    if "gated" in r4:
        out["config4_2048x1024"].update(gated=r4["gated"], gated_vs_plain_fp64=r4["gated"] / r4["fp64"],
                                        gated_vs_split=r4["gated"] / r4["split"])
    # config 3: the 3-D air/helium shock-bubble at 256^3, split precision,
    # against plain FP64 on the same case (states of 1 GB per register: no
    # L2 reuse between steps)
    c3 = cases.shock_bubble_3d(N=256, steps=500, precision="split")
    r3, v3 = {}, {}
    for prec3, n3 in (("split", 10), ("fp64", 2)):
        with Simulation(c3.replace(precision=prec3), ic="device") as s:
            v3[prec3], _ = s.tune(2)
            s.select_variant(v3[prec3])
            if prec3 == "split":
                tma3 = bool(s.variant_features(v3[prec3]) & _lib.MFC_VARIANT_TMA)
            st = torch.cuda.ExternalStream(s.stream)
            r3[prec3] = c3.cells * n3 / _time_steps(s, st, flush, n3, 2, c3.dt)
    out["split_3d"] = {"workload": "3-D air/helium shock-bubble 256^3, 2 fluids, WENO5-JS + HLLC + TVD-RK3",
                       "value": r3["split"], "unit": "cell-updates/s", "steps": 10, "tile_variant": v3["split"],
                       "tma_staging": tma3, "plain_fp64": r3["fp64"], "vs_plain_fp64": r3["split"] / r3["fp64"]}
    # config 5: 64 cases, nx in {128,256,384,512}, ny = nx/2, seed 0
    prec = "gated" if params is not None else "split"
    cl = random_droplet_cases(count=64, seed=0, steps=500, precision=prec)
    with Ensemble(cl) as ens:
        if params is not None:
            ens.set_gate(params)
        variant, _ = ens.tune(reps=3)
        ens_tma = bool(ens.variant_features(variant) & _lib.MFC_VARIANT_TMA)
        ens.run(0, 3, use_graph=True)  # warm-up (advances the state; timing only)
        torch.cuda.synchronize()
        nsteps = 20
        est = torch.cuda.ExternalStream(ens.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(est)  # 64 states (0.7 GB) exceed the L2: no flush needed
        ens.run(3, 3 + nsteps, use_graph=True)
        e1.record(est)
        torch.cuda.synchronize()
        t_ens = e0.elapsed_time(e1) / 1e3
        ens_rate = ens.cells * nsteps / t_ens
    # 64 sequential plain FP64 runs: measured per size class
    seq_time = 0.0
    per_class = {}
    for c in cl:
        key = c.m + 1
        if key not in per_class:
            with Simulation(c.replace(precision="fp64")) as s:
                s.tune(3)
                st = torch.cuda.ExternalStream(s.stream)
                per_class[key] = _time_steps(s, st, flush, 3, 3, c.dt) / 3
        seq_time += per_class[key]
    seq_rate = sum(c.cells for c in cl) / seq_time
    out["ensemble"] = {"cases": len(cl), "cells": int(sum(c.cells for c in cl)), "precision": prec,
                       "value": ens_rate, "unit": "cell-updates/s", "steps": nsteps, "graph": True,
                       "tile_variant": variant, "tma_staging": ens_tma,
                       "timing": "CUDA events on the ensemble stream around 20 graph-replayed steps",
                       "sequential_plain_fp64": seq_rate, "vs_sequential_plain_fp64": ens_rate / seq_rate}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "split", "gated", "fp64_fma"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--nx", type=int, default=NX, help="cells in x (profiling runs; the benchmark is 1024)")
    ap.add_argument("--ny", type=int, default=NY, help="cells in y (profiling runs; the benchmark is 512)")
    ap.add_argument("--no-modes", action="store_true", help="skip the split/gated/ensemble figures")
    ap.add_argument("--variant", type=int, default=None,
                    help="pin this tile variant instead of running the autotuner (profiling runs)")
    ap.add_argument("--case", default="droplet2d", choices=["droplet2d", "bubble3d"],
                    help="profiling runs only: bubble3d is the 3-D shock-bubble at --nx^3 cells (the benchmark "
                         "workload is droplet2d); no modes, no compute roofline")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch
    import torch.distributed as dist
    from microfc_gb300 import Simulation, _lib, cases, preprocess

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    fp64_peak, fp32_peak = _lib.measure_peaks(local)
    if args.case == "bubble3d":
        case = cases.shock_bubble_3d(N=args.nx if args.nx != NX else 256, precision=args.precision)
        sim = Simulation(case, ic="device", device=local)
        q0 = sim.download()
        x_cb = y_cb = None
        args.no_modes = True
    else:
        case = cases.shock_droplet_2d(nx=args.nx, ny=args.ny, precision=args.precision)
        x_cb, y_cb, _, q0 = preprocess.generate(case)
        sim = Simulation(case, x_cb, y_cb, q_cons=q0, device=local)
    if args.precision == "gated":
        from microfc_gb300 import gate
        sim.set_gate(gate.load())
    if args.variant is None:
        variant, _ = sim.tune(5)  # the library's autotuner picks the tile shape
    else:
        variant = args.variant
        sim.select_variant(variant)
    tile = sim.select_variant(variant)
    stream = torch.cuda.ExternalStream(sim.stream, device=torch.device("cuda", local))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            dist.barrier()

    # ---- device-resident timing -------------------------------------------------
    for _ in range(args.warmup):
        sim.tvd_rk(0, case.dt)
    barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    l0 = sim.launches
    with ClockSampler(local) as clk:
        with torch.cuda.stream(stream):
            for i in range(args.steps):
                flush.fill_(float(i))  # evict the state from L2 between timed steps
                ev[i][0].record(stream)
                sim.tvd_rk(0, case.dt)
                ev[i][1].record(stream)
        barrier()
    launches = sim.launches - l0
    ms = [a.elapsed_time(b) for a, b in ev]
    t_total = sum(ms) / 1e3
    cells = case.cells
    value, t_total = replica_rate(t_total, cells * args.steps, ws)
    ms_step = 1e3 * t_total / args.steps
    if sim.status() != 0:
        raise RuntimeError("device flagged a non-finite state during the benchmark")

    # ---- end to end through the public API with host buffers --------------------
    host = torch.empty(case.shape, dtype=torch.float64, pin_memory=True).numpy()
    host[...] = q0
    e2e_steps = max(3, min(args.steps, 10))
    sim.upload(host)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sim.upload(host)
        sim.tvd_rk(0, case.dt)
        sim.download(host)
    t_e2e = time.perf_counter() - t0
    e2e, t_e2e = replica_rate(t_e2e, cells * e2e_steps, ws)
    state_bytes = int(np.prod(case.shape)) * 8

    # ---- rooflines ---------------------------------------------------------------------
    hbm, peak_kind = _peaks()
    per_launch_s = t_total / launches  # every timed launch is the stage kernel (2-D)
    bytes_per_update = 64 * case.sys_size  # 448 B for the benchmark's 2-D workload
    # algorithmic bytes of the timed steps over their time (in 2-D: one
    # launch's bytes over the launch's average duration)
    achieved = bytes_per_update * cells * args.steps / t_total / 1e9
    # the headline configuration, or a profiling run that names its own workload
    headline = args.case == "droplet2d" and args.precision == "fp64" and (args.nx, args.ny) == (NX, NY)
    prec_label = "plain FP64" if args.precision == "fp64" else args.precision
    if args.case == "droplet2d":
        workload = WORKLOAD if (args.nx, args.ny) == (NX, NY) else WORKLOAD.replace(f"{NX}x{NY}", f"{args.nx}x{args.ny}")
        workload = workload.replace("plain FP64", prec_label)
    else:
        workload = f"3-D shock-bubble {case.m + 1}^3, 2 fluids, WENO5-JS + HLLC + TVD-RK3, {prec_label} (profiling run)"
    metric = METRIC if headline else f"cell-updates/s ({workload})"
    # DRAM bytes per launch measured by ncu for the headline kernel only
    traffic = _profile_value("stage_kernel_fp64_droplet_1024x512.md", "dram_bytes_per_launch") if headline else None
    flops = _profile_value("flop_count_droplet_1024x512.md", "algorithmic_flops_per_cell_update")
    hbm_roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": traffic, "bytes_per_cell_update": bytes_per_update,
                "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback"}
    line = {
        "metric": metric, "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": {"fp64": "f64", "fp64_fma": "f64 (multiply-add contraction)", "split": "f64 state / f32 WENO+HLLC",
                  "gated": "f64 state / f32 WENO+HLLC + learned gate"}[args.precision],
        "data": "synthetic (reference-style case inputs, generated in-process)",
        "config": {"workload": workload,
                   "cells": cells, "equations": case.sys_size, "dt": case.dt,
                   "l2": "flushed between timed steps (256 MiB write)", "parallelism": f"replicas x{ws}",
                   "tile": {"variant": variant, "tx": tile[0], "ty": tile[1], "threads": tile[2],
                            "tma_staging": bool(sim.variant_features(variant) & _lib.MFC_VARIANT_TMA)}},
        "e2e": {"value": e2e, "unit": "cell-updates/s", "h2d_bytes_per_step": state_bytes,
                "d2h_bytes_per_step": state_bytes, "steps": e2e_steps},
        "roofline": hbm_roof,
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if flops and args.case == "droplet2d":
        # algorithmic flops of one launch (a third of a cell-update per cell)
        # over the launch's average CUDA-event duration
        fp64_bound = args.precision in ("fp64", "fp64_fma")
        peak = fp64_peak if fp64_bound else fp32_peak
        ach = flops * cells / 3 / per_launch_s / 1e12
        compute = {
            "bound": "fp64" if fp64_bound else "fp32", "achieved": ach, "peak": peak,
            "unit": "TFLOP/s", "frac": ach / peak, "traffic": traffic, "flops_per_cell_update": flops,
            "peak_kind": "measured in-process (FMA chains, mfc_gpu_measure_peaks; MEASURED_PEAKS.json has no "
                         "FP64/FP32 entry)",
            "peaks_measured": {"fp64_tflops": fp64_peak, "fp32_tflops": fp32_peak}}
        if args.precision == "fp64":
            # the peak counts an FMA as 2 flops; the bit-faithful path may fuse
            # nothing, so each algorithmic add or mul needs its own FP64 pipe
            # instruction (divisions run on the integer pipes): its ceiling is
            # half the flop peak
            compute["no_fma_ceiling_frac"] = ach / (peak / 2.0)
        # the slower-of roofline: the bound the kernel is closer to
        if compute["frac"] >= hbm_roof["frac"]:
            line["roofline"] = dict(compute, hbm=hbm_roof)
        else:
            line["roofline"] = dict(hbm_roof, compute=compute)
    sim.close()
    if not args.no_modes and args.precision == "fp64":
        line["modes"] = other_modes(args, case, x_cb, y_cb, q0, flush, value / ws)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
