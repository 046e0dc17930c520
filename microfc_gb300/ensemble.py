"""Ensemble mode: many independent 2-D cases advanced together.

``Ensemble(cases)`` uploads every case and advances all of them with one
persistent launch per RK stage (C ABI ``mfc_gpu_ensemble_*``); ``run``
replays the stage launches of a step from a CUDA graph; ``tune`` runs the
project's autotuner over the compiled tile shapes.  Each case keeps its own
grid, boundary conditions, fluids and dt, and gets the same bits it would
get from a ``Simulation`` of its own.

``random_droplet_cases`` builds the seeded ensemble of 2-D shock-droplet
cases: nx drawn from {128, 256, 384, 512}, ny = nx/2, Mach uniform in
[1.2, 2.5], droplet radius uniform in [1, 3] mm (numpy default_rng(seed)).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib, cases, preprocess
from .solver import _dp, make_params


def random_droplet_cases(count: int = 64, seed: int = 0, steps: int = 500, precision: str = "split",
                         sizes=(128, 256, 384, 512)):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        nx = int(rng.choice(sizes))
        mach = float(rng.uniform(1.2, 2.5))
        radius = float(rng.uniform(1e-3, 3e-3))
        out.append(cases.shock_droplet_2d(nx=nx, ny=nx // 2, mach=mach, radius=radius, steps=steps,
                                          precision=precision))
    return out


class Ensemble:
    def __init__(self, case_list, states=None, device: int = 0, ic: str = "host"):
        """states: initial states per case; without them the cases' patches
        give the initial condition, built on the host (ic="host") or written
        in place by the device generator (ic="device", no host arrays)."""
        if ic not in ("host", "device"):
            raise ValueError("ic must be 'host' or 'device'")
        self.cases = list(case_list)
        self.L = _lib.load()
        params = (_lib.MfcParams * len(self.cases))()
        self._keep = []
        self.grids = []
        qs = []
        on_device = states is None and ic == "device"
        for i, c in enumerate(self.cases):
            c.check()
            if on_device:
                x_cb, y_cb, _ = preprocess.grid(c)
                q = None
            else:
                x_cb, y_cb, _, q = preprocess.generate(c)
                if states is not None:
                    q = states[i]
                q = np.ascontiguousarray(q, dtype=np.float64)
            P, cb = make_params(c, x_cb, y_cb, None, device)
            params[i] = P
            self._keep.append(cb)
            self.grids.append((x_cb, y_cb))
            qs.append(q)
        if any(c.viscous and c.weno_re_flux for c in self.cases):
            raise ValueError("the ensemble's viscous terms use the finite-difference gradients "
                             "(weno_Re_flux = F)")
        dts = np.array([c.dt for c in self.cases], dtype=np.float64)
        h = ctypes.c_void_p()
        _lib.check(self.L.mfc_gpu_ensemble_init(params, _dp(dts), len(self.cases), ctypes.byref(h)))
        self._h = h
        if any(c.viscous for c in self.cases):
            self.set_viscosity([c.re_shear for c in self.cases], [c.re_bulk for c in self.cases])
        for i, q in enumerate(qs):
            if on_device:
                self.generate_ic(i)
            else:
                self.upload(i, q)

    def generate_ic(self, i: int) -> None:
        """pre_process of case i on the device, straight into its state."""
        arr, dom = preprocess.device_patches(self.cases[i])
        _lib.check(self.L.mfc_gpu_ensemble_generate_ic(self._h, int(i), arr, len(arr),
                                                       None if dom is None else _dp(dom)))

    def close(self):
        if getattr(self, "_h", None):
            self.L.mfc_gpu_ensemble_finalize(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def cells(self) -> int:
        return sum(c.cells for c in self.cases)

    def upload(self, i: int, q: np.ndarray) -> None:
        a = np.ascontiguousarray(q, dtype=np.float64).reshape(self.cases[i].shape)
        _lib.check(self.L.mfc_gpu_ensemble_upload(self._h, int(i), _dp(a)))

    def download(self, i: int) -> np.ndarray:
        a = np.empty(self.cases[i].shape)
        _lib.check(self.L.mfc_gpu_ensemble_download(self._h, int(i), _dp(a)))
        return a

    def set_viscosity(self, re_shear, re_bulk) -> None:
        """fluid_pp(f)%Re(1:2) of every case (one sequence of num_fluids
        values per case; mfc_gpu_ensemble_set_viscosity).  Every case must be
        viscous, or none."""
        nf = self.cases[0].num_fluids

        def table(rows):
            a = np.zeros((len(self.cases), nf))
            for i, r in enumerate(rows):
                a[i, :len(r)] = r
            return a

        a, b = table(re_shear), table(re_bulk)
        _lib.check(self.L.mfc_gpu_ensemble_set_viscosity(self._h, _dp(a), _dp(b)))

    def set_gate(self, params) -> None:
        """Parameters of the learned gate (precision "gated")."""
        w = np.ascontiguousarray(params, dtype=np.float32)
        _lib.check(self.L.mfc_gpu_ensemble_set_gate(self._h, w.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    def select_variant(self, variant: int):
        """Pin a tile variant (mfc_gpu_ensemble_select_variant); returns (tx, ty, threads)."""
        tx, ty, nt = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        _lib.check(self.L.mfc_gpu_ensemble_select_variant(self._h, int(variant), ctypes.byref(tx), ctypes.byref(ty),
                                                          ctypes.byref(nt)))
        return tx.value, ty.value, nt.value

    def variant_features(self, variant: int) -> int:
        """MFC_VARIANT_* bits of a tile variant (mfc_gpu_ensemble_variant_features)."""
        f = ctypes.c_uint32(0)
        _lib.check(self.L.mfc_gpu_ensemble_variant_features(self._h, int(variant), ctypes.byref(f)))
        return f.value

    def tune(self, reps: int = 5):
        v, ms = ctypes.c_int(-1), ctypes.c_double(0)
        _lib.check(self.L.mfc_gpu_ensemble_tune(self._h, int(reps), ctypes.byref(v), ctypes.byref(ms)))
        return v.value, ms.value

    def run(self, t_step_start: int, t_step_stop: int, use_graph: bool = True) -> None:
        _lib.check(self.L.mfc_gpu_ensemble_run(self._h, int(t_step_start), int(t_step_stop), int(bool(use_graph))))

    @property
    def stream(self) -> int:
        return self.L.mfc_gpu_ensemble_stream(self._h) or 0

    @property
    def launches(self) -> int:
        return self.L.mfc_gpu_ensemble_launch_count(self._h)
