"""Python host of the GB300 hot path, mirroring the reference's simulation
interfaces.

=====================================  =========================================
reference (src/simulation/...)         here
=====================================  =========================================
s_initialize_*_module                  ``Simulation(case, ...)`` -> mfc_gpu_init
!$acc update device(q_cons_ts(1))      ``Simulation.upload``    -> mfc_gpu_upload_state
!$acc update host(q_cons_ts(1))        ``Simulation.download``  -> mfc_gpu_download_state
s_compute_rhs (m_rhs.fpp:405)          ``Simulation.s_compute_rhs``
s_weno (m_weno.fpp:365)                ``Simulation.s_weno``    -> mfc_gpu_weno
s_hllc_riemann_solver                  ``Simulation.s_hllc_riemann_solver`` -> mfc_gpu_riemann
s_1st/2nd/3rd_order_tvd_rk             ``Simulation.s_1st_order_tvd_rk`` ...
p_main time loop (p_main.fpp:196-318)  ``Simulation.run``       -> mfc_gpu_run
s_finalize_*_module                    ``Simulation.close``     -> mfc_gpu_finalize
=====================================  =========================================

Every call goes through the C ABI of ``libmfc_gpu.so``; there is no CPU path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from . import preprocess
from .case import Case


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_params(case: Case, x_cb, y_cb=None, z_cb=None, device: int = 0):
    """The mfc_params block of a case; returns (params, arrays it points to)."""
    cb = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (x_cb, y_cb, z_cb)]
    P = _lib.MfcParams()
    P.m, P.n, P.p = case.m, case.n, case.p
    P.num_fluids = case.num_fluids
    P.weno_order = case.weno_order
    P.weno_eps = case.weno_eps
    P.time_stepper = case.time_stepper
    P.bc_x_beg, P.bc_x_end = case.bc_x
    P.bc_y_beg, P.bc_y_end = case.bc_y
    P.bc_z_beg, P.bc_z_end = case.bc_z
    for i in range(case.num_fluids):
        P.gammas[i] = case.gammas[i]
        P.pi_infs[i] = case.pi_infs[i]
    P.x_cb = _dp(cb[0])
    P.y_cb = _dp(cb[1]) if cb[1] is not None else None
    P.z_cb = _dp(cb[2]) if cb[2] is not None else None
    P.precision = {"fp64": _lib.MFC_PREC_FP64, "split": _lib.MFC_PREC_SPLIT,
                   "gated": _lib.MFC_PREC_GATED, "fp64_fma": _lib.MFC_PREC_FP64_FMA}[case.precision]
    P.device = device
    return P, cb


class Simulation:
    """Device-resident state of one case (q_cons_ts, rhs, grid, WENO tables)."""

    def __init__(self, case: Case, x_cb=None, y_cb=None, z_cb=None, q_cons=None, device: int = 0,
                 check: bool = True, ic: str = "host"):
        """ic: where the initial condition comes from when q_cons is None --
        "host" (preprocess.generate, then an upload) or "device"
        (mfc_gpu_generate_ic writes it in place)."""
        if check:
            case.check()
        if ic not in ("host", "device"):
            raise ValueError("ic must be 'host' or 'device'")
        self.case = case
        on_device = q_cons is None and ic == "device"
        if on_device:
            gx, gy, gz = preprocess.grid(case)
            x_cb = gx if x_cb is None else x_cb
            y_cb = gy if y_cb is None else y_cb
            z_cb = gz if z_cb is None else z_cb
        elif x_cb is None or q_cons is None:
            gx, gy, gz, gq = preprocess.generate(case)
            x_cb = gx if x_cb is None else x_cb
            y_cb = gy if y_cb is None else y_cb
            z_cb = gz if z_cb is None else z_cb
            q_cons = gq if q_cons is None else q_cons
        self.L = _lib.load()
        P, self._cb = make_params(case, x_cb, y_cb, z_cb, device)
        self._params = P
        h = ctypes.c_void_p()
        _lib.check(self.L.mfc_gpu_init(ctypes.byref(P), ctypes.byref(h)))
        self._h = h
        self.S = self.L.mfc_gpu_sys_size(h)
        self.dt = case.dt
        if case.viscous:
            self.set_viscosity(case.re_shear, case.re_bulk)
            if case.weno_re_flux:
                self.set_viscous_gradients(True)
        if case.char_decomp:
            self.set_reconstruction("characteristic")
        if on_device:
            self.generate_ic()
        else:
            self.upload(q_cons)

    def generate_ic(self, case: Case | None = None) -> None:
        """pre_process on the device: the case's patches straight into q_cons_ts(1)."""
        arr, dom = preprocess.device_patches(case or self.case)
        _lib.check(self.L.mfc_gpu_generate_ic(self._h, arr, len(arr), None if dom is None else _dp(dom)))

    # -- life cycle -----------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self.L.mfc_gpu_finalize(self._h)
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

    # -- state transfer -------------------------------------------------------
    def upload(self, q: np.ndarray) -> None:
        a = np.ascontiguousarray(q, dtype=np.float64).reshape(self.case.shape)
        _lib.check(self.L.mfc_gpu_upload_state(self._h, _dp(a)))

    def download(self, out: np.ndarray | None = None) -> np.ndarray:
        a = out if out is not None else np.empty(self.case.shape, dtype=np.float64)
        _lib.check(self.L.mfc_gpu_download_state(self._h, _dp(a)))
        return a

    def snapshot(self, slot: int = 0) -> None:
        """Start an asynchronous copy of the current state into pinned slot 0 or 1
        (mfc_gpu_snapshot); time steps issued afterwards overlap with it."""
        _lib.check(self.L.mfc_gpu_snapshot(self._h, int(slot)))

    def snapshot_wait(self, slot: int = 0) -> np.ndarray:
        """The state of the slot's last snapshot, once it has landed.  A view of
        pinned memory, valid until the slot's next snapshot or close()."""
        ptr = ctypes.POINTER(ctypes.c_double)()
        _lib.check(self.L.mfc_gpu_snapshot_wait(self._h, int(slot), ctypes.byref(ptr)))
        return np.ctypeslib.as_array(ptr, shape=self.case.shape)

    def upload_var(self, var: int, sf: np.ndarray, ld_y: int, ld_z: int = 0) -> None:
        """Copy one equation from a host array laid out like q_cons_vf(var)%sf."""
        _lib.check(self.L.mfc_gpu_upload(self._h, int(var), _dp(sf), int(ld_y), int(ld_z)))

    def download_var(self, var: int, sf: np.ndarray, ld_y: int, ld_z: int = 0) -> None:
        _lib.check(self.L.mfc_gpu_download(self._h, int(var), _dp(sf), int(ld_y), int(ld_z)))

    # -- the hot path -----------------------------------------------------------
    def s_compute_rhs(self):
        """RHS and primitive variables of the current state (both [S,p+1,n+1,m+1])."""
        rhs = np.empty(self.case.shape)
        prim = np.empty(self.case.shape)
        _lib.check(self.L.mfc_gpu_compute_rhs(self._h, _dp(rhs), _dp(prim)))
        return rhs, prim

    def face_shape(self, direction: int, faces: bool = False) -> tuple:
        """Shape of the face window of a direction: [S, p+1, n+1, m+1] with
        the extent along it widened to the cells -1 .. s+1 (faces=False) or
        the faces -1/2 .. s+1/2 (faces=True)."""
        shape = list(self.case.shape)
        shape[3 - direction] += 1 if faces else 2
        return tuple(shape)

    def s_weno(self, direction: int):
        """s_weno of the current state along a direction over the face window:
        (vL, vR), the left- and right-face values of every cell."""
        shape = self.face_shape(direction)
        vl, vr = np.empty(shape), np.empty(shape)
        _lib.check(self.L.mfc_gpu_weno(self._h, int(direction), _dp(vl), _dp(vr)))
        return vl, vr

    def s_hllc_riemann_solver(self, direction: int, qL_rs, qR_rs):
        """s_hllc_riemann_solver along a direction: qL_rs(j) is the state left
        of face j+1/2, qR_rs(j+1) the state right of it (s_compute_rhs passes
        vR and vL of s_weno).  Returns (flux [S, ...], flux_src [...]) over the
        faces -1/2 .. s+1/2."""
        shape = self.face_shape(direction)
        a = np.ascontiguousarray(qL_rs, dtype=np.float64).reshape(shape)
        b = np.ascontiguousarray(qR_rs, dtype=np.float64).reshape(shape)
        fshape = self.face_shape(direction, faces=True)
        flux, src = np.empty(fshape), np.empty(fshape[1:])
        _lib.check(self.L.mfc_gpu_riemann(self._h, int(direction), _dp(a), _dp(b), _dp(flux), _dp(src)))
        return flux, src

    def tvd_rk(self, t_step: int, dt: float | None = None) -> None:
        """One call of the configured s_*_order_tvd_rk (asynchronous)."""
        last = int(t_step == self.case.t_step_stop)
        _lib.check(self.L.mfc_gpu_tvd_rk(self._h, float(self.dt if dt is None else dt), last))

    s_1st_order_tvd_rk = s_2nd_order_tvd_rk = s_3rd_order_tvd_rk = tvd_rk

    def run(self, t_step_start: int | None = None, t_step_stop: int | None = None) -> float:
        """The p_main time loop; returns the (possibly trimmed) final dt."""
        a = self.case.t_step_start if t_step_start is None else t_step_start
        b = self.case.t_step_stop if t_step_stop is None else t_step_stop
        dt = ctypes.c_double(self.case.dt)
        _lib.check(self.L.mfc_gpu_run(self._h, int(a), int(b), ctypes.byref(dt)))
        self.dt = dt.value
        return dt.value

    def tune(self, reps: int = 5):
        """Autotune the tile variant (mfc_gpu_tune); returns (index, ms per stage)."""
        v, ms = ctypes.c_int(-1), ctypes.c_double(0)
        _lib.check(self.L.mfc_gpu_tune(self._h, int(reps), ctypes.byref(v), ctypes.byref(ms)))
        return v.value, ms.value

    def set_viscosity(self, re_shear=(), re_bulk=()) -> None:
        """fluid_pp(i)%Re(1:2) of the case's fluids (mfc_gpu_set_viscosity);
        all zero switches back to the inviscid kernels."""
        nf = self.case.num_fluids
        a = np.zeros(nf)
        b = np.zeros(nf)
        a[:len(re_shear)] = re_shear
        b[:len(re_bulk)] = re_bulk
        _lib.check(self.L.mfc_gpu_set_viscosity(self._h, _dp(a), _dp(b)))

    def set_viscous_gradients(self, weno_re_flux: bool = True) -> None:
        """weno_Re_flux: the viscous stresses from WENO-reconstructed velocity
        gradients (True) or the default finite differences (False);
        mfc_gpu_set_viscous_gradients."""
        _lib.check(self.L.mfc_gpu_set_viscous_gradients(self._h, int(bool(weno_re_flux))))

    def set_reconstruction(self, variables: str = "primitive") -> None:
        """WENO of the "primitive" variables (the reference's choice) or of
        the "characteristic" fields (mfc_gpu_set_reconstruction)."""
        code = {"primitive": _lib.MFC_RECON_PRIMITIVE, "characteristic": _lib.MFC_RECON_CHARACTERISTIC}[variables]
        _lib.check(self.L.mfc_gpu_set_reconstruction(self._h, code))

    def set_uniform_coefficients(self, enable: bool = True) -> int:
        """Split/gated WENO5 on a uniform grid reads one shared coefficient
        record per direction (on by default, identical results); returns the
        directions using it as a bit mask (x 1, y 2, z 4)."""
        used = ctypes.c_int(0)
        _lib.check(self.L.mfc_gpu_set_uniform_coefficients(self._h, int(bool(enable)), ctypes.byref(used)))
        return used.value

    def select_variant(self, variant: int):
        """Pin a tile variant (mfc_gpu_select_variant); returns (tx, ty, threads)."""
        tx, ty, nt = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        _lib.check(self.L.mfc_gpu_select_variant(self._h, int(variant), ctypes.byref(tx), ctypes.byref(ty),
                                                 ctypes.byref(nt)))
        return tx.value, ty.value, nt.value

    def variant_features(self, variant: int) -> int:
        """MFC_VARIANT_* bits of a tile variant (mfc_gpu_variant_features)."""
        f = ctypes.c_uint32(0)
        _lib.check(self.L.mfc_gpu_variant_features(self._h, int(variant), ctypes.byref(f)))
        return f.value

    def set_monitor(self, on: bool = True) -> None:
        """Fused ICFL monitor (the reference's run-time information)."""
        _lib.check(self.L.mfc_gpu_set_monitor(self._h, int(bool(on))))

    def icfl(self, reset: bool = False) -> float:
        v = ctypes.c_double(0)
        _lib.check(self.L.mfc_gpu_icfl(self._h, ctypes.byref(v), int(bool(reset))))
        return v.value

    def run_cfl(self, num_steps: int, cfl: float, dt: float | None = None, time: float = 0.0):
        """num_steps steps at a constant CFL number; returns (next dt, time)."""
        d = ctypes.c_double(self.case.dt if dt is None else dt)
        t = ctypes.c_double(time)
        _lib.check(self.L.mfc_gpu_run_cfl(self._h, int(num_steps), float(cfl), ctypes.byref(d), ctypes.byref(t)))
        return d.value, t.value

    def set_gate(self, params) -> None:
        """Parameters (FP32, mfc_gate_param_count values) of the learned gate."""
        w = np.ascontiguousarray(params, dtype=np.float32)
        _lib.check(self.L.mfc_gpu_set_gate(self._h, w.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    def gate_samples(self, direction: int, x_dev_ptr: int, dev_dev_ptr: int) -> None:
        """Gate training samples of the current state into device buffers."""
        _lib.check(self.L.mfc_gpu_gate_samples(self._h, int(direction), ctypes.c_void_p(x_dev_ptr),
                                               ctypes.c_void_p(dev_dev_ptr)))

    def status(self, clear: bool = False) -> int:
        f = ctypes.c_uint32(0)
        _lib.check(self.L.mfc_gpu_status(self._h, ctypes.byref(f), int(clear)))
        return f.value

    @property
    def stream(self) -> int:
        """The cudaStream_t the context launches on (as an integer handle)."""
        return self.L.mfc_gpu_stream(self._h) or 0

    @property
    def launches(self) -> int:
        return self.L.mfc_gpu_launch_count(self._h)
