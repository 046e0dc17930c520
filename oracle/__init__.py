"""ctypes binding of the MicroFC oracle -- test infrastructure only.

The oracle is a CPU restatement of MicroFC's RHS + TVD-RK step (see
``mfc_oracle.hpp`` for the reference files it follows).  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import
this module, and only as the checker.  Parity against the reference's own
build is unpinned: the reference is Fortran and no Fortran compiler is
available; the oracle is pinned by analytic known-answer tests instead.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libmfc_oracle.so")
# the same sources built with the reference's Release flags (-O3, -march /
# -mcpu=native, default FMA contraction): the timed CPU baseline, and the
# stand-in for a default-flag CPU build of the reference
_LIB_NATIVE_PATH = os.path.join(_HERE, "libmfc_oracle_native.so")
_PATHS = {"exact": _LIB_PATH, "native": _LIB_NATIVE_PATH}
_lock = threading.Lock()
_libs = {}

MAX_FLUIDS = 4
MAX_PATCHES = 10


class MfoParams(ctypes.Structure):
    _fields_ = [
        ("m", ctypes.c_int), ("n", ctypes.c_int), ("p", ctypes.c_int),
        ("num_fluids", ctypes.c_int),
        ("weno_order", ctypes.c_int),
        ("weno_eps", ctypes.c_double),
        ("time_stepper", ctypes.c_int),
        ("bc_x_beg", ctypes.c_int), ("bc_x_end", ctypes.c_int),
        ("bc_y_beg", ctypes.c_int), ("bc_y_end", ctypes.c_int),
        ("bc_z_beg", ctypes.c_int), ("bc_z_end", ctypes.c_int),
        ("gammas", ctypes.c_double * MAX_FLUIDS),
        ("pi_infs", ctypes.c_double * MAX_FLUIDS),
        ("re_shear", ctypes.c_double * MAX_FLUIDS),
        ("re_bulk", ctypes.c_double * MAX_FLUIDS),
        ("char_decomp", ctypes.c_int),
        ("weno_re_flux", ctypes.c_int),
    ]


class MfoPatch(ctypes.Structure):
    _fields_ = [
        ("geometry", ctypes.c_int),
        ("x_centroid", ctypes.c_double), ("y_centroid", ctypes.c_double), ("z_centroid", ctypes.c_double),
        ("length_x", ctypes.c_double), ("length_y", ctypes.c_double), ("length_z", ctypes.c_double),
        ("radius", ctypes.c_double),
        ("smoothen", ctypes.c_int),
        ("smooth_patch_id", ctypes.c_int),
        ("smooth_coeff", ctypes.c_double),
        ("alter_patch", ctypes.c_int * (MAX_PATCHES + 1)),
        ("alpha_rho", ctypes.c_double * MAX_FLUIDS),
        ("alpha", ctypes.c_double * MAX_FLUIDS),
        ("vel", ctypes.c_double * 3),
        ("pres", ctypes.c_double),
        ("normal", ctypes.c_double * 3),
        ("radii", ctypes.c_double * 3),
        ("epsilon", ctypes.c_double),
    ]


def build(force: bool = False) -> str:
    """Compile both oracle builds with their Makefile (g++ only; seconds)."""
    with _lock:
        if force or any(not os.path.exists(p) or _stale(p) for p in _PATHS.values()):
            subprocess.run(["make", "-s", "-C", _HERE, "-j4"], check=True)
    return _LIB_PATH


def _stale(path: str) -> bool:
    t = os.path.getmtime(path)
    for f in os.listdir(_HERE):
        if f.endswith((".cpp", ".hpp", "Makefile")) and os.path.getmtime(os.path.join(_HERE, f)) > t:
            return True
    return False


def lib(variant: str = "exact"):
    """The oracle library: "exact" (no FMA contraction; the parity oracle) or
    "native" (the reference's Release flags)."""
    if variant not in _libs:
        build()
        L = ctypes.CDLL(_PATHS[variant])
        dp = ctypes.POINTER(ctypes.c_double)
        L.mfo_create.restype = ctypes.c_void_p
        L.mfo_create.argtypes = [ctypes.POINTER(MfoParams), dp, dp, dp]
        L.mfo_destroy.argtypes = [ctypes.c_void_p]
        L.mfo_sys_size.argtypes = [ctypes.c_void_p]
        L.mfo_set_state.argtypes = [ctypes.c_void_p, ctypes.c_int, dp]
        L.mfo_get_state.argtypes = [ctypes.c_void_p, ctypes.c_int, dp]
        L.mfo_compute_rhs.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, dp]
        L.mfo_tvd_rk.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int]
        L.mfo_run.restype = ctypes.c_double
        L.mfo_run.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.mfo_set_threads.argtypes = [ctypes.c_int]
        L.mfo_get_threads.restype = ctypes.c_int
        L.mfo_generate_ic.restype = ctypes.c_int
        L.mfo_generate_ic.argtypes = [ctypes.POINTER(MfoParams), ctypes.POINTER(MfoPatch), ctypes.c_int,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_double, dp, dp, dp, dp, dp]
        L.mfo_weno.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, dp, dp]
        L.mfo_riemann.argtypes = [ctypes.c_void_p, ctypes.c_int, dp, dp, dp, dp]
        L.mfo_count_ops.restype = ctypes.c_int
        L.mfo_count_ops.argtypes = [ctypes.POINTER(MfoParams), dp, dp, dp, dp, ctypes.c_double, dp]
        _libs[variant] = L
    return _libs[variant]


def _dp(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def params_from_case(case) -> MfoParams:
    """Build the oracle's parameter block from a ``microfc_gb300`` case."""
    q = MfoParams()
    q.m, q.n, q.p = case.m, case.n, case.p
    q.num_fluids = case.num_fluids
    q.weno_order = case.weno_order
    q.weno_eps = case.weno_eps
    q.time_stepper = case.time_stepper
    q.bc_x_beg, q.bc_x_end = case.bc_x
    q.bc_y_beg, q.bc_y_end = case.bc_y
    q.bc_z_beg, q.bc_z_end = case.bc_z
    for i, (g, pi) in enumerate(zip(case.gammas, case.pi_infs)):
        q.gammas[i] = g
        q.pi_infs[i] = pi
    for i, r in enumerate(getattr(case, "re_shear", ())):
        q.re_shear[i] = r
    for i, r in enumerate(getattr(case, "re_bulk", ())):
        q.re_bulk[i] = r
    q.char_decomp = int(bool(getattr(case, "char_decomp", False)))
    q.weno_re_flux = int(bool(getattr(case, "weno_re_flux", False)))
    return q


class Oracle:
    """The oracle solver for one case (state of shape [S, p+1, n+1, m+1])."""

    def __init__(self, case, x_cb, y_cb=None, z_cb=None, threads: int = 0, build: str = "exact"):
        self._L = L = lib(build)
        self.build = build
        if threads:
            L.mfo_set_threads(int(threads))
        self.case = case
        self._q = params_from_case(case)
        self._cb = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None
                    for a in (x_cb, y_cb, z_cb)]
        self._h = L.mfo_create(ctypes.byref(self._q), *(_dp(a) for a in self._cb))
        if not self._h:
            raise ValueError("oracle creation failed (missing cell boundaries of a used direction, or no memory)")
        self.S = L.mfo_sys_size(self._h)
        self.shape = (self.S, case.p + 1, case.n + 1, case.m + 1)

    def close(self):
        if getattr(self, "_h", None):
            self._L.mfo_destroy(self._h)
            self._h = None

    __del__ = close

    def set_state(self, q, reg: int = 0):
        a = np.ascontiguousarray(q, dtype=np.float64).reshape(self.shape)
        self._L.mfo_set_state(self._h, reg, _dp(a))

    def get_state(self, reg: int = 0):
        a = np.empty(self.shape, dtype=np.float64)
        self._L.mfo_get_state(self._h, reg, _dp(a))
        return a

    def compute_rhs(self, reg: int = 0):
        rhs = np.empty(self.shape, dtype=np.float64)
        prim = np.empty(self.shape, dtype=np.float64)
        self._L.mfo_compute_rhs(self._h, reg, _dp(rhs), _dp(prim))
        return rhs, prim

    def face_shape(self, dir: int, faces: bool = False):
        """[S, p+1, n+1, m+1] with the extent along dir widened to the face
        window: cells -1 .. s+1 (faces=False) or faces -1/2 .. s+1/2."""
        shape = list(self.shape)
        shape[3 - dir] += 1 if faces else 2
        return tuple(shape)

    def weno(self, dir: int, reg: int = 0):
        """s_weno of register reg along dir over the face window: (vL, vR)."""
        shape = self.face_shape(dir)
        vl, vr = np.empty(shape), np.empty(shape)
        self._L.mfo_weno(self._h, reg, dir, _dp(vl), _dp(vr))
        return vl, vr

    def riemann(self, dir: int, qL_rs, qR_rs):
        """s_hllc_riemann_solver along dir: (flux [S, ...], flux_src [...])."""
        shape = self.face_shape(dir)
        a = np.ascontiguousarray(qL_rs, dtype=np.float64).reshape(shape)
        b = np.ascontiguousarray(qR_rs, dtype=np.float64).reshape(shape)
        fshape = self.face_shape(dir, faces=True)
        flux, src = np.empty(fshape), np.empty(fshape[1:])
        self._L.mfo_riemann(self._h, dir, _dp(a), _dp(b), _dp(flux), _dp(src))
        return flux, src

    def tvd_rk(self, dt: float, last_step: bool = False):
        self._L.mfo_tvd_rk(self._h, float(dt), int(bool(last_step)))

    def run(self, t_step_start: int, t_step_stop: int, dt: float) -> float:
        return self._L.mfo_run(self._h, int(t_step_start), int(t_step_stop), float(dt))

    def count_ops(self, state, dt: float):
        """Operation counts per interior cell for one full time step."""
        a = np.ascontiguousarray(state, dtype=np.float64).reshape(self.shape)
        out = np.zeros(5, dtype=np.float64)
        self._L.mfo_count_ops(ctypes.byref(self._q), *(_dp(c) for c in self._cb), _dp(a), float(dt), _dp(out))
        return dict(zip(("add", "mul", "div", "sqrt", "cmp"), out.tolist()))


def generate_ic(case):
    """pre_process restatement: returns (x_cb, y_cb, z_cb, cons[S,p+1,n+1,m+1])."""
    L = lib()
    q = params_from_case(case)
    P = len(case.patches)
    arr = (MfoPatch * P)()
    for i, pt in enumerate(case.patches):
        a = arr[i]
        a.geometry = pt.geometry
        a.x_centroid, a.y_centroid, a.z_centroid = pt.centroid
        a.length_x, a.length_y, a.length_z = pt.length
        a.radius = pt.radius
        a.smoothen = int(pt.smoothen)
        a.smooth_patch_id = pt.smooth_patch_id if pt.smooth_patch_id else i + 1
        a.smooth_coeff = pt.smooth_coeff
        for j in range(MAX_PATCHES + 1):
            a.alter_patch[j] = 1 if j in pt.alter_patch or j == 0 else 0
        for f in range(case.num_fluids):
            a.alpha_rho[f] = pt.alpha_rho[f]
            a.alpha[f] = pt.alpha[f]
        for d in range(3):
            a.vel[d] = pt.vel[d] if d < len(pt.vel) else 0.0
            a.normal[d] = pt.normal[d] if d < len(pt.normal) else 0.0
            a.radii[d] = pt.radii[d] if d < len(pt.radii) else 0.0
        a.pres = pt.pres
        a.epsilon = pt.epsilon
    S = case.sys_size
    x_cb = np.zeros(case.m + 2)
    y_cb = np.zeros(case.n + 2)
    z_cb = np.zeros(case.p + 2)
    cons = np.zeros((S, case.p + 1, case.n + 1, case.m + 1))
    (xb, xe), (yb, ye), (zb, ze) = case.x_domain, case.y_domain, case.z_domain
    st = np.zeros(8)
    for k, s in enumerate((case.stretch_x, case.stretch_y)):
        if s:
            st[4 * k: 4 * k + 4] = s
    rc = L.mfo_generate_ic(ctypes.byref(q), arr, P, xb, xe, yb, ye, zb, ze, _dp(st),
                           _dp(x_cb), _dp(y_cb), _dp(z_cb), _dp(cons))
    if rc != 0:
        raise ValueError(f"oracle IC generation failed ({rc})")
    return x_cb, (y_cb if case.n > 0 else None), (z_cb if case.p > 0 else None), cons
