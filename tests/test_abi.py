"""The C ABI library builds, loads, and exports every declared entry point;
host-side validation rejects bad cases before any device call (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

from microfc_gb300 import _lib, cases, preprocess
from microfc_gb300 import build as mbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "mfc_gpu.h")).read()
    return sorted(set(re.findall(r"\b(mfc_(?:gpu|gate)_\w+)\s*\(", text)))


def test_library_builds_and_exports_every_declared_symbol():
    mbuild.build()
    L = _lib.load()
    decl = declared_symbols()
    assert set(decl) == set(_lib.EXPORTS)
    for name in decl:
        assert hasattr(L, name), name
    assert L.mfc_gpu_abi_version() == 1


def _params(case, x_cb, y_cb=None):
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
    P.x_cb = x_cb.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    if y_cb is not None:
        P.y_cb = y_cb.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    return P


@pytest.mark.parametrize("field,value,msg", [
    ("m", 0, "Unsupported value of m"),
    ("weno_order", 4, "weno_order"),
    ("weno_eps", 1e-3, "weno_eps"),
    ("time_stepper", 4, "time_stepper"),
    ("bc_x_beg", -13, "Unsupported boundary condition"),
    ("bc_x_beg", -1, "Periodic"),
    ("num_fluids", 5, "num_fluids"),
])
def test_init_rejects_invalid_cases_without_touching_the_device(field, value, msg):
    L = _lib.load()
    case = cases.sod_1d(m=99, steps=10, dt=1e-4)
    x_cb, _, _, _ = preprocess.generate(case)
    P = _params(case, x_cb)
    setattr(P, field, value)
    h = ctypes.c_void_p()
    rc = L.mfc_gpu_init(ctypes.byref(P), ctypes.byref(h))
    assert rc == _lib.MFC_ERR_INVALID
    assert not h.value
    assert msg in L.mfc_gpu_last_error().decode()


def test_null_context_calls_fail_cleanly():
    L = _lib.load()
    assert L.mfc_gpu_tvd_rk(None, 1.0, 0) == _lib.MFC_ERR_INVALID
    assert L.mfc_gpu_finalize(None) == _lib.MFC_OK
    assert L.mfc_gpu_sys_size(None) == 0
    buf = np.zeros(4)
    assert L.mfc_gpu_upload_state(None, buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == _lib.MFC_ERR_INVALID
