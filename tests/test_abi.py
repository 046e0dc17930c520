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


def _fortran_bridge():
    return open(os.path.join(ROOT, "microfc_gb300", "fortran", "m_gpu_bridge.f90")).read()


def test_fortran_bridge_binds_only_declared_and_exported_entry_points():
    """The bind(C) names of the (uncompiled) Fortran bridge are entry points
    of include/mfc_gpu.h that the library exports, and every entry point the
    bridge calls has its interface there."""
    text = _fortran_bridge()
    bound = set(re.findall(r"bind\(C,\s*name='(\w+)'\)", text))
    assert {"mfc_gpu_init", "mfc_gpu_upload", "mfc_gpu_download", "mfc_gpu_tvd_rk", "mfc_gpu_status",
            "mfc_gpu_finalize", "mfc_gpu_set_viscosity", "mfc_gpu_set_viscous_gradients"} <= bound
    assert bound <= set(declared_symbols())
    mbuild.build()
    L = _lib.load()
    for name in bound:
        assert hasattr(L, name), name
    called = set(re.findall(r"\b(mfc_gpu_\w+)\(", re.sub(r"(?m)^\s*!.*$", "", text)))
    assert called <= bound, called - bound


def test_fortran_bridge_params_type_mirrors_the_header_struct():
    """mfc_params_t (bind(C)) lists the members of mfc_params in the same
    order with the same kinds, and its fluid arrays have MFC_MAX_FLUIDS
    elements, so the two layouts agree."""
    text = _fortran_bridge()
    body = re.search(r"type, bind\(C\) :: mfc_params_t\n(.*?)end type mfc_params_t", text, re.S).group(1)
    f_fields = []
    for kind, names in re.findall(r"^\s*(integer\(c_int32_t\)|real\(c_double\)|type\(c_ptr\))\s*::\s*(.+)$", body,
                                  re.M):
        for nm in names.split(","):
            nm = nm.strip()
            size = re.search(r"\((\d+)\)", nm)
            f_fields.append((re.sub(r"\(.*\)", "", nm), {"integer(c_int32_t)": "int32_t", "real(c_double)": "double",
                                                          "type(c_ptr)": "ptr"}[kind],
                             int(size.group(1)) if size else 1))
    header = open(os.path.join(ROOT, "include", "mfc_gpu.h")).read()
    max_fluids = int(re.search(r"#define MFC_MAX_FLUIDS (\d+)", header).group(1))
    struct = re.search(r"typedef struct mfc_params \{(.*?)\} mfc_params;", header, re.S).group(1)
    c_fields = []
    for line in struct.splitlines():
        line = re.sub(r"/\*.*?\*/", "", line).strip()
        if not line:
            continue
        m = re.match(r"(const double\*|int32_t|double)\s+(.+);", line)
        kind = {"const double*": "ptr", "int32_t": "int32_t", "double": "double"}[m.group(1)]
        for nm in m.group(2).split(","):
            nm = nm.strip()
            arr = re.search(r"\[(\w+)\]", nm)
            n = (max_fluids if arr.group(1) == "MFC_MAX_FLUIDS" else int(arr.group(1))) if arr else 1
            c_fields.append((re.sub(r"\[.*\]", "", nm), kind, n))
    assert f_fields == c_fields
    assert [f[0] for f in c_fields] == [f[0] for f in _lib.MfcParams._fields_]
