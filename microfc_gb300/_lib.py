"""ctypes binding of ``libmfc_gpu.so`` (the C ABI in include/mfc_gpu.h).

The library is built in-tree by :mod:`microfc_gb300.build`.  There is no CPU
fallback: if the library cannot be built or loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

MFC_MAX_FLUIDS = 4
MFC_OK, MFC_ERR_INVALID, MFC_ERR_CUDA, MFC_ERR_NOMEM, MFC_ERR_STATE = 0, 1, 2, 3, 4
MFC_FLAG_NAN, MFC_FLAG_NEG_PRESSURE, MFC_FLAG_TIMEOUT = 0x1, 0x2, 0x4
MFC_PREC_FP64, MFC_PREC_SPLIT = 0, 1

# every symbol include/mfc_gpu.h declares (checked by the tests)
EXPORTS = (
    "mfc_gpu_abi_version", "mfc_gpu_last_error", "mfc_gpu_init", "mfc_gpu_sys_size",
    "mfc_gpu_upload", "mfc_gpu_download", "mfc_gpu_upload_state", "mfc_gpu_download_state",
    "mfc_gpu_compute_rhs", "mfc_gpu_weno", "mfc_gpu_riemann", "mfc_gpu_set_reconstruction", "mfc_gpu_tvd_rk", "mfc_gpu_run", "mfc_gpu_status", "mfc_gpu_stream",
    "mfc_gpu_launch_count", "mfc_gpu_finalize", "mfc_gpu_measure_peaks", "mfc_gpu_tvd_rk_noalloc",
    "mfc_gpu_selftest_div",
    "mfc_gpu_tune", "mfc_gpu_ensemble_init", "mfc_gpu_ensemble_upload", "mfc_gpu_ensemble_download",
    "mfc_gpu_ensemble_tune", "mfc_gpu_ensemble_run", "mfc_gpu_ensemble_stream", "mfc_gpu_ensemble_launch_count",
    "mfc_gpu_ensemble_finalize", "mfc_gpu_ensemble_set_gate", "mfc_gpu_ensemble_set_viscosity", "mfc_gate_param_count", "mfc_gate_workspace_floats",
    "mfc_gpu_set_gate", "mfc_gpu_gate_samples", "mfc_gate_gradients", "mfc_gate_train_step", "mfc_gate_infer",
    "mfc_gpu_set_monitor", "mfc_gpu_icfl", "mfc_gpu_run_cfl", "mfc_gpu_generate_ic", "mfc_gpu_ensemble_generate_ic",
    "mfc_gpu_snapshot", "mfc_gpu_snapshot_wait", "mfc_gpu_select_variant", "mfc_gpu_variant_features",
    "mfc_gpu_rk_stage", "mfc_gpu_halo_buffer", "mfc_gpu_halo_pack", "mfc_gpu_set_halo_widths",
    "mfc_gpu_set_viscosity", "mfc_gpu_set_viscous_gradients", "mfc_gpu_set_uniform_coefficients", "mfc_gpu_ensemble_select_variant", "mfc_gpu_ensemble_variant_features",
)
MFC_PREC_GATED = 2
MFC_PREC_FP64_FMA = 3
MFC_RECON_PRIMITIVE, MFC_RECON_CHARACTERISTIC = 0, 1
MFC_VARIANT_TMA = 0x1


class MfcParams(ctypes.Structure):
    _fields_ = [
        ("m", ctypes.c_int32), ("n", ctypes.c_int32), ("p", ctypes.c_int32),
        ("num_fluids", ctypes.c_int32),
        ("weno_order", ctypes.c_int32),
        ("weno_eps", ctypes.c_double),
        ("time_stepper", ctypes.c_int32),
        ("bc_x_beg", ctypes.c_int32), ("bc_x_end", ctypes.c_int32),
        ("bc_y_beg", ctypes.c_int32), ("bc_y_end", ctypes.c_int32),
        ("bc_z_beg", ctypes.c_int32), ("bc_z_end", ctypes.c_int32),
        ("gammas", ctypes.c_double * MFC_MAX_FLUIDS),
        ("pi_infs", ctypes.c_double * MFC_MAX_FLUIDS),
        ("x_cb", ctypes.POINTER(ctypes.c_double)),
        ("y_cb", ctypes.POINTER(ctypes.c_double)),
        ("z_cb", ctypes.POINTER(ctypes.c_double)),
        ("precision", ctypes.c_int32),
        ("device", ctypes.c_int32),
    ]


MFC_MAX_PATCHES = 10


class MfcPatch(ctypes.Structure):
    """mfc_patch: one patch_icpp(i) of the case file (device initial condition)."""
    _fields_ = [
        ("geometry", ctypes.c_int32),
        ("x_centroid", ctypes.c_double), ("y_centroid", ctypes.c_double), ("z_centroid", ctypes.c_double),
        ("length_x", ctypes.c_double), ("length_y", ctypes.c_double), ("length_z", ctypes.c_double),
        ("radius", ctypes.c_double),
        ("smoothen", ctypes.c_int32),
        ("smooth_patch_id", ctypes.c_int32),
        ("smooth_coeff", ctypes.c_double),
        ("alter_patch", ctypes.c_int32 * (MFC_MAX_PATCHES + 1)),
        ("alpha_rho", ctypes.c_double * MFC_MAX_FLUIDS),
        ("alpha", ctypes.c_double * MFC_MAX_FLUIDS),
        ("vel", ctypes.c_double * 3),
        ("pres", ctypes.c_double),
        ("normal", ctypes.c_double * 3),
        ("radii", ctypes.c_double * 3),
        ("epsilon", ctypes.c_double),
    ]


class MfcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[mfc_gpu error {code}] {msg}")
        self.code = code


_lib = None


def lib_path() -> str:
    from . import build
    return build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) the in-tree CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    from . import build
    if build_if_missing and not build.up_to_date():
        build.build()
    if not os.path.exists(build.LIB):
        raise MfcError(MFC_ERR_CUDA, f"{build.LIB} is missing: build it with python -m microfc_gb300.build")
    L = ctypes.CDLL(build.LIB)
    dp = ctypes.POINTER(ctypes.c_double)
    vp = ctypes.c_void_p
    i64 = ctypes.c_int64
    L.mfc_gpu_abi_version.restype = ctypes.c_int
    L.mfc_gpu_last_error.restype = ctypes.c_char_p
    L.mfc_gpu_init.argtypes = [ctypes.POINTER(MfcParams), ctypes.POINTER(vp)]
    L.mfc_gpu_sys_size.argtypes = [vp]
    L.mfc_gpu_upload.argtypes = [vp, ctypes.c_int, dp, i64, i64]
    L.mfc_gpu_download.argtypes = [vp, ctypes.c_int, dp, i64, i64]
    L.mfc_gpu_upload_state.argtypes = [vp, dp]
    L.mfc_gpu_download_state.argtypes = [vp, dp]
    L.mfc_gpu_compute_rhs.argtypes = [vp, dp, dp]
    L.mfc_gpu_weno.argtypes = [vp, ctypes.c_int, dp, dp]
    L.mfc_gpu_set_reconstruction.argtypes = [vp, ctypes.c_int]
    L.mfc_gpu_riemann.argtypes = [vp, ctypes.c_int, dp, dp, dp, dp]
    L.mfc_gpu_tvd_rk.argtypes = [vp, ctypes.c_double, ctypes.c_int]
    L.mfc_gpu_run.argtypes = [vp, ctypes.c_int, ctypes.c_int, dp]
    L.mfc_gpu_status.argtypes = [vp, ctypes.POINTER(ctypes.c_uint32), ctypes.c_int]
    L.mfc_gpu_stream.argtypes = [vp]
    L.mfc_gpu_stream.restype = vp
    L.mfc_gpu_launch_count.argtypes = [vp]
    L.mfc_gpu_launch_count.restype = i64
    L.mfc_gpu_finalize.argtypes = [vp]
    L.mfc_gpu_measure_peaks.argtypes = [ctypes.c_int, dp, dp]
    L.mfc_gpu_selftest_div.argtypes = [vp, vp, vp, vp, ctypes.c_longlong, vp]
    L.mfc_gpu_tvd_rk_noalloc.argtypes = [ctypes.POINTER(MfcParams), vp, vp, i64, ctypes.c_double, vp]
    ip = ctypes.POINTER(ctypes.c_int)
    L.mfc_gpu_tune.argtypes = [vp, ctypes.c_int, ip, dp]
    L.mfc_gpu_ensemble_init.argtypes = [ctypes.POINTER(MfcParams), dp, ctypes.c_int, ctypes.POINTER(vp)]
    L.mfc_gpu_ensemble_upload.argtypes = [vp, ctypes.c_int, dp]
    ip = ctypes.POINTER(ctypes.c_int)
    L.mfc_gpu_select_variant.argtypes = [vp, ctypes.c_int, ip, ip, ip]
    L.mfc_gpu_variant_features.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_uint32)]
    L.mfc_gpu_rk_stage.argtypes = [vp, ctypes.c_int, ctypes.c_double]
    L.mfc_gpu_set_viscosity.argtypes = [vp, dp, dp]
    L.mfc_gpu_set_viscous_gradients.argtypes = [vp, ctypes.c_int]
    L.mfc_gpu_set_uniform_coefficients.argtypes = [vp, ctypes.c_int, ip]
    L.mfc_gpu_ensemble_select_variant.argtypes = [vp, ctypes.c_int, ip, ip, ip]
    L.mfc_gpu_ensemble_variant_features.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_uint32)]
    L.mfc_gpu_halo_buffer.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                                      ctypes.POINTER(ctypes.c_int64)]
    L.mfc_gpu_halo_pack.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp]
    L.mfc_gpu_set_halo_widths.argtypes = [vp, ctypes.c_int, ctypes.c_int, dp, ctypes.c_int]
    L.mfc_gpu_snapshot.argtypes = [vp, ctypes.c_int]
    L.mfc_gpu_snapshot_wait.argtypes = [vp, ctypes.c_int, ctypes.POINTER(dp)]
    L.mfc_gpu_generate_ic.argtypes = [vp, ctypes.POINTER(MfcPatch), ctypes.c_int, dp]
    L.mfc_gpu_ensemble_generate_ic.argtypes = [vp, ctypes.c_int, ctypes.POINTER(MfcPatch), ctypes.c_int, dp]
    L.mfc_gpu_ensemble_download.argtypes = [vp, ctypes.c_int, dp]
    L.mfc_gpu_ensemble_tune.argtypes = [vp, ctypes.c_int, ip, dp]
    L.mfc_gpu_ensemble_run.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.mfc_gpu_ensemble_stream.argtypes = [vp]
    L.mfc_gpu_ensemble_stream.restype = vp
    L.mfc_gpu_ensemble_launch_count.argtypes = [vp]
    L.mfc_gpu_ensemble_launch_count.restype = i64
    L.mfc_gpu_ensemble_finalize.argtypes = [vp]
    fp = ctypes.POINTER(ctypes.c_float)
    L.mfc_gpu_ensemble_set_gate.argtypes = [vp, fp]
    L.mfc_gpu_ensemble_set_viscosity.argtypes = [vp, dp, dp]
    L.mfc_gate_param_count.restype = ctypes.c_int
    L.mfc_gate_workspace_floats.argtypes = [ctypes.c_int]
    L.mfc_gpu_set_gate.argtypes = [vp, fp]
    L.mfc_gpu_gate_samples.argtypes = [vp, ctypes.c_int, vp, vp]
    L.mfc_gate_gradients.argtypes = [vp, vp, ctypes.c_int, vp, ctypes.c_float, vp, vp, vp, vp]
    L.mfc_gate_train_step.argtypes = [vp, vp, ctypes.c_int, vp, vp, vp, vp, vp, ctypes.c_int, ctypes.c_float,
                                      ctypes.c_float, vp, vp]
    L.mfc_gate_infer.argtypes = [vp, ctypes.c_int, vp, vp, vp, vp]
    L.mfc_gpu_set_monitor.argtypes = [vp, ctypes.c_int]
    L.mfc_gpu_icfl.argtypes = [vp, dp, ctypes.c_int]
    L.mfc_gpu_run_cfl.argtypes = [vp, ctypes.c_int, ctypes.c_double, dp, dp]
    _lib = L
    return L


def measure_peaks(device: int = 0):
    """(fp64, fp32) FMA throughput of the device in TFLOP/s."""
    a, b = ctypes.c_double(0), ctypes.c_double(0)
    check(load().mfc_gpu_measure_peaks(int(device), ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


def check(rc: int) -> None:
    if rc != MFC_OK:
        msg = load().mfc_gpu_last_error().decode(errors="replace")
        raise MfcError(rc, msg)
