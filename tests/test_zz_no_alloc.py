"""mfc_gpu_tvd_rk_noalloc: the time step for callers that cannot allocate.

Some hosts cannot let a library call cudaMalloc: their device memory belongs
to another allocator (a framework's caching pool, an OpenACC runtime that
owns the state arrays), or they must avoid the device-wide synchronisation
that cudaMalloc/cudaFree can cause.  This entry point takes their device
arrays for the state before and after the step and keeps its one
intermediate RK register and grid tables in a fixed file-scope device array
(about 58 MiB; at most 7*2^20 doubles of state and 4096 cells per direction).

The GPU test checks it against the regular entry point (mfc_gpu_init +
mfc_gpu_tvd_rk) on two calls in a row, at the tolerance of the other parity
tests (relative L1 <= 1e-10 per field; both the FP64 and the split path give
the same bits for any row pitch and tile variant, so the results are
expected to be identical), in FP64 and split precision.  This file is collected last so a run
that stops at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_l1
from microfc_gb300 import Simulation, _lib, cases, preprocess

TOL = 1e-10


def _params(case, x_cb, y_cb, precision=None):
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
    P.precision = _lib.MFC_PREC_FP64 if precision is None else precision
    P.device = 0
    return P


FP64, SPLIT, FP64_FMA = _lib.MFC_PREC_FP64, _lib.MFC_PREC_SPLIT, _lib.MFC_PREC_FP64_FMA
PREC_NAMES = {FP64: "fp64", SPLIT: "split", FP64_FMA: "fp64_fma"}


@pytest.mark.gpu
@pytest.mark.parametrize("builder,precision,pad", [
    (lambda: cases.shock_droplet_2d(nx=96, ny=64, steps=2), FP64, 3),
    (lambda: cases.sod_1d(m=299, steps=2, dt=1e-4), FP64, 3),
    (lambda: cases.shock_droplet_2d(nx=64, ny=40, steps=2).replace(time_stepper=2, bc_x=(-2, -4)), FP64, 3),
    # split precision: an odd row pitch (no tensor map; plain tile loads) and
    # an even one (interior tiles staged by the TMA copy over the caller's array)
    (lambda: cases.shock_droplet_2d(nx=96, ny=64, steps=2), SPLIT, 3),
    (lambda: cases.shock_droplet_2d(nx=96, ny=64, steps=2), SPLIT, 4),
    (lambda: cases.sod_1d(m=299, steps=2, dt=1e-4), SPLIT, 3),
    # the opt-in contracted FP64 kernels (2-D WENO5)
    (lambda: cases.shock_droplet_2d(nx=96, ny=64, steps=2), FP64_FMA, 3),
], ids=["droplet-fp64", "sod-fp64", "droplet-rk2-fp64", "droplet-split-odd", "droplet-split-even", "sod-split",
        "droplet-fp64-fma"])
def test_noalloc_step_matches_regular_entry_point_twice_in_a_row(builder, precision, pad):
    import torch

    case = builder()
    x_cb, y_cb, _, q0 = preprocess.generate(case)
    L = _lib.load()
    P = _params(case, x_cb, y_cb, precision)
    ld_y = case.m + 1 + pad  # a row pitch other than the regular path's
    shape = (case.sys_size, case.p + 1, case.n + 1, ld_y)
    host = np.zeros(shape)
    host[..., : case.m + 1] = q0
    dev = torch.device("cuda", 0)
    a = torch.from_numpy(host).to(dev)
    b = torch.zeros(shape, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize(dev)

    # two calls in a row: a -> b, then b -> a
    rc = L.mfc_gpu_tvd_rk_noalloc(ctypes.byref(P), ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()),
                                  ld_y, case.dt, ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, L.mfc_gpu_last_error().decode()
    one = b.cpu().numpy()[..., : case.m + 1].copy()
    rc = L.mfc_gpu_tvd_rk_noalloc(ctypes.byref(P), ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(a.data_ptr()),
                                  ld_y, case.dt, ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, L.mfc_gpu_last_error().decode()
    two = a.cpu().numpy()[..., : case.m + 1].copy()

    regular = case.replace(precision=PREC_NAMES[precision])
    with Simulation(regular, x_cb, y_cb, q_cons=q0) as sim:
        sim.tvd_rk(0)
        ref1 = sim.download()
        sim.tvd_rk(1)
        ref2 = sim.download()

    for got, ref in ((one, ref1), (two, ref2)):
        assert np.all(np.isfinite(got))
        assert rel_l1(got, ref).max() <= TOL
    assert np.array_equal(one, ref1) and np.array_equal(two, ref2)


def test_noalloc_rejects_cases_beyond_its_scratch():
    """Oversized requests fail with a clear error before touching a device."""
    L = _lib.load()
    case = cases.shock_droplet_2d(nx=64, ny=32, steps=2, dt=1e-9)
    x_cb, y_cb, _, _ = preprocess.generate(case)
    P = _params(case, x_cb, y_cb)
    fake_in, fake_out = ctypes.c_void_p(0x1000), ctypes.c_void_p(0x2000)
    # 7 equations x 32 rows x ld_y doubles > 7*2^20
    rc = L.mfc_gpu_tvd_rk_noalloc(ctypes.byref(P), fake_in, fake_out, 40000, 1e-9, None)
    assert rc == _lib.MFC_ERR_INVALID
    assert "fixed scratch" in L.mfc_gpu_last_error().decode()
    big = cases.sod_1d(m=4999, steps=2, dt=1e-4)
    xb, _, _, _ = preprocess.generate(big)
    Pb = _params(big, xb, None)
    rc = L.mfc_gpu_tvd_rk_noalloc(ctypes.byref(Pb), fake_in, fake_out, 5000, 1e-4, None)
    assert rc == _lib.MFC_ERR_INVALID
    assert "4096 cells" in L.mfc_gpu_last_error().decode()
    rc = L.mfc_gpu_tvd_rk_noalloc(ctypes.byref(P), fake_in, fake_in, 64, 1e-9, None)
    assert rc == _lib.MFC_ERR_INVALID


def test_noalloc_refuses_the_gated_precision_before_any_device_call():
    """The gate's parameters live in a context, so the no-allocation step has
    none to give the gated kernel: it must refuse the precision up front
    (the fake device pointers below are never dereferenced)."""
    L = _lib.load()
    case = cases.shock_droplet_2d(nx=64, ny=32, steps=2, dt=1e-9)
    x_cb, y_cb, _, _ = preprocess.generate(case)
    P = _params(case, x_cb, y_cb, _lib.MFC_PREC_GATED)
    rc = L.mfc_gpu_tvd_rk_noalloc(ctypes.byref(P), ctypes.c_void_p(0x1000), ctypes.c_void_p(0x2000), 64, 1e-9, None)
    assert rc == _lib.MFC_ERR_INVALID
    assert "gate" in L.mfc_gpu_last_error().decode()
