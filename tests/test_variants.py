"""Every compiled tile variant the autotuner can pick gives the same bits: the
per-cell arithmetic does not depend on the tile shape, so a tuned run must
equal the default one (and, for FP64, the CPU oracle) exactly.  Ragged grids
exercise partial edge tiles.  (Every unit is compiled without FMA
contraction and the FP32 path writes its FMAs explicitly, so no register
cap can make two variants fuse differently.)"""
import numpy as np
import pytest

from microfc_gb300 import cases, gate, preprocess

pytestmark = pytest.mark.gpu


def _variant_runs(case, steps, params=None):
    from microfc_gb300 import Simulation
    from microfc_gb300._lib import MfcError
    x, y, z, q = preprocess.generate(case)
    outs, shapes = [], []
    v = 0
    while True:
        with Simulation(case, x, y, z, q_cons=q) as sim:
            if params is not None:
                sim.set_gate(params)
            try:
                shapes.append(sim.select_variant(v))
            except MfcError:
                break
            sim.run(0, steps)
            outs.append(sim.download())
        v += 1
    return outs, shapes


@pytest.mark.parametrize("kind", ["1d_fp64", "1d_split", "2d_fp64", "2d_split", "2d_gated", "3d_fp64", "3d_split"])
def test_all_tile_variants_agree_bitwise(kind):
    nd, prec = kind.split("_")
    params = None
    if nd == "1d":
        c = cases.sod_1d(m=299, steps=6, dt=1e-4).replace(precision=prec)
    elif nd == "2d":
        c = cases.shock_droplet_2d(nx=100, ny=60, steps=6, precision=prec)
        if prec == "gated":
            params = gate.load()
    else:
        c = cases.shock_bubble_3d(N=28, steps=6, precision=prec).replace(m=28, n=26, p=27)
    outs, shapes = _variant_runs(c, 6, params)
    assert len(outs) >= 1
    for o, s in zip(outs[1:], shapes[1:]):
        assert np.array_equal(o.view(np.uint64), outs[0].view(np.uint64)), s


@pytest.mark.parametrize("kind", ["1d_split", "2d_split", "2d_gated", "3d_split"])
def test_uniform_coefficient_record_matches_per_cell_records(kind):
    """On a uniform grid the split kernels read one shared coefficient record
    per direction from their parameters; the per-cell records give the same
    bits."""
    from microfc_gb300 import Simulation
    nd, prec = kind.split("_")
    params = None
    if nd == "1d":
        c = cases.sod_1d(m=299, steps=6, dt=1e-4).replace(precision=prec)
    elif nd == "2d":
        c = cases.shock_droplet_2d(nx=100, ny=60, steps=6, precision=prec)
        params = gate.load() if prec == "gated" else None
    else:
        c = cases.shock_bubble_3d(N=28, steps=6, precision=prec).replace(m=28, n=26, p=27)
    full = {"1d": 1, "2d": 3, "3d": 7}[nd]
    x, y, z, q = preprocess.generate(c)
    outs = []
    for enable in (True, False):
        with Simulation(c, x, y, z, q_cons=q) as sim:
            if params is not None:
                sim.set_gate(params)
            assert sim.set_uniform_coefficients(enable) == (full if enable else 0)
            sim.run(0, 6)
            outs.append(sim.download())
    assert np.array_equal(outs[0].view(np.uint64), outs[1].view(np.uint64))


@pytest.mark.parametrize("prec", ["fp64", "split", "gated", "3d_fp64", "3d_split"])
@pytest.mark.parametrize("uniform", [True, False], ids=["uniform", "records"])
def test_tma_staged_variants_match_plain_loads(prec, uniform):
    """Variants that stage interior tiles with one TMA bulk tensor copy give
    the bits of the first plain-load variant and no bounded wait gives up,
    with the shared coefficient record of a uniform grid and with per-cell
    records (staged beside the copy's landing area)."""
    from microfc_gb300 import Simulation
    from microfc_gb300._lib import MFC_FLAG_TIMEOUT, MFC_VARIANT_TMA, MfcError
    if prec.endswith("fp64") and not uniform:
        pytest.skip("the FP64 kernels have no shared record to switch off: they always stage their own "
                    "coefficients (stretched grids: test_gpu_parity.py::test_stretched_grid_matches_oracle)")
    if prec.startswith("3d"):
        # interior tiles in every sweep: x tiles of 32 cells, y and z of 16
        c = cases.shock_bubble_3d(N=40, steps=4, precision=prec[3:])
        c = c.replace(m=71, dt=c.dt / 2)
    else:
        c = cases.shock_droplet_2d(nx=160, ny=96, steps=4, precision=prec)
    params = gate.load() if prec == "gated" else None
    x, y, z, q = preprocess.generate(c)
    ref, staged_out = None, []
    v = 0
    while True:
        with Simulation(c, x, y, z, q_cons=q) as sim:
            if params is not None:
                sim.set_gate(params)
            if not uniform:
                sim.set_uniform_coefficients(False)
            try:
                shape = sim.select_variant(v)
            except MfcError:
                break
            staged = bool(sim.variant_features(v) & MFC_VARIANT_TMA)
            if staged or ref is None:
                sim.run(0, 4)
                out = sim.download()
                assert not sim.status() & MFC_FLAG_TIMEOUT
                if staged:
                    staged_out.append((shape, out))
                else:
                    ref = out
        v += 1
    assert ref is not None and staged_out
    for shape, out in staged_out:
        assert np.array_equal(out.view(np.uint64), ref.view(np.uint64)), shape
