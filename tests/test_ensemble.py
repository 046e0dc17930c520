"""Ensemble mode: every case advanced in the ensemble gets the bits it gets
from its own Simulation (FP64 and split precision), with and without graph
replay and after autotuning."""
import ctypes

import numpy as np
import pytest

from microfc_gb300 import Simulation, _lib, cases
from microfc_gb300.ensemble import Ensemble, random_droplet_cases
from microfc_gb300.solver import make_params


def _mixed(precision):
    return [
        cases.shock_droplet_2d(nx=64, ny=32, steps=6, precision=precision),
        cases.shock_droplet_2d(nx=96, ny=48, mach=2.2, radius=1.5e-3, steps=6, precision=precision),
        cases.shock_droplet_2d(nx=48, ny=40, mach=1.3, radius=2.5e-3, steps=6, precision=precision).replace(
            bc_x=(-2, -4), bc_y=(-1, -1)),
    ]


def _single(case, steps):
    with Simulation(case) as sim:
        sim.run(0, steps)
        return sim.download()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "split"])
@pytest.mark.parametrize("use_graph", [True, False])
def test_ensemble_matches_single_case_runs(precision, use_graph):
    cl = _mixed(precision)
    with Ensemble(cl) as ens:
        ens.run(0, 6, use_graph=use_graph)
        assert ens.launches == 3 * 6
        got = [ens.download(i) for i in range(len(cl))]
    for c, g in zip(cl, got):
        ref = _single(c, 6)
        assert np.isfinite(g).all()
        assert np.array_equal(g, ref), c.name


@pytest.mark.gpu
def test_ensemble_autotuner_keeps_results():
    cl = _mixed("split")
    with Ensemble(cl) as ens:
        v, ms = ens.tune(reps=3)
        assert v >= 0 and ms > 0
        ens.run(0, 6)
        got = [ens.download(i) for i in range(len(cl))]
    for c, g in zip(cl, got):
        assert np.array_equal(g, _single(c, 6))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["split", "gated"])
def test_every_ensemble_variant_gives_the_same_bits(precision):
    from microfc_gb300 import gate
    from microfc_gb300._lib import MfcError
    cl = _mixed(precision)
    params = gate.load() if precision == "gated" else None
    refs = []
    for c in cl:
        with Simulation(c) as sim:
            if params is not None:
                sim.set_gate(params)
            sim.run(0, 6)
            refs.append(sim.download())
    from microfc_gb300._lib import MFC_VARIANT_TMA
    v, tma = 0, 0
    while True:
        with Ensemble(cl) as ens:
            if params is not None:
                ens.set_gate(params)
            try:
                shape = ens.select_variant(v)
            except MfcError:
                break
            tma += bool(ens.variant_features(v) & MFC_VARIANT_TMA)
            ens.run(0, 6)
            for i, ref in enumerate(refs):
                assert np.array_equal(ens.download(i).view(np.uint64), ref.view(np.uint64)), (v, shape, i)
        v += 1
    assert v >= 2 and tma >= 1  # the TMA-staged variants are among them


@pytest.mark.gpu
def test_single_case_autotuner_keeps_results():
    c = cases.shock_droplet_2d(nx=128, ny=64, steps=4)
    with Simulation(c) as sim:
        v, ms = sim.tune(reps=3)
        assert v >= 0 and ms > 0
        sim.run(0, 4)
        got = sim.download()
    assert np.array_equal(got, _single(c, 4))


def test_random_ensemble_is_seeded():
    a = random_droplet_cases(count=6, seed=3, steps=10)
    b = random_droplet_cases(count=6, seed=3, steps=10)
    assert [(c.m, c.n, c.dt) for c in a] == [(c.m, c.n, c.dt) for c in b]
    assert all(c.m + 1 in (128, 256, 384, 512) and (c.n + 1) * 2 == c.m + 1 for c in a)


def test_ensemble_rejects_mixed_configurations_before_touching_a_device():
    L = _lib.load()
    c1 = cases.shock_droplet_2d(nx=64, ny=32, steps=2)
    c2 = c1.replace(weno_order=3)
    keep = []
    arr = (_lib.MfcParams * 2)()
    for i, c in enumerate((c1, c2)):
        from microfc_gb300 import preprocess
        x, y, _, _ = preprocess.generate(c)
        P, cb = make_params(c, x, y)
        keep.append(cb)
        arr[i] = P
    dts = np.array([c1.dt, c2.dt])
    h = ctypes.c_void_p()
    rc = L.mfc_gpu_ensemble_init(arr, dts.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 2, ctypes.byref(h))
    assert rc == _lib.MFC_ERR_INVALID and not h.value
    assert "must share" in L.mfc_gpu_last_error().decode()


def _viscous_mixed(precision):
    re = dict(re_shear=(1.0 / 1e-1, 1.0 / 2e-3), re_bulk=(0.0, 1.0 / 5e-3))
    return [c.replace(**re) for c in _mixed(precision)]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "split", "gated"])
def test_viscous_ensemble_matches_single_case_runs(precision):
    """Viscous cases (mfc_gpu_ensemble_set_viscosity) get the bits of their
    own viscous Simulation, with graph replay and after autotuning."""
    from microfc_gb300 import gate
    params = gate.load() if precision == "gated" else None

    def single(c):
        with Simulation(c) as sim:
            if params is not None:
                sim.set_gate(params)
            sim.run(0, 6)
            return sim.download()

    cl = _viscous_mixed(precision)
    with Ensemble(cl) as ens:
        if params is not None:
            ens.set_gate(params)
        ens.tune(reps=2)
        ens.run(0, 6, use_graph=True)
        got = [ens.download(i) for i in range(len(cl))]
    for c, g in zip(cl, got):
        ref = single(c)
        assert np.isfinite(g).all()
        assert np.array_equal(g, ref), c.name
    # and the viscous terms acted: the inviscid run differs
    inv = single(_mixed(precision)[0])
    assert not np.array_equal(got[0], inv)


@pytest.mark.gpu
def test_ensemble_refuses_a_mix_of_viscous_and_inviscid_cases():
    cl = _mixed("fp64")
    cl[1] = cl[1].replace(re_shear=(10.0, 10.0))
    with pytest.raises(_lib.MfcError):
        Ensemble(cl)
