"""The learned WENO gate: oracle gradients pinned by finite differences, GPU
training kernels against the oracle, tensor-core inference, sample
extraction, and what the trained network gains over the method without it."""
import numpy as np
import pytest

from conftest import rel_l1
from oracle import gate_mlp


def _rand(seed, B=64):
    rng = np.random.default_rng(seed)
    X = rng.uniform(0, 1, (B, 10))
    t = (rng.uniform(size=B) < 0.3).astype(np.float64)
    p = rng.normal(0, 0.4, gate_mlp.N_PARAMS)
    return X, t, p


def test_oracle_gradient_matches_finite_differences():
    X, t, p = _rand(0)
    g = gate_mlp.gradient(X, t, p, pos_weight=2.0)
    h = 1e-6
    idx = np.random.default_rng(1).choice(gate_mlp.N_PARAMS, 60, replace=False)
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        fd = (gate_mlp.loss(X, t, p + e, 2.0) - gate_mlp.loss(X, t, p - e, 2.0)) / (2 * h) / len(X)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_label_separates_smooth_from_discontinuous_stencils():
    x = np.linspace(-1, 1, 5)
    smooth = np.stack([np.sin(0.05 * x + s) for s in np.linspace(0, 3, 20)])
    step = np.stack([np.where(x > c, 1.0, 0.0) + 0.01 * x for c in (-0.6, -0.1, 0.1, 0.6)])
    tiny = 1.0 + 1e-9 * np.random.default_rng(0).normal(size=(20, 5))  # round-off on a flat field
    assert gate_mlp.weight_deviation(gate_mlp.norm5(smooth, 1e-30)).max() < 1e-3
    assert gate_mlp.weight_deviation(gate_mlp.norm5(step, 1e-30)).min() > 1e-3
    assert gate_mlp.weight_deviation(gate_mlp.norm5(tiny, 1e-30)).max() < 1e-3


@pytest.mark.gpu
def test_gpu_backward_kernels_match_oracle():
    from microfc_gb300 import gate
    X, t, p = _rand(2, B=1000)
    g, loss = gate.gradients(X.astype(np.float32), t.astype(np.float32), p.astype(np.float32), pos_weight=2.0)
    p32 = p.astype(np.float32).astype(np.float64)
    X32 = X.astype(np.float32).astype(np.float64)
    gref = gate_mlp.gradient(X32, t, p32, pos_weight=2.0)
    lref = gate_mlp.loss(X32, t, p32, 2.0)
    assert abs(loss - lref) <= 1e-4 * abs(lref)
    scale = np.abs(gref).max()
    assert np.abs(g - gref).max() <= 1e-4 * scale, np.abs(g - gref).max() / scale


@pytest.mark.gpu
def test_tensor_core_inference_matches_fp16_oracle():
    from microfc_gb300 import gate
    X, _, p = _rand(3, B=1000)
    z = gate.infer(X.astype(np.float32), p.astype(np.float32))
    zref = gate_mlp.forward_fp16(X, p)
    scale = np.abs(zref).max()
    assert np.abs(z - zref).max() <= 2e-3 * scale
    decided = np.abs(zref) > 1e-2 * scale
    assert np.array_equal(z[decided] > 0, zref[decided] > 0)


@pytest.mark.gpu
def test_gate_samples_match_oracle_features():
    import torch
    from microfc_gb300 import Simulation, cases, preprocess
    c = cases.shock_droplet_2d(nx=128, ny=64, steps=30, precision="split")
    x_cb, y_cb, _, q = preprocess.generate(c)
    with Simulation(c, x_cb, y_cb, q_cons=q) as sim:
        sim.run(0, 30)
        state = sim.download()
        X = torch.empty((c.cells, 10), dtype=torch.float32, device="cuda")
        D = torch.empty((c.cells,), dtype=torch.float32, device="cuda")
        sim.gate_samples(0, X.data_ptr(), D.data_ptr())
        Xg, Dg = X.cpu().numpy(), D.cpu().numpy()
    prim = preprocess.to_primitive(c, state)
    a = prim[c.adv_idx, 0]
    pr = prim[c.E_idx, 0]
    # x stencils with extrapolation boundaries
    idx = np.clip(np.arange(c.m + 1)[:, None] + np.arange(-2, 3)[None, :], 0, c.m)
    feat = gate_mlp.features(a[:, idx], pr[:, idx]).reshape(-1, 10)
    assert np.abs(Xg - feat).max() <= 2e-3
    # labels: the FP64 weight deviation of the kernel's own normalised stencils
    X64 = Xg.astype(np.float64)
    dref = np.maximum(gate_mlp.weight_deviation(X64[:, :5]), gate_mlp.weight_deviation(X64[:, 5:]))
    assert np.abs(Dg - dref).max() <= 1e-6
    assert Dg.min() >= 0 and 0.01 < (Dg > 1e-3).mean() < 0.5


@pytest.mark.gpu
def test_training_learns_and_the_gate_gains_over_the_method_without_it():
    """Train on solver-generated states, then compare, against FP64 WENO:
    the gated solver, plain split WENO everywhere, and linear weights
    everywhere (the method without the network's judgement)."""
    from microfc_gb300 import Simulation, cases, gate, preprocess
    train_cases = gate.training_cases(count=3, seed=5, nx=256, ny=128, steps=300)
    X, y = gate.collect_samples(train_cases, per_snapshot=3000)
    params, losses = gate.train(X, y, epochs=15, batch=2048)
    assert losses[-1] < 0.5 * losses[0], losses
    acc = ((gate.infer(X, params) > 0) == (y > 0.5)).mean()
    assert acc > 0.9, acc

    test = cases.shock_droplet_2d(nx=256, ny=128, mach=2.0, radius=2e-3, steps=300)
    x_cb, y_cb, _, q = preprocess.generate(test)

    def run(precision, p=None):
        with Simulation(test.replace(precision=precision), x_cb, y_cb, q_cons=q) as sim:
            if p is not None:
                sim.set_gate(p)
            sim.run(0, 300)
            return sim.download()

    ref = run("fp64")
    split = run("split")
    gated = run("gated", params)
    linear = run("gated", gate.all_linear_params())
    cols = [0, 1, test.adv_idx, test.adv_idx + 1]
    e_split = rel_l1(split, ref)[cols].max()
    e_gated = rel_l1(gated, ref)[cols].max()
    e_lin = rel_l1(linear, ref)[cols].max() if np.isfinite(linear).all() else np.inf
    print(f"rel L1 vs FP64: split {e_split:.3e} gated {e_gated:.3e} all-linear {e_lin:.3e}")
    assert e_gated <= 1e-3
    assert e_lin > 3 * e_gated


@pytest.mark.gpu
@pytest.mark.slow
def test_config4_gated_against_plain_fp64_and_ungated_split():
    """Config 4 at its stated size: the droplet at 2048 x 1024 for 2000 steps.
    The gated form must stay within density / volume-fraction L1 <= 1e-3 of
    plain FP64 WENO everywhere (the fallback and the judge; the FP64 GPU path
    is the oracle bit for bit) and run at >= 2x its cell-updates/s.  Beside
    it, the method without the network: plain split WENO everywhere (its
    accuracy and speed are printed with the gated form's), and linear
    weights everywhere over a shorter run (the network's accuracy gain)."""
    import torch
    from microfc_gb300 import Simulation, cases, gate

    params = gate.load()
    case = cases.shock_droplet_2d(nx=2048, ny=1024, steps=2000)

    def run(precision, p=None, steps=2000):
        with Simulation(case.replace(precision=precision), ic="device") as sim:
            if p is not None:
                sim.set_gate(p)
            sim.tune(3)
            st = torch.cuda.ExternalStream(sim.stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(st)
            sim.run(0, steps)
            e1.record(st)
            torch.cuda.synchronize()
            rate = case.cells * steps / (e0.elapsed_time(e1) / 1e3)
            assert sim.status() == 0
            return sim.download(), rate

    ref, r_fp64 = run("fp64")
    split, r_split = run("split")
    gated, r_gated = run("gated", params)
    cols = [0, 1, case.adv_idx, case.adv_idx + 1]
    e_split = rel_l1(split, ref)[cols].max()
    e_gated = rel_l1(gated, ref)[cols].max()
    print(f"2048x1024 x 2000 steps: cell-updates/s fp64 {r_fp64:.3e} split {r_split:.3e} gated {r_gated:.3e} "
          f"(gated/fp64 {r_gated / r_fp64:.1f}x, gated/split {r_gated / r_split:.2f}); "
          f"max density/alpha rel L1 split {e_split:.2e} gated {e_gated:.2e}")
    assert e_gated <= 1e-3
    assert r_gated >= 2.0 * r_fp64
    # the network's gain over linear weights everywhere, on the first 200 steps
    short_ref, _ = run("fp64", steps=200)
    short_gated, _ = run("gated", params, steps=200)
    short_lin, _ = run("gated", gate.all_linear_params(), steps=200)
    e_g = rel_l1(short_gated, short_ref)[cols].max()
    e_l = rel_l1(short_lin, short_ref)[cols].max() if np.isfinite(short_lin).all() else np.inf
    print(f"200 steps: max density/alpha rel L1 gated {e_g:.2e} all-linear {e_l:.2e}")
    assert e_l > 3 * e_g
