"""The learned WENO gate: sample collection, GPU training, persistence.

The network (10 -> 32 -> 32 -> 1, ReLU, sigmoid) reads one cell's 5-point
stencils of alpha_1 and p along one direction, each shifted by its minimum
and divided by its range, and predicts whether the cell needs the nonlinear
WENO5 weights.  Label: max_k |omega_k - d_k| > 1e-3 over alpha_1 and p and
both faces, the weights evaluated in FP64 on those same normalised stencils
with epsilon = 1e-2, so variations under ~1e-3 of a variable's magnitude
count as flat (with the case's epsilon on the raw fields, round-off in the
pressure recovery alone would flag nearly every cell); the inputs come
from the split path's FP32 primitives, as the gated kernel sees them.  Smooth
cells then use the
optimal linear weights d_k; plain WENO everywhere stays the fallback
(precision "split") and the measure of the gated form's error (FP64,
precision "fp64").

Training data are states the solver itself generates: seeded runs of the
2-D shock-droplet case (Mach uniform in [1.2, 2.5], droplet radius uniform
in [1, 3] mm), sampled at several times along both directions.  Training
runs on the GPU through the library's own forward/backward/Adam kernels
(mfc_gate_train_step); torch is used only to hold device buffers.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib, cases, preprocess
from .solver import Simulation

N_IN, N_H = 10, 32
N_PARAMS = N_IN * N_H + N_H + N_H * N_H + N_H + N_H + 1  # 1441
LABEL_TOL = 1e-3
WEIGHTS_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "gate_params.npz")


def init_params(seed: int = 0) -> np.ndarray:
    """He-initialised FP32 parameter vector."""
    rng = np.random.default_rng(seed)
    w = np.zeros(N_PARAMS, dtype=np.float32)
    o = 0
    for fan_in, fan_out in ((N_IN, N_H), (N_H, N_H), (N_H, 1)):
        w[o:o + fan_in * fan_out] = rng.normal(0.0, np.sqrt(2.0 / fan_in), fan_in * fan_out)
        o += fan_in * fan_out + fan_out  # weights then biases (zero)
    return w


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def collect_samples(case_list, snapshots=(0.25, 0.5, 0.75, 1.0), per_snapshot=4096, seed=0, device=0,
                    positive_fraction=0.5):
    """(X, labels) sampled from solver states of the given cases.

    Each case runs in split precision; at every snapshot fraction of its
    t_step_stop both directions are sampled: all flagged cells up to
    positive_fraction * per_snapshot, the rest drawn from the smooth cells.
    """
    import torch
    dev = torch.device("cuda", device)
    rng = np.random.default_rng(seed)
    xs, ys = [], []
    for case in case_list:
        c = case.replace(precision="split")
        x_cb, y_cb, _, q = preprocess.generate(c)
        stops = sorted({max(1, int(round(f * c.t_step_stop))) for f in snapshots})
        with Simulation(c, x_cb, y_cb, q_cons=q, device=device) as sim:
            t = 0
            X = torch.empty((c.cells, N_IN), dtype=torch.float32, device=dev)
            D = torch.empty((c.cells,), dtype=torch.float32, device=dev)
            for s in stops:
                sim.run(t, s)
                t = s
                for d in (0, 1):
                    sim.gate_samples(d, X.data_ptr(), D.data_ptr())
                    lab = (D > LABEL_TOL).cpu().numpy()
                    xn = X.cpu().numpy()
                    pos = np.flatnonzero(lab)
                    neg = np.flatnonzero(~lab)
                    npos = min(len(pos), int(positive_fraction * per_snapshot))
                    nneg = min(len(neg), per_snapshot - npos)
                    pick = np.concatenate([rng.choice(pos, npos, replace=False) if npos else pos[:0],
                                           rng.choice(neg, nneg, replace=False) if nneg else neg[:0]])
                    xs.append(xn[pick])
                    ys.append(lab[pick].astype(np.float32))
    return np.concatenate(xs), np.concatenate(ys)


def train(X: np.ndarray, y: np.ndarray, epochs: int = 20, batch: int = 4096, lr: float = 3e-3,
          pos_weight: float = 1.0, seed: int = 0, device: int = 0, params: np.ndarray | None = None):
    """Adam on the GPU with the library's kernels; returns (params, losses)."""
    import torch
    L = _lib.load()
    dev = torch.device("cuda", device)
    n = len(X)
    Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).to(dev)
    yd = torch.from_numpy(np.ascontiguousarray(y, dtype=np.float32)).to(dev)
    w = torch.from_numpy(init_params(seed) if params is None else np.asarray(params, np.float32).copy()).to(dev)
    g = torch.zeros_like(w)
    m = torch.zeros_like(w)
    v = torch.zeros_like(w)
    work = torch.empty(L.mfc_gate_workspace_floats(batch), dtype=torch.float32, device=dev)
    loss = torch.zeros(1, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    gen = torch.Generator(device="cpu").manual_seed(seed)
    step, losses = 0, []
    for _ in range(epochs):
        perm = torch.randperm(n, generator=gen).to(dev)
        tot = 0.0
        for b0 in range(0, n - batch + 1, batch):
            idx = perm[b0:b0 + batch]
            xb = Xd[idx].contiguous()
            yb = yd[idx].contiguous()
            step += 1
            _lib.check(L.mfc_gate_train_step(_vp(xb), _vp(yb), batch, _vp(w), _vp(g), _vp(m), _vp(v), _vp(work),
                                             step, float(lr), float(pos_weight), _vp(loss),
                                             ctypes.c_void_p(stream.cuda_stream)))
            tot += float(loss.item()) / batch
        losses.append(tot / max(1, n // batch))
    return w.cpu().numpy(), losses


def gradients(X: np.ndarray, y: np.ndarray, params: np.ndarray, pos_weight: float = 1.0, device: int = 0):
    """(grad, summed loss) of one batch from the library's backward kernels."""
    import torch
    L = _lib.load()
    dev = torch.device("cuda", device)
    B = len(X)
    Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).to(dev)
    yd = torch.from_numpy(np.ascontiguousarray(y, dtype=np.float32)).to(dev)
    w = torch.from_numpy(np.asarray(params, dtype=np.float32).copy()).to(dev)
    g = torch.zeros_like(w)
    work = torch.empty(L.mfc_gate_workspace_floats(B), dtype=torch.float32, device=dev)
    loss = torch.zeros(1, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    _lib.check(L.mfc_gate_gradients(_vp(Xd), _vp(yd), B, _vp(w), float(pos_weight), _vp(g), _vp(work), _vp(loss),
                                    ctypes.c_void_p(stream.cuda_stream)))
    return g.cpu().numpy(), float(loss.item())


def infer(X: np.ndarray, params: np.ndarray, device: int = 0) -> np.ndarray:
    """Logits from the tensor-core inference kernel (FP16 weights)."""
    import torch
    L = _lib.load()
    dev = torch.device("cuda", device)
    Xd = torch.from_numpy(np.ascontiguousarray(X, dtype=np.float32)).to(dev)
    w = torch.from_numpy(np.asarray(params, dtype=np.float32).copy()).to(dev)
    wh = torch.empty(N_PARAMS, dtype=torch.float16, device=dev)
    out = torch.empty(len(X), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    _lib.check(L.mfc_gate_infer(_vp(Xd), len(X), _vp(w), _vp(wh), _vp(out), ctypes.c_void_p(stream.cuda_stream)))
    return out.cpu().numpy()


def training_cases(count: int = 16, seed: int = 0, nx: int = 1024, ny: int = 512, steps: int = 1000):
    """The seeded shock-droplet runs the training data come from."""
    rng = np.random.default_rng(seed)
    return [cases.shock_droplet_2d(nx=nx, ny=ny, mach=float(rng.uniform(1.2, 2.5)),
                                   radius=float(rng.uniform(1e-3, 3e-3)), steps=steps) for _ in range(count)]


def all_linear_params() -> np.ndarray:
    """Parameters whose logit is always negative: every cell takes the
    linear weights (the method without the learned gate's judgement)."""
    w = np.zeros(N_PARAMS, dtype=np.float32)
    w[-1] = -1.0
    return w


def save(params: np.ndarray, path: str = WEIGHTS_FILE, **meta) -> None:
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez(path, params=np.asarray(params, dtype=np.float32), **meta)


def load(path: str = WEIGHTS_FILE) -> np.ndarray:
    return np.load(path)["params"].astype(np.float32)


def main():
    """Train the committed gate: 16 seeded 1024x512 runs, 2e6 samples."""
    import argparse
    import json
    ap = argparse.ArgumentParser()
    ap.add_argument("--cases", type=int, default=16)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--per-snapshot", type=int, default=15625)  # 16 cases x 4 snapshots x 2 dirs -> 2e6
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--out", default=WEIGHTS_FILE)
    a = ap.parse_args()
    cl = training_cases(a.cases, steps=a.steps)
    X, y = collect_samples(cl, per_snapshot=a.per_snapshot)
    perm = np.random.default_rng(1).permutation(len(X))
    X, y = X[perm], y[perm]
    ntest = len(X) // 10
    params, losses = train(X[ntest:], y[ntest:], epochs=a.epochs)
    logits = infer(X[:ntest], params)
    pred = logits > 0
    lab = y[:ntest] > 0.5
    stats = {"samples": int(len(X)), "positive_fraction": float(y.mean()), "final_loss": losses[-1],
             "test_accuracy": float((pred == lab).mean()),
             "test_recall_nonsmooth": float(pred[lab].mean()) if lab.any() else None,
             "test_flagged_fraction": float(pred.mean())}
    save(params, a.out, losses=np.array(losses), stats=json.dumps(stats))
    print(json.dumps(stats))


if __name__ == "__main__":
    main()
