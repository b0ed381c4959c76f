"""Learned Johnson-Cook return map: training pairs from the plain GPU path,
normalisation, training on the GPU, and its installation in a simulation.

Data.  Taylor-bar runs (3-D TLMPM, MUSL, cubic B-spline) of the copper bar
with A, B, n and C drawn uniformly within +-spread of their nominal values,
executed together as one independent batch.  While they run, the stress
kernel logs a hashed fraction of the plastic particle-steps: the network's 15
inputs and the closed-form return map's 7 outputs.  The network has no
material inputs, so every logged input row is labelled again with the return
map of the material the network will stand in for (``kmpm_jc_label``); rows
that are elastic under that material are dropped.  The perturbed runs thus
widen the envelope of visited states (strain paths, rates, stress levels)
while the labels stay a single-valued function of the inputs.

Training.  ``Mlp.train``: FP32 forward / backward / Adam kernels of the
library, mean squared error in normalised output units, batches drawn with
replacement, cosine learning-rate decay.  Inference in the simulation is
BF16 on the tensor cores with FP32 accumulation (``kmpm_set_surrogate``).
"""
from __future__ import annotations

import json

import numpy as np

from . import workloads as W
from .batch import Batch
from .gpu import MLP_NIN, MLP_NNORM, MLP_NOUT, Mlp

PERTURBED = ("A", "B", "n", "C")


def taylor_training_runs(cellsize=0.4, instances=8, spread=0.2, seed=0):
    """The nominal bar and instances - 1 bars with A, B, n, C perturbed."""
    rng = np.random.default_rng(seed)
    sims, params = [], []
    for i in range(instances):
        p = {} if i == 0 else {k: W.COPPER[k] * float(rng.uniform(1 - spread, 1 + spread)) for k in PERTURBED}
        sim = W.taylor_bar(None, cellsize=cellsize, params=p)
        W.taylor_bar_wall(sim)
        sims.append(sim)
        params.append(p)
    return sims, params


def collect_pairs(sims, steps, capacity, fraction, seed=0, label_material=0):
    """Run the scripts as one independent batch with logging on; returns
    (X [n, 15], Y [n, 7]) CUDA tensors labelled by material label_material
    (material 0 is the first script's, the nominal one) and the raw log."""
    batch = Batch(sims, track_strain=False)
    be = batch.backend
    be.log_start(capacity, fraction, seed)
    batch.run(steps)
    raw = be.log_data()
    be.log_stop()
    X = raw[:, :MLP_NIN].contiguous()
    lab = be.jc_label(label_material, X)
    keep = lab[:, MLP_NOUT] > 0.5
    return X[keep].contiguous(), lab[keep, :MLP_NOUT].contiguous(), raw, batch


def fit_norm(X, Y, margin=0.05):
    """Normalisation vector (include/kmpm.h layout): per-feature mean / std,
    and the envelope = the normalised range of the training inputs widened by
    margin of its width on each side."""
    import torch
    Xd, Yd = X.double(), Y.double()
    in_mean, in_std = Xd.mean(0), Xd.std(0)
    in_std = torch.where(in_std > 1e-12 * (in_mean.abs() + 1), in_std, torch.zeros_like(in_std))
    out_mean, out_scale = Yd.mean(0), Yd.std(0).clamp_min(1e-12)
    istd = torch.where(in_std > 0, 1.0 / torch.where(in_std > 0, in_std, torch.ones_like(in_std)),
                       torch.zeros_like(in_std))
    Xn = (Xd - in_mean) * istd
    lo, hi = Xn.min(0).values, Xn.max(0).values
    w = (hi - lo).clamp_min(1e-6)
    env_lo, env_hi = lo - margin * w, hi + margin * w
    norm = torch.cat([in_mean, in_std, out_mean, out_scale, env_lo, env_hi]).float().cpu().numpy()
    assert norm.size == MLP_NNORM
    return norm


def train_surrogate(X, Y, steps=20000, batch=8192, lr=2e-3, seed=0, holdout=0.05, report_every=0):
    """A trained :class:`Mlp` and its hold-out statistics."""
    import torch
    n = X.shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    perm = torch.randperm(n, generator=g).to(X.device)
    nh = max(1, int(n * holdout))
    te, tr = perm[:nh], perm[nh:]
    Xtr, Ytr = X[tr].contiguous(), Y[tr].contiguous()
    mlp = Mlp(batch=batch, seed=seed)
    mlp.norm = fit_norm(Xtr, Ytr)
    loss = mlp.train(Xtr, Ytr, steps=steps, batch=min(batch, Xtr.shape[0]), lr=lr, seed=seed,
                     report_every=report_every)
    stats = evaluate(mlp, X[te].contiguous(), Y[te].contiguous())
    stats["train_loss"] = loss
    stats["n_train"], stats["n_holdout"] = int(Xtr.shape[0]), int(nh)
    return mlp, stats


def evaluate(mlp, X, Y):
    """Relative L2 errors of the FP32 and tensor-core predictions of the
    stress correction and the plastic strain increment."""
    yf = mlp.predict(X)
    yt, inside = mlp.predict_tc(X)

    def rel(a, b):
        return float((a - b).norm() / b.norm().clamp_min(1e-30))

    return {"fp32_rel_l2_stress": rel(yf[:, :6], Y[:, :6]), "fp32_rel_l2_dep": rel(yf[:, 6], Y[:, 6]),
            "tc_rel_l2_stress": rel(yt[:, :6], Y[:, :6]), "tc_rel_l2_dep": rel(yt[:, 6], Y[:, 6]),
            "tc_vs_fp32": rel(yt, yf), "inside": float(inside.float().mean())}


def residual_pass(X, Y, P, G, tols=(1e-3, 3e-3, 1e-2)):
    """Share of rows whose predicted answer P passes the learned kernel's
    acceptance test (radial projection, yield and flow-rule residuals) at each
    tolerance; X, Y are inputs and closed-form outputs of plastic rows."""
    import torch
    X, Y, P = X.double(), Y.double(), P.double()
    s = X[:, 6:12] + 2 * G * X[:, 0:6]
    tr = s[:, :3].mean(1, keepdim=True)
    s = torch.cat([s[:, :3] - tr, s[:, 3:]], 1)
    w = torch.tensor([1, 1, 1, 2, 2, 2.], dtype=torch.float64, device=X.device)
    ss = (w * s * s).sum(1)
    J2tr = torch.sqrt(1.5 * ss)
    ys = J2tr - 3 * G * Y[:, 6]
    f1 = 1 + (w * P[:, :6] * s).sum(1) / ss
    J2n = J2tr * f1.abs()
    r_y = (J2n - ys).abs() / ys
    r_f = (J2tr - J2n - 3 * G * P[:, 6]).abs() / ys
    out = {}
    for tol in tols:
        ok = (r_y <= tol) & (r_f <= tol) & (P[:, 6] >= 0) & (f1 > 0)
        out[f"{tol:g}"] = float(ok.double().mean())
    return out


def save_network(mlp, path, meta):
    np.savez(path, params=mlp.params, norm=mlp.norm, meta=json.dumps(meta))


def load_network(path, batch=256):
    """An :class:`Mlp` with the parameters and normalisation saved by ``save_network``."""
    d = np.load(path)
    mlp = Mlp(batch=batch, seed=0)
    mlp.params = d["params"]
    mlp.norm = d["norm"]
    return mlp, json.loads(str(d["meta"]))


def train_taylor_network(out, steps=100000, seed=0, nominal_cellsize=0.1, nominal_steps=1500,
                         sweep_cellsize=0.2, sweep_instances=8, sweep_steps=4000, capacity=16_000_000,
                         sweep_fraction=0.002, nominal_fraction=0.008, report_every=10000):
    """The network of the Taylor-bar benchmark: pairs from the nominal bar at
    the benchmark's resolution and from a batch of bars with A, B, n, C
    perturbed by +-20% at twice the cell size (relabelled with the nominal
    material), trained on the GPU; saved with its hold-out statistics."""
    import time
    import torch
    t0 = time.time()
    sims, params = taylor_training_runs(cellsize=sweep_cellsize, instances=sweep_instances, spread=0.2, seed=seed)
    Xa, Ya, _, _ = collect_pairs(sims, steps=sweep_steps, capacity=capacity, fraction=sweep_fraction, seed=seed + 1)
    nominal = [W.taylor_bar(None, cellsize=nominal_cellsize)]
    W.taylor_bar_wall(nominal[0])
    Xb, Yb, _, _ = collect_pairs(nominal, steps=nominal_steps, capacity=capacity, fraction=nominal_fraction,
                                 seed=seed + 2)
    X, Y = torch.cat([Xa, Xb]).contiguous(), torch.cat([Ya, Yb]).contiguous()
    t1 = time.time()
    mlp, stats = train_surrogate(X, Y, steps=steps, batch=8192, lr=2e-3, seed=seed, report_every=report_every)
    t2 = time.time()
    G = W.COPPER["E"] / (2 * (1 + W.COPPER["nu"]))
    idx = torch.arange(0, X.shape[0], 13, device=X.device)
    P, _ = mlp.predict_tc(X[idx].contiguous())
    stats["tc_pass"] = residual_pass(X[idx], Y[idx], P, G)
    stats.update(collect_s=t1 - t0, train_s=t2 - t1, n_pairs=int(X.shape[0]), n_sweep=int(Xa.shape[0]),
                 n_nominal=int(Xb.shape[0]), steps=steps,
                 perturbed_params=params, nominal_cellsize=nominal_cellsize, sweep_cellsize=sweep_cellsize)
    save_network(mlp, out, stats)
    return mlp, stats


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description="train the learned return map of the Taylor-bar benchmark")
    ap.add_argument("--out", required=True)
    ap.add_argument("--steps", type=int, default=100000)
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args()
    _, st = train_taylor_network(a.out, steps=a.steps, seed=a.seed)
    print(json.dumps(st), flush=True)
