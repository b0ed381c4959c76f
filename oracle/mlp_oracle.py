"""FP64 CPU restatement of the learned return map's network and of the
closed-form Johnson-Cook return map it is trained on.

TEST INFRASTRUCTURE: only the tests may import this module, as the checker of
the CUDA kernels (karamelo_gb300/csrc/kmpm_mlp.cu, kmpm_learn.cu).  It is never
the thing measured and never part of the product path.

Network: 15 -> 128 -> 128 -> 128 -> 7, ReLU hidden layers, the flat parameter
layout of include/kmpm.h (W1[128x15] b1 W2 b2 W3 b3 W4[7x128] b4, row-major
out x in), inputs and outputs normalised by the affine maps of the
normalisation vector, loss = mean squared error in normalised output units.

Return map: StrengthJohnsonCook::update_deviatoric_stress
(src/strength_jc.cpp:100-184) on one particle-step without damage, written in
terms of the network's inputs (strain increment dt*D, stress, eps_p, T,
log(1 + epsdot/epsdot0)).
"""
from __future__ import annotations

import numpy as np

NIN, NOUT, HID = 15, 7, 128
SIZES = [(HID, NIN), (HID, HID), (HID, HID), (NOUT, HID)]


def unpack(params):
    """List of (W, b) in float64."""
    p = np.asarray(params, np.float64)
    out, o = [], 0
    for n_out, n_in in SIZES:
        W = p[o:o + n_out * n_in].reshape(n_out, n_in)
        o += n_out * n_in
        b = p[o:o + n_out]
        o += n_out
        out.append((W, b))
    assert o == p.size
    return out


def split_norm(norm):
    n = np.asarray(norm, np.float64)
    in_mean, in_std = n[:NIN], n[NIN:2 * NIN]
    out_mean, out_scale = n[2 * NIN:2 * NIN + NOUT], n[2 * NIN + NOUT:2 * NIN + 2 * NOUT]
    env_lo = n[2 * NIN + 2 * NOUT:3 * NIN + 2 * NOUT]
    env_hi = n[3 * NIN + 2 * NOUT:]
    return in_mean, in_std, out_mean, out_scale, env_lo, env_hi


def normalise_inputs(X, norm):
    in_mean, in_std = split_norm(norm)[:2]
    istd = np.where(in_std > 0, 1.0 / np.where(in_std > 0, in_std, 1.0), 0.0)
    return (np.asarray(X, np.float64) - in_mean) * istd


def forward(params, Xn):
    """Activations of every layer (normalised inputs in, normalised outputs out)."""
    acts = [np.asarray(Xn, np.float64)]
    layers = unpack(params)
    for li, (W, b) in enumerate(layers):
        z = acts[-1] @ W.T + b
        acts.append(np.maximum(z, 0.0) if li < 3 else z)
    return acts


def predict(params, norm, X):
    out_mean, out_scale = split_norm(norm)[2:4]
    return forward(params, normalise_inputs(X, norm))[-1] * out_scale + out_mean


def loss_grad(params, norm, X, Y):
    """Mean squared error in normalised output units and its gradient (float64)."""
    out_mean, out_scale = split_norm(norm)[2:4]
    Xn = normalise_inputs(X, norm)
    Yn = (np.asarray(Y, np.float64) - out_mean) / out_scale
    acts = forward(params, Xn)
    B = Xn.shape[0]
    d = acts[-1] - Yn
    loss = float(np.mean(d * d))
    dz = 2.0 * d / (B * NOUT)
    grads = []
    layers = unpack(params)
    for li in range(3, -1, -1):
        W, _ = layers[li]
        a_in = acts[li]
        grads.append((dz.T @ a_in, dz.sum(axis=0)))
        if li > 0:
            dz = (dz @ W) * (a_in > 0)
    flat = []
    for dW, db in reversed(grads):
        flat += [dW.ravel(), db]
    return loss, np.concatenate(flat)


def jc_flow_stress(p, epsp, epsdot, T):
    """p = (G, A, B, n, epsdot0, C, m, Tr, Tm) (src/strength_jc.cpp:120-150)."""
    G, A, B, n, epsdot0, C, m, Tr, Tm = p
    ratio = np.maximum(epsdot / epsdot0, 1.0)
    ys = np.where(epsp < 1e-10, A, A + B * np.power(np.maximum(epsp, 0.0), n))
    if C != 0:
        ys = ys * np.power(1.0 + ratio, C)
    if m != 0:
        hot = (T >= Tr) & (T < Tm)
        ys = np.where(hot, ys * (1.0 - np.power(np.clip((T - Tr) / (Tm - Tr), 0, None), m)), ys)
    return np.where(T < Tm, ys, 0.0)


def jc_label(p, X):
    """Closed-form return map on input rows: [n, 8] = s_new - s_trial (6), dep, plastic flag."""
    X = np.asarray(X, np.float64)
    G = p[0]
    epsdot = p[4] * np.expm1(X[:, 14])
    ys = jc_flow_stress(p, X[:, 12], epsdot, X[:, 13])
    s = X[:, 6:12] + 2.0 * G * X[:, 0:6]
    tr = (s[:, 0] + s[:, 1] + s[:, 2]) / 3.0
    s[:, 0:3] -= tr[:, None]
    nrm = np.sqrt(s[:, 0] ** 2 + s[:, 1] ** 2 + s[:, 2] ** 2 + 2 * (s[:, 3] ** 2 + s[:, 4] ** 2 + s[:, 5] ** 2))
    J2 = np.sqrt(1.5) * nrm
    pl = ~(J2 < ys)
    sc = np.where(pl, ys / np.where(J2 > 0, J2, 1.0), 1.0)
    Y = np.zeros((X.shape[0], 8))
    Y[:, :6] = s * sc[:, None] - s
    Y[:, 6] = np.where(pl, (J2 - ys) / (3 * G), 0.0)
    Y[:, 7] = pl
    return Y
