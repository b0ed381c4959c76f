"""The FP64 network oracle pinned by finite differences, and the closed-form
return-map oracle pinned by the radial-return identities (CPU only)."""
import numpy as np

import mlp_oracle as MO


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    npar = sum(o * i + o for o, i in MO.SIZES)
    params = rng.normal(0, 0.3, npar)
    norm = np.zeros(74)
    norm[:15] = rng.normal(0, 1, 15)
    norm[15:30] = rng.uniform(0.5, 2, 15)
    norm[30:37] = rng.normal(0, 1, 7)
    norm[37:44] = rng.uniform(0.5, 2, 7)
    X = rng.normal(0, 2, (16, 15))
    Y = rng.normal(0, 1, (16, 7))
    _, g = MO.loss_grad(params, norm, X, Y)
    idx = rng.choice(npar, 60, replace=False)
    h = 1e-6
    for k in idx:
        pp, pm = params.copy(), params.copy()
        pp[k] += h
        pm[k] -= h
        fd = (MO.loss_grad(pp, norm, X, Y)[0] - MO.loss_grad(pm, norm, X, Y)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 + 1e-5 * abs(fd), (k, fd, g[k])


def test_oracle_return_map_identities():
    """On plastic rows: |s_new| = flow stress, stress drop = 3 G dep, radial."""
    rng = np.random.default_rng(1)
    p = np.array([43.9, 0.09, 0.292, 0.31, 1e-3, 0.025, 0.0, 25.0, 1600.0])
    n = 500
    X = np.zeros((n, 15))
    X[:, 0:6] = rng.normal(0, 2e-3, (n, 6))
    X[:, 6:12] = rng.normal(0, 0.1, (n, 6))
    X[:, 12] = rng.uniform(0, 1, n)
    X[:, 14] = rng.uniform(0, 10, n)
    Y = MO.jc_label(p, X)
    pl = Y[:, 7] > 0.5
    assert 50 < pl.sum() < n
    s = X[:, 6:12] + 2 * p[0] * X[:, 0:6]
    s[:, :3] -= s[:, :3].mean(1, keepdims=True)
    vm = lambda a: np.sqrt(1.5 * (a[:, 0] ** 2 + a[:, 1] ** 2 + a[:, 2] ** 2 + 2 * (a[:, 3:6] ** 2).sum(1)))
    sn = s + Y[:, :6]
    ys = MO.jc_flow_stress(p, X[:, 12], p[4] * np.expm1(X[:, 14]), X[:, 13])
    assert np.allclose(vm(sn)[pl], ys[pl], rtol=1e-12)
    assert np.allclose((vm(s) - vm(sn))[pl], 3 * p[0] * Y[pl, 6], rtol=1e-10, atol=1e-14)
    assert np.allclose(sn[pl] * vm(s)[pl, None], s[pl] * vm(sn)[pl, None], rtol=1e-10, atol=1e-14)
    assert np.all(Y[~pl, :7] == 0)
