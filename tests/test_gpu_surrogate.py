"""Learned Johnson-Cook return map: training kernels against the FP64 oracle,
the tensor-core inference against a PyTorch reference of the same BF16
arithmetic, the logged training pairs against the closed form, and the
learned Taylor bar against the plain GPU path and the FP64 oracle."""
import numpy as np
import pytest

import mlp_oracle as MO

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _lib(gpu_lib):
    return gpu_lib


def _rand_norm(rng):
    norm = np.zeros(MO.NIN * 4 + MO.NOUT * 2, np.float32)
    norm[:15] = rng.normal(0, 0.5, 15)                    # in_mean
    norm[15:30] = rng.uniform(0.5, 2.0, 15)               # in_std
    norm[30:37] = rng.normal(0, 0.2, 7)                   # out_mean
    norm[37:44] = rng.uniform(0.5, 2.0, 7)                # out_scale
    norm[44:59], norm[59:74] = -1e30, 1e30                # envelope
    return norm


def test_mlp_gradient_matches_oracle():
    """Forward + backward kernels (FP32) vs the FP64 oracle on one batch."""
    from karamelo_gb300.gpu import Mlp
    rng = np.random.default_rng(1)
    mlp = Mlp(batch=256, seed=7)
    mlp.norm = _rand_norm(rng)
    X = rng.normal(0, 1.5, (200, 15)).astype(np.float32)
    Y = rng.normal(0, 1.0, (200, 7)).astype(np.float32)
    loss, g = mlp.loss_grad(torch.tensor(X, device="cuda"), torch.tensor(Y, device="cuda"))
    lo, go = MO.loss_grad(mlp.params, mlp.norm, X, Y)
    assert abs(loss - lo) <= 1e-5 * abs(lo)
    # per-tensor relative error of the gradient (FP32 accumulation over 200 rows)
    o = 0
    for n_out, n_in in MO.SIZES:
        for size in (n_out * n_in, n_out):
            a, b = g[o:o + size], go[o:o + size]
            assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b) + 1e-9, (o, size)
            o += size


def _bf16(t):
    return t.to(torch.bfloat16).to(torch.float32)


def _tc_reference(params, norm, X):
    """PyTorch reference of the tensor-core arithmetic: BF16 operands
    (weights, normalised inputs, hidden activations), FP32 accumulation,
    FP32 bias + ReLU epilogue; layer 1 as hi/lo BF16 pairs with the bias
    carried as a column."""
    p = [(torch.tensor(W, dtype=torch.float32), torch.tensor(b, dtype=torch.float32)) for W, b in MO.unpack(params)]
    nm = torch.tensor(norm, dtype=torch.float32)
    in_mean, in_std, out_mean, out_scale = nm[:15], nm[15:30], nm[30:37], nm[37:44]
    istd = torch.where(in_std > 0, 1.0 / torch.where(in_std > 0, in_std, torch.ones_like(in_std)), 0 * in_std)
    xn = (torch.tensor(X) - in_mean) * istd
    # layer 1 with the hi/lo split of inputs and weights (bias as a column)
    x = torch.cat([xn, torch.ones(xn.shape[0], 1)], 1)
    xh = _bf16(x)
    xl = _bf16(x - xh)
    W = torch.cat([p[0][0], p[0][1][:, None]], 1)
    Wh = _bf16(W)
    Wl = _bf16(W - Wh)
    z = xh.double() @ Wh.double().T + xl.double() @ Wh.double().T + xh.double() @ Wl.double().T
    h = _bf16(torch.relu(z).float())
    for li in (1, 2):
        h = _bf16(torch.relu((h.double() @ _bf16(p[li][0]).double().T).float() + p[li][1]))
    y = (h.double() @ _bf16(p[3][0]).double().T).float() + p[3][1]
    return (y * out_scale + out_mean).numpy()


def test_mlp_tensor_core_matches_torch_reference():
    """tcgen05 BF16 inference vs the PyTorch reference of the same arithmetic,
    over several CTAs and a ragged last tile."""
    from karamelo_gb300.gpu import Mlp
    rng = np.random.default_rng(2)
    mlp = Mlp(batch=256, seed=11)
    norm = _rand_norm(rng)
    mlp.norm = norm
    n = 3 * 512 + 77
    X = rng.normal(0, 1.5, (n, 15)).astype(np.float32)
    yt, inside = mlp.predict_tc(torch.tensor(X, device="cuda"))
    yt = yt.cpu().numpy()
    ref = _tc_reference(mlp.params, mlp.norm, X)
    err = np.linalg.norm(yt - ref) / np.linalg.norm(ref)
    assert err < 2e-3, err
    assert np.max(np.abs(yt - ref)) < 2e-2 * np.max(np.abs(ref))
    assert bool(inside.all())
    # and against the FP32 network (BF16 rounding only)
    yf = mlp.predict(torch.tensor(X, device="cuda")).cpu().numpy()
    assert np.linalg.norm(yt - yf) / np.linalg.norm(yf) < 3e-2


def test_mlp_envelope_flags():
    from karamelo_gb300.gpu import Mlp
    rng = np.random.default_rng(3)
    mlp = Mlp(batch=64, seed=1)
    norm = _rand_norm(rng)
    norm[15:30] = 1.0
    norm[:15] = 0.0
    norm[44:59], norm[59:74] = -1.0, 1.0
    mlp.norm = norm
    X = rng.uniform(-0.9, 0.9, (600, 15)).astype(np.float32)
    X[::7, 3] = 1.5
    _, inside = mlp.predict_tc(torch.tensor(X, device="cuda"))
    expect = np.ones(600, np.int8)
    expect[::7] = 0
    assert np.array_equal(inside.cpu().numpy(), expect)


def test_mlp_training_reduces_loss():
    """The training kernels fit a smooth function of the inputs."""
    from karamelo_gb300.gpu import Mlp
    rng = np.random.default_rng(4)
    n = 20000
    X = rng.uniform(-1, 1, (n, 15)).astype(np.float32)
    Y = np.stack([np.sin(X[:, 0]) + X[:, 1] * X[:, 2], np.maximum(X[:, 3], 0), X[:, 4] ** 2,
                  X[:, 5] - X[:, 6], np.tanh(X[:, 7] + X[:, 8]), X[:, 9] * 0.5, X[:, 10] * X[:, 11]], 1)
    Y = Y.astype(np.float32)
    mlp = Mlp(batch=1024, seed=3)
    norm = np.zeros(74, np.float32)
    norm[15:30], norm[37:44] = 1.0, 1.0
    norm[44:59], norm[59:74] = -1e30, 1e30
    mlp.norm = norm
    Xt, Yt = torch.tensor(X, device="cuda"), torch.tensor(Y, device="cuda")
    l0, _ = mlp.loss_grad(Xt[:1024], Yt[:1024])
    mlp.train(Xt, Yt, steps=1500, batch=1024, lr=2e-3, seed=5)
    l1, _ = mlp.loss_grad(Xt[:1024], Yt[:1024])
    assert l1 < 0.02 * l0, (l0, l1)


def test_logged_pairs_are_the_closed_form():
    """Pairs logged by the stress kernel equal the closed-form return map of
    the run's material (GPU labelling kernel and the FP64 oracle)."""
    from karamelo_gb300 import workloads as W
    from karamelo_gb300.gpu import GpuBackend
    sim = W.taylor_bar(None, cellsize=0.8)
    sim.backend = GpuBackend(sim.s, track_strain=False)
    sim.run(1)
    W.taylor_bar_wall(sim)
    be = sim.backend
    be.log_start(200000, 0.25, seed=3)
    sim.run(600)
    raw = be.log_data()
    be.log_stop()
    assert raw.shape[0] > 1000
    X, Yk = raw[:, :15].contiguous(), raw[:, 15:]
    lab = be.jc_label(0, X)
    assert bool((lab[:, 7] > 0.5).all())            # logged rows are plastic
    # same FP32 arithmetic in a different order: agreement to FP32 rounding of the trial stress
    assert float((lab[:, :7] - Yk).abs().max()) <= 1e-5 * float(Yk.abs().max())
    # FP64 oracle of the closed form on the same inputs
    m = sim.s.materials[0]
    p = np.array([m.str_p[k] for k in range(9)], np.float64)
    ref = MO.jc_label(p, X.double().cpu().numpy())
    got = lab.cpu().numpy()
    assert np.linalg.norm(got[:, :6] - ref[:, :6]) <= 1e-4 * np.linalg.norm(ref[:, :6])
    assert np.linalg.norm(got[:, 6] - ref[:, 6]) <= 1e-4 * np.linalg.norm(ref[:, 6])


@pytest.fixture(scope="module")
def trained(gpu_lib):
    from karamelo_gb300 import surrogate as S
    sims, _ = S.taylor_training_runs(cellsize=0.8, instances=6, spread=0.2, seed=0)
    X, Y, raw, _ = S.collect_pairs(sims, steps=2500, capacity=2_000_000, fraction=0.5, seed=1)
    mlp, stats = S.train_surrogate(X, Y, steps=20000, batch=4096, lr=2e-3, seed=0)
    return mlp, stats, X, Y


def _learned_bar(mlp, steps, tol=1e-3, cellsize=0.8):
    from karamelo_gb300 import workloads as W
    from karamelo_gb300.gpu import GpuBackend
    sim = W.taylor_bar(None, cellsize=cellsize)
    sim.backend = GpuBackend(sim.s, track_strain=False)
    sim.run(1)
    W.taylor_bar_wall(sim)
    if mlp is not None:
        sim.backend.set_surrogate(mlp, tol)
    sim.run(steps)
    return sim


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_learned_taylor_bar_matches_plain_and_oracle(trained):
    """The learned path (network where its residuals pass, closed form
    elsewhere) stays within 1e-3 relative L2 of the plain GPU path and of the
    FP64 oracle in stress and bar length, and the network serves plastic
    particle-steps."""
    import oracle as orc
    from karamelo_gb300 import workloads as W
    mlp, stats, _, _ = trained
    steps = 1500
    learned = _learned_bar(mlp, steps)
    plain = _learned_bar(None, steps)
    ref = W.taylor_bar(lambda s: orc.OracleBackend(s), cellsize=0.8, method="tlmpm")
    ref.run(1)
    W.taylor_bar_wall(ref)
    ref.run(steps)
    st = learned.backend.surrogate_stats()
    assert st["plastic"] > 0 and st["network"] > 0, st
    sl, sp, so = (s.particles(0, "sigma") for s in (learned, plain, ref))
    xl, xp, xo = (s.particles(0, "x") for s in (learned, plain, ref))
    assert _rel(sl, so) <= 1e-3 and _rel(sl, sp) <= 1e-3
    length = lambda x: x[:, 0].max() - x[:, 0].min()
    assert abs(length(xl) - length(xo)) <= 1e-3 * length(xo)
    assert _rel(xl, xo) <= 1e-3


def test_trained_network_gain(trained):
    """What training buys: the share of plastic return maps the network
    answers within a 1e-2 residual tolerance, trained vs the same network
    untrained (He initialisation with the trained normalisation); the closed
    form covers the rest."""
    from karamelo_gb300.gpu import Mlp
    mlp, stats, _, _ = trained
    untrained = Mlp(batch=256, seed=0)
    untrained.norm = mlp.norm
    steps = 1200
    a = _learned_bar(mlp, steps, tol=1e-2).backend.surrogate_stats()
    b = _learned_bar(untrained, steps, tol=1e-2).backend.surrogate_stats()
    share = lambda s: s["network"] / max(1, s["plastic"])
    assert share(a) > 0.1, (a, stats)
    assert share(b) < 0.005, b
    assert share(a) > 20 * share(b)


def test_queued_network_matches_fused_kernel(trained):
    """Two schedules of the learned return map: the plain stress kernel
    queueing the plastic steps for a separate network kernel (the default for
    linear EOS + Johnson-Cook), and the network fused into the stress kernel
    (KMPM_SUR_FUSED=1).  Both apply the same tests to the same answers, so
    they serve about the same steps and end at the same state."""
    import os
    mlp, _, _, _ = trained
    steps = 800
    a = _learned_bar(mlp, steps)
    os.environ["KMPM_SUR_FUSED"] = "1"
    try:
        b = _learned_bar(mlp, steps)
    finally:
        del os.environ["KMPM_SUR_FUSED"]
    sa, sb = a.backend.surrogate_stats(), b.backend.surrogate_stats()
    assert sa["network"] > 0 and sb["network"] > 0, (sa, sb)
    assert abs(sa["plastic"] - sb["plastic"]) <= 0.01 * sb["plastic"], (sa, sb)
    assert abs(sa["network"] - sb["network"]) <= 0.02 * sb["network"], (sa, sb)
    for f, tol in (("sigma", 1e-4), ("x", 1e-6), ("eps_p", 1e-4)):
        assert _rel(a.particles(0, f), b.particles(0, f)) <= tol, f
