"""Scalar-potential surrogate: the oracle's gradient and double
backpropagation against finite differences (CPU); the device's gradient pass
and training gradients against the oracle, a training run on a known
potential, and exactness when it drives the sampler (GPU).

Tolerances: oracle vs central differences 1e-6 (FP64).  Device vs oracle:
the device rounds inputs, weights, activations and deltas to BF16 (2^-8
relative) at the same points as the oracle's predict form, so the predicted
gradient agrees to 1e-4 median / 2e-2 max of its scale; the training
gradients, whose oracle is unrounded FP64, to 3 % (Frobenius)."""
import numpy as np
import pytest

from oracle import mlp_oracle as MO


def small_params(rng, d=7, h1=9, h2=8):
    P = dict(W1=rng.normal(size=(h1, d)) / 3, b1=rng.normal(size=h1) / 3, W2=rng.normal(size=(h2, h1)) / 3,
             b2=rng.normal(size=h2) / 3, w3=rng.normal(size=h2))
    A = rng.normal(size=(d, d))
    return P, 0.5 * (A + A.T), rng.normal(size=d)


def test_oracle_gradient_is_the_derivative_of_the_potential():
    rng = np.random.default_rng(0)
    P, A, beta = small_params(rng)
    x = rng.normal(size=(5, 7))
    g = MO.potential_grad(x, **P, A=A, beta=beta)
    eps = 1e-6
    for i in range(7):
        e = np.zeros(7)
        e[i] = eps
        fd = (MO.potential_value(x + e, **P, A=A, beta=beta) - MO.potential_value(x - e, **P, A=A, beta=beta)) / (2 * eps)
        np.testing.assert_allclose(fd, g[:, i], rtol=1e-6, atol=1e-8)
    # a gradient field: its Jacobian is symmetric
    J = np.stack([(MO.potential_grad(x + np.eye(7)[i] * eps, **P, A=A, beta=beta)
                   - MO.potential_grad(x - np.eye(7)[i] * eps, **P, A=A, beta=beta)) / (2 * eps) for i in range(7)], 2)
    np.testing.assert_allclose(J, np.swapaxes(J, 1, 2), atol=1e-6)


def test_oracle_double_backpropagation_matches_finite_differences():
    rng = np.random.default_rng(1)
    P, A, beta = small_params(rng)
    x, t = rng.normal(size=(5, 7)), rng.normal(size=(5, 7))
    sc, sh = rng.uniform(0.5, 2, size=7), rng.normal(size=7)
    _, G = MO.potential_loss_grads(x, t, sc, sh, **P, A=A, beta=beta)
    eps = 1e-6
    for k, v in P.items():
        for idx in rng.choice(v.size, size=min(6, v.size), replace=False):
            Pp = {kk: vv.copy() for kk, vv in P.items()}
            Pm = {kk: vv.copy() for kk, vv in P.items()}
            Pp[k].reshape(-1)[idx] += eps
            Pm[k].reshape(-1)[idx] -= eps
            lp, _ = MO.potential_loss_grads(x, t, sc, sh, **Pp, A=A, beta=beta)
            lm, _ = MO.potential_loss_grads(x, t, sc, sh, **Pm, A=A, beta=beta)
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - G[k].reshape(-1)[idx]) <= 1e-6 * max(1.0, abs(fd)), (k, idx)


# ---------------------------------------------------------------------------
def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def h(t):
    return t.double().cpu().numpy()


def _fitted(torch, d, hidden, n, seed, grad):
    from hmclab_gb300 import surrogate as S

    rng = np.random.default_rng(seed)
    data = S.TrainingSet(d, n)
    Q = rng.normal(size=(d, n))
    for k in range(n // 256):
        qc = Q[:, k * 256:(k + 1) * 256]
        assert data.record(torch.from_numpy(qc.copy()).float().cuda(), torch.from_numpy(grad(qc)).float().cuda(),
                           torch.cuda.current_stream().cuda_stream)
    net = S.PotentialSurrogate(d, hidden=hidden, seed=seed)
    net.fit_normalization(data)
    return net, data, Q, rng


def _oracle_params(net):
    return dict(W1=h(net.params["W1"]), b1=h(net.params["b1"]), W2=h(net.params["W2"]), b2=h(net.params["b2"]),
                w3=h(net.params["w3"]), A=h(net.A), beta=h(net.beta))


@pytest.mark.gpu
def test_device_potential_gradient_matches_oracle():
    """grad_q f on the sampler's [d][C] layout against the oracle with the
    same weights and BF16 rounding points, after a few training steps."""
    torch = _torch()
    d, C = 80, 300
    net, data, _, rng = _fitted(torch, d, (128, 64), 1024, 4, lambda q: 2.0 * q + np.sin(q))
    net.train(data, steps=20, batch=128, lr=1e-3)
    qt = rng.normal(size=(d, C)).astype(np.float32)
    out = torch.zeros((d, C), dtype=torch.float32, device="cuda")
    net.freeze().predict_into(torch.from_numpy(qt).cuda(), out, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    net.check_status()
    ref = MO.potential_predict(qt.astype(np.float64), h(net.mu_q), 1.0 / h(net.inv_q), h(net.mu_g), h(net.sig_g),
                               **_oracle_params(net))
    err = np.abs(h(out) - ref) / (np.abs(ref).max() + 1e-30)
    assert np.median(err) < 1e-4 and err.max() < 2e-2, (np.median(err), err.max())


@pytest.mark.gpu
def test_device_training_gradients_match_oracle():
    """One training step with a zero learning rate: the device's weight and
    bias gradients (double backpropagation through BF16 contractions)
    against the oracle's FP64 gradients on the same minibatch."""
    torch = _torch()
    d, B = 48, 128
    net, data, _, rng = _fitted(torch, d, (64, 64), 512, 6, lambda q: 1.5 * q + np.tanh(2 * q))
    net.train(data, steps=10, batch=B, lr=1e-3)  # non-trivial weights
    idx = rng.integers(0, 512, size=B)
    net.train_step(data, idx, lr=0.0)
    torch.cuda.synchronize()
    net.check_status()
    q = h(data.q[torch.from_numpy(idx).cuda()])
    g = h(data.g[torch.from_numpy(idx).cuda()])
    x = (q - h(net.mu_q)) * h(net.inv_q)
    t = (g - h(net.mu_g)) * h(net.inv_g)
    scale = h(net.scale)
    shift = -h(net.mu_g) / h(net.sig_g)
    loss, G = MO.potential_loss_grads(x, t, scale, shift, **_oracle_params(net))
    assert abs(float(net.loss_buf[0]) - loss) <= 0.02 * loss
    for k, ref in G.items():
        got = h(net.grads[k])
        rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        print(f"{k}: relative error {rel:.2e}")
        assert rel < 0.03, (k, rel)


@pytest.mark.gpu
def test_potential_learns_a_potential():
    """Gradients of U(q) = q^T P q / 2 + sum_k log cosh(3 w_k . q) * 2/3 in 64-D:
    the trained potential's held-out gradient error must fall well below the
    quadratic (ridge) start."""
    torch = _torch()
    d = 64
    rng0 = np.random.default_rng(3)
    L = rng0.normal(size=(d, d)) / np.sqrt(d)
    P = L @ L.T + np.eye(d)
    Wd = rng0.normal(size=(4, d)) / np.sqrt(d) * 2

    def grad(q):
        return P @ q + 2.0 * Wd.T @ np.tanh(3 * Wd @ q)

    net, data, Q, rng = _fitted(torch, d, (256, 256), 8192, 2, grad)
    held = torch.arange(7680, 8192, device="cuda")
    e0 = net.relative_error(data, held)
    net.train(data, steps=1500, batch=256, lr=2e-3, rows=7680)
    e1 = net.relative_error(data, held)
    print(f"held-out relative error: quadratic start {e0:.3f} -> trained {e1:.3f}")
    net.check_status()
    assert e1 < 0.5 * e0 and e1 < 0.1


@pytest.mark.gpu
def test_potential_surrogate_keeps_the_exact_posterior():
    """A potential fitted to 1.3x the true gradient drives the leapfrog; the
    exact accept test keeps chains started at posterior draws distributed as
    the posterior."""
    torch = _torch()
    import hmclab_gb300 as H
    from hmclab_gb300 import surrogate as S
    from hmclab_gb300 import problems

    d0 = 32
    G, dat, _ = problems.dense_linear(64, d0, 1.0 / np.sqrt(d0), 0.2, 0)
    post = H.Distributions.BayesRule([H.Distributions.Normal(np.zeros((d0, 1)), np.ones((d0, 1))),
                                      H.Distributions.LinearMatrix(G, dat, 0.04)])
    mean, cov = problems.gaussian_posterior(G, dat, 0.04, 0.0, 1.0)
    d, C = 32, 4096
    rng = np.random.default_rng(2)
    Lc = np.linalg.cholesky(cov)
    data = S.TrainingSet(d, 8192)
    for _ in range(8):
        qb = torch.from_numpy(mean + 1.5 * Lc @ rng.normal(size=(d, 1024))).float().cuda().contiguous()
        data.record(qb, 1.3 * post.gradient_batch(qb), torch.cuda.current_stream().cuda_stream)
    net = S.PotentialSurrogate(d, hidden=(64, 64), seed=0)
    net.fit(data, steps=300, batch=256, lr=1e-3)
    net.freeze()
    w = np.sqrt(np.linalg.eigvalsh(np.linalg.inv(cov)).max())
    q0 = mean + Lc @ rng.normal(size=(d, C))
    smp = H.Samplers.HMC(seed=4).sample(None, post, stepsize=0.5 / w, amount_of_steps=8, initial_model=q0,
                                        proposals=30, chains=C, dtype="float32", surrogate=net)
    acc = np.mean(smp.accepted_proposals) / 30
    assert 0.05 < acc < 0.95, acc
    q = smp.current_model
    sd = np.sqrt(np.diag(cov))
    z_mean = np.abs(q.mean(axis=1) - mean[:, 0]) / (sd / np.sqrt(C))
    var_ratio = q.var(axis=1) / np.diag(cov)
    print(f"acceptance {acc:.3f}; max |mean error| {z_mean.max():.2f} standard errors; variance ratio "
          f"{var_ratio.min():.3f}..{var_ratio.max():.3f}")
    assert z_mean.max() < 5.0
    assert np.all(np.abs(var_ratio - 1.0) < 5.0 * np.sqrt(2.0 / C))


@pytest.mark.gpu
def test_fit_skips_non_finite_pairs():
    """Pairs recorded from diverged trajectories (non-finite gradient) are
    left out of the normalisation, the ridge start and the loss."""
    torch = _torch()
    from hmclab_gb300 import surrogate as S

    d = 32

    def grad(q):
        return 2.0 * q + np.sin(q)

    for kind in (S.PotentialSurrogate, S.MLPSurrogate):
        data = S.TrainingSet(d, 2048)
        rng = np.random.default_rng(9)
        for k in range(8):
            q = rng.normal(size=(d, 256))
            g = grad(q)
            if k == 3:
                g[:, :40] = np.nan
                g[0, 40:50] = np.inf
            data.record(torch.from_numpy(q).float().cuda(), torch.from_numpy(g).float().cuda(),
                        torch.cuda.current_stream().cuda_stream)
        net = kind(d, hidden=(64, 64), seed=1)
        fit = net.fit(data, steps=200, batch=128)
        assert fit["skipped_pairs"] == 50
        assert np.isfinite(fit["best_heldout"]) and fit["best_heldout"] < fit["heldout"][0][1] + 1e-12
        qt = torch.from_numpy(rng.normal(size=(d, 64))).float().cuda()
        out = torch.empty_like(qt)
        net.freeze().predict_into(qt, out, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert torch.isfinite(out).all()


def test_quadratic_fit_recovers_a_quadratic_potential():
    """The fixed part of the potential surrogate: the symmetrised ridge fit
    of gradients recovers the Hessian and linear term of a quadratic (host,
    no device)."""
    from hmclab_gb300.surrogate import quadratic_fit

    rng = np.random.default_rng(4)
    d, n = 12, 4000
    L = rng.normal(size=(d, d))
    H = L @ L.T / d + np.eye(d)
    b = rng.normal(size=d)
    x = rng.normal(size=(n, d))
    A, beta = quadratic_fit(x, x @ H + b, ridge=1e-9)
    np.testing.assert_allclose(A, H, atol=1e-6)
    np.testing.assert_allclose(beta, b, atol=1e-6)
    # a non-symmetric linear field is projected onto its symmetric part
    M = rng.normal(size=(d, d))
    A2, _ = quadratic_fit(x, x @ M.T, ridge=1e-9)
    np.testing.assert_allclose(A2, 0.5 * (M + M.T), atol=1e-6)


def test_oracle_value_loss_gradients_match_finite_differences():
    rng = np.random.default_rng(8)
    P, _, _ = small_params(rng)
    x = rng.normal(size=(6, 7))
    t = rng.normal(size=6) * 3
    loss, G = MO.potential_value_loss_grads(x, t, 0.7, **P)
    eps = 1e-6
    for k in P:
        for idx in list(np.ndindex(P[k].shape))[:5]:
            Pp = {kk: v.copy() for kk, v in P.items()}
            Pm = {kk: v.copy() for kk, v in P.items()}
            Pp[k][idx] += eps
            Pm[k][idx] -= eps
            fd = (MO.potential_value_loss_grads(x, t, 0.7, **Pp)[0] - MO.potential_value_loss_grads(x, t, 0.7, **Pm)[0])
            fd /= 2 * eps
            assert abs(fd - G[k][idx]) <= 1e-6 * max(1.0, abs(fd)), (k, idx, fd, G[k][idx])


@pytest.mark.gpu
def test_device_value_matching_gradients_match_oracle():
    """With values matched, a training step adds the value loss's weight
    gradients (csrc/potential.cu value kernels + tensor-core WGRAD) to the
    gradient-matching ones: the difference of the two steps' gradients
    against the oracle's FP64 backpropagation on the same minibatch (BF16
    activations and deltas on the device: 3 % Frobenius)."""
    torch = _torch()
    from hmclab_gb300 import surrogate as S

    d, B, n = 48, 128, 512
    rng = np.random.default_rng(12)
    data = S.TrainingSet(d, n, values=True)
    Q = rng.normal(size=(d, n))

    def U(q):
        return 0.75 * np.sum(q * q, axis=0) + np.sum(np.log(np.cosh(2 * q[:5])), axis=0)

    def grad(q):
        g = 1.5 * q
        g[:5] += 2 * np.tanh(2 * q[:5])
        return g

    st = torch.cuda.current_stream().cuda_stream
    for k in range(n // 256):
        qc = Q[:, k * 256:(k + 1) * 256]
        data.record(torch.from_numpy(qc.copy()).float().cuda(), torch.from_numpy(grad(qc)).float().cuda(), st,
                    torch.from_numpy(U(qc)).cuda())
    torch.cuda.synchronize()
    assert torch.isfinite(data.x[:n]).all()
    net = S.PotentialSurrogate(d, hidden=(64, 64), seed=1)
    net.value_weight = 0.5
    net.fit_normalization(data)
    net.train(data, steps=10, batch=B, lr=1e-3)
    idx = rng.integers(0, n, size=B)
    w = net._vt_w
    net._vt_w = 0.0
    net.train_step(data, idx, lr=0.0)
    g_grad = {k: h(v) for k, v in net.grads.items()}
    net._vt_w = w
    net.train_step(data, idx, lr=0.0)
    torch.cuda.synchronize()
    net.check_status()
    q = h(data.q[torch.from_numpy(idx).cuda()])
    x = (q - h(net.mu_q)) * h(net.inv_q)
    t = h(net._vt)[idx]
    P = _oracle_params(net)
    loss, G = MO.potential_value_loss_grads(x, t, w, P["W1"], P["b1"], P["W2"], P["b2"], P["w3"])
    assert abs(float(net.value_loss[0]) - loss) <= 0.02 * loss
    for k, ref in G.items():
        got = h(net.grads[k]) - g_grad[k]
        rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        print(f"value loss {k}: relative error {rel:.2e}")
        assert rel < 0.03, (k, rel)
    # the held-out value error is measured and finite
    ve = net.value_error(data, np.arange(256))
    assert ve is not None and np.isfinite(ve)
