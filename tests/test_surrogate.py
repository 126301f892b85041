"""MLP surrogate kernels (tensor-core forward/backward, Adam) against the FP64
numpy oracle, stage by stage on the device's own stage inputs, and a training
run that must fit a known map.

Tolerances: contractions 2e-5 of sum |a||b| (FP32 accumulation of BF16
products); BF16 outputs within one BF16 ulp (2^-8 relative); Adam 1e-6."""
import numpy as np
import pytest

from oracle import mlp_oracle as MO

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def h(t):
    return t.double().cpu().numpy()


def close_contraction(got, a, b, ref, tol=2e-5):
    scale = np.abs(a) @ np.abs(b).T
    assert np.all(np.abs(got - ref) <= tol * scale + 1e-7), np.abs(got - ref).max()


def close_bf16(got, ref):
    """Equal up to one BF16 ulp (FP32 vs FP64 GELU may round across a BF16
    boundary): |got - ref| <= 2^-7 max(|got|, |ref|)."""
    bound = 2.0**-7 * np.maximum(np.abs(got), np.abs(ref)) * 1.0001 + 1e-30
    bad = np.abs(got - ref) > bound
    if bad.any():
        k = np.unravel_index(np.argmax(np.abs(got - ref) - bound), got.shape)
        raise AssertionError(f"{bad.sum()} of {bad.size} differ; worst at {k}: got {got[k]!r}, ref {ref[k]!r}")


def test_oracle_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0], dtype=np.float32)
    r = MO.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125 and abs(r[3] + 3.140625) < 1e-9 and r[4] == 0.0
    t = torch.tensor(x).to(torch.bfloat16).double().numpy()
    np.testing.assert_array_equal(r, t)


def test_training_step_matches_oracle():
    from hmclab_gb300 import surrogate as S

    d, B = 96, 160
    net = S.MLPSurrogate(d, hidden=(128, 64), seed=1)
    data = S.TrainingSet(d, 512)
    rng = np.random.default_rng(0)
    q = rng.normal(size=(d, 512))
    A = rng.normal(size=(d, d)) / np.sqrt(d)
    g = A @ q + 0.1 * np.tanh(q)
    for k in range(4):
        qc = torch.from_numpy(q[:, k * 128:(k + 1) * 128].copy()).float().cuda()
        gc = torch.from_numpy(g[:, k * 128:(k + 1) * 128].copy()).float().cuda()
        assert data.record(qc, gc, torch.cuda.current_stream().cuda_stream)
    net.fit_normalization(data)
    W0 = [h(w) for w in net.W]
    b0 = [h(x) for x in net.b]
    idx = rng.integers(0, 512, size=B)
    net.train_step(data, idx, lr=1e-3)
    torch.cuda.synchronize()
    bu = net._bufs[(B, True)]
    # inputs and targets
    qs, gs = h(data.q), h(data.g)
    x_ref = MO.bf16((qs[idx] - h(net.mu_q)) * h(net.inv_q))
    X = h(bu["X"])[:, :d]
    np.testing.assert_allclose(X, x_ref, rtol=2.0**-7)
    np.testing.assert_array_equal(h(bu["Xt"])[:, :B], X.T)
    T = h(bu["T"])
    np.testing.assert_allclose(T, (gs[idx] - h(net.mu_g)) * h(net.inv_g), rtol=1e-6, atol=1e-6)
    W16 = [MO.bf16(w) for w in W0]
    # layer 1 and 2 (pre-activations from the device inputs)
    Z1 = h(bu["Z1"])
    close_contraction(Z1 - b0[0], X, W16[0], X @ W16[0].T)
    A1 = h(bu["A1"])[:, :128]
    close_bf16(A1, MO.bf16(MO.gelu(Z1)))
    Z2 = h(bu["Z2"])
    close_contraction(Z2 - b0[1], A1, W16[1], A1 @ W16[1].T)
    A2 = h(bu["A2"])[:, :64]
    close_bf16(A2, MO.bf16(MO.gelu(Z2)))
    # the output layer reads [h2 | x] (linear skip path)
    A2x = h(bu["A2"])[:, :64 + d]
    np.testing.assert_array_equal(A2x[:, 64:], X)
    np.testing.assert_array_equal(h(bu["A2t"])[:, :B], A2x.T)
    Y = h(bu["Y"])
    close_contraction(Y - b0[2], A2x, W16[2], A2x @ W16[2].T)
    # loss and output delta
    loss = float(net.loss_buf[0].item())
    np.testing.assert_allclose(loss, 0.5 / B * np.sum((Y - T) ** 2), rtol=1e-6)
    dY = h(bu["dY"])[:, :d]
    close_bf16(dY, MO.bf16(((Y - T) / B).astype(np.float32)))
    # weight gradients from the device deltas and activations
    gW = [h(x) for x in net.gW]
    close_contraction(gW[2], dY.T, A2x.T, dY.T @ A2x)
    dZ2 = h(bu["dZ2"])[:, :64]
    close_bf16(dZ2, MO.back(dY, W16[2][:, :64], Z2))
    close_contraction(gW[1], dZ2.T, A1.T, dZ2.T @ A1)
    dZ1 = h(bu["dZ1"])[:, :128]
    close_bf16(dZ1, MO.back(dZ2, W16[1], Z1))
    close_contraction(gW[0], dZ1.T, X.T, dZ1.T @ X)
    gb = [h(x) for x in net.gb]
    np.testing.assert_allclose(gb[2], dY.sum(axis=0), rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(gb[0], dZ1.sum(axis=0), rtol=1e-5, atol=1e-7)
    # Adam step on the master weights
    for l in range(3):
        w1, _, _ = MO.adam(W0[l], gW[l], 0.0, 0.0, 1e-3, 0.9, 0.999, 1e-8, 1)
        np.testing.assert_allclose(h(net.W[l]), w1, rtol=1e-6, atol=1e-7)
    net.check_status()


def test_predict_matches_oracle():
    """The sampler-facing inference path (state layout [d][C] in, [d][C] out)
    against the FP64 oracle forward of the same weights, after a few
    training steps so that every weight block is non-trivial."""
    from hmclab_gb300 import surrogate as S

    d, C = 80, 300
    net = S.MLPSurrogate(d, hidden=(128, 64), seed=4)
    data = S.TrainingSet(d, 1024)
    rng = np.random.default_rng(5)
    q = rng.normal(size=(d, 1024))
    g = 2.0 * q + np.sin(q)
    for k in range(4):
        sl = slice(k * 256, (k + 1) * 256)
        assert data.record(torch.from_numpy(q[:, sl].copy()).float().cuda(),
                           torch.from_numpy(g[:, sl].copy()).float().cuda(), torch.cuda.current_stream().cuda_stream)
    net.fit_normalization(data)
    net.train(data, steps=20, batch=128, lr=1e-3)
    qt = rng.normal(size=(d, C)).astype(np.float32)
    out = torch.zeros((d, C), dtype=torch.float32, device="cuda")
    net.freeze().predict_into(torch.from_numpy(qt).cuda(), out, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    ref = MO.predict(qt.astype(np.float64), h(net.mu_q), h(net.inv_q), h(net.mu_g), h(net.sig_g),
                     [h(w) for w in net.W], [h(x) for x in net.b])
    err = np.abs(h(out) - ref) / (np.abs(ref).max() + 1e-30)
    # BF16 activations may round across a BF16 boundary (one ulp, 2^-8) in
    # a few entries; the output is an FP32 sum over 64 + d such products
    assert np.median(err) < 1e-4 and err.max() < 2e-2, (np.median(err), err.max())


def test_surrogate_learns_a_gradient_field():
    """Train on (q, grad U) pairs of a 64-D target: an anisotropic Gaussian
    plus four log-cosh ridges, grad U = P q + 2 sum_k w_k tanh(3 w_k.q).  The
    linear skip starts at the least-squares linear fit (held-out error ~0.19
    here); the trained network must fall below 8% held-out relative error and
    below 40% of the linear fit's.  An FP32 PyTorch model of the same
    architecture, initialisation and schedule reaches 0.040 on this problem."""
    from hmclab_gb300 import surrogate as S

    d = 64
    rng = np.random.default_rng(3)
    L = rng.normal(size=(d, d)) / np.sqrt(d)
    P = L @ L.T + np.eye(d)
    Wd = rng.normal(size=(4, d)) / np.sqrt(d) * 2

    def grad(q):
        return P @ q + 2.0 * Wd.T @ np.tanh(3 * Wd @ q)

    net = S.MLPSurrogate(d, hidden=(256, 256), seed=2)
    data = S.TrainingSet(d, 8192)
    Q = rng.normal(size=(d, 8192))
    for k in range(32):
        qc = Q[:, k * 256:(k + 1) * 256]
        assert data.record(torch.from_numpy(qc.copy()).float().cuda(), torch.from_numpy(grad(qc)).float().cuda(),
                           torch.cuda.current_stream().cuda_stream)
    net.fit_normalization(data)
    hist = net.train(data, steps=1500, batch=256, lr=2e-3)
    assert hist[-1][1] < 0.25 * hist[0][1], hist
    qt = rng.normal(size=(d, 512))
    g = torch.zeros((d, 512), dtype=torch.float32, device="cuda")
    net.freeze().predict_into(torch.from_numpy(qt).float().cuda().contiguous(), g,
                              torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    ref = grad(qt)
    rel = np.linalg.norm(h(g) - ref) / np.linalg.norm(ref)
    gq = torch.zeros((d, 512), dtype=torch.float32, device="cuda")
    net.predict_into(torch.from_numpy(Q[:, :512].copy()).float().cuda(), gq, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    rel_train = np.linalg.norm(h(gq) - grad(Q[:, :512])) / np.linalg.norm(grad(Q[:, :512]))
    print(f"training-point relative error {rel_train:.3f}")
    # linear least-squares fit on the same training pairs, for comparison
    A = np.c_[Q.T, np.ones(Q.shape[1])]
    coef, *_ = np.linalg.lstsq(A, grad(Q).T, rcond=None)
    lin = np.linalg.norm((np.c_[qt.T, np.ones(512)] @ coef).T - ref) / np.linalg.norm(ref)
    print(f"surrogate held-out relative error {rel:.3f} (linear fit {lin:.3f}), "
          f"loss {hist[0][1]:.3e} -> {hist[-1][1]:.3e}")
    assert rel < 0.08 and rel < 0.4 * lin
