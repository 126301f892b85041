"""Surrogate-driven HMC through Samplers.HMC: the recorded burn-in pairs are
exact gradients, a frozen surrogate (even a wrong one) leaves the exact
posterior invariant, and on a small elastic FWI posterior the trained network
makes proposals much cheaper at a comparable acceptance rate."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def linear_problem(d=32, n=64, seed=0):
    import hmclab_gb300 as H
    from hmclab_gb300 import problems

    G, dat, _ = problems.dense_linear(n, d, 1.0 / np.sqrt(d), 0.2, seed)
    prior = H.Distributions.Normal(np.zeros((d, 1)), np.ones((d, 1)))
    lik = H.Distributions.LinearMatrix(G, dat, 0.04)
    post = H.Distributions.BayesRule([prior, lik])
    mean, cov = problems.gaussian_posterior(G, dat, 0.04, 0.0, 1.0)
    return post, mean, cov


def test_training_set_records_exact_gradients():
    import hmclab_gb300 as H
    from hmclab_gb300 import surrogate as S

    post, mean, cov = linear_problem()
    d, C, L, P = 32, 128, 5, 3
    data = S.TrainingSet(d, P * L * C)
    q0 = mean + np.linalg.cholesky(cov) @ np.random.default_rng(1).normal(size=(d, C))
    smp = H.Samplers.HMC(seed=3).sample(None, post, stepsize=0.1, amount_of_steps=L, initial_model=q0, proposals=P,
                                        chains=C, dtype="float32", training_set=data)
    assert not smp.use_graph  # recording runs uncaptured
    assert data.count == P * L * C
    q = data.q[: data.count].t().contiguous()
    g_ref = post.gradient_batch(q)
    err = (data.g[: data.count].t() - g_ref).abs().max().item()
    assert err <= 1e-5 * g_ref.abs().max().item(), err
    # positions differ between records (they follow the trajectories)
    assert torch.unique(data.q[: data.count, 0]).numel() > data.count // 2


def test_wrong_surrogate_keeps_the_exact_posterior():
    """A surrogate fitted to 1.3x the true gradient drives the trajectories;
    the exact misfit in the accept test keeps chains that start at exact
    posterior draws distributed as the posterior.  (A chain accepting with
    the surrogate's own energy would shrink the variance towards 1/1.3.)"""
    import hmclab_gb300 as H
    from hmclab_gb300 import surrogate as S

    post, mean, cov = linear_problem()
    d, C = 32, 4096
    rng = np.random.default_rng(2)
    Lc = np.linalg.cholesky(cov)
    # training pairs on posterior-like positions, targets 1.3 x the gradient
    data = S.TrainingSet(d, 8192)
    for _ in range(8):
        qb = torch.from_numpy(mean + 1.5 * Lc @ rng.normal(size=(d, 1024))).float().cuda().contiguous()
        data.record(qb, 1.3 * post.gradient_batch(qb), torch.cuda.current_stream().cuda_stream)
    net = S.MLPSurrogate(d, hidden=(64, 64), seed=0)
    net.fit(data, steps=300, batch=256, lr=1e-3)
    net.freeze()
    w = np.sqrt(np.linalg.eigvalsh(np.linalg.inv(cov)).max())
    q0 = mean + Lc @ rng.normal(size=(d, C))
    smp = H.Samplers.HMC(seed=4).sample(None, post, stepsize=0.5 / w, amount_of_steps=8, initial_model=q0,
                                        proposals=30, chains=C, dtype="float32", surrogate=net)
    acc = np.mean(smp.accepted_proposals) / 30
    assert 0.05 < acc < 0.95, acc
    q = smp.current_model  # d x C, each column a posterior draw after 30 proposals
    sd = np.sqrt(np.diag(cov))
    z_mean = np.abs(q.mean(axis=1) - mean[:, 0]) / (sd / np.sqrt(C))
    var_ratio = q.var(axis=1) / np.diag(cov)
    print(f"acceptance {acc:.3f}; max |mean error| {z_mean.max():.2f} standard errors; variance ratio "
          f"{var_ratio.min():.3f}..{var_ratio.max():.3f}")
    assert z_mean.max() < 5.0
    assert np.all(np.abs(var_ratio - 1.0) < 5.0 * np.sqrt(2.0 / C))


def test_surrogate_cheapens_small_fwi_proposals():
    """Small elastic FWI (56x40 simulation grid, 300 steps, 2 shots, 45 blob
    parameters, 2% prior): the surrogate trained on exact burn-in pairs cuts
    the device time of a proposal by > 3x and keeps the acceptance rate
    within a factor 2 of plain HMC at the same step size and length."""
    import hmclab_gb300 as H
    from hmclab_gb300 import fwi as FW
    from hmclab_gb300 import problems
    from hmclab_gb300 import surrogate as S

    cfg = FW.ElasticConfig(nx=40, nz=24, pad=8, h=5.0, dt=5e-4, nt=300, f0=25.0, sponge=0.05,
                           src_x=(60.0, 140.0), src_z=20.0, rec_x=np.linspace(15.0, 185.0, 9), rec_z=20.0)
    pb = problems.elastic_fwi(cfg, 5, 3, prior_fraction=0.02, noise_fraction=0.5, seed=1)
    post, d, C, L = pb["posterior"], 45, 64, 10
    mass = H.MassMatrices.Diagonal(1.0 / pb["prior_std"] ** 2)
    rng = np.random.default_rng(5)
    # largest curvature of the prior-whitened posterior at the true model
    # (power iteration on central differences of the gradient) sets the step
    s = torch.from_numpy(pb["prior_std"]).float().cuda()[:, None]
    m0 = torch.from_numpy(pb["m_true"]).float().cuda()[:, None]
    v = torch.randn(d, 1, device="cuda")
    for _ in range(15):
        v = v / v.norm()
        hv = s * (post.gradient_batch((m0 + 1e-2 * s * v).contiguous())
                  - post.gradient_batch((m0 - 1e-2 * s * v).contiguous())) / 2e-2
        lam = float((v * hv).sum())
        v = hv
    eps = 0.8 / np.sqrt(max(lam, 1.0))
    q0 = pb["m_true"][:, None] + 0.2 * pb["prior_std"][:, None] * rng.normal(size=(d, C))
    kw = dict(stepsize=eps, amount_of_steps=L, mass_matrix=mass, chains=C, dtype="float32")
    data = S.TrainingSet(d, 8 * L * C)
    burn = H.Samplers.HMC(seed=6).sample(None, post, initial_model=q0, proposals=8, training_set=data, **kw)
    net = S.MLPSurrogate(d, hidden=(128, 128), seed=0)
    fit = net.fit(data, steps=1500, batch=256, lr=1e-3)
    net.freeze()

    def timed(surrogate, n=10):
        smp = H.Samplers.HMC(seed=7).prepare(None, post, initial_model=burn.current_model, proposals=n,
                                            surrogate=surrogate, **kw)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(smp.stream)
        smp.run(n)
        ev1.record(smp.stream)
        smp.finish()
        return ev0.elapsed_time(ev1) / n, np.mean(smp.accepted_proposals) / n

    t_plain, acc_plain = timed(None)
    t_sur, acc_sur = timed(net)
    print(f"largest whitened curvature {lam:.1f}, stepsize {eps:.4f}; "
          f"held-out gradient error {fit['best_heldout']:.4f}; plain {t_plain:.2f} ms/proposal, acceptance "
          f"{acc_plain:.2f}; surrogate {t_sur:.2f} ms/proposal, acceptance {acc_sur:.2f}")
    assert fit["best_heldout"] < 0.05
    assert t_sur < t_plain / 3.0
    assert acc_sur > 0.5 * acc_plain


def test_refresh_appends_exact_pairs_and_retrains_between_blocks():
    """refresh_interval: after every block the exact gradient and misfit at
    each chain's position join the training set (checked against the
    target), the potential trains further with its values matched, and the
    chains stay on the exact posterior."""
    import hmclab_gb300 as H
    from hmclab_gb300 import surrogate as S

    post, mean, cov = linear_problem()
    d, C, L = 32, 512, 5
    rng = np.random.default_rng(7)
    Lc = np.linalg.cholesky(cov)
    q0 = mean + Lc @ rng.normal(size=(d, C))
    data = S.TrainingSet(d, 3 * L * C + 3 * C, values=True)
    kw = dict(stepsize=0.1, amount_of_steps=L, chains=C, dtype="float32")
    burn = H.Samplers.HMC(seed=1).sample(None, post, initial_model=q0, proposals=3, training_set=data, **kw)
    n0 = data.count
    assert n0 == 3 * L * C and torch.isfinite(data.x[:n0]).all()
    x_ref = post.misfit_batch(data.q[:n0].t().contiguous())
    assert torch.allclose(data.x[:n0], x_ref, rtol=1e-5)
    net = S.PotentialSurrogate(d, hidden=(64, 64), seed=0)
    net.value_weight = 1.0
    net.fit(data, steps=400, batch=256)
    steps0 = net.steps
    smp = H.Samplers.HMC(seed=2).sample(None, post, initial_model=burn.current_model, proposals=40,
                                        surrogate=net.freeze(), training_set=data, refresh_interval=10,
                                        refresh_steps=50, keep_samples=True, **kw)
    assert smp.refreshes == 3  # after proposals 10, 20, 30 (not after the last)
    assert data.count == n0 + 3 * C and net.steps == steps0 + 150 and net.frozen
    g_ref = post.gradient_batch(data.q[n0:data.count].t().contiguous())
    err = (data.g[n0:data.count].t() - g_ref).abs().max().item()
    assert err <= 1e-5 * g_ref.abs().max().item()
    assert net._vt.numel() == data.count
    q = smp.samples_numpy()[:, :-1, :]  # C, d, N
    z = (q[:, :, -1].mean(axis=0) - mean[:, 0]) / (np.sqrt(np.diag(cov)) / np.sqrt(C))
    assert np.abs(z).max() < 5.0
    assert 0.2 < np.mean(np.atleast_1d(smp.accepted_proposals)) / 40
