"""Persistent fused proposals (one launch per block of proposals, one warp
per chain) against the launch-per-step path on the same inputs and the same
Philox draws: FP64 chains to 1e-12, FP32 chains to 1e-5 relative with equal
accept decisions, for every prior kind, unit and diagonal mass, and the
leapfrog and 3-stage integrators."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _problem(d, prior, seed):
    import hmclab_gb300 as H

    rng = np.random.default_rng(seed)
    n = 2 * d
    G = rng.normal(size=(n, d)) / np.sqrt(d)
    m = rng.normal(size=(d, 1))
    dat = G @ m + 0.1 * rng.normal(size=(n, 1))
    lik = H.Distributions.LinearMatrix(G, dat, 0.01, dtype=np.float64)
    if prior == "none":
        post = lik
    elif prior == "normal":
        post = H.Distributions.BayesRule([H.Distributions.Normal(np.zeros((d, 1)), np.full((d, 1), 2.0)), lik])
    else:
        post = H.Distributions.BayesRule([H.Distributions.Laplace(np.zeros((d, 1)), np.ones((d, 1))), lik])
    w = np.sqrt(np.linalg.eigvalsh(G.T @ G / 0.01).max())
    return post, m, 0.5 / w


@pytest.mark.parametrize("d,prior,mass,integrator", [
    (24, "normal", "unit", "lf"), (50, "laplace", "diag", "lf"), (97, "none", "diag", "3s"), (128, "normal", "unit", "4s"),
    (40, "normal", "full", "lf"), (80, "laplace", "full", "3s"),
])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_persistent_matches_launch_per_step(d, prior, mass, integrator, dtype):
    import hmclab_gb300 as H

    post, m, eps = _problem(d, prior, seed=d)
    C, P = 96, 7
    rng = np.random.default_rng(1)
    q0 = m + 0.02 * rng.normal(size=(d, C))
    if mass == "unit":
        mm = None
    elif mass == "diag":
        mm = H.MassMatrices.Diagonal(rng.uniform(0.5, 2.0, size=(d, 1)))
    else:
        A = rng.normal(size=(d, d)) / np.sqrt(d)
        mm = H.MassMatrices.Full(A @ A.T + np.eye(d))
    runs = []
    for persistent in (True, False):
        smp = H.Samplers.HMC(seed=11).sample(
            None, post, stepsize=eps, amount_of_steps=6, initial_model=q0, proposals=P, chains=C, dtype=dtype,
            mass_matrix=mm, integrator=integrator, keep_samples=True, proposals_per_graph=4, persistent=persistent)
        assert (smp._persistent is not None) == persistent
        runs.append(smp)
    a, b = (r.samples_numpy() for r in runs)  # C, d+1, N
    differ = np.sum(np.asarray(runs[0].accepted_proposals) != np.asarray(runs[1].accepted_proposals))
    # FP64: identical decisions; FP32 (the other path may use the tensor-core
    # step for d >= 64): at most one chain on a decision within rounding of u
    assert differ == 0 if dtype == "float64" else differ <= 1
    acc = np.mean(runs[0].accepted_proposals) / P
    assert 0.1 < acc <= 1.0, acc
    # FP32 at d >= 64: the launch-per-step path contracts on the tensor cores
    # (BF16 hi/lo products, ~1e-6 per gradient), and 42 kicks compound it
    tol = 1e-12 if dtype == "float64" else (1e-5 if d < 64 else 5e-5)
    same = np.asarray(runs[0].accepted_proposals) == np.asarray(runs[1].accepted_proposals)
    err = np.abs(a - b) / np.abs(b).max(axis=(0, 2), keepdims=True)
    if dtype == "float32":
        err = err[same]
    assert np.max(err) < tol, np.max(err)
    assert runs[0].kernel_launches < runs[1].kernel_launches / 5


def test_persistent_counts_proposals_and_thins():
    """The proposal counter advances by the block, so the draws of the next
    block differ; thinned records land in the same slots as the
    launch-per-step path's."""
    import hmclab_gb300 as H

    post, m, eps = _problem(32, "normal", seed=3)
    rng = np.random.default_rng(2)
    q0 = m + 0.02 * rng.normal(size=(32, 64))
    out = []
    for persistent in (True, False):
        smp = H.Samplers.HMC(seed=5).sample(None, post, stepsize=eps, amount_of_steps=4, initial_model=q0,
                                            proposals=24, online_thinning=3, chains=64, dtype="float64",
                                            keep_samples=True, proposals_per_graph=6, persistent=persistent)
        out.append(smp.samples_numpy())
        assert int(smp.control.cpu()[0]) == 24
    assert out[0].shape == (64, 33, 8)
    assert np.max(np.abs(out[0] - out[1])) < 1e-10
    assert not np.allclose(out[0][:, :-1, 0], out[0][:, :-1, -1])


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_targets_of_uneven_dimension_in_one_launch(dtype):
    """Three posteriors (d = 20, 50, 97; 64, 33 and 128 chains) advanced
    together, one launch per block of proposals, give the chains each one
    gives alone."""
    import hmclab_gb300 as H

    specs = [(20, 64, 1), (50, 33, 2), (97, 128, 3)]

    def prepared(d, C, seed):
        post, m, eps = _problem(d, "normal", seed=seed)
        q0 = m + 0.02 * np.random.default_rng(seed).normal(size=(d, C))
        return H.Samplers.HMC(seed=seed).prepare(None, post, stepsize=eps, amount_of_steps=5, initial_model=q0,
                                                 proposals=12, chains=C, dtype=dtype, keep_samples=True,
                                                 proposals_per_graph=6)

    alone = []
    for d, C, seed in specs:
        smp = prepared(d, C, seed)
        smp.run(12)
        smp.finish()
        alone.append(smp.samples_numpy())
    group = [prepared(d, C, seed) for d, C, seed in specs]
    H.Samplers.run_together(group, 12)
    for smp, ref in zip(group, alone):
        smp.finish()
        assert smp.current_proposal == 11
        got = smp.samples_numpy()
        assert got.shape == ref.shape
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-13 * np.abs(ref).max())
