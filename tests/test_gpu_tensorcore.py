"""Tensor-core (tcgen05) dense contraction: gradient, fused leapfrog step and
residual misfit in FP32 against FP64 references.

Error model: each BF16 hi/lo split product has relative error <= 2^-15
(3.1e-5) of |a||b|; the operands hold q - c (c = least-squares centre), so
the gradient error is bounded by 3.1e-5 * (|GtG| |q - c|) elementwise plus
FP32 accumulation; misfits carry FP64 per-chain sums."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import hmclab_gb300 as H  # noqa: E402
from hmclab_gb300 import _lib  # noqa: E402
from oracle import hmc_oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu
SPLIT_REL = 2.0**-15


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.load()


def problem(n, d, seed=0, noise=0.05):
    rng = np.random.default_rng(seed)
    G = rng.normal(size=(n, d)) / np.sqrt(d)
    m = rng.normal(size=(d, 1))
    dat = G @ m + noise * rng.normal(size=(n, 1))
    return G, dat, m


@pytest.mark.parametrize("n,d,C", [(400, 200, 300), (2000, 1000, 256), (240, 120, 3), (130, 64, 129)])
def test_tc_gradient_and_misfit(n, d, C):
    G, dat, m = problem(n, d, seed=n + d)
    lik = H.Distributions.LinearMatrix(G, dat, 0.05**2)
    assert lik.premultiplication and lik._use_tc("float32", C)
    rng = np.random.default_rng(1)
    ops_probe = m + 0.05 * rng.normal(size=(d, C))
    M32 = torch.from_numpy(ops_probe).to("cuda", torch.float32)
    Mh = M32.double().cpu().numpy()  # the FP32-rounded positions, exactly
    g = lik.gradient_batch(M32)
    x = lik.misfit_batch(M32)
    torch.cuda.synchronize()
    ops = lik._tc_operands(C, M32.device)
    ops.check_status()
    g_ref = lik.GtG @ Mh - lik.Gtd0
    c = ops.center.double().cpu().numpy()[:, None]
    bound = SPLIT_REL * (np.abs(lik.GtG) @ np.abs(Mh - c)) * 1.5 + 1e-5 * np.abs(g_ref).max()
    err = np.abs(g.double().cpu().numpy() - g_ref)
    assert np.all(err <= bound), f"max err {err.max():.3e}, max bound {bound.max():.3e}"
    r = lik.G @ Mh - lik.d
    x_ref = 0.5 * np.sum(r * r * lik.inv_var, axis=0)
    rel = np.abs(x.cpu().numpy() - x_ref) / x_ref
    assert rel.max() < 1e-5, f"misfit relative error {rel.max():.3e}"
    print(f"n={n} d={d} C={C}: gradient max err {err.max():.3e} (max |g| {np.abs(g_ref).max():.2f}), "
          f"misfit rel err {rel.max():.2e}")


def test_fused_step_matches_unfused_reference():
    """One fused kick+drift (gradient + Normal prior in the epilogue) equals
    p -= eps*g, q += eps*M^-1 p computed in FP64 from the same state."""
    n, d, C = 600, 300, 256
    G, dat, m = problem(n, d, seed=5)
    lik = H.Distributions.LinearMatrix(G, dat, 0.05**2)
    prior = H.Distributions.Normal(np.zeros((d, 1)), np.full((d, 1), 2.0))
    post = H.Distributions.BayesRule([prior, lik])
    rng = np.random.default_rng(2)
    diag = rng.uniform(0.5, 2.0, size=(d, 1))
    q0 = m + 0.03 * rng.normal(size=(d, C))
    smp = H.Samplers.HMC(seed=3)
    smp.prepare(None, post, stepsize=0.004, amount_of_steps=1, mass_matrix=H.MassMatrices.Diagonal(diag),
                initial_model=q0, proposals=1, chains=C, dtype="float32", graph=False)
    assert smp._fused is not None
    h = smp.stream.cuda_stream
    _lib.call("hmc_begin_trajectory", smp._state_ref, 0.5, h)
    smp._fused.after_begin(h)
    smp.stream.synchronize()
    q = smp.q.double().cpu().numpy()
    p = smp.p.double().cpu().numpy()
    eps = smp.eps_local.double().cpu().numpy()[None, :]
    smp._fused.kick_drift(1.0, 1.0, h)
    smp.stream.synchronize()
    smp._fused.ops.check_status()
    g = lik.GtG @ q - lik.Gtd0 + 0.5 * q
    p1 = p - eps * g
    q1 = q + eps * (p1 / diag)
    gq = smp.q.double().cpu().numpy()
    gp = smp.p.double().cpu().numpy()
    c = smp._fused.ops.center.double().cpu().numpy()[:, None]
    gbound = SPLIT_REL * (np.abs(lik.GtG) @ np.abs(q - c)) * 1.5 + 1e-5 * np.abs(g).max()
    assert np.all(np.abs(gp - p1) <= eps * gbound + 1e-6 * np.abs(p1).max())
    assert np.all(np.abs(gq - q1) <= eps * eps * gbound / diag + 1e-6 * np.abs(q1).max())
    smp.finish()


def test_fused_sampler_tracks_fp64_oracle(golden):
    """cfg2-small through the fused tensor-core sampler path in FP32 against
    the FP64 oracle under the same random streams."""
    g = golden("cfg2_small_normal.npz")
    d = g["G"].shape[1]
    lik = H.Distributions.LinearMatrix(g["G"], g["d"], 0.0025, dtype=np.float64)
    post = H.Distributions.BayesRule([H.Distributions.Normal(np.zeros((d, 1)), np.ones((d, 1))), lik])
    P = 8
    smp = H.Samplers.HMC(seed=0)
    smp.sample(None, post, stepsize=float(g["stepsize"]), amount_of_steps=20,
               mass_matrix=H.MassMatrices.Diagonal(g["diag"]), initial_model=g["q0"], proposals=P, chains=3,
               dtype="float32", rng_streams=(g["z"], g["f"], g["u"]), keep_samples=True, proposals_per_graph=4,
               persistent=False)
    assert smp._fused is not None
    opost = O.Sum([O.NormalDiag(np.zeros(d), np.ones(d)), O.DensePremul(g["G"], g["d"], 0.0025)])
    res = O.run_chains(opost, O.Mass("diag", diag=g["diag"]), g["q0"], float(g["stepsize"]), (g["z"], g["f"], g["u"]),
                       P, amount_of_steps=20)
    got = smp.samples_numpy()[:, :-1]
    ref = np.transpose(res["samples"][:, :-1], (2, 1, 0))
    assert np.array_equal(np.atleast_1d(smp.accepted_proposals), res["accepted"])
    rel = np.abs(got - ref).max() / np.abs(ref).max()
    print(f"fused FP32 chains vs FP64 oracle: max relative deviation {rel:.2e}")
    assert rel < 1e-5
    xr = np.transpose(res["samples"][:, -1], (1, 0))
    np.testing.assert_allclose(smp.samples_numpy()[:, -1], xr, rtol=1e-5)


def test_persistent_fp32_sampler_tracks_fp64_oracle(golden):
    """The same cfg2-small chains through the persistent kernel (FP32, one
    launch per block of proposals) against the FP64 oracle."""
    g = golden("cfg2_small_normal.npz")
    d = g["G"].shape[1]
    lik = H.Distributions.LinearMatrix(g["G"], g["d"], 0.0025, dtype=np.float64)
    post = H.Distributions.BayesRule([H.Distributions.Normal(np.zeros((d, 1)), np.ones((d, 1))), lik])
    P = 8
    smp = H.Samplers.HMC(seed=0).sample(
        None, post, stepsize=float(g["stepsize"]), amount_of_steps=20, mass_matrix=H.MassMatrices.Diagonal(g["diag"]),
        initial_model=g["q0"], proposals=P, chains=3, dtype="float32", rng_streams=(g["z"], g["f"], g["u"]),
        keep_samples=True, proposals_per_graph=4)
    assert smp._persistent is not None
    opost = O.Sum([O.NormalDiag(np.zeros(d), np.ones(d)), O.DensePremul(g["G"], g["d"], 0.0025)])
    res = O.run_chains(opost, O.Mass("diag", diag=g["diag"]), g["q0"], float(g["stepsize"]), (g["z"], g["f"], g["u"]),
                       P, amount_of_steps=20)
    got = smp.samples_numpy()[:, :-1]
    ref = np.transpose(res["samples"][:, :-1], (2, 1, 0))
    assert np.array_equal(np.atleast_1d(smp.accepted_proposals), res["accepted"])
    rel = np.abs(got - ref).max() / np.abs(ref).max()
    print(f"persistent FP32 chains vs FP64 oracle: max relative deviation {rel:.2e}")
    assert rel < 1e-5


@pytest.mark.parametrize("prior,C", [("normal", 160), ("laplace", 160), ("normal", 162)])
def test_two_pass_step_equals_fused_step_bitwise(prior, C):
    """hmc_tc_step_split (contraction, then a streaming update: 16-byte
    accesses when C is a multiple of 4, scalar otherwise) and the fused
    hmc_tc_step give bitwise-equal chains, bounds reflection included: the
    autotuner may pick either."""
    rng = np.random.default_rng(11)
    n, d = 300, 192
    G = rng.normal(size=(n, d)) / np.sqrt(d)
    dat = G @ rng.normal(size=(d, 1)) + 0.05 * rng.normal(size=(n, 1))
    lik = H.Distributions.LinearMatrix(G, dat, 0.05**2)
    pri = (H.Distributions.Normal(np.zeros((d, 1)), np.ones((d, 1)), lower_bounds=np.full((d, 1), -1.5),
                                  upper_bounds=np.full((d, 1), 1.5)) if prior == "normal"
           else H.Distributions.Laplace(np.zeros((d, 1)), np.ones((d, 1))))
    post = H.Distributions.BayesRule([pri, lik])
    q0 = np.clip(rng.normal(size=(d, C)) * 0.3, -1.4, 1.4)
    runs = []
    for entry in ("hmc_tc_step", "hmc_tc_step_split"):
        smp = H.Samplers.HMC(seed=5)
        smp.prepare(None, post, stepsize=0.05, amount_of_steps=8, initial_model=q0, proposals=6, chains=C,
                    dtype="float32", keep_samples=True, persistent=False, graph=False)
        assert smp._fused is not None
        smp._fused.entry = entry
        smp.run(6)
        smp.finish()
        smp._fused.ops.check_status()
        runs.append((smp.samples_numpy(), np.atleast_1d(smp.accepted_proposals)))
    assert np.array_equal(runs[0][0], runs[1][0])
    assert np.array_equal(runs[0][1], runs[1][1])
