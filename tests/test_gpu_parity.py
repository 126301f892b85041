"""GPU parity tests: the CUDA path (through the C ABI) against the reference's
own outputs (golden fixtures) and the CPU oracle, on the same inputs and the
same injected random streams.

Tolerances (stated per test): FP64 path 1e-12 relative (misfits of the
premultiplied dense form are compared relative to the magnitude of the terms
that cancel in them); FP32 path 1e-5 relative against FP64 references.
Accept decisions must agree except where |dH - log u| < 1e-9."""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

torch = pytest.importorskip("torch")

import hmclab_gb300 as H  # noqa: E402
from hmclab_gb300 import _lib  # noqa: E402
from oracle import hmc_oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-12
FP32_RTOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.load()


def dev(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to("cuda", dtype)


# ---------------------------------------------------------------------------
def test_philox_known_answers_on_device():
    out = torch.zeros(4, dtype=torch.int32, device="cuda")
    for ctr, key, expect in O.PHILOX_KAT:
        _lib.call("hmc_philox_raw", 1, *ctr, *key, out.data_ptr(), None)
        got = tuple(int(x) & 0xFFFFFFFF for x in out.cpu().numpy())
        assert got == expect


def test_philox_normals_match_oracle_and_moments():
    rows, C = 37, 129
    for dtype, oracle_fn, tol in (
        (torch.float64, O.philox_normal_f64, 1e-12),
        (torch.float32, O.philox_normal_f32, 2e-5),
    ):
        out = torch.empty((rows, C), dtype=dtype, device="cuda")
        code = _lib.HMC_F64 if dtype == torch.float64 else _lib.HMC_F32
        _lib.call("hmc_philox_normal", code, rows, C, 12345, 7, 0, out.data_ptr(), None)
        ref = oracle_fn(12345, rows, C, 7)
        np.testing.assert_allclose(out.double().cpu().numpy(), ref, rtol=tol, atol=tol)
    big = torch.empty((1000, 4096), dtype=torch.float32, device="cuda")
    _lib.call("hmc_philox_normal", _lib.HMC_F32, 1000, 4096, 99, 3, 0, big.data_ptr(), None)
    x = big.double().cpu().numpy()
    assert abs(x.mean()) < 5e-3 and abs(x.std() - 1) < 5e-3


# ---------------------------------------------------------------------------
def _posteriors(golden):
    """(name, hmclab_gb300 posterior, golden) for every fixture with probes."""
    out = []
    g = golden("cfg1_dense_lf.npz")
    lik = H.Distributions.LinearMatrix(g["G"], g["d"], 0.01, dtype=np.float64)
    out.append(("cfg1", H.Distributions.BayesRule([H.Distributions.Normal(np.zeros((50, 1)), np.ones((50, 1))), lik]), g))
    for prior in ("normal", "laplace"):
        g = golden(f"cfg2_small_{prior}.npz")
        d = g["G"].shape[1]
        lik = H.Distributions.LinearMatrix(g["G"], g["d"], 0.0025, dtype=np.float64)
        pr = (
            H.Distributions.Normal(np.zeros((d, 1)), np.ones((d, 1)))
            if prior == "normal"
            else H.Distributions.Laplace(np.zeros((d, 1)), np.ones((d, 1)))
        )
        out.append((f"cfg2_{prior}", H.Distributions.BayesRule([pr, lik]), g))
    g = golden("tomo_small.npz")
    G = sp.csr_matrix((g["data"], g["indices"], g["indptr"]), shape=tuple(g["shape"]))
    n = G.shape[1]
    post = H.Distributions.BayesRule(
        [H.Distributions.Normal(g["background"], np.full((n, 1), 0.05**2)), H.Distributions.LinearMatrix(G, g["d"], 1e-4)]
    )
    out.append(("tomo", post, g))
    g = golden("srcloc_small.npz")
    out.append(("srcloc", H.Distributions.SourceLocation3D(g["rx"], g["ry"], g["rz"], g["obs"], g["std"]), g))
    g = golden("fullmass_bounds.npz")
    post = H.Distributions.BayesRule(
        [
            H.Distributions.Normal(g["mean"], g["cov"], lower_bounds=g["lower"], upper_bounds=g["upper"]),
            H.Distributions.Laplace(g["mean"], np.full((6, 1), 2.0)),
        ]
    )
    out.append(("fullmass", post, g))
    return out


def _misfit_tolerance(post, M):
    """Premultiplied dense misfits cancel terms of size |m^T GtG m|; compare
    relative to that magnitude (and to the misfit itself elsewhere)."""
    for part in getattr(post, "separate_distributions", [post]):
        if isinstance(part, H.Distributions.LinearMatrix) and part.premultiplication:
            return np.abs(np.sum(M * (part.GtG @ M), axis=0)) + np.abs(part.dtd)
    return None


def test_misfit_and_gradient_fp64_match_reference(golden):
    for name, post, g in _posteriors(golden):
        M = g["probe_m"]
        x = post.misfit_batch(dev(M)).cpu().numpy()
        scale = _misfit_tolerance(post, M)
        if scale is None:
            np.testing.assert_allclose(x, g["probe_misfit"], rtol=FP64_RTOL, err_msg=name)
        else:
            assert np.all(np.abs(x - g["probe_misfit"]) <= FP64_RTOL * scale), name
        gr = post.gradient_batch(dev(M)).cpu().numpy()
        gscale = np.abs(g["probe_grad"]).max()
        np.testing.assert_allclose(gr, g["probe_grad"], rtol=FP64_RTOL, atol=FP64_RTOL * gscale, err_msg=name)
        # single-vector reference API
        x0 = post.misfit(M[:, :1])
        assert abs(x0 - g["probe_misfit"][0]) <= FP64_RTOL * (scale[0] if scale is not None else abs(x0)), name
        np.testing.assert_allclose(post.gradient(M[:, :1])[:, 0], g["probe_grad"][:, 0], rtol=FP64_RTOL,
                                   atol=FP64_RTOL * gscale, err_msg=name)


def test_misfit_and_gradient_fp32_within_1e5(golden):
    """FP32 kernels against the reference's FP64 values: 1e-5 relative."""
    for name, post, g in _posteriors(golden):
        M = g["probe_m"]
        x = post.misfit_batch(dev(M, torch.float32)).cpu().numpy()
        np.testing.assert_allclose(x, g["probe_misfit"], rtol=FP32_RTOL, err_msg=name)
        gr = post.gradient_batch(dev(M, torch.float32)).double().cpu().numpy()
        gscale = np.abs(g["probe_grad"]).max()
        np.testing.assert_allclose(gr, g["probe_grad"], rtol=FP32_RTOL, atol=FP32_RTOL * gscale, err_msg=name)


# ---------------------------------------------------------------------------
def test_first_trajectory_fp64_step_by_step(golden):
    """cfg1: positions and gradients of every leapfrog step of the first
    trajectory, through hmc_begin_trajectory / hmc_kick_drift."""
    g = golden("cfg1_dense_lf.npz")
    post = _posteriors(golden)[0][1]
    smp = H.Samplers.HMC(seed=0)
    smp._parse(None, post, 0.01, True, 10, None, "lf", g["q0"], 1, 1, False, False, None, False, 0.65, 0.75, 1,
               "float64", (g["z"], g["f"][:, None], g["u"][:, None]), False, None, False)
    smp._setup_device()
    h = smp.stream.cuda_stream
    smp._load_streams(0, 1)
    first, steps = smp._schedule
    _lib.call("hmc_begin_trajectory", smp._state_ref, first, h)
    for k, (needs, kick, drift) in enumerate(steps):
        post._device_gradient(smp.q, smp.g, False, "float64", h)
        smp.stream.synchronize()
        q = smp.q.cpu().numpy()[:, 0]
        gr = smp.g.cpu().numpy()[:, 0]
        np.testing.assert_allclose(q, g["traj_q"][k], rtol=FP64_RTOL, atol=FP64_RTOL)
        np.testing.assert_allclose(gr, g["traj_g"][k], rtol=1e-11, atol=1e-12 * np.abs(g["traj_g"][k]).max())
        _lib.call("hmc_kick_drift", smp._state_ref, kick, drift, h)


def _accept_ties(H0, H1, u):
    return np.abs((H0 - H1) - np.log(u)) < 1e-9


def _run_case(post, g, mass, dtype="float64", graph=True, **kw):
    z, f, u = g["z"], g["f"], g["u"]
    C = g["q0"].shape[1]
    if z.ndim == 2:
        z, f, u = z[..., None], f[:, None], u[:, None]
    P = kw.pop("P", None) or g["samples"].shape[1]
    smp = H.Samplers.HMC(seed=0)
    smp.sample(None, post, stepsize=float(g["stepsize"]), amount_of_steps=int(g["amount_of_steps"]),
               mass_matrix=mass, initial_model=g["q0"], proposals=P, chains=C, dtype=dtype,
               rng_streams=(z, f, u), graph=graph, keep_samples=True, proposals_per_graph=10 if P % 10 == 0 else P,
               **kw)
    return smp


CASES = ["cfg1", "cfg2_normal", "cfg2_laplace", "tomo", "srcloc", "fullmass"]


@pytest.mark.parametrize("case", CASES)
def test_sampler_fp64_matches_reference_chains(golden, case):
    """Whole chains: samples (d+1, N) per chain and accepted counts equal the
    reference's HMC(seed) output to 1e-12 under the same random streams."""
    name, post, g = [c for c in _posteriors(golden) if c[0] == case][0]
    mass = None
    kw = {}
    if case.startswith("cfg2"):
        mass = H.MassMatrices.Diagonal(g["diag"])
    if case == "fullmass":
        mass = H.MassMatrices.Full(g["mass"])
        kw["randomize_stepsize"] = False
    smp = _run_case(post, g, mass, **kw)
    got = smp.samples_numpy()  # C, d+1, N
    ref = np.moveaxis(g["samples"], -1, 0)
    scale = np.abs(ref).max()
    np.testing.assert_allclose(got[:, :-1], ref[:, :-1], rtol=FP64_RTOL * 10, atol=FP64_RTOL * 10 * scale)
    np.testing.assert_allclose(got[:, -1], ref[:, -1], rtol=1e-9)
    acc = np.atleast_1d(smp.accepted_proposals)
    assert np.array_equal(acc, g["accepted"]), (acc, g["accepted"])


def test_graph_and_direct_launches_agree(golden):
    name, post, g = _posteriors(golden)[1]
    mass = H.MassMatrices.Diagonal(g["diag"])
    a = _run_case(post, g, mass, graph=True).samples_numpy()
    b = _run_case(post, g, mass, graph=False).samples_numpy()
    assert np.array_equal(a, b)


def test_integrators_and_autotune_match_reference(golden):
    g = golden("integrators_autotune.npz")
    post = H.Distributions.Normal(g["mean"], g["var"])
    for integ in ("3s", "4s"):
        smp = H.Samplers.HMC(seed=0).sample(
            None, post, stepsize=0.4, amount_of_steps=4, integrator=integ, initial_model=g["q0"], proposals=50,
            rng_streams=(g["z"][..., None], g["f"][:, None], g["u"][:, None]), keep_samples=True,
            proposals_per_graph=10,
        )
        np.testing.assert_allclose(smp.samples_numpy(0), g[f"samples_{integ}"][..., 0], rtol=1e-12, atol=1e-12)
        assert smp.accepted_proposals == g[f"accepted_{integ}"][0]
    smp = H.Samplers.HMC(seed=0).sample(
        None, post, stepsize=1.5, amount_of_steps=3, initial_model=g["q0"], proposals=60, autotuning=True,
        online_thinning=3, target_acceptance_rate=0.7, learning_rate=0.6,
        rng_streams=(g["za"][..., None], g["fa"][:, None], g["ua"][:, None]), keep_samples=True, proposals_per_graph=12,
    )
    np.testing.assert_allclose(smp.samples_numpy(0), g["samples_auto"][..., 0], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(smp.stepsizes[:, 0], g["auto_stepsizes"], rtol=1e-13)
    # acceptance rates are exp(dH): compare dH itself (absolute 1e-9, the
    # accept-decision tolerance), since tiny rates amplify dH round-off.
    np.testing.assert_allclose(np.log(smp.acceptance_rates[1:, 0]), np.log(g["auto_rates"][1:]), rtol=0, atol=1e-9)
    np.testing.assert_allclose(smp.stepsize, g["auto_final_stepsize"], rtol=1e-13)


def test_fp32_chains_track_fp64_oracle(golden):
    """cfg2-small in FP32: trajectories agree with the FP64 oracle to 1e-5
    relative while accept decisions agree (ties |dH - log u| < 1e-9 excepted)."""
    g = golden("cfg2_small_normal.npz")
    name, post, _ = _posteriors(golden)[1]
    mass = H.MassMatrices.Diagonal(g["diag"])
    P = 8
    smp = _run_case(post, g, mass, dtype="float32", P=P)
    lik = O.DensePremul(g["G"], g["d"], 0.0025)
    opost = O.Sum([O.NormalDiag(np.zeros(120), np.ones(120)), lik])
    res = O.run_chains(opost, O.Mass("diag", diag=g["diag"]), g["q0"], float(g["stepsize"]), (g["z"], g["f"], g["u"]),
                       P, amount_of_steps=20)
    got = smp.samples_numpy()[:, :-1]  # C, d, N
    ref = np.transpose(res["samples"][:, :-1], (2, 1, 0))
    # until the first accept-decision difference both chains are the same
    ties = _accept_ties(res["H0"], res["H1"], g["u"][:P])
    assert not ties.any()
    np.testing.assert_allclose(got, ref, rtol=FP32_RTOL, atol=FP32_RTOL * np.abs(ref).max())


def test_philox_mode_targets_the_analytic_posterior(golden):
    """cfg1 with device Philox streams: posterior mean and std of 4096 short
    chains agree with the analytic Gaussian posterior."""
    g = golden("cfg1_dense_lf.npz")
    post = _posteriors(golden)[0][1]
    C = 2048
    smp = H.Samplers.HMC(seed=11).sample(
        None, post, stepsize=0.01, amount_of_steps=10, initial_model=g["post_mean"], proposals=60, chains=C,
        dtype="float64", keep_samples=True, proposals_per_graph=20,
    )
    s = smp.samples_numpy()[:, :-1, 20:]  # C, d, N
    x = s.transpose(1, 0, 2).reshape(50, -1)
    mean, std = x.mean(axis=1), x.std(axis=1)
    ref_std = np.sqrt(np.diag(g["post_cov"]))
    assert np.max(np.abs(mean - g["post_mean"][:, 0]) / ref_std) < 0.1
    assert np.max(np.abs(std / ref_std - 1)) < 0.1
    assert 0.2 < np.mean(np.atleast_1d(smp.accepted_proposals)) / 60 < 1.0


def test_split_k_product_matches_numpy_and_is_deterministic():
    """hmc_gemm_splitk (the FWI grid-to-blob projection shape: m=200, n=64,
    k=33600) against numpy in FP64 to 1e-12 and FP32 to 1e-5 of sum |a||b|;
    two launches give bit-identical results; accumulate adds to out."""
    rng = np.random.default_rng(11)
    m, n, k = 200, 64, 33600
    A = rng.normal(size=(m, k))
    B = rng.normal(size=(k, n))
    ref = A @ B
    scale = np.abs(A) @ np.abs(B)
    h = torch.cuda.current_stream().cuda_stream
    for dt, code, tol in ((torch.float64, _lib.HMC_F64, 1e-12), (torch.float32, _lib.HMC_F32, 1e-5)):
        a, b = dev(A, dt), dev(B, dt)
        work = torch.empty(64 * m * n, dtype=dt, device="cuda")
        outs = []
        for _ in range(2):
            out = torch.zeros((m, n), dtype=dt, device="cuda")
            _lib.call("hmc_gemm_splitk", code, m, n, k, 0.5, a.data_ptr(), b.data_ptr(), out.data_ptr(), 0,
                      work.data_ptr(), work.numel(), h)
            outs.append(out.clone())
        got = outs[0].double().cpu().numpy()
        assert np.all(np.abs(got - 0.5 * ref) <= tol * 0.5 * scale)
        assert torch.equal(outs[0], outs[1])
        _lib.call("hmc_gemm_splitk", code, m, n, k, 1.0, a.data_ptr(), b.data_ptr(), out.data_ptr(), 1,
                  work.data_ptr(), m * n * 3, h)  # three splits at most, accumulated onto 0.5 A B
        got = out.double().cpu().numpy()
        assert np.all(np.abs(got - 1.5 * ref) <= tol * 1.5 * scale)
    with pytest.raises(ValueError):
        _lib.call("hmc_gemm_splitk", _lib.HMC_F32, m, n, k, 1.0, a.data_ptr(), b.data_ptr(), out.data_ptr(), 0,
                  work.data_ptr(), m * n - 1, h)
