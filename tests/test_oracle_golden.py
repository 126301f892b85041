"""Pins the CPU oracle (oracle/hmc_oracle.py) against the golden fixtures the
reference itself produced (tests/golden/make_golden.py), and Philox against
the Random123 known-answer vectors."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import hmc_oracle as O


def test_philox_known_answers():
    for ctr, key, expect in O.PHILOX_KAT:
        r = O.philox4x32_10(np.array(ctr, np.uint32), np.array(key, np.uint32))
        assert tuple(int(x) for x in r) == expect


def test_reference_streams_replay_numpy_generator():
    z, f, u = O.reference_streams(7, 3, 2)
    rng = np.random.default_rng(7)
    assert np.array_equal(z[0], rng.normal(size=(3, 1))[:, 0])
    assert f[0] == rng.uniform(0.5, 1.5)
    assert u[0] == rng.uniform(0, 1)


def _check_run(g, dist, mass, **kw):
    res = O.run_chains(
        dist,
        mass,
        g["q0"],
        float(g["stepsize"]),
        (g["z"], g["f"], g["u"]),
        g["samples"].shape[1],
        amount_of_steps=int(g["amount_of_steps"]),
        **kw,
    )
    ref = np.moveaxis(g["samples"], 1, 0)  # N, d+1, C
    np.testing.assert_allclose(res["samples"], ref, rtol=1e-9, atol=1e-9)
    assert np.array_equal(res["accepted"], g["accepted"])
    return res


def test_cfg1_dense_fp64(golden):
    g = golden("cfg1_dense_lf.npz")
    lik = O.DensePremul(g["G"], g["d"], 0.01)
    post = O.Sum([O.NormalDiag(np.zeros(50), np.ones(50)), lik])
    np.testing.assert_allclose(post.misfit(g["probe_m"]), g["probe_misfit"], rtol=1e-12)
    np.testing.assert_allclose(post.gradient(g["probe_m"]), g["probe_grad"], rtol=1e-12, atol=1e-9)
    # first trajectory: positions at which the gradient was evaluated
    rec = []
    z = g["z"][0]
    O.trajectory(post, O.Mass("unit"), g["q0"], z, g["f"][0] * 0.01, "lf", 10, record=rec)
    for k, (q, gr) in enumerate(rec):
        np.testing.assert_allclose(q[:, 0], g["traj_q"][k], rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(gr[:, 0], g["traj_g"][k], rtol=1e-11, atol=1e-9)
    _check_run(g, post, O.Mass("unit"))


@pytest.mark.parametrize("prior", ["normal", "laplace"])
def test_cfg2_small(golden, prior):
    g = golden(f"cfg2_small_{prior}.npz")
    d = g["G"].shape[1]
    lik = O.DensePremul(g["G"], g["d"], 0.0025)
    pr = O.NormalDiag(np.zeros(d), np.ones(d)) if prior == "normal" else O.Laplace(np.zeros(d), np.ones(d))
    post = O.Sum([pr, lik])
    np.testing.assert_allclose(post.misfit(g["probe_m"]), g["probe_misfit"], rtol=1e-12)
    np.testing.assert_allclose(post.gradient(g["probe_m"]), g["probe_grad"], rtol=1e-10, atol=1e-8)
    _check_run(g, post, O.Mass("diag", diag=g["diag"]))


def test_public_linearmatrix_quirk(golden):
    """The reference's public LinearMatrix rounds G to FP32 for GtG but uses the
    unrounded G for Gtd0 (LinearMatrix.py:148-177)."""
    g = golden("linearmatrix_public.npz")
    G, dd, var = g["G"], g["d"], float(g["var"])
    G32 = G.astype(np.float32).astype(np.float64)
    d32 = dd.astype(np.float32).astype(np.float64)
    GtG = G32.T @ G32 / var
    Gtd0 = G.T @ d32 / var
    dtd = (d32.T @ d32 / var).item()
    M = g["probe_m"]
    mis = 0.5 * (np.sum(M * (GtG @ M - 2 * Gtd0), axis=0) + dtd)
    np.testing.assert_allclose(mis, g["probe_misfit"], rtol=1e-12)
    np.testing.assert_allclose(GtG @ M - Gtd0, g["probe_grad"], rtol=1e-12, atol=1e-9)


def test_tomography_small(golden):
    g = golden("tomo_small.npz")
    G = sp.csr_matrix((g["data"], g["indices"], g["indptr"]), shape=tuple(g["shape"]))
    n = G.shape[1]
    # reference default dtype: CSR values and data rounded to FP32, FP64 arithmetic
    G32 = sp.csr_matrix((g["data"].astype(np.float32).astype(np.float64), g["indices"], g["indptr"]), shape=G.shape)
    d32 = g["d"].astype(np.float32).astype(np.float64)
    lik = O.SparseLinear(G32, d32, 1e-4)
    post = O.Sum([O.NormalDiag(g["background"], np.full(n, 0.05**2)), lik])
    np.testing.assert_allclose(post.misfit(g["probe_m"]), g["probe_misfit"], rtol=1e-11)
    np.testing.assert_allclose(post.gradient(g["probe_m"]), g["probe_grad"], rtol=1e-9, atol=1e-7)
    _check_run(g, post, O.Mass("unit"))


def test_source_location_small(golden):
    g = golden("srcloc_small.npz")
    dist = O.SourceLocation3D(g["rx"], g["ry"], g["rz"], g["obs"], g["std"], infer_velocity=True)
    np.testing.assert_allclose(dist.misfit(g["probe_m"]), g["probe_misfit"], rtol=1e-12)
    np.testing.assert_allclose(dist.gradient(g["probe_m"]), g["probe_grad"], rtol=1e-10, atol=1e-9)
    fixed = O.SourceLocation3D(g["rx"], g["ry"], g["rz"], g["obs"], g["std"], infer_velocity=False, medium_velocity=5.0)
    np.testing.assert_allclose(fixed.misfit(g["probe_fixed_m"]), g["probe_fixed_misfit"], rtol=1e-12)
    np.testing.assert_allclose(fixed.gradient(g["probe_fixed_m"]), g["probe_fixed_grad"], rtol=1e-10, atol=1e-9)
    _check_run(g, dist, O.Mass("unit"))


def test_full_mass_bounds(golden):
    g = golden("fullmass_bounds.npz")
    post = O.Sum([O.NormalFull(g["mean"], g["cov"]), O.Laplace(g["mean"], np.full(6, 2.0))])
    np.testing.assert_allclose(post.misfit(g["probe_m"]), g["probe_misfit"], rtol=1e-12)
    np.testing.assert_allclose(post.gradient(g["probe_m"]), g["probe_grad"], rtol=1e-12, atol=1e-12)
    _check_run(g, post, O.Mass("full", full=g["mass"]), randomize_stepsize=False, lower=g["lower"], upper=g["upper"])


def test_integrators_and_autotune(golden):
    g = golden("integrators_autotune.npz")
    post = O.NormalDiag(g["mean"], g["var"])
    for integ in ("3s", "4s"):
        res = O.run_chains(post, O.Mass("unit"), g["q0"], 0.4, (g["z"], g["f"], g["u"]), 50, integrator=integ, amount_of_steps=4)
        np.testing.assert_allclose(res["samples"], np.moveaxis(g[f"samples_{integ}"], 1, 0), rtol=1e-12, atol=1e-12)
        assert res["accepted"][0] == g[f"accepted_{integ}"][0]
    res = O.run_chains(
        post, O.Mass("unit"), g["q0"], 1.5, (g["za"], g["fa"], g["ua"]), 60, amount_of_steps=3,
        autotuning=True, online_thinning=3, target_acceptance_rate=0.7, learning_rate=0.6,
    )
    np.testing.assert_allclose(res["samples"], np.moveaxis(g["samples_auto"], 1, 0), rtol=1e-12, atol=1e-12)
    # The reference keeps records[:current_proposal] (Samplers.py:1421-1423), i.e.
    # it drops the last proposal's entry; compare the entries it kept.
    n = len(g["auto_stepsizes"])
    assert n == 59
    np.testing.assert_allclose(res["stepsizes"][:n, 0], g["auto_stepsizes"], rtol=1e-13)
    np.testing.assert_allclose(res["acceptance_rates"][:n, 0], g["auto_rates"], rtol=1e-12)
    np.testing.assert_allclose(res["stepsize"][0], g["auto_final_stepsize"], rtol=1e-13)


def test_oracle_replica_exchange_matches_reference_parallel_sampler(golden):
    """The oracle's parallel-tempering restatement replays the reference's
    own ParallelSampleSMP run (fixture from the reference: schedule, samples
    files, per-chain streams) to 1e-12: same pairing convention, exchange
    after proposals 0, interval, ..., same acceptance, samples recorded after
    the exchange (with the pre-swap misfit the reference keeps)."""
    g = golden("replica_exchange.npz")
    d = g["mean"].shape[0]
    beta = 1.0 / g["temps"]
    C = beta.size
    P = g["z"].shape[0]
    q0 = np.repeat(g["mean"], C, axis=1)
    samples, decisions = O.run_tempered_exchange(
        O.NormalDiag(g["mean"][:, 0], g["var"][:, 0]), beta, O.Mass("unit"), q0, float(g["stepsize"]),
        (g["z"], g["f"], g["u"]), P, int(g["interval"]), g["schedule"], g["exchange_u"],
        amount_of_steps=int(g["amount_of_steps"]))
    ref = np.transpose(g["samples"], (1, 0, 2))  # N, d+1, C
    np.testing.assert_allclose(samples, ref, rtol=1e-12, atol=1e-12)
    assert decisions.any() and not decisions.all()  # the fixture exercises both outcomes
