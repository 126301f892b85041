"""Effective sample size: the oracle against the analytic AR(1) value (CPU),
and the device kernel against the oracle (GPU)."""
import numpy as np
import pytest

from oracle import hmc_oracle as O


def ar1(N, d, C, phi, seed=0):
    rng = np.random.default_rng(seed)
    phi = np.asarray(phi, float)[:, None]
    x = np.zeros((N, d, C))
    x[0] = rng.normal(size=(d, C)) / np.sqrt(1 - phi**2)
    for t in range(1, N):
        x[t] = phi * x[t - 1] + rng.normal(size=(d, C))
    return x


def test_oracle_ess_matches_ar1_theory():
    phi = [0.0, 0.5, 0.8]
    x = ar1(400, 3, 64, phi)
    e, rhat = O.ess_split(x, 100)
    ref = O.ar1_ess(np.array(phi), 400 * 64)
    np.testing.assert_allclose(np.abs(e), ref, rtol=0.15)
    assert np.all(np.abs(rhat - 1) < 0.06)


def test_oracle_ess_detects_unmixed_chains():
    x = ar1(200, 1, 8, [0.5])
    x[:, :, :4] += 10.0  # half the chains in another mode
    e, rhat = O.ess_split(x, 50)
    assert rhat[0] > 1.5 and np.abs(e[0]) < 0.05 * 200 * 8


@pytest.mark.gpu
def test_device_ess_and_moments_match_oracle():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from hmclab_gb300 import diagnostics

    x = ar1(300, 5, 96, [0.0, 0.3, 0.6, 0.9, -0.4], seed=3)
    # the kernel stages draws in FP32 shared memory: 1e-6 relative for FP64 input
    for dtype, tol in ((torch.float64, 1e-6), (torch.float32, 1e-4)):
        t = torch.from_numpy(x).to("cuda", dtype)
        e, rh = diagnostics.ess(t, lags=80, return_rhat=True)
        xr = t.double().cpu().numpy()
        e_ref, rh_ref = O.ess_split(xr, 80)
        np.testing.assert_allclose(e, e_ref, rtol=tol)
        np.testing.assert_allclose(rh, rh_ref, rtol=tol)
        mean, std = diagnostics.moments(t)
        np.testing.assert_allclose(mean, xr.mean(axis=(0, 2)), rtol=1e-9, atol=1e-12)
        np.testing.assert_allclose(std, xr.std(axis=(0, 2)), rtol=1e-9)


@pytest.mark.gpu
def test_device_ess_of_one_long_chain_matches_oracle():
    """A single chain of 6000 draws (halves longer than the staged path
    holds): the draws are read in place; same estimate as the oracle."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from hmclab_gb300 import diagnostics

    x = ar1(6000, 3, 1, [0.0, 0.5, 0.95], seed=4)
    t = torch.from_numpy(x).to("cuda", torch.float64)
    e = diagnostics.ess(t, lags=300)
    e_ref, _ = O.ess_split(t.double().cpu().numpy(), 300)
    np.testing.assert_allclose(e, e_ref, rtol=1e-6)


def test_oracle_rank_normalised_ess():
    """Rank-normalised bulk-ESS: close to the plain estimate for Gaussian
    AR(1) chains, unchanged by a monotone transformation of the draws, and
    finite for heavy-tailed draws whose variance does not exist."""
    phi = [0.0, 0.5, 0.8]
    x = ar1(400, 3, 64, phi, seed=5)
    e_plain, _ = O.ess_split(x, 100)
    e_rank, rh = O.ess_split(O.rank_normalize(x), 100)
    np.testing.assert_allclose(np.abs(e_rank), np.abs(e_plain), rtol=0.1)
    assert np.all(np.abs(rh - 1) < 0.06)
    e_mono, _ = O.ess_split(O.rank_normalize(np.exp(3 * x) + x**3), 100)
    np.testing.assert_array_equal(e_mono, e_rank)
    # Cauchy draws: independent, so the bulk-ESS is close to N C
    rng = np.random.default_rng(6)
    c = rng.standard_cauchy(size=(400, 2, 64))
    e_c, _ = O.ess_split(O.rank_normalize(c), 100)
    assert np.all(np.abs(e_c) > 0.8 * 400 * 64)
    # ties get their average rank: a constant parameter maps to z = 0
    z = O.rank_normalize(np.ones((10, 1, 4)))
    np.testing.assert_allclose(z, 0.0, atol=1e-15)


@pytest.mark.gpu
def test_device_rank_normalisation_matches_oracle():
    """Normal scores and rank-normalised ESS / split-R-hat of the device
    against the oracle (FP64 and FP32 draws, with ties), and the invariance
    of the device estimate under a monotone transformation."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from hmclab_gb300 import diagnostics

    x = ar1(300, 4, 96, [0.0, 0.3, 0.6, 0.9], seed=7)
    x[:, 3] = np.round(x[:, 3] * 4) / 4  # many ties
    for dtype in (torch.float64, torch.float32):
        t = torch.from_numpy(x).to("cuda", dtype)
        xr = t.double().cpu().numpy()
        z = diagnostics.rank_normalize(t).cpu().numpy()
        z_ref = O.rank_normalize(xr)
        np.testing.assert_allclose(z, z_ref, rtol=0, atol=1e-12)
        e, rh = diagnostics.ess(t, lags=80, return_rhat=True, rank_normalize=True)
        e_ref, rh_ref = O.ess_split(z_ref, 80)
        np.testing.assert_allclose(e, e_ref, rtol=1e-9)
        np.testing.assert_allclose(rh, rh_ref, rtol=1e-9)
    t = torch.from_numpy(x).to("cuda", torch.float64)
    e1 = diagnostics.ess(t, lags=80, rank_normalize=True)
    e2 = diagnostics.ess(torch.exp(2 * t) + t, lags=80, rank_normalize=True)
    np.testing.assert_array_equal(e1, e2)
