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
