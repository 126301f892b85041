"""Bounded device waits: a wait that runs out is reported on the host as
DeviceTimeoutError, and the CUDA context stays usable.

The failure is made by the library's wait-limit hook (hmc_set_wait_limits):
block 0 of each launch that stages operands through tensor-copy barriers
initialises its barrier but never arms it and issues no copy, so its wait
runs out after the shortened limit (1 ms) with nothing in flight.  Nothing
faults, traps or spins without a bound.  Covered: the tcgen05 contraction
(csrc/dense_tc.cu) and the staged elastic stencils (csrc/fwi.cu)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import hmclab_gb300 as H  # noqa: E402
from hmclab_gb300 import _lib  # noqa: E402
from hmclab_gb300 import fwi as FW  # noqa: E402
from hmclab_gb300.Helpers.CustomExceptions import DeviceTimeoutError  # noqa: E402

pytestmark = pytest.mark.gpu
LIMIT_NS = 1_000_000  # 1 ms


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.load()


def test_tensor_core_wait_runs_out_and_the_context_survives():
    rng = np.random.default_rng(0)
    n, d, C = 300, 128, 256
    G = rng.normal(size=(n, d)) / np.sqrt(d)
    dat = G @ rng.normal(size=(d, 1)) + 0.05 * rng.normal(size=(n, 1))
    lik = H.Distributions.LinearMatrix(G, dat, 0.05**2)
    assert lik._use_tc("float32", C)
    M = torch.from_numpy(rng.normal(size=(d, C))).to("cuda", torch.float32)
    g_ref = lik.gradient_batch(M).clone()
    lik.check_device_status()
    with _lib.wait_limits(LIMIT_NS, withhold=True):
        lik.gradient_batch(M)
        torch.cuda.synchronize()
    with pytest.raises(DeviceTimeoutError):
        lik.check_device_status()
    lik.check_device_status()  # the status word was cleared by the raise
    g = lik.gradient_batch(M)
    torch.cuda.synchronize()
    lik.check_device_status()
    assert torch.equal(g, g_ref)


def test_tensor_core_short_limit_without_withholding_changes_nothing():
    rng = np.random.default_rng(1)
    n, d, C = 260, 96, 130
    G = rng.normal(size=(n, d)) / np.sqrt(d)
    dat = G @ rng.normal(size=(d, 1))
    lik = H.Distributions.LinearMatrix(G, dat, 0.01)
    M = torch.from_numpy(rng.normal(size=(d, C))).to("cuda", torch.float32)
    g_ref = lik.gradient_batch(M).clone()
    with _lib.wait_limits(50_000_000, withhold=False):  # 50 ms: far above a launch's duration
        g = lik.gradient_batch(M)
        torch.cuda.synchronize()
    lik.check_device_status()
    assert torch.equal(g, g_ref)


def _fwi(cfg, C):
    rng = np.random.default_rng(3)
    zeros = np.zeros((cfg.n_shots, cfg.nt, cfg.n_rec))
    obs = zeros + 1e-3 * rng.normal(size=zeros.shape)
    dist = H.Distributions.ElasticFullWaveform2D(cfg, obs, obs, data_std=1e-3, free_parameter_grid=[5, 3])
    M = torch.from_numpy(rng.normal(size=(45, C)) * 20.0).to("cuda", torch.float32)
    return dist, M


def test_elastic_tile_wait_runs_out_and_the_context_survives():
    cfg = FW.ElasticConfig(nx=40, nz=24, pad=8, h=5.0, dt=5e-4, nt=20, f0=25.0, sponge=0.05,
                           src_x=(60.0, 140.0), src_z=20.0, rec_x=np.linspace(15.0, 185.0, 9), rec_z=20.0)
    C = 32  # a multiple of 32: the staged-tile kernels run
    dist, M = _fwi(cfg, C)
    x_ref = dist.misfit_batch(M).clone()
    dist.check_device_status()
    # a fresh copy captures its per-shot graphs under the hook
    hooked = H.Distributions.ElasticFullWaveform2D(dist)
    with _lib.wait_limits(LIMIT_NS, withhold=True):
        hooked.misfit_batch(M)
        torch.cuda.synchronize()
    with pytest.raises(DeviceTimeoutError):
        hooked.check_device_status()
    del hooked
    x = dist.misfit_batch(M)
    torch.cuda.synchronize()
    dist.check_device_status()
    assert torch.equal(x, x_ref)
    fresh = H.Distributions.ElasticFullWaveform2D(dist)
    assert torch.equal(fresh.misfit_batch(M), x_ref)
    fresh.check_device_status()
