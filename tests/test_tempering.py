"""Tempered chains and replica exchange on the device: the exchange kernel
against the oracle's restatement of the reference's exchange rule
(Samplers.py:589-669), and tempered levels that keep their own
distributions while they swap models."""
import ctypes

import numpy as np
import pytest

from oracle import hmc_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_exchange_kernel_matches_oracle(dtype):
    from hmclab_gb300 import _lib

    rng = np.random.default_rng(4)
    d, C = 7, 301
    q = rng.normal(size=(d, C))
    x = rng.uniform(0, 20, size=C)
    beta = 1.0 / rng.choice([1.0, 2.0, 4.0, 8.0], size=C)
    perm = rng.permutation(C)[: 2 * (C // 2)]
    pairs = perm.reshape(-1, 2)
    u = rng.uniform(size=len(pairs))
    tdt = torch.float64 if dtype == "float64" else torch.float32
    qd = torch.from_numpy(q).to("cuda", tdt).contiguous()
    xd = torch.from_numpy(x).cuda()
    bd = torch.from_numpy(beta).cuda()
    pd = torch.from_numpy(perm.astype(np.int32)).cuda()
    ud = torch.from_numpy(u).cuda()
    sw = torch.zeros(len(pairs), dtype=torch.int32, device="cuda")
    tot = torch.zeros(1, dtype=torch.int64, device="cuda")
    st = _lib.HmcChains()
    st.dtype = _lib.HMC_F64 if dtype == "float64" else _lib.HMC_F32
    st.dims, st.chains = d, C
    st.q_cur, st.x_cur, st.beta = qd.data_ptr(), xd.data_ptr(), bd.data_ptr()
    _lib.call("hmc_exchange", ctypes.byref(st), len(pairs), pd.data_ptr(), ud.data_ptr(), sw.data_ptr(),
              tot.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    q_ref, x_ref, s_ref = O.exchange(q.astype(np.float32).astype(np.float64) if dtype == "float32" else q, x, beta,
                                     pairs, u)
    np.testing.assert_array_equal(sw.cpu().numpy().astype(bool), s_ref)
    assert int(tot.item()) == int(s_ref.sum()) and 0 < s_ref.sum() < len(pairs)
    np.testing.assert_array_equal(qd.double().cpu().numpy(), q_ref)
    np.testing.assert_array_equal(xd.cpu().numpy(), x_ref)
    with pytest.raises(ValueError):
        _lib.call("hmc_exchange", ctypes.byref(st), C, pd.data_ptr(), ud.data_ptr(), sw.data_ptr(), None,
                  torch.cuda.current_stream().cuda_stream)


def test_tempered_levels_keep_their_distributions_while_swapping():
    """Four temperature levels of a Normal target (variance T sigma^2 at
    level T), 1024 chains each, started at exact draws of their level and
    exchanged after every proposal: after 30 proposals every level still has
    its mean and variance (a swap rule that ignored the temperatures would
    pull hot models into the cold level and inflate its variance)."""
    import hmclab_gb300 as H

    d, per = 4, 1024
    temps = np.repeat([1.0, 2.0, 4.0, 8.0], per)
    C = temps.size
    rng = np.random.default_rng(9)
    mu = rng.normal(size=(d, 1))
    var = rng.uniform(0.5, 2.0, size=(d, 1))
    post = H.Distributions.Normal(mu, var)
    q0 = mu + np.sqrt(var * temps[None, :]) * rng.normal(size=(d, C))
    eps = 0.5 * np.sqrt(var.min() * temps)
    smp = H.Samplers.HMC(seed=3).sample(None, post, stepsize=eps, amount_of_steps=5, initial_model=q0,
                                        proposals=30, chains=C, dtype="float32", temperatures=temps,
                                        exchange_interval=1)
    assert smp.exchanges_accepted > 0
    q = smp.current_model
    for k, T in enumerate([1.0, 2.0, 4.0, 8.0]):
        sl = slice(k * per, (k + 1) * per)
        qm = q[:, sl]
        sd = np.sqrt(var[:, 0] * T)
        z = np.abs(qm.mean(axis=1) - mu[:, 0]) / (sd / np.sqrt(per))
        ratio = qm.var(axis=1) / (var[:, 0] * T)
        print(f"T={T}: max |z| {z.max():.2f}, variance ratios {ratio.round(3)}")
        assert z.max() < 5.0
        assert np.all(np.abs(ratio - 1.0) < 5.0 * np.sqrt(2.0 / per))


def test_device_parallel_tempering_matches_reference_parallel_sampler(golden):
    """The device sampler with temperatures and exchanges replays the
    reference's own ParallelSampleSMP run (forked chains exchanging over
    pipes; fixture made by the reference itself) under the same streams:
    positions of every recorded sample to 1e-12, for all four tempered
    chains.  Recorded misfits agree except right after a swap, where the
    reference's file keeps the chain's pre-swap misfit (its exchange leaves
    current_x alone, Samplers.py:589-678) and the device records the misfit
    of the swapped-in model."""
    import hmclab_gb300 as H

    g = golden("replica_exchange.npz")
    temps = g["temps"]
    C = temps.size
    post = H.Distributions.Normal(g["mean"], g["var"])
    P = g["z"].shape[0]
    smp = H.Samplers.HMC(seed=0).sample(
        None, post, stepsize=float(g["stepsize"]), amount_of_steps=int(g["amount_of_steps"]),
        initial_model=np.repeat(g["mean"], C, axis=1), proposals=P, chains=C, dtype="float64", temperatures=temps,
        exchange_interval=int(g["interval"]), rng_streams=(g["z"], g["f"], g["u"]),
        exchange_streams=(g["schedule"], g["exchange_u"]), keep_samples=True)
    got = smp.samples_numpy()  # C, d+1, N
    ref = np.moveaxis(g["samples"], -1, 0)
    np.testing.assert_allclose(got[:, :-1], ref[:, :-1], rtol=1e-12, atol=1e-12)
    # misfits: equal wherever the recorded model is the chain's own
    beta = 1.0 / temps
    own = np.isclose(got[:, -1], ref[:, -1], rtol=1e-12, atol=0)
    assert own.mean() > 0.5
    x_model = np.stack([beta[c] * 0.5 * np.sum((got[c, :-1] - g["mean"]) ** 2 / g["var"], axis=0) for c in range(C)])
    np.testing.assert_allclose(got[:, -1], x_model, rtol=1e-12)  # the device records the model's own misfit
    assert smp.exchanges_accepted > 0
