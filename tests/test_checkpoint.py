"""Checkpoint / resume of the batched sampler: `checkpoint(path)` after a run
and `sample(..., resume=path)` continue the chains bit for bit (positions,
misfits, thinned samples, adapted step sizes, the Philox streams and a
surrogate's weights), on the launch-per-step, tensor-core and persistent
paths.  The reference saves no chain or random state (Samples.py:280-335
leaves only a readable partial file), so this has no reference counterpart;
the test is an uninterrupted run of the same length.

CPU: the checkpoint's argument checks; GPU: the bitwise continuations."""
import numpy as np
import pytest

import hmclab_gb300 as H


def _fake_checkpoint(path, **over):
    ck = dict(format=np.array("hmclab_gb300.checkpoint.v1"), q=np.zeros((4, 2)), eps=np.full(2, 0.1),
              proposals_done=np.array(8, np.int64), philox_seed=np.array(5, np.uint64),
              dimensions=np.array(4, np.int64), chains=np.array(2, np.int64), dtype=np.array("float32"),
              online_thinning=np.array(1, np.int64))
    ck.update(over)
    np.savez(path, **ck)
    return str(path)


def test_resume_argument_checks(tmp_path):
    post = H.Distributions.Normal(np.zeros((4, 1)), np.ones((4, 1)))
    ok = _fake_checkpoint(tmp_path / "ok.npz")
    smp = H.Samplers.HMC(seed=0)
    with pytest.raises(ValueError, match="exclude each other"):
        smp.prepare(None, post, resume=ok, initial_model=np.zeros((4, 2)))
    with pytest.raises(ValueError, match="rng_streams"):
        smp.prepare(None, post, resume=ok, rng_streams="numpy")
    with pytest.raises(ValueError, match="chains"):
        smp.prepare(None, post, resume=ok, chains=3)
    with pytest.raises(ValueError, match="dimensions"):
        smp.prepare(None, H.Distributions.Normal(np.zeros((5, 1)), np.ones((5, 1))), resume=ok)
    with pytest.raises(ValueError, match="not an hmclab_gb300 sampler checkpoint"):
        smp.prepare(None, post, resume=_fake_checkpoint(tmp_path / "bad.npz", format=np.array("other")))
    with pytest.raises(ValueError, match="multiple of online_thinning"):
        smp.prepare(None, post, resume=ok, online_thinning=3)
    a = {"chains": None, "dtype": None, "initial_model": None, "rng_streams": None, "online_thinning": 1,
         "stepsize": 0.5}
    ck = smp._read_checkpoint(ok, post, a)
    assert a["chains"] == 2 and a["dtype"] == "float32" and a["initial_model"].shape == (4, 2)
    assert np.array_equal(a["stepsize"], np.full(2, 0.1)) and int(ck["proposals_done"]) == 8


# ---------------------------------------------------------------------------
def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _dense_posterior(n, d, seed):
    rng = np.random.default_rng(seed)
    G = rng.normal(size=(n, d)) / np.sqrt(d)
    dat = G @ rng.normal(size=(d, 1)) + 0.1 * rng.normal(size=(n, 1))
    return H.Distributions.BayesRule([H.Distributions.Normal(np.zeros((d, 1)), np.ones((d, 1))),
                                      H.Distributions.LinearMatrix(G, dat, 0.01, dtype=np.float64)])


@pytest.mark.gpu
@pytest.mark.parametrize("path,d,dtype,extra", [
    ("launch per step", 40, "float64", dict(persistent=False, autotuning=True)),
    ("tensor-core fused step", 200, "float32", dict(autotuning=True)),
    ("persistent kernel", 50, "float32", dict()),
])
def test_resume_continues_bit_for_bit(tmp_path, path, d, dtype, extra):
    torch = _cuda()
    post = _dense_posterior(3 * d, d, d)
    C, P1, P2 = 64, 12, 20
    kw = dict(stepsize=0.02, amount_of_steps=6, chains=C, dtype=dtype, keep_samples=True, proposals_per_graph=4,
              **extra)
    q0 = np.zeros((d, C))
    full = H.Samplers.HMC(seed=9).sample(None, post, initial_model=q0, proposals=P1 + P2, **kw)
    first = H.Samplers.HMC(seed=9).sample(None, post, initial_model=q0, proposals=P1, **kw)
    ck = first.checkpoint(str(tmp_path / "state.npz"))
    rest = H.Samplers.HMC(seed=123).sample(None, post, proposals=P2, resume=ck, **kw)
    assert np.array_equal(rest.current_model, full.current_model), path
    assert np.array_equal(np.atleast_1d(rest.current_x), np.atleast_1d(full.current_x))
    got = rest.samples_numpy()  # C, d+1, P2
    want = full.samples_numpy()[:, :, P1:]
    assert np.array_equal(got, want), path
    if extra.get("autotuning"):
        assert np.array_equal(rest.stepsize, full.stepsize)
        assert np.array_equal(rest.stepsizes, full.stepsizes[P1:P1 + P2 - 1])
    assert rest._persistent is not None if path == "persistent kernel" else True
    torch.cuda.synchronize()


@pytest.mark.gpu
def test_resume_with_a_surrogate_restores_its_state(tmp_path):
    """A surrogate-driven run resumed with a freshly built surrogate of the
    same architecture: the checkpoint restores its weights, normalisation and
    Adam moments, so the continued chains and further training are equal."""
    torch = _cuda()
    from hmclab_gb300 import surrogate as S

    d, C = 64, 32
    post = _dense_posterior(3 * d, d, 3)
    data = S.TrainingSet(d, 6 * 4 * C)
    q0 = np.zeros((d, C))
    kw = dict(stepsize=0.02, amount_of_steps=4, chains=C, dtype="float32")
    H.Samplers.HMC(seed=1).sample(None, post, initial_model=q0, proposals=6, training_set=data, **kw)
    net = S.PotentialSurrogate(d, hidden=(64, 64), seed=0)
    net.train(data, steps=50, batch=64)
    net.freeze()
    P1, P2 = 5, 7
    full = H.Samplers.HMC(seed=4).sample(None, post, initial_model=q0, proposals=P1 + P2, surrogate=net,
                                         keep_samples=True, **kw)
    first = H.Samplers.HMC(seed=4).sample(None, post, initial_model=q0, proposals=P1, surrogate=net, **kw)
    ck = first.checkpoint(str(tmp_path / "s.npz"))
    fresh = S.PotentialSurrogate(d, hidden=(64, 64), seed=99)
    rest = H.Samplers.HMC(seed=0).sample(None, post, proposals=P2, resume=ck, surrogate=fresh, keep_samples=True,
                                         **kw)
    assert fresh.frozen and fresh.steps == net.steps
    assert np.array_equal(rest.current_model, full.current_model)
    assert np.array_equal(rest.samples_numpy(), full.samples_numpy()[:, :, P1:])
    # training continues identically from the restored Adam moments
    net.frozen = fresh.frozen = False
    idx = np.arange(64)
    la = net.train_step(data, idx, lr=1e-3)
    lb = fresh.train_step(data, idx, lr=1e-3)
    torch.cuda.synchronize()
    assert float(la[0]) == float(lb[0])
    for k in net.params:
        assert torch.equal(net.params[k], fresh.params[k]), k
