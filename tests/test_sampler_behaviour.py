"""Sampler behaviour the reference's own tests pin, run through the CUDA
path: finite-difference gradients of the default distributions
(test_distributions.py:171-215, test_mass_matrices.py:85-120), bit-identical
runs for identical seeds (test_sampling_reproducibility.py:22-123), thinned
file shapes and existing-file handling (test_sampling.py, Samples.py:102-110),
`max_time` and interrupts ending a run cleanly (test_break.py:11-63).

Tolerance of the finite-difference checks: central differences in FP64 agree
with the device gradient to 1e-6 relative (the reference accepts 1e-2)."""
import _thread
import threading
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _fd_check(dist, m, rng, h=1e-6):
    g = dist.gradient(m)
    assert g.shape == m.shape and g.dtype == np.float64
    for _ in range(3):
        v = rng.normal(size=m.shape)
        fd = (dist.misfit(m + h * v) - dist.misfit(m - h * v)) / (2 * h)
        an = float(np.sum(g * v))
        assert abs(fd - an) <= 1e-6 * max(abs(fd), abs(an), 1e-8), (type(dist).__name__, fd, an)


@pytest.mark.parametrize("dims", [1, 10, 50])
def test_default_distributions_gradients_match_finite_differences(dims):
    import hmclab_gb300 as H
    from hmclab_gb300 import problems

    rng = np.random.default_rng(dims)
    np.random.seed(dims)
    for cls in (H.Distributions.Normal, H.Distributions.Laplace, H.Distributions.LinearMatrix):
        dist = cls.create_default(dims)
        m = rng.normal(size=(dims, 1)) + 3.0  # away from the Laplace kinks at the means (in [0, 1])
        _fd_check(dist, m, rng)
    t = problems.source_location(n_events=2, n_stations=12, seed=dims)
    sl = H.Distributions.SourceLocation3D(t["rx"], t["ry"], t["rz"], t["obs"], 0.05)
    _fd_check(sl, t["m_true"] + 0.1 * rng.normal(size=t["m_true"].shape), rng, h=1e-5)


def test_mass_matrix_kinetic_gradients_match_finite_differences():
    import hmclab_gb300 as H

    rng = np.random.default_rng(0)
    d = 6
    A = rng.normal(size=(d, d))
    for mm in (H.MassMatrices.Unit(d), H.MassMatrices.Diagonal(rng.uniform(0.5, 2.0, size=(d, 1))),
               H.MassMatrices.Full(A @ A.T + d * np.eye(d))):
        p = rng.normal(size=(d, 1))
        g = mm.kinetic_energy_gradient(p)
        v = rng.normal(size=(d, 1))
        h = 1e-6
        fd = (mm.kinetic_energy(p + h * v) - mm.kinetic_energy(p - h * v)) / (2 * h)
        assert abs(fd - float(np.sum(g * v))) <= 1e-7 * abs(fd)
        with pytest.raises(ValueError):
            mm.kinetic_energy(np.zeros((d + 1, 1)))


def _post(d=8):
    import hmclab_gb300 as H

    np.random.seed(3)
    return H.Distributions.BayesRule([H.Distributions.Normal.create_default(d),
                                      H.Distributions.LinearMatrix.create_default(d)])


def test_identical_seeds_give_identical_chains(tmp_path):
    import hmclab_gb300 as H

    post = _post()
    files = [str(tmp_path / f"{k}.npy") for k in "abc"]
    for f, seed in zip(files, (1, 1, 2)):
        H.Samplers.HMC(seed=seed).sample(f, post, stepsize=0.2, amount_of_steps=5, proposals=40, online_thinning=2,
                                         disable_progressbar=True)
    a, b, c = (np.array(H.Samples(f).numpy) for f in files)
    assert a.shape == (9, 20)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c)
    # batched FP32 chains with device Philox draws
    runs = [H.Samplers.HMC(seed=s).sample(None, post, stepsize=0.2, amount_of_steps=5, proposals=12, chains=256,
                                          keep_samples=True) for s in (5, 5, 6)]
    s0, s1, s2 = (r.samples_numpy() for r in runs)
    assert np.array_equal(s0, s1) and not np.array_equal(s0, s2)


def test_thinned_samples_file_and_existing_file(tmp_path):
    import hmclab_gb300 as H

    post = _post(5)
    f = str(tmp_path / "s.npy")
    smp = H.Samplers.HMC(seed=2).sample(f, post, stepsize=0.2, amount_of_steps=4, proposals=30, online_thinning=3)
    with H.Samples(f) as s:
        arr = np.array(s.numpy)
        assert arr.shape == (6, 10)
        assert s.read_attribute("online_thinning") == 3
    # the last row holds the misfit of the column above it
    for k in (0, 5, 9):
        assert abs(arr[-1, k] - post.misfit(arr[:-1, k:k + 1])) <= 1e-9 * max(1.0, abs(arr[-1, k]))
    assert smp.current_proposal == 29
    with pytest.raises(FileExistsError):
        H.Samplers.HMC(seed=2).sample(f, post, proposals=3)
    H.Samplers.HMC(seed=2).sample(f, post, proposals=3, overwrite_existing_file=True)
    assert H.Samples(f).numpy.shape == (6, 3)


class _SlowNormal:
    """A Normal target whose gradient takes 20 ms on the host."""

    @staticmethod
    def make(d):
        import hmclab_gb300 as H

        class SlowNormal(H.Distributions.Normal):
            graph_safe = False

            def _device_gradient(self, M, out, accumulate, dtype, stream):
                time.sleep(0.02)
                super()._device_gradient(M, out, accumulate, dtype, stream)

        return SlowNormal(np.zeros((d, 1)), np.ones((d, 1)))


def test_max_time_ends_the_run_early(tmp_path):
    import hmclab_gb300 as H

    post = _SlowNormal.make(4)
    f = str(tmp_path / "t.npy")
    t0 = time.time()
    smp = H.Samplers.HMC(seed=1).sample(f, post, stepsize=0.3, amount_of_steps=5, proposals=10000, max_time=1.0,
                                        proposals_per_graph=1)
    assert time.time() - t0 < 10.0
    assert 0 < smp.current_proposal < 9999
    assert H.Samples(f).numpy.shape[1] == smp.current_proposal + 1


def test_interrupt_ends_the_run_cleanly(tmp_path):
    import hmclab_gb300 as H

    post = _SlowNormal.make(4)
    f = str(tmp_path / "i.npy")
    timer = threading.Timer(0.8, _thread.interrupt_main)
    timer.start()
    try:
        smp = H.Samplers.HMC(seed=1).sample(f, post, stepsize=0.3, amount_of_steps=5, proposals=10000,
                                            proposals_per_graph=1)
    finally:
        timer.cancel()
    assert 0 < smp.current_proposal < 9999
    n = H.Samples(f).numpy.shape[1]
    assert n == smp.current_proposal + 1


def test_diagnostic_mode_times_every_phase(capsys):
    """diagnostic_mode (reference Samplers.py:449-460, 499-527, 759-764):
    CUDA-event timers per phase with the reference's timer attributes, call
    counts that follow the proposal structure, and the printed split."""
    import hmclab_gb300 as H

    rng = np.random.default_rng(4)
    d, C, P, L = 30, 16, 6, 5
    G = rng.normal(size=(60, d)) / np.sqrt(d)
    dat = G @ rng.normal(size=(d, 1))
    post = H.Distributions.BayesRule([H.Distributions.Normal(np.zeros((d, 1)), np.ones((d, 1))),
                                      H.Distributions.LinearMatrix(G, dat, 0.01, dtype=np.float64)])
    smp = H.Samplers.HMC(seed=2).sample(None, post, stepsize=0.01, amount_of_steps=L, proposals=P, chains=C,
                                        dtype="float64", diagnostic_mode=True, initial_model=np.zeros((d, C)))
    timers = {t.function.__name__: t for t in smp.get_diagnostics()}
    assert timers["generate_momentum"].calls == P
    assert timers["gradient"].calls == P * L  # position Verlet: L gradients per trajectory
    assert timers["integrator"].calls == P * L  # one kick+drift per gradient
    assert timers["misfit"].calls == P and timers["_evaluate_acceptance"].calls == P
    for name in ("generate_momentum", "gradient", "integrator", "misfit", "_evaluate_acceptance"):
        assert timers[name].time_spent > 0.0, name
    assert sum(t.time_spent for t in timers.values()) <= smp.runtime_seconds
    out = capsys.readouterr().out
    assert "Detailed statistics:" in out and "gradient" in out
    # the same launch-per-step run without the timers (graph-captured) gives the same chains
    ref = H.Samplers.HMC(seed=2).sample(None, post, stepsize=0.01, amount_of_steps=L, proposals=P, chains=C,
                                        dtype="float64", initial_model=np.zeros((d, C)), persistent=False)
    assert np.array_equal(ref.current_model, smp.current_model)
