"""Host-side logic that needs no GPU: argument validation with the reference's
exception classes, integrator schedules, samples files, synthetic problems,
and the loud failure when no device is present."""
import os

import numpy as np
import pytest

import hmclab_gb300 as H
from hmclab_gb300 import Samplers, problems
from hmclab_gb300.Helpers.CustomExceptions import DeviceUnavailableError
from oracle import hmc_oracle as O

torch = pytest.importorskip("torch")
NO_GPU = not torch.cuda.is_available()


@pytest.mark.parametrize("integrator", ["lf", "3s", "4s"])
@pytest.mark.parametrize("L", [1, 3, 10])
def test_integrator_ops_match_oracle(integrator, L):
    assert Samplers.integrator_ops(integrator, L) == O.integrator_schedule(integrator, L)


def test_schedule_compiles_to_fused_kick_drift():
    first, steps = Samplers.compile_schedule(Samplers.integrator_ops("lf", 4))
    assert first == 0.5
    assert steps == [(True, 1.0, 1.0)] * 3 + [(True, 1.0, 0.5)]
    first, steps = Samplers.compile_schedule(Samplers.integrator_ops("3s", 2))
    # 3 kicks per stage, a bare drift where two stages meet
    assert sum(s[0] for s in steps) == 6
    assert sum(1 for s in steps if not s[0]) == 1


def test_unknown_integrator_raises_value_error():
    with pytest.raises(ValueError):
        Samplers.integrator_ops("rk4", 3)


def _normal(d=3):
    return H.Distributions.Normal(np.zeros((d, 1)), np.ones((d, 1)))


@pytest.mark.parametrize(
    "kwargs,exc",
    [
        (dict(proposals=0), AssertionError),
        (dict(proposals=10, online_thinning=3), AssertionError),
        (dict(stepsize=-1.0), AssertionError),
        (dict(amount_of_steps=2.5), AssertionError),
        (dict(integrator="xx"), ValueError),
        (dict(mass_matrix=H.MassMatrices.Unit(5)), AssertionError),
        (dict(autotuning=True, learning_rate=0.3), AssertionError),
        (dict(initial_model=np.zeros((4, 1))), AssertionError),
        (dict(max_time=-1.0), AssertionError),
    ],
)
def test_sampler_argument_validation(kwargs, exc):
    """Invalid arguments are rejected before any device work, with the
    reference's exception types (Samplers.py:347-441, 1335-1384)."""
    base = dict(proposals=10)
    base.update(kwargs)
    with pytest.raises(exc):
        Samplers.HMC(seed=1)._parse(
            None, _normal(), base.get("stepsize", 0.1), True, base.get("amount_of_steps", 10),
            base.get("mass_matrix"), base.get("integrator", "lf"), base.get("initial_model"), base["proposals"],
            base.get("online_thinning", 1), False, False, base.get("max_time"), base.get("autotuning", False),
            0.65, base.get("learning_rate", 0.75), None, None, None, True, None, False,
        )


@pytest.mark.skipif(not NO_GPU, reason="checks the no-device behaviour")
def test_device_calls_fail_loudly_without_gpu():
    with pytest.raises(DeviceUnavailableError):
        _normal().misfit(np.zeros((3, 1)))
    with pytest.raises(DeviceUnavailableError):
        H.Samplers.HMC(seed=0).sample(None, _normal(), proposals=2)


def test_distribution_bounds_validation():
    d = _normal(2)
    with pytest.raises(ValueError):
        d.update_bounds(lower=np.zeros((3, 1)))
    with pytest.raises(ValueError):
        d.update_bounds(lower=np.ones((2, 1)), upper=np.zeros((2, 1)))
    d.update_bounds(lower=-np.ones((2, 1)), upper=np.ones((2, 1)))
    assert d.misfit_bounds(np.zeros((2, 1))) == 0.0
    assert d.misfit_bounds(np.full((2, 1), 2.0)) == np.inf
    q, p = np.array([[-1.5], [0.5]]), np.ones((2, 1))
    d.corrector(q, p)
    assert np.allclose(q, [[-0.5], [0.5]]) and np.allclose(p, [[-1.0], [1.0]])


def test_bayes_rule_collapses_bounds():
    a = H.Distributions.Normal(np.zeros((2, 1)), np.ones((2, 1)), lower_bounds=np.array([[-1.0], [-2.0]]))
    b = H.Distributions.Laplace(np.zeros((2, 1)), np.ones((2, 1)), lower_bounds=np.array([[-3.0], [-1.0]]),
                                upper_bounds=np.array([[4.0], [5.0]]))
    post = H.Distributions.BayesRule([a, b])
    assert np.array_equal(post.lower_bounds, [[-1.0], [-1.0]])
    assert np.array_equal(post.upper_bounds, [[4.0], [5.0]])


def test_linear_matrix_reproduces_reference_quirks(golden):
    g = golden("linearmatrix_public.npz")
    lik = H.Distributions.LinearMatrix(g["G"].copy(), g["d"].copy(), float(g["var"]))
    assert lik.premultiplication
    M = g["probe_m"]
    mis = 0.5 * (np.sum(M * (lik.GtG @ M - 2 * lik.Gtd0), axis=0) + lik.dtd)
    np.testing.assert_allclose(mis, g["probe_misfit"], rtol=1e-12)
    np.testing.assert_allclose(lik.GtG @ M - lik.Gtd0, g["probe_grad"], rtol=1e-12, atol=1e-9)


def test_samples_file_roundtrip(tmp_path):
    fn = str(tmp_path / "s.npy")
    w = H.Samples(fn, mode="w")
    a = np.arange(12.0).reshape(4, 3)
    w.append_columns(a)
    w.append_columns(a + 100)
    w.write_attribute("proposals", 6)
    w.close()
    arr = np.load(fn)
    assert arr.shape == (6, 4)  # rows are samples, like the reference's file
    with H.Samples(fn) as r:
        assert r.numpy.shape == (4, 6)
        np.testing.assert_array_equal(r.numpy[:, :3], a)
        assert r.read_attribute("write_index") == 6
    with pytest.raises(FileExistsError):
        H.Samples(fn, mode="w")
    H.Samples(fn, mode="w", overwrite=True).close()


def test_siddon_lengths_sum_to_segment_length():
    rng = np.random.default_rng(0)
    for _ in range(50):
        x0, y0, x1, y1 = rng.uniform(0, 16, size=4)
        idx, lens = problems.ray_cell_lengths(x0, y0, x1, y1, 16, 16, 1.0)
        assert np.isclose(lens.sum(), np.hypot(x1 - x0, y1 - y0), rtol=1e-12)
        assert len(np.unique(idx)) == len(idx)
    # axis-aligned ray along a grid line interior
    idx, lens = problems.ray_cell_lengths(0.0, 2.5, 16.0, 2.5, 16, 16, 1.0)
    assert len(idx) == 16 and np.allclose(lens, 1.0)


def test_tomography_problem_shape():
    t = problems.tomography(nx=32, ny=32, n_rays=200, seed=1)
    G = t["G"]
    assert G.shape == (200, 1024)
    nnz = np.diff(G.indptr)
    assert nnz.min() > 0 and 20 < nnz.mean() < 64 * 2
    bg = t["background"]
    assert bg.min() >= 0.2 - 1e-12 and bg.max() <= 0.5 + 1e-12


class _FakeSurrogate:
    def __init__(self, d, frozen=True):
        self.d, self.frozen = d, frozen


def _parsed(d=3, chains=4, dtype="float32"):
    smp = Samplers.HMC(seed=1)
    smp._parse(None, _normal(d), 0.1, True, 10, None, "lf", None, 10, 1, False, False, None, False, 0.65, 0.75,
               chains, dtype, None, True, None, False)
    return smp


@pytest.mark.parametrize(
    "make,msg",
    [
        (lambda: (_parsed(dtype="float64"), _FakeSurrogate(3)), "float32"),
        (lambda: (_parsed(), _FakeSurrogate(5)), "dimensions"),
        (lambda: (_parsed(), _FakeSurrogate(3, frozen=False)), "freeze"),
    ],
)
def test_surrogate_argument_validation(make, msg):
    """A surrogate must be frozen, match the target's dimension and drive
    float32 chains; checked on the host before any device work."""
    smp, sur = make()
    with pytest.raises(AssertionError, match=msg):
        smp._parse_surrogate(sur, None)


def test_training_set_disables_graph_capture():
    """Recording exact gradients needs the host between launches, so the
    sampler runs uncaptured; a frozen surrogate alone keeps the graphs."""
    smp = _parsed()
    smp._parse_surrogate(_FakeSurrogate(3), None)
    assert smp.use_graph is True
    smp = _parsed()
    smp._parse_surrogate(None, _FakeSurrogate(3))
    assert smp.use_graph is False


@pytest.mark.parametrize(
    "temps,interval,msg",
    [
        ([1.0, 2.0, 4.0], None, "one temperature per chain"),
        ([1.0, 2.0, 0.0, 4.0], None, "positive"),
        ([1.0, 2.0, np.inf, 4.0], None, "finite"),
        ([1.0, 2.0, 3.0, 4.0], 0, "positive int"),
        ([1.0, 2.0, 3.0, 4.0], 2.5, "positive int"),
    ],
)
def test_tempering_argument_validation(temps, interval, msg):
    smp = _parsed(chains=4)
    with pytest.raises(AssertionError, match=msg):
        smp._parse_tempering(temps, interval)


def test_replica_exchange_needs_two_chains_and_a_thinning_multiple():
    with pytest.raises(AssertionError, match="two chains"):
        _parsed(chains=1)._parse_tempering(None, 5)
    smp = Samplers.HMC(seed=1)
    smp._parse(None, _normal(3), 0.1, True, 10, None, "lf", None, 12, 3, False, False, None, False, 0.65, 0.75,
               4, "float32", None, True, None, False)
    with pytest.raises(AssertionError, match="multiple of online_thinning"):
        smp._parse_tempering(None, 4)
    smp._parse_tempering([1.0, 1.5, 2.0, 3.0], 6)
    assert smp.exchange_interval == 6 and np.allclose(smp._temperatures, [1.0, 1.5, 2.0, 3.0])


def _linear_post(d=6, n=12, prior="normal", sparse=False):
    import scipy.sparse as sp

    rng = np.random.default_rng(0)
    G = rng.normal(size=(n, d))
    if sparse:
        G = sp.csr_matrix(G)
    lik = H.Distributions.LinearMatrix(G, rng.normal(size=(n, 1)), 0.1)
    if prior is None:
        return lik
    pr = _normal(d) if prior == "normal" else H.Distributions.Laplace(np.zeros((d, 1)), np.ones((d, 1)))
    return H.Distributions.BayesRule([pr, lik])


def _parsed_for(post, chains=8, dtype="float32", proposals=10, autotuning=False):
    smp = Samplers.HMC(seed=1)
    smp._parse(None, post, 0.1, True, 10, None, "lf", None, proposals, 1, False, False, None, autotuning, 0.65,
               0.75, chains, dtype, None, True, None, False)
    smp._parse_surrogate(None, None)
    smp._parse_tempering(None, None)
    # the device set-up uploads the bounds; these targets have none
    smp.lower = smp.upper = None
    return smp


@pytest.mark.parametrize(
    "case",
    ["too_large", "autotuning", "surrogate", "sparse", "no_linear", "two_priors", "opted_out"],
)
def test_persistent_kernel_declines_unsupported_runs(case):
    """The persistent path applies only to small dense linear-Gaussian (or
    Laplace-prior) targets without bounds, autotuning, tempering or a
    surrogate; every other run keeps the launch-per-step path.  Host logic,
    no device allocation."""
    from hmclab_gb300._persistent import PersistentDense

    if case == "too_large":
        smp = _parsed_for(_linear_post(d=200, n=300))
    elif case == "autotuning":
        smp = _parsed_for(_linear_post(), autotuning=True)
    elif case == "surrogate":
        smp = _parsed_for(_linear_post())
        smp.surrogate = _FakeSurrogate(6)
    elif case == "sparse":
        smp = _parsed_for(_linear_post(sparse=True))
    elif case == "no_linear":
        smp = _parsed_for(_normal(6))
    elif case == "two_priors":
        post = H.Distributions.BayesRule([_normal(6), _normal(6), _linear_post(prior=None)])
        smp = _parsed_for(post)
    else:
        smp = _parsed_for(_linear_post())
        smp.use_persistent = False
    assert PersistentDense.applies(smp) is None


def test_persistent_shared_memory_budget():
    from hmclab_gb300._persistent import MAX_D, _SMEM, _smem

    # GtG with an odd row stride plus one vector per warp; a full mass adds
    # its inverse and Cholesky factor
    assert _smem(50, False, 4, 4) == (50 * 51 + 4 * 50) * 4
    assert _smem(64, True, 2, 8) == (3 * 64 * 65 + 2 * 64) * 8
    # the largest supported dimension fits in FP32 with a unit or diagonal
    # mass; in FP64 with a full mass it does not, and the path declines it
    assert _smem(MAX_D, False, 16, 4) <= _SMEM
    assert _smem(MAX_D, True, 1, 8) > _SMEM


@pytest.mark.parametrize("case", ["float64", "full_mass", "small", "sparse", "tempered", "two_priors"])
def test_fused_tensor_core_step_declines_unsupported_runs(case):
    """The fused tensor-core leapfrog step applies to FP32 chains of a dense
    premultiplied LinearMatrix with d >= 64 and at most one diagonal Normal
    or Laplace prior, under a unit or diagonal mass and no tempering."""
    from hmclab_gb300._dense_tc import FusedDenseStep

    d = 16 if case == "small" else 80
    post = _linear_post(d=d, n=2 * d, sparse=case == "sparse")
    if case == "two_priors":
        post = H.Distributions.BayesRule([_normal(d), _normal(d), _linear_post(d=d, n=2 * d, prior=None)])
    smp = _parsed_for(post, dtype="float64" if case == "float64" else "float32")
    if case == "full_mass":
        smp.mass_matrix = H.MassMatrices.Full(np.eye(d))
    if case == "tempered":
        smp.beta = object()
    assert FusedDenseStep.applies(smp) is None


def test_moment_error():
    from hmclab_gb300 import diagnostics

    me, se = diagnostics.moment_error(np.array([1.0, 2.0]), np.array([1.0, 4.0]), [[1.1], [2.0]], [[2.0], [5.0]])
    assert me == pytest.approx(0.05) and se == pytest.approx(0.5)


def test_batched_calls_reject_host_arrays_and_wrong_shapes():
    torch = pytest.importorskip("torch")
    dist = _normal(4)
    with pytest.raises(ValueError, match="CUDA tensor"):
        dist.misfit_batch(torch.zeros(4, 3))
    with pytest.raises(ValueError, match="CUDA tensor"):
        dist.gradient_batch(np.zeros((4, 3)))


def test_get_diagnostics_needs_diagnostic_mode():
    import hmclab_gb300 as H
    from hmclab_gb300.Helpers.CustomExceptions import InvalidCaseError

    with pytest.raises(InvalidCaseError):
        H.Samplers.HMC(seed=0).get_diagnostics()
    t = H.Samplers.DeviceTimer("gradient")
    t.add_host_seconds(0.25)
    assert t.function.__name__ == "gradient" and t.calls == 1 and t.time_spent == 0.25
    assert "gradient" in str(t)


def test_samples_file_opens_with_the_reference_reader(tmp_path):
    """A file written by hmclab_gb300's Samples writer (the one the sampler
    drains thinned samples into) is opened unchanged by the reference's own
    `Samples` reader (hmclab/Samples.py:23-278): same (d+1, N) layout, same
    attributes, burn-in slicing and misfit row."""
    from oracle import ref_shim

    ref = ref_shim.load()
    if ref is None:
        pytest.skip("reference sources not present on this machine")
    from hmclab.Samples import Samples as RefSamples

    fn = str(tmp_path / "chain.npy")
    rng = np.random.default_rng(3)
    d, N = 5, 40
    cols = rng.normal(size=(d + 1, N))
    w = H.Samples(fn, mode="w")
    for k in range(0, N, 8):
        w.append_columns(cols[:, k:k + 8])
    for name, value in (("stepsize", 0.1), ("amount_of_steps", 10), ("mass_matrix", "Unit"),
                        ("integrator", "leapfrog"), ("proposals", N), ("online_thinning", 1), ("sampler", "HMC")):
        w.write_attribute(name, value)
    w.close()
    with RefSamples(fn, burn_in=10) as r:
        assert r.numpy.shape == (d + 1, N - 10)
        np.testing.assert_array_equal(r.samples, cols[:-1, 10:])
        np.testing.assert_array_equal(r.misfits, cols[-1, 10:])
        assert r.read_attribute("write_index") == N
        assert r.read_attribute("proposals") == N and r.read_attribute("sampler") == "HMC"
        # the reference's [] applies the burn-in on top of `numpy`, which already has it
        np.testing.assert_array_equal(r[:, :3], cols[:, 20:23])


def test_bound_handling_matches_the_reference_contract():
    """corrector / update_bounds / misfit_bounds against the reference's own
    methods (hmclab/Distributions/base.py:239-374) on the same inputs:
    reflections, momentum flips, the lower-then-upper order, error messages
    and that rejected bounds leave the old ones in place."""
    from oracle import ref_shim

    ref = ref_shim.load()
    if ref is None:
        pytest.skip("reference sources not present on this machine")
    rng = np.random.default_rng(5)
    d = 7
    mine = H.Distributions.Normal(np.zeros((d, 1)), np.ones((d, 1)))
    theirs = ref.Distributions.Normal(np.zeros((d, 1)), np.ones((d, 1)))
    lo, hi = -np.ones((d, 1)), np.ones((d, 1))
    for dist in (mine, theirs):
        dist.update_bounds(lower=list(lo[:, 0]), upper=hi)
    for _ in range(20):
        q = rng.normal(size=(d, 1)) * 2.5  # some beyond both reflections
        p = rng.normal(size=(d, 1))
        q1, p1, q2, p2 = q.copy(), p.copy(), q.copy(), p.copy()
        mine.corrector(q1, p1)
        theirs.corrector(q2, p2)
        np.testing.assert_array_equal(q1, q2)
        np.testing.assert_array_equal(p1, p2)
        assert mine.misfit_bounds(q) == theirs.misfit_bounds(q)
    for args in ({"lower": "x"}, {"upper": 3.0}, {"lower": np.zeros((d + 1, 1))}, {"lower": hi, "upper": lo}):
        msgs = []
        for dist in (mine, theirs):
            with pytest.raises(ValueError) as e:
                dist.update_bounds(**args)
            msgs.append(str(e.value))
            np.testing.assert_array_equal(dist.lower_bounds, lo)
            np.testing.assert_array_equal(dist.upper_bounds, hi)
        assert msgs[0] == msgs[1]
