"""BFGS mass matrix (host-side, reference MassMatrices.py:330-522): the
inverse-Hessian update, its bookkeeping, and its hand-over to the device
sampler as an exact Full mass matrix.  No GPU."""
import numpy as np
import pytest

import hmclab_gb300 as H
from hmclab_gb300 import Samplers
from hmclab_gb300.MassMatrices import BFGS, Full


def quadratic(d=8, seed=0):
    rng = np.random.default_rng(seed)
    L = rng.normal(size=(d, d))
    return L @ L.T / d + np.eye(d), rng


def test_updates_recover_the_inverse_hessian_of_a_quadratic():
    d = 8
    Hs, rng = quadratic(d)
    x = rng.normal(size=(d, 1))
    b = BFGS(d, x, Hs @ x)
    for _ in range(10 * d):
        x = x + 0.5 * rng.normal(size=(d, 1))
        b.update(x, Hs @ x)
    b.accept()
    np.testing.assert_allclose(b.Minv, np.linalg.inv(Hs), rtol=0, atol=1e-3)
    np.testing.assert_allclose(b.matrix, Hs, atol=1e-2)
    assert b.succesful_updates == b.attempted_updates == 10 * d


def test_secant_condition_and_rejected_curvature():
    d = 5
    Hs, rng = quadratic(d, 1)
    m0 = rng.normal(size=(d, 1))
    b = BFGS(d, m0, Hs @ m0)
    m1 = m0 + rng.normal(size=(d, 1))
    b._update(m1, Hs @ m1)
    s, y = m1 - m0, Hs @ (m1 - m0)
    np.testing.assert_allclose(b.Minv @ y, s, atol=1e-10)  # secant condition
    # non-positive curvature s^T y <= 0: Minv kept, the pair still advances
    before = b.Minv.copy()
    m2 = m1 + rng.normal(size=(d, 1))
    b._update(m2, Hs @ m1 - (m2 - m1))
    np.testing.assert_array_equal(b.Minv, before)
    np.testing.assert_array_equal(b.m, m2)
    assert b.attempted_updates_current == 2


def test_reject_restores_and_queued_updates_apply_once():
    d = 4
    Hs, rng = quadratic(d, 2)
    x = rng.normal(size=(d, 1))
    b = BFGS(d, x, Hs @ x)
    for _ in range(3):
        x = x + rng.normal(size=(d, 1))
        b.update(x, Hs @ x)
    b.reject()
    np.testing.assert_array_equal(b.Minv, np.eye(d))
    assert b.ms == [] and b.attempted_updates == 0
    for _ in range(3):
        x = x + rng.normal(size=(d, 1))
        b.update(x, Hs @ x)
    b.accept()
    first = b.Minv.copy()
    b.accept()  # nothing queued: no change
    np.testing.assert_array_equal(b.Minv, first)
    assert b.attempted_updates == 3


def test_greedy_updates_and_kinetic_energy():
    d = 3
    Hs, rng = quadratic(d, 3)
    x = rng.normal(size=(d, 1))
    b = BFGS(d, x, Hs @ x, greedy=True, rng=np.random.default_rng(0))
    x2 = x + rng.normal(size=(d, 1))
    b.update(x2, Hs @ x2)
    assert b.attempted_updates_current == 1 and b.ms == []
    p = rng.normal(size=(d, 1))
    assert b.kinetic_energy(p) == pytest.approx(0.5 * (p.T @ b.Minv @ p).item())
    np.testing.assert_allclose(b.kinetic_energy_gradient(p), b.Minv @ p)
    with pytest.raises(ValueError):
        b.kinetic_energy(np.zeros((d + 1, 1)))
    # momenta have covariance M = Minv^-1
    z = b.generate_momentum(repeat=200000)
    np.testing.assert_allclose(np.cov(z), np.linalg.inv(b.Minv), atol=0.02 * np.abs(np.linalg.inv(b.Minv)).max())


def test_freeze_and_cast_to_full():
    d = 4
    Hs, rng = quadratic(d, 4)
    x = rng.normal(size=(d, 1))
    b = BFGS(d, x, Hs @ x)
    for _ in range(20):
        x = x + rng.normal(size=(d, 1))
        b.update(x, Hs @ x)
    b.accept()
    full = b.freeze(cast=True)
    assert isinstance(full, Full) and full.dimensions == d
    np.testing.assert_allclose(full.matrix, np.linalg.inv(b.Minv), rtol=1e-10)
    frozen = b.freeze()
    x = x + rng.normal(size=(d, 1))
    before = frozen.Minv.copy()
    frozen.update(x, Hs @ x)
    frozen.accept()
    np.testing.assert_array_equal(frozen.Minv, before)
    assert BFGS.create_default(6).Minv.shape == (6, 6)


def test_device_sampler_rejects_bfgs():
    d = 3
    prior = H.Distributions.Normal(np.zeros((d, 1)), np.ones((d, 1)))
    with pytest.raises(NotImplementedError, match="freeze"):
        Samplers.HMC(seed=1)._parse(None, prior, 0.1, True, 10, BFGS.create_default(d), "lf", None, 10, 1, False,
                                    False, None, False, 0.65, 0.75, None, None, None, True, None, False)
