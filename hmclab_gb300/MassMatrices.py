"""Mass matrices (kinetic-energy metrics) of the HMC sampler.

Same classes and single-vector API as the reference (larsgeb/hmclab,
`hmclab/MassMatrices.py:27-327`): `kinetic_energy(p)`,
`kinetic_energy_gradient(p)`, `generate_momentum()`, `accept()`/`reject()`,
`matrix`, `create_default`.  The single-vector energy calls run the FP64
kernels on the GPU; the sampler applies the same formulas for all chains
inside its trajectory kernels (the mass matrix is handed to the device as
`mass_kind` plus its diagonal, or its Cholesky factor and inverse).  `BFGS`
(reference `MassMatrices.py:330-522`) is host-side: it learns a metric from
(position, gradient) pairs and hands it to the sampler as a `Full` mass
matrix through `freeze(cast=True)`.
"""
import ctypes as _ct

import numpy as _numpy

from hmclab_gb300 import _device as _dev
from hmclab_gb300 import _lib
from hmclab_gb300.Helpers.CustomExceptions import AbstractMethodError as _AbstractMethodError


class _AbstractMassMatrix:
    name: str = "mass matrix abstract base class"
    dimensions: int = -1
    rng: _numpy.random.Generator = _numpy.random.default_rng()
    kind: int = -1

    def full_name(self) -> str:
        raise _AbstractMethodError()

    def accept(self):
        pass

    def reject(self):
        pass

    def _check(self, momentum):
        if _numpy.shape(momentum) != (self.dimensions, 1):
            raise ValueError()

    # ---- device parameters -------------------------------------------------
    def device_params(self, dtype):
        cache = self.__dict__.setdefault("_param_cache", {})
        if dtype not in cache:
            cache[dtype] = self._make_params(dtype)
        return cache[dtype]

    def _make_params(self, dtype):
        return {}

    def __getstate__(self):
        state = self.__dict__.copy()
        state.pop("_param_cache", None)
        return state

    def _device_energy(self, momentum, gradient=False):
        p = _dev.upload(momentum.reshape(self.dimensions, 1), "float64")
        prm = self.device_params("float64")
        st = _lib.HmcChains()
        st.dtype = _lib.HMC_F64
        st.mass_kind = self.kind
        st.dims = self.dimensions
        st.chains = 1
        st.mass_inv_diag = _dev.ptr(prm.get("inv_diag"))
        st.mass_diag = _dev.ptr(prm.get("diag"))
        st.mass_chol = _dev.ptr(prm.get("chol"))
        st.mass_inv = _dev.ptr(prm.get("inv"))
        work = _dev.empty((self.dimensions, 1), "float64", p.device)
        st.v = work.data_ptr()
        stream = _dev.stream_handle()
        if gradient:
            out = _dev.empty((self.dimensions, 1), "float64", p.device)
            _lib.call("hmc_kinetic_energy_gradient", _ct.byref(st), p.data_ptr(), out.data_ptr(), stream)
            return out.cpu().numpy()
        out = _dev.empty((1,), "float64", p.device)
        _lib.call("hmc_kinetic_energy", _ct.byref(st), p.data_ptr(), out.data_ptr(), stream)
        return float(out.cpu()[0])

    def kinetic_energy(self, momentum: _numpy.ndarray) -> float:
        """K(p) = 0.5 p^T M^-1 p (FP64, on the GPU)."""
        self._check(momentum)
        return self._device_energy(_numpy.asarray(momentum, _numpy.float64))

    def kinetic_energy_gradient(self, momentum: _numpy.ndarray, position=None, g=None) -> _numpy.ndarray:
        """dK/dp = M^-1 p (FP64, on the GPU)."""
        self._check(momentum)
        return self._device_energy(_numpy.asarray(momentum, _numpy.float64), gradient=True)


class Unit(_AbstractMassMatrix):
    """Identity mass matrix (reference `MassMatrices.py:82-156`)."""

    kind = _lib.HMC_MASS_UNIT

    def __init__(self, dimensions: int = -1, rng: _numpy.random.Generator = None):
        self.name = "unit mass matrix"
        self.dimensions = dimensions
        if rng is not None:
            self.rng = rng

    def generate_momentum(self) -> _numpy.ndarray:
        return self.rng.normal(size=(self.dimensions, 1))

    @property
    def matrix(self) -> _numpy.ndarray:
        return _numpy.eye(self.dimensions)

    @staticmethod
    def create_default(dimensions: int, rng=None) -> "Unit":
        return Unit(dimensions, rng)


class Diagonal(_AbstractMassMatrix):
    """Diagonal mass matrix (reference `MassMatrices.py:159-238`)."""

    kind = _lib.HMC_MASS_DIAG

    def __init__(self, diagonal: _numpy.ndarray, rng: _numpy.random.Generator = None):
        self.name = "diagonal mass matrix"
        diagonal = _numpy.asarray(diagonal, dtype=_numpy.float64).reshape(-1, 1)
        self.dimensions = diagonal.size
        self.diagonal = diagonal
        self.inverse_diagonal = 1.0 / self.diagonal
        if rng is not None:
            self.rng = rng

    def _make_params(self, dtype):
        return {"diag": _dev.upload(self.diagonal[:, 0], dtype), "inv_diag": _dev.upload(self.inverse_diagonal[:, 0], dtype)}

    def generate_momentum(self) -> _numpy.ndarray:
        return _numpy.sqrt(self.diagonal) * self.rng.normal(size=(self.dimensions, 1))

    @property
    def matrix(self) -> _numpy.ndarray:
        return _numpy.diagflat(self.diagonal)

    @staticmethod
    def create_default(dimensions: int, rng=None) -> "Diagonal":
        return Diagonal(_numpy.ones((dimensions, 1)), rng=rng)


class Full(_AbstractMassMatrix):
    """Full (dense SPD) mass matrix (reference `MassMatrices.py:241-327`).
    The device uses the lower Cholesky factor L (momenta p = L z) and the
    explicit inverse M^-1 (formed once in FP64 from L)."""

    kind = _lib.HMC_MASS_FULL

    def __init__(self, full: _numpy.ndarray, rng: _numpy.random.Generator = None, do_hermitian_check=True):
        self.name = "full mass matrix"
        self.mass_matrix = _numpy.asarray(full, dtype=_numpy.float64)
        if do_hermitian_check:
            assert _numpy.allclose(self.mass_matrix, self.mass_matrix.T)
        self.cholesky = _numpy.linalg.cholesky(self.mass_matrix)
        self.dimensions = self.mass_matrix.shape[0]
        eye = _numpy.eye(self.dimensions)
        linv = _numpy.linalg.solve(self.cholesky, eye)
        self.inverse = linv.T @ linv
        if rng is not None:
            self.rng = rng

    def _make_params(self, dtype):
        return {"chol": _dev.upload(self.cholesky, dtype), "inv": _dev.upload(self.inverse, dtype)}

    def generate_momentum(self, repeat=1) -> _numpy.ndarray:
        return self.cholesky @ self.rng.normal(size=(self.dimensions, repeat))

    @property
    def matrix(self) -> _numpy.ndarray:
        return self.mass_matrix

    @staticmethod
    def create_default(dimensions: int, rng=None) -> "Full":
        m = _numpy.eye(dimensions) + 0.1 * _numpy.eye(dimensions, k=-1) + 0.1 * _numpy.eye(dimensions, k=1)
        return Full(m, rng=rng)


class BFGS(_AbstractMassMatrix):
    """Quasi-Newton inverse mass matrix (reference `MassMatrices.py:330-522`):
    Minv approximates the posterior covariance (the inverse Hessian of the
    misfit) through BFGS updates from successive (position, gradient) pairs,
        s = m - m_prev,  y = g - g_prev,  rho = 1 / (s^T y)  (only if s^T y > 0),
        Minv <- (I - rho s y^T) Minv (I - rho y s^T) + rho s s^T
    (Nocedal & Wright, Numerical Optimization, eq. 6.17), kept only when the
    result still has a Cholesky factor.

    The reference updates Minv at every leapfrog step inside the trajectory,
    which leaves the leapfrog neither volume-preserving nor reversible, so the
    chain no longer targets the posterior exactly; the batched device
    sampler does not do that, and `sample()` rejects a BFGS mass matrix with
    NotImplementedError.  Use it on the host to learn a metric — feed it
    (position, gradient) pairs with `update` / `kinetic_energy_gradient(p,
    position, g)`, e.g. the pairs a `surrogate.TrainingSet` recorded during
    burn-in — and sample with `freeze(cast=True)`, a `Full` mass matrix with
    M = Minv^-1, which is exact.  Host-side FP64 numpy.  Queued updates are
    applied once by `consolidate_updates` (the queue is then emptied)."""

    kind = None

    def __init__(self, dimensions: int, m: _numpy.ndarray, g: _numpy.ndarray, Minv: _numpy.ndarray = None,
                 greedy: bool = False, rng: _numpy.random.Generator = None):
        self.name = "BFGS-optimized mass matrix"
        self.greedy = greedy
        if rng is not None:
            self.rng = rng
        self.dimensions = dimensions
        assert m.shape == (self.dimensions, 1), f"{m.shape}"
        assert g.shape == (self.dimensions, 1), f"{g.shape}"
        self.Minv = _numpy.eye(dimensions) if Minv is None else _numpy.array(Minv, dtype=_numpy.float64)
        self._factor()
        self.m = _numpy.array(m, dtype=_numpy.float64)
        self.g = _numpy.array(g, dtype=_numpy.float64)
        self.ms, self.gs = [], []
        self.succesful_updates = self.attempted_updates = 0
        self.succesful_updates_current = self.attempted_updates_current = 0
        self.frozen = False
        self.save()

    def _factor(self):
        # Minv = L L^T; momenta p = L^-T z have covariance (L L^T)^-1 = M
        chol = _numpy.linalg.cholesky(self.Minv)
        self.LTinv = _numpy.linalg.inv(chol.T)

    # ---- energies (host) -----------------------------------------------------
    def kinetic_energy(self, momentum: _numpy.ndarray) -> float:
        self._check(momentum)
        return 0.5 * (momentum.T @ self.Minv @ momentum).item()

    def kinetic_energy_gradient(self, momentum: _numpy.ndarray, position=None, g=None) -> _numpy.ndarray:
        """Minv p; with a position and its gradient, first updates Minv."""
        self._check(momentum)
        if position is not None and g is not None:
            self._update(position, g)
        return self.Minv @ momentum

    def generate_momentum(self, repeat=1) -> _numpy.ndarray:
        return self.LTinv @ self.rng.normal(size=(self.dimensions, repeat))

    @property
    def matrix(self) -> _numpy.ndarray:
        return _numpy.linalg.inv(self.Minv)

    # ---- updates -------------------------------------------------------------
    def update(self, m, g):
        """Queue a (position, gradient) pair; applied at once when greedy."""
        if self.frozen:
            return
        self.ms.append(_numpy.array(m, dtype=_numpy.float64))
        self.gs.append(_numpy.array(g, dtype=_numpy.float64))
        if self.greedy:
            self.consolidate_updates()

    def consolidate_updates(self):
        for m, g in zip(self.ms, self.gs):
            self._update(m, g)
        self.ms, self.gs = [], []

    def _update(self, m, g):
        if self.frozen:
            return
        before = self.Minv.copy(), self.m.copy(), self.g.copy()
        s = m - self.m
        y = g - self.g
        self.m, self.g = _numpy.array(m, dtype=_numpy.float64), _numpy.array(g, dtype=_numpy.float64)
        sy = (s.T @ y).item()
        if sy > 0.0:
            rho = 1.0 / sy
            left = _numpy.eye(self.dimensions) - rho * (s @ y.T)
            self.Minv = left @ self.Minv @ left.T + rho * (s @ s.T)
        self.attempted_updates_current += 1
        try:
            self._factor()
            self.succesful_updates_current += 1
        except _numpy.linalg.LinAlgError:
            self.Minv, self.m, self.g = before
            self._factor()

    def save(self):
        self.backup = self.Minv.copy(), self.m.copy(), self.g.copy()

    def reset(self):
        self.Minv, self.m, self.g = (a.copy() for a in self.backup)
        self._factor()
        self.ms, self.gs = [], []

    def accept(self):
        if self.frozen:
            return
        self.consolidate_updates()
        self.save()
        self.attempted_updates += self.attempted_updates_current
        self.succesful_updates += self.succesful_updates_current
        self.attempted_updates_current = self.succesful_updates_current = 0

    def reject(self):
        if self.frozen:
            return
        self.reset()
        self.attempted_updates_current = self.succesful_updates_current = 0

    def freeze(self, cast=False):
        """Stop updating; with cast=True return the equivalent `Full` mass
        matrix M = Minv^-1 for the device sampler."""
        if cast:
            M = _numpy.linalg.inv(self.Minv)
            return Full(0.5 * (M + M.T), rng=self.rng)
        self.frozen = True
        return self

    @staticmethod
    def create_default(dimensions: int, rng: _numpy.random.Generator = None) -> "BFGS":
        return BFGS(dimensions, _numpy.zeros((dimensions, 1)), _numpy.ones((dimensions, 1)), _numpy.eye(dimensions),
                    rng=rng)
