"""Mass matrices (kinetic-energy metrics) of the HMC sampler.

Same classes and single-vector API as the reference (larsgeb/hmclab,
`hmclab/MassMatrices.py:27-327`): `kinetic_energy(p)`,
`kinetic_energy_gradient(p)`, `generate_momentum()`, `accept()`/`reject()`,
`matrix`, `create_default`.  The single-vector energy calls run the FP64
kernels on the GPU; the sampler applies the same formulas for all chains
inside its trajectory kernels (the mass matrix is handed to the device as
`mass_kind` plus its diagonal, or its Cholesky factor and inverse).
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
