"""Target distributions of the HMC hot path, evaluated on the GPU.

The classes keep the reference's plugin API (larsgeb/hmclab,
`hmclab/Distributions/base.py:21-374`): an integer `dimensions`,
`misfit(m) -> float` and `gradient(m) -> (d,1) ndarray` on column vectors,
optional `lower_bounds` / `upper_bounds`, `corrector`, `update_bounds`,
`misfit_bounds`, `misfit_v`.  Single-vector calls run the FP64 kernels on one
chain.  The batched API takes a device tensor M of shape (d, C) (one chain per
column, chain index fastest in memory) and is what the sampler calls:

    misfit_batch(M)   -> float64 tensor (C,)
    gradient_batch(M) -> tensor (d, C) of M's dtype

Every evaluation goes through the CUDA library; there is no CPU fallback.
"""
from abc import abstractmethod as _abstractmethod
from typing import List as _List, Union as _Union

import numpy as _numpy
import scipy.sparse as _sparse

from hmclab_gb300 import _device as _dev
from hmclab_gb300 import _lib
from hmclab_gb300.Helpers.CustomExceptions import AbstractMethodError as _AbstractMethodError
from hmclab_gb300.Helpers.CustomExceptions import InvalidCaseError as _InvalidCaseError

__all__ = [
    "_AbstractDistribution",
    "Normal",
    "Laplace",
    "AdditiveDistribution",
    "BayesRule",
    "LinearMatrix",
    "SourceLocation3D",
]


def _column(coordinates, dimensions):
    m = _numpy.asarray(coordinates, dtype=_numpy.float64)
    if m.size != dimensions:
        raise ValueError(f"coordinates of size {m.size} do not match dimensions {dimensions}")
    return m.reshape(dimensions, 1)


class _AbstractDistribution:
    """Plugin base class (reference `base.py:21-374`).

    Subclasses set `self.dimensions` and implement `_device_misfit` and
    `_device_gradient`, which write (or accumulate into) device buffers for a
    (d, C) batch of models."""

    name: str = None
    lower_bounds: _Union[_numpy.ndarray, None] = None
    upper_bounds: _Union[_numpy.ndarray, None] = None
    normalized: bool = False
    normalization_constant: float = 0.0
    # arithmetic type of the single-vector misfit()/gradient() calls
    single_dtype: str = "float64"
    # False when the device calls launch CUDA graphs of their own or need the
    # host between launches: the sampler then issues proposals uncaptured
    graph_safe: bool = True

    # ---- reference-facing single-vector API -------------------------------
    def misfit(self, coordinates: _numpy.ndarray) -> float:
        """chi(m) for one column vector (d,1), on the GPU in `single_dtype`
        (FP64 unless the target's kernels are FP32 only; reference
        `base.py:70-105`); +inf outside the bounds."""
        m = _column(coordinates, self.dimensions)
        x = self.misfit_batch(_dev.upload(m, self.single_dtype))
        return float(x.cpu()[0]) + self.normalization_constant + self.misfit_bounds(m)

    def gradient(self, coordinates: _numpy.ndarray) -> _numpy.ndarray:
        """d chi / d m for one column vector, on the GPU in `single_dtype`
        (reference `base.py:140-168`), returned as FP64; the bound misfit (0 or
        +inf) is added like the reference does."""
        m = _column(coordinates, self.dimensions)
        g = self.gradient_batch(_dev.upload(m, self.single_dtype))
        return g.double().cpu().numpy().reshape(self.dimensions, 1) + self.misfit_bounds(m)

    def misfit_v(self, coordinates: _numpy.ndarray, vectors_in_dim=None):
        """Misfits of many vectors at once (reference `base.py:107-138`), as
        one batched launch instead of a Python loop."""
        c = _numpy.asarray(coordinates, dtype=_numpy.float64)
        if c.size == self.dimensions:
            return self.misfit(c)
        if vectors_in_dim is None:
            if c.ndim != 2:
                raise AttributeError("Can only take 1D or 2D arrays as input if not specifying vector input dimension")
            if c.shape[0] == self.dimensions:
                vectors_in_dim = 0
            elif c.shape[1] == self.dimensions:
                vectors_in_dim = 1
            else:
                raise AttributeError(f"Don't know what to do with input of shape {c.shape}.")
        M = _numpy.moveaxis(c, vectors_in_dim, 0).reshape(self.dimensions, -1)
        x = self.misfit_batch(_dev.upload(M, "float64")).cpu().numpy()
        x = x + self.normalization_constant + _numpy.array([self.misfit_bounds(M[:, [k]]) for k in range(M.shape[1])])
        return x.reshape(_numpy.moveaxis(c, vectors_in_dim, 0).shape[1:])

    # ---- batched device API -------------------------------------------------
    def _check_batch(self, M):
        if not (hasattr(M, "is_cuda") and M.is_cuda):
            raise ValueError("batched evaluation needs a CUDA tensor of shape (dimensions, chains)")
        if M.dim() != 2 or M.shape[0] != self.dimensions:
            raise ValueError(f"expected shape ({self.dimensions}, C), got {tuple(M.shape)}")
        if not M.is_contiguous():
            raise ValueError("the model batch must be contiguous (chains fastest)")
        return _dev.normalise_dtype(M.dtype)

    def misfit_batch(self, M, out=None, accumulate=False, stream=None):
        """chi for every column of M (device, (d, C)); returns float64 (C,).
        Bounds are not applied here (the sampler tracks them per chain)."""
        dtype = self._check_batch(M)
        if out is None:
            out = _dev.zeros((M.shape[1],), "float64", M.device)
        self._device_misfit(M, out, bool(accumulate), dtype, _dev.stream_handle(stream))
        return out

    def gradient_batch(self, M, out=None, accumulate=False, stream=None):
        """d chi / d m for every column of M; returns a (d, C) tensor of M's dtype."""
        dtype = self._check_batch(M)
        if out is None:
            out = _dev.zeros(tuple(M.shape), dtype, M.device)
        self._device_gradient(M, out, bool(accumulate), dtype, _dev.stream_handle(stream))
        return out

    def check_device_status(self):
        """Raise DeviceTimeoutError if one of this target's kernels gave up a
        bounded wait since the last check (synchronises with the device).
        Targets whose kernels never wait have nothing to check."""

    @_abstractmethod
    def _device_misfit(self, M, out, accumulate, dtype, stream):
        raise _AbstractMethodError()

    @_abstractmethod
    def _device_gradient(self, M, out, accumulate, dtype, stream):
        raise _AbstractMethodError()

    def _device_misfit_after_gradient(self, M, out, accumulate, dtype, stream):
        """The misfit at M, called right after _device_gradient at the same
        M (targets whose gradient runs a forward simulation reuse it)."""
        self._device_misfit(M, out, accumulate, dtype, stream)

    # ---- device parameter / scratch caches ---------------------------------
    def _params(self, dtype):
        cache = self.__dict__.setdefault("_param_cache", {})
        if dtype not in cache:
            cache[dtype] = self._make_params(dtype)
        return cache[dtype]

    def _make_params(self, dtype):
        return {}

    def _scratch(self, name, shape, dtype, device):
        cache = self.__dict__.setdefault("_scratch_cache", {})
        key = (name, tuple(shape), dtype)
        t = cache.get(key)
        if t is None:
            t = _dev.empty(shape, dtype, device)
            cache[key] = t
        return t

    def __getstate__(self):
        state = self.__dict__.copy()
        state.pop("_param_cache", None)
        state.pop("_scratch_cache", None)
        state.pop("_last_gradient_descriptor", None)
        return state

    # ---- reference API kept as is -----------------------------------------
    def normalize(self):
        raise AttributeError("This distribution is not normalizable.")

    def generate(self, repeat=1, rng=_numpy.random.default_rng()) -> _numpy.ndarray:
        raise NotImplementedError("Generating samples from this distribution is not implemented or supported.")

    @staticmethod
    def create_default(dimensions: int) -> "_AbstractDistribution":
        raise NotImplementedError()

    def corrector(self, coordinates: _numpy.ndarray, momentum: _numpy.ndarray):
        """Mirror every coordinate that crossed a bound back inside it and
        reverse its momentum, in place (the reference's contract,
        `base.py:239-270`: the lower bound first, then the upper one).  The
        sampler applies the same rule on the device after every drift."""
        for bound, crossed in ((self.lower_bounds, _numpy.less), (self.upper_bounds, _numpy.greater)):
            if bound is None:
                continue
            hit = crossed(coordinates, bound)
            coordinates[hit] += 2 * (bound[hit] - coordinates[hit])
            momentum[hit] *= -1.0

    def update_bounds(self, lower=None, upper=None):
        """Replace the bounds (either may be None: unbounded).  Lists become
        column vectors; anything else must be a (dimensions, 1) array with
        every upper bound above its lower bound.  A rejected pair raises
        ValueError with the reference's messages (`base.py:272-359`) and
        leaves the current bounds in place."""

        def column(b):
            return _numpy.array(b)[:, None] if type(b) == list else b

        lower, upper = column(lower), column(upper)
        for b, which in ((lower, "Lower"), (upper, "Upper")):
            if b is not None and type(b) is not _numpy.ndarray:
                raise ValueError(f"{which} bounds object not understood.")
        if any(b is not None and b.shape != (self.dimensions, 1) for b in (lower, upper)):
            raise ValueError("Bounds vectors are of incorrect size.")
        if lower is not None and upper is not None and _numpy.any(upper <= lower):
            raise ValueError("Bounds vectors are incompatible.")
        self.lower_bounds, self.upper_bounds = lower, upper

    def misfit_bounds(self, coordinates: _numpy.ndarray) -> float:
        """+inf when any coordinate lies outside the bounds, else 0
        (`base.py:361-374`)."""
        outside = (self.lower_bounds is not None and bool(_numpy.any(coordinates < self.lower_bounds))) or (
            self.upper_bounds is not None and bool(_numpy.any(coordinates > self.upper_bounds)))
        return _numpy.inf if outside else 0.0


# ---------------------------------------------------------------------------
class Normal(_AbstractDistribution):
    """Normal distribution (reference `base.py:427-643`): diagonal (scalar or
    (d,1) variances) or full (d,d) covariance."""

    def __init__(self, means, covariance, inverse_covariance=None, lower_bounds=None, upper_bounds=None):
        self.name = "Gaussian (normal) distribution"
        if type(means) == list:
            means = _numpy.array(means)[:, None]
        if type(covariance) == list:
            covariance = _numpy.array(covariance)[:, None]
        if type(means) == float or type(means) == int:
            self.dimensions = 1
            means = _numpy.ones((1, 1)) * means
        else:
            self.dimensions = int(means.size)
            means = _numpy.asarray(means, dtype=_numpy.float64).reshape(self.dimensions, 1)
        self.means = means
        self.normalization_constant = 0.0
        self.generate_ready = False
        if isinstance(covariance, (float, int, _numpy.floating)):
            covariance = _numpy.float64(covariance)
            self.diagonal = True
        elif covariance.shape == (means.size, means.size):
            self.diagonal = False
        else:
            self.diagonal = True
            covariance = _numpy.asarray(covariance, dtype=_numpy.float64).reshape(self.dimensions, 1)
        self.covariance = covariance
        if inverse_covariance is not None:
            self.inverse_covariance = inverse_covariance
        elif self.diagonal:
            self.inverse_covariance = 1.0 / self.covariance
        else:
            self.inverse_covariance = _numpy.linalg.inv(self.covariance)
        if self.dimensions == 1:
            self.diagonal = True
        self.update_bounds(lower_bounds, upper_bounds)

    def _make_params(self, dtype):
        if self.diagonal:
            iv = _numpy.broadcast_to(_numpy.asarray(self.inverse_covariance, _numpy.float64).reshape(-1, 1),
                                     (self.dimensions, 1))
            return {"mean": _dev.upload(self.means[:, 0], dtype), "iv": _dev.upload(iv[:, 0], dtype)}
        return {
            "mean": _dev.upload(self.means[:, 0], dtype),
            "icov": _dev.upload(_numpy.asarray(self.inverse_covariance), dtype),
        }

    def _device_misfit(self, M, out, accumulate, dtype, stream):
        p = self._params(dtype)
        d, C = M.shape
        if self.diagonal:
            _lib.call("hmc_normal_diag_misfit", _dev.dtype_code(dtype), d, C, M.data_ptr(), p["mean"].data_ptr(),
                      p["iv"].data_ptr(), out.data_ptr(), int(accumulate), stream)
        else:
            work = self._scratch("work2", (2, d, C), dtype, M.device)
            _lib.call("hmc_normal_full_misfit", _dev.dtype_code(dtype), d, C, M.data_ptr(), p["mean"].data_ptr(),
                      p["icov"].data_ptr(), work.data_ptr(), out.data_ptr(), int(accumulate), stream)

    def _device_gradient(self, M, out, accumulate, dtype, stream):
        p = self._params(dtype)
        d, C = M.shape
        if self.diagonal:
            _lib.call("hmc_normal_diag_gradient", _dev.dtype_code(dtype), d, C, M.data_ptr(), p["mean"].data_ptr(),
                      p["iv"].data_ptr(), out.data_ptr(), int(accumulate), stream)
        else:
            work = self._scratch("work1", (d, C), dtype, M.device)
            _lib.call("hmc_normal_full_gradient", _dev.dtype_code(dtype), d, C, M.data_ptr(), p["mean"].data_ptr(),
                      p["icov"].data_ptr(), work.data_ptr(), out.data_ptr(), int(accumulate), stream)

    def normalize(self):
        cov = self.covariance
        if isinstance(cov, (float, int, _numpy.floating)):
            det = cov**self.dimensions
        elif cov.shape == (self.means.size, self.means.size):
            det = _numpy.linalg.det(cov)
        else:
            det = _numpy.prod(cov)
        self.normalization_constant = 0.5 * (_numpy.log(_numpy.abs(det)) + self.dimensions * _numpy.log(2 * _numpy.pi))
        self.normalized = True

    def generate(self, repeat=1, rng=_numpy.random.default_rng()) -> _numpy.ndarray:
        if self.diagonal:
            return rng.normal(size=(self.dimensions, repeat)) * _numpy.sqrt(self.covariance) + self.means
        return _numpy.linalg.cholesky(self.covariance) @ rng.normal(size=(self.dimensions, repeat)) + self.means

    @staticmethod
    def create_default(dimensions: int, diagonal=True) -> "Normal":
        means = _numpy.random.rand(dimensions, 1)
        std = _numpy.random.rand(dimensions, 1) + 1
        return Normal(means, std * std)


class Laplace(_AbstractDistribution):
    """Laplace (L1) distribution (reference `base.py:646-744`)."""

    def __init__(self, means, dispersions, lower_bounds=None, upper_bounds=None):
        if type(means) == list:
            means = _numpy.array(means)[:, None]
        if type(dispersions) == list:
            dispersions = _numpy.array(dispersions)[:, None]
        means = _numpy.asarray(means, dtype=_numpy.float64)
        self.dimensions = int(means.size)
        self.means = means.reshape(self.dimensions, 1)
        dispersions = _numpy.asarray(dispersions, dtype=_numpy.float64)
        if dispersions.size == 1:
            dispersions = _numpy.full((self.dimensions, 1), float(dispersions.reshape(-1)[0]))
        self.dispersions = dispersions.reshape(self.dimensions, 1)
        self.inverse_dispersions = 1.0 / self.dispersions
        self.normalization_constant = 0.0
        self.update_bounds(lower_bounds, upper_bounds)

    def _make_params(self, dtype):
        return {"mean": _dev.upload(self.means[:, 0], dtype), "iw": _dev.upload(self.inverse_dispersions[:, 0], dtype)}

    def _device_misfit(self, M, out, accumulate, dtype, stream):
        p = self._params(dtype)
        _lib.call("hmc_laplace_misfit", _dev.dtype_code(dtype), M.shape[0], M.shape[1], M.data_ptr(),
                  p["mean"].data_ptr(), p["iw"].data_ptr(), out.data_ptr(), int(accumulate), stream)

    def _device_gradient(self, M, out, accumulate, dtype, stream):
        p = self._params(dtype)
        _lib.call("hmc_laplace_gradient", _dev.dtype_code(dtype), M.shape[0], M.shape[1], M.data_ptr(),
                  p["mean"].data_ptr(), p["iw"].data_ptr(), out.data_ptr(), int(accumulate), stream)

    def normalize(self):
        self.normalization_constant = _numpy.log(
            1.0 / (2.0 * (_numpy.prod(self.dispersions) ** (1.0 / self.dimensions)))
        )
        self.normalized = True

    def generate(self, repeat=1, rng=_numpy.random.default_rng()) -> _numpy.ndarray:
        return rng.laplace(loc=self.means, scale=self.dispersions, size=(self.dimensions, repeat))

    @staticmethod
    def create_default(dimensions: int) -> "Laplace":
        return Laplace(_numpy.random.rand(dimensions, 1), 10 ** _numpy.random.rand(dimensions, 1))


class Uniform(_AbstractDistribution):
    """Uniform distribution between `lower_bounds` and `upper_bounds`
    (reference `base.py:747-800`): misfit and gradient are zero inside the
    bounds (one memset on the device), +inf outside through misfit_bounds;
    the sampler keeps every chain inside them by reflection."""

    def __init__(self, lower_bounds, upper_bounds):
        self.name = "uniform distribution"
        lower = _numpy.asarray(lower_bounds, dtype=_numpy.float64)
        lower = _numpy.resize(lower, (lower.size, 1))
        upper = _numpy.asarray(upper_bounds, dtype=_numpy.float64)
        upper = _numpy.resize(upper, (upper.size, 1))
        self.dimensions = int(lower.size)
        self.update_bounds(lower, upper)

    def _device_misfit(self, M, out, accumulate, dtype, stream):
        if not accumulate:
            _lib.call("hmc_fill_zero", out.data_ptr(), out.numel() * out.element_size(), stream)

    def _device_gradient(self, M, out, accumulate, dtype, stream):
        if not accumulate:
            _lib.call("hmc_fill_zero", out.data_ptr(), out.numel() * out.element_size(), stream)

    def generate(self, repeat=1, rng=_numpy.random.default_rng()) -> _numpy.ndarray:
        return rng.uniform(self.lower_bounds, self.upper_bounds, (self.dimensions, repeat))

    @staticmethod
    def create_default(dimensions: int) -> "Uniform":
        lower = _numpy.random.rand(dimensions, 1) * 5 - 10
        upper = _numpy.random.rand(dimensions, 1) * 5 + 10
        return Uniform(lower, upper)


class AdditiveDistribution(_AbstractDistribution):
    """Sum of misfits and gradients of several distributions, with bounds
    collapsed to the tightest set (reference `base.py:1005-1142`)."""

    def __init__(self, list_of_distributions: _List[_AbstractDistribution], lower_bounds=None, upper_bounds=None):
        self.name = "additive distribution"
        self.dimensions = list_of_distributions[0].dimensions
        self.separate_distributions = list(list_of_distributions)
        for dist in self.separate_distributions:
            assert dist.dimensions == self.dimensions
        self.lower_bounds = lower_bounds
        self.upper_bounds = upper_bounds
        self.collapse_bounds()

    @property
    def single_dtype(self):
        dts = {d.single_dtype for d in self.separate_distributions}
        return "float32" if "float32" in dts else "float64"

    @property
    def graph_safe(self):
        return all(d.graph_safe for d in self.separate_distributions)

    def misfit(self, coordinates):
        m = _column(coordinates, self.dimensions)
        x = self.misfit_batch(_dev.upload(m, self.single_dtype))
        const = sum(d.normalization_constant for d in self.separate_distributions)
        bounds = sum(d.misfit_bounds(m) for d in self.separate_distributions)
        return float(x.cpu()[0]) + const + bounds + self.misfit_bounds(m)

    def _device_misfit(self, M, out, accumulate, dtype, stream):
        for k, dist in enumerate(self.separate_distributions):
            dist._device_misfit(M, out, accumulate or k > 0, dtype, stream)

    def _device_gradient(self, M, out, accumulate, dtype, stream):
        for k, dist in enumerate(self.separate_distributions):
            dist._device_gradient(M, out, accumulate or k > 0, dtype, stream)

    def _device_misfit_after_gradient(self, M, out, accumulate, dtype, stream):
        for k, dist in enumerate(self.separate_distributions):
            dist._device_misfit_after_gradient(M, out, accumulate or k > 0, dtype, stream)

    def check_device_status(self):
        for dist in self.separate_distributions:
            dist.check_device_status()

    def collapse_bounds(self):
        for dist in self.separate_distributions:
            if dist.lower_bounds is not None:
                assert dist.lower_bounds.shape == (self.dimensions, 1)
                self.lower_bounds = (
                    dist.lower_bounds if self.lower_bounds is None else _numpy.maximum(self.lower_bounds, dist.lower_bounds)
                )
            if dist.upper_bounds is not None:
                assert dist.upper_bounds.shape == (self.dimensions, 1)
                self.upper_bounds = (
                    dist.upper_bounds if self.upper_bounds is None else _numpy.minimum(self.upper_bounds, dist.upper_bounds)
                )

    def add_distribution(self, distribution: _AbstractDistribution):
        assert distribution.dimensions == self.dimensions
        self.separate_distributions.append(distribution)
        self.collapse_bounds()


class BayesRule(AdditiveDistribution):
    """Unnormalised Bayes' rule: the sum of prior and likelihood misfits."""


# ---------------------------------------------------------------------------
class LinearMatrix(_AbstractDistribution):
    """Linear forward model G m = d with Gaussian data errors (reference
    `LinearMatrix.py:15-135`): dense or sparse G with a scalar or (n,1) data
    variance.  Full data covariances are not part of the HMC path built here
    and raise NotImplementedError.

    Precision follows the reference: G and d are rounded to `dtype` (default
    single) as the reference's `_LinearMatrix_*_simple_covariance` classes do
    (`LinearMatrix.py:148-177, 318-323`), while the premultiplied GtG, Gtd0 and
    dtd are formed in FP64 exactly as there (Gtd0 from the unrounded G).  FP64
    chains use the reference's formulas; FP32 chains use GtG for the gradient
    and the residual form for the misfit, with FP64 per-chain sums."""

    def __init__(self, G, d, data_covariance, dtype=None, premultiplication: bool = None, use_mkl: bool = False):
        d = _numpy.asarray(d)
        if not (d.ndim == 2 and d.shape == (d.size, 1)):
            raise ValueError("Didn't understand the data vector object. Should be a NumPy column vector.")
        self.dense = not _sparse.issparse(G)
        if self.dense and not (isinstance(G, _numpy.ndarray) and G.ndim == 2 and G.shape[0] == d.size):
            raise ValueError("Didn't understand the forward model matrix object.")
        if not self.dense and G.shape[0] != d.size:
            raise ValueError("Didn't understand the forward model matrix object.")
        self.dimensions = int(G.shape[1])
        self.n_data = int(d.size)
        if isinstance(data_covariance, (float, _numpy.floating)):
            var = _numpy.full((self.n_data, 1), float(data_covariance))
            scalar_variance = True
        elif isinstance(data_covariance, _numpy.ndarray) and data_covariance.shape == (d.size, 1):
            var = _numpy.asarray(data_covariance, dtype=_numpy.float64)
            scalar_variance = False
        elif isinstance(data_covariance, _numpy.ndarray) and data_covariance.shape == (d.size, d.size):
            raise NotImplementedError("full data covariance matrices are not on the GPU HMC path")
        else:
            raise ValueError("Didn't understand the data covariance object.")
        store = _numpy.dtype(dtype) if dtype is not None else _numpy.dtype(_numpy.single)
        self.storage_dtype = store
        if not scalar_variance:
            var = var.astype(store).astype(_numpy.float64)
        self.data_variance = var
        self.inv_var = 1.0 / var
        if self.dense:
            G = _numpy.asarray(G)
            self.G = G.astype(store).astype(_numpy.float64)
        else:
            Gc = _sparse.csr_matrix(G, dtype=store)
            Gc.sort_indices()
            self.G = Gc.astype(_numpy.float64)
        self.d = d.astype(store).astype(_numpy.float64)
        self.premultiplication = (
            premultiplication if premultiplication is not None else self.G.shape[0] > self.G.shape[1]
        )
        if self.premultiplication:
            iv = self.inv_var
            if self.dense:
                self.GtG = self.G.T @ (iv * self.G)
                self.Gtd0 = _numpy.asarray(G, dtype=_numpy.float64).T @ (iv * self.d)
            else:
                self.GtG = (self.G.T @ _sparse.diags(iv[:, 0]) @ self.G).toarray()
                self.Gtd0 = _sparse.csr_matrix(G).astype(_numpy.float64).T @ (iv * self.d)
            self.dtd = (self.d.T @ (iv * self.d)).item()

    def forward(self, coordinates):
        return self.G @ coordinates

    def _make_params(self, dtype):
        p = {}
        if self.dense:
            p["G"] = _dev.upload(self.G, dtype)
            if not self.premultiplication or dtype == "float32":
                p["Gt"] = _dev.upload(self.G.T, dtype)
        else:
            G = self.G
            Gt = self.G.T.tocsr()
            Gt.sort_indices()
            # the device kernels index the dense operand with these columns
            for A in (G, Gt):
                if A.nnz and not (0 <= int(A.indices.min()) and int(A.indices.max()) < A.shape[1]):
                    raise ValueError("sparse matrix column index out of range")
                if len(A.indptr) != A.shape[0] + 1 or int(A.indptr[-1]) != A.nnz or _numpy.any(_numpy.diff(A.indptr) < 0):
                    raise ValueError("malformed sparse row pointers")
            p["rp"], p["col"], p["val"] = _dev.upload_int32(G.indptr), _dev.upload_int32(G.indices), _dev.upload(G.data, dtype)
            p["trp"], p["tcol"], p["tval"] = (
                _dev.upload_int32(Gt.indptr),
                _dev.upload_int32(Gt.indices),
                _dev.upload(Gt.data, dtype),
            )
        p["data"] = _dev.upload(self.d[:, 0], dtype)
        p["iv"] = _dev.upload(self.inv_var[:, 0], dtype)
        if self.premultiplication:
            p["GtG"] = _dev.upload(self.GtG, dtype)
            p["Gtd0"] = _dev.upload(self.Gtd0[:, 0], dtype)
        return p

    def _tc_operands(self, C, device):
        """BF16 hi/lo operands of the tensor-core path for a batch of C chains."""
        from hmclab_gb300 import _dense_tc

        cache = self.__dict__.setdefault("_scratch_cache", {})
        key = ("tc", int(C))
        if key not in cache:
            cache[key] = _dense_tc.DenseOperands(self, C, device)
        return cache[key]

    def check_device_status(self):
        """The tensor-core contractions wait on tensor-copy barriers with a
        bound; raise DeviceTimeoutError if one of them ran out since the last
        check (synchronises with the device)."""
        for key, ops in list(self.__dict__.get("_scratch_cache", {}).items()):
            if isinstance(key, tuple) and key[0] == "tc":
                ops.check_status()

    def _csr_plan(self, C, device, stream):
        """Slab-staged FP32 products of the sparse G for C chains, with the
        launch shapes the autotuner picked (timed on the first call)."""
        from hmclab_gb300 import _csr

        cache = self.__dict__.setdefault("_scratch_cache", {})
        key = ("csr_slab", int(C))
        if key not in cache:
            cache[key] = _csr.CsrSlabPlan(self, C, device, stream)
        return cache[key]

    def _use_tc(self, dtype, C):
        from hmclab_gb300 import _dense_tc

        return dtype == "float32" and _dense_tc.usable(self, C)

    def _device_misfit(self, M, out, accumulate, dtype, stream):
        p = self._params(dtype)
        d, C = M.shape
        code = _dev.dtype_code(dtype)
        if self._use_tc(dtype, C):
            self._tc_operands(C, M.device).misfit(M, out, accumulate, stream)
            return
        if self.premultiplication and dtype == "float64":
            work = self._scratch("work", (d, C), dtype, M.device)
            _lib.call("hmc_dense_premul_misfit", code, d, C, M.data_ptr(), p["GtG"].data_ptr(), p["Gtd0"].data_ptr(),
                      float(self.dtd), work.data_ptr(), out.data_ptr(), int(accumulate), stream)
            return
        resid = self._scratch("resid", (self.n_data, C), dtype, M.device)
        if self.dense:
            _lib.call("hmc_dense_resid_misfit", code, self.n_data, d, C, M.data_ptr(), p["G"].data_ptr(),
                      p["data"].data_ptr(), p["iv"].data_ptr(), resid.data_ptr(), out.data_ptr(), int(accumulate), stream)
        elif dtype == "float32":
            self._csr_plan(C, M.device, stream).misfit(M, resid, out, accumulate, stream)
        else:
            _lib.call("hmc_csr_misfit", code, self.n_data, d, C, M.data_ptr(), p["rp"].data_ptr(), p["col"].data_ptr(),
                      p["val"].data_ptr(), p["data"].data_ptr(), p["iv"].data_ptr(), resid.data_ptr(), out.data_ptr(),
                      int(accumulate), stream)

    def _device_gradient(self, M, out, accumulate, dtype, stream):
        p = self._params(dtype)
        d, C = M.shape
        code = _dev.dtype_code(dtype)
        if self.premultiplication and self._use_tc(dtype, C):
            self._tc_operands(C, M.device).gradient(M, out, accumulate, stream)
            return
        if self.premultiplication:
            _lib.call("hmc_dense_premul_gradient", code, d, C, M.data_ptr(), p["GtG"].data_ptr(),
                      p["Gtd0"].data_ptr(), out.data_ptr(), int(accumulate), stream)
            return
        resid = self._scratch("resid", (self.n_data, C), dtype, M.device)
        if self.dense:
            _lib.call("hmc_dense_resid_gradient", code, self.n_data, d, C, M.data_ptr(), p["G"].data_ptr(),
                      p["Gt"].data_ptr(), p["data"].data_ptr(), p["iv"].data_ptr(), resid.data_ptr(), out.data_ptr(),
                      int(accumulate), stream)
        elif dtype == "float32":
            self._csr_plan(C, M.device, stream).gradient(M, resid, out, accumulate, stream)
        else:
            _lib.call("hmc_csr_gradient", code, self.n_data, d, C, M.data_ptr(), p["rp"].data_ptr(),
                      p["col"].data_ptr(), p["val"].data_ptr(), p["trp"].data_ptr(), p["tcol"].data_ptr(),
                      p["tval"].data_ptr(), p["data"].data_ptr(), p["iv"].data_ptr(), resid.data_ptr(),
                      out.data_ptr(), int(accumulate), stream)

    @staticmethod
    def create_default(dimensions: int, dtype=_numpy.dtype("float64")) -> "LinearMatrix":
        return LinearMatrix(_numpy.eye(dimensions, dtype=dtype), _numpy.ones(dimensions)[:, None], 1.0, dtype=dtype)


# ---------------------------------------------------------------------------
class SourceLocation3D(_AbstractDistribution):
    """Earthquake location with straight rays in a homogeneous medium
    (reference `SourceLocation.py:369-713`).  Parameters are interleaved
    x1, y1, z1, t1, ..., xn, yn, zn, tn (, v when `infer_velocity`)."""

    name = "Earthquake source location in 3D"

    def __init__(self, receiver_array_x, receiver_array_y, receiver_array_z, observed_data, data_std,
                 infer_velocity: bool = True, medium_velocity=None):
        rx = _numpy.array(receiver_array_x, dtype=_numpy.float64).reshape(1, -1)
        ry = _numpy.array(receiver_array_y, dtype=_numpy.float64).reshape(1, -1)
        rz = _numpy.array(receiver_array_z, dtype=_numpy.float64).reshape(1, -1)
        self.receiver_array_x, self.receiver_array_y, self.receiver_array_z = rx, ry, rz
        self.infer_velocity = infer_velocity
        if not infer_velocity:
            assert medium_velocity is not None
            self.medium_velocity = float(_numpy.asarray(medium_velocity).reshape(-1)[0])
        else:
            self.medium_velocity = None
        observed_data = _numpy.array(observed_data, dtype=_numpy.float64)
        assert observed_data.size % rx.size == 0
        self.number_of_events = int(observed_data.size // rx.size)
        self.number_of_stations = int(rz.size)
        self.number_of_datums = self.number_of_events * self.number_of_stations
        shape = (self.number_of_events, self.number_of_stations)
        if observed_data.shape != shape:
            observed_data = observed_data.T
            assert observed_data.shape == shape, "Wrong shape for the observed data, not sure what to do."
        self.observed_data = observed_data
        if isinstance(data_std, float):
            data_std = _numpy.ones_like(observed_data) * data_std
        data_std = _numpy.array(data_std, dtype=_numpy.float64)
        if data_std.shape != shape:
            data_std = data_std.T
            assert data_std.shape == shape, "Wrong shape for the data uncertainty, not sure what to do."
        self.data_std = data_std
        self.dimensions = self.number_of_events * 4 + int(self.infer_velocity)

    def _make_params(self, dtype):
        return {
            "rx": _dev.upload(self.receiver_array_x[0], dtype),
            "ry": _dev.upload(self.receiver_array_y[0], dtype),
            "rz": _dev.upload(self.receiver_array_z[0], dtype),
            "obs": _dev.upload(self.observed_data, dtype),
            "iv": _dev.upload(1.0 / self.data_std**2, dtype),
        }

    def _args(self, M, dtype):
        p = self._params(dtype)
        return (_dev.dtype_code(dtype), self.number_of_events, self.number_of_stations, M.shape[1], M.data_ptr(),
                p["rx"].data_ptr(), p["ry"].data_ptr(), p["rz"].data_ptr(), p["obs"].data_ptr(), p["iv"].data_ptr(),
                int(self.infer_velocity), float(self.medium_velocity or 0.0))

    def _device_misfit(self, M, out, accumulate, dtype, stream):
        _lib.call("hmc_srcloc3d_misfit", *self._args(M, dtype), out.data_ptr(), int(accumulate), stream)

    def _device_gradient(self, M, out, accumulate, dtype, stream):
        _lib.call("hmc_srcloc3d_gradient", *self._args(M, dtype), out.data_ptr(), int(accumulate), stream)

    @staticmethod
    def split_vector(model_vector, velocity=None):
        if velocity is None:
            assert model_vector.size % 4 == 1
            return (model_vector[0:-1:4], model_vector[1:-1:4], model_vector[2:-1:4], model_vector[3:-1:4],
                    model_vector[-1])
        assert model_vector.size % 4 == 0
        return model_vector[0::4], model_vector[1::4], model_vector[2::4], model_vector[3::4], velocity

    @staticmethod
    def forward(x, y, z, T, v, receiver_array_x, receiver_array_y, receiver_array_z):
        return T + ((x - receiver_array_x) ** 2 + (y - receiver_array_y) ** 2 + (z - receiver_array_z) ** 2) ** 0.5 / v


# ---------------------------------------------------------------------------
class ElasticFullWaveform2D(_AbstractDistribution):
    """2-D elastic P-SV full-waveform misfit (reference
    `ElasticFullWaveform2D.py:12-226`), computed by the project's own FP32
    finite-difference kernels instead of psvWave, for C chains at once.

    `_input` is the path of a psvWave .ini file (read by
    `hmclab_gb300.fwi.read_ini`, as the reference hands it to psvWave), an
    `hmclab_gb300.fwi.ElasticConfig`, or another ElasticFullWaveform2D to
    copy; anything else raises ValueError, and so does a new object without
    observed data.  Observed records `ux_obs`, `uz_obs` are
    [shots][nt][receivers].  The misfit is 0.5 * sum (u - u_obs)^2 /
    data_std^2 / temperature.  Without `free_parameter_grid` the model vector
    is psvWave's: absolute (vp, vs, rho) of every cell (or npx x npz block)
    of the free-parameter region (`fwi.CellBasis`); `free_parameter_grid=
    [nx, nz]` / `make_blob` switches to Gaussian-blob amplitudes relative to
    the background (`fwi.BlobBasis`), m = [vp | vs | rho] either way.  The
    gradient is the exact derivative of the discrete misfit (chain rule
    through the parametrisation); `gradient_projection="least_squares"`
    applies the reference's (C^T C)^-1 C^T map to blob gradients instead
    (ElasticFullWaveform2D.py:159, 329-330).  With the configuration's
    `snapshot_interval` k > 1 (psvWave's; set before the first evaluation)
    the forward pass keeps the wavefield of every k-th step only and the
    gradient correlates at those steps, weighted by k: a k-times smaller
    store and cheaper adjoint steps, and a gradient that is exact up to the
    aliasing of the correlation's spectrum above 1 / (2 k dt) (the misfit
    stays exact, so HMC still targets the exact posterior)."""

    temperature: float = 1.0
    # the stencils run in FP32 only; single-vector calls use one FP32 chain
    single_dtype = "float32"
    # each shot is a CUDA graph of its own, replayed from the host
    graph_safe = False
    # forward stencils read their neighbourhoods from shared-memory tiles
    # staged by the tensor memory accelerator (chain counts that are a
    # multiple of 32); False selects the direct-load kernels, which give the
    # same records.  Set before the first evaluation.
    staged_tiles: bool = True

    def __init__(self, _input, ux_obs=None, uz_obs=None, temperature=None, omp_threads_override=None,
                 free_parameter_grid=None, data_std=1.0, background=None, gradient_projection="chain_rule"):
        from hmclab_gb300 import fwi as _fwi

        if isinstance(_input, ElasticFullWaveform2D):
            src = _input
            self.config = src.config
            self.background = src.background
            ux_obs = src.ux_obs if ux_obs is None else ux_obs
            uz_obs = src.uz_obs if uz_obs is None else uz_obs
            temperature = src.temperature if temperature is None else temperature
            data_std = src.data_std
            if free_parameter_grid is None and isinstance(src.blob, _fwi.BlobBasis):
                free_parameter_grid = [src.blob.nbx, src.blob.nbz]
            gradient_projection = src.gradient_projection
        elif isinstance(_input, (str, _fwi.ElasticConfig)) or hasattr(_input, "__fspath__"):
            self.config = _input if isinstance(_input, _fwi.ElasticConfig) else _fwi.ElasticConfig.from_ini(_input)
            self.background = background if background is not None else _fwi.background_model(self.config)
        else:
            raise ValueError(f"Incorrect initialization. Passed argument `{_input}` can not create an FWI object.")
        if ux_obs is None or uz_obs is None:
            raise ValueError("No passed observed data. Could not construct an inverse problem.")
        cfg = self.config
        self.ux_obs = _numpy.asarray(ux_obs, dtype=_numpy.float64).reshape(cfg.n_shots, cfg.nt, cfg.n_rec)
        self.uz_obs = _numpy.asarray(uz_obs, dtype=_numpy.float64).reshape(cfg.n_shots, cfg.nt, cfg.n_rec)
        self.temperature = 1.0 if temperature is None else float(temperature)
        self.data_std = float(data_std)
        self.gradient_projection = gradient_projection
        if free_parameter_grid is not None:
            self.make_blob(*free_parameter_grid)
        else:
            self.blob = _fwi.CellBasis(cfg, *cfg.cell_block)
            self.dimensions = self.blob.free_parameters

    @property
    def use_blob_par(self):
        from hmclab_gb300 import fwi as _fwi

        return isinstance(self.blob, _fwi.BlobBasis)

    def make_blob(self, nx, nz):
        from hmclab_gb300 import fwi as _fwi

        self.blob = _fwi.BlobBasis(self.config, nx, nz)
        self.dimensions = self.blob.free_parameters
        self.__dict__.pop("_param_cache", None)
        self.__dict__.pop("_scratch_cache", None)

    @property
    def weight(self):
        return 1.0 / (self.data_std**2 * self.temperature)

    def fine_model(self, m):
        """Physical (vp, vs, rho) fields [nz][nx] of a model vector (host)."""
        m = _numpy.asarray(m, dtype=_numpy.float64).reshape(3, -1)
        cfg = self.config
        return tuple((self.blob.to_physical(m[f]) + self.blob.base_field(self.background[f]).reshape(-1))
                     .reshape(cfg.nz, cfg.nx) for f in range(3))

    # ---- device parameters ------------------------------------------------
    def _make_params(self, dtype):
        cfg = self.config
        # the fields the parameters add to, on the simulation grid
        rows = cfg.extension_matrix_rows()
        bg = []
        for f in range(3):
            base = self.blob.base_field(self.background[f]).reshape(-1)
            full = cfg.extend(_numpy.asarray(self.background[f], _numpy.float64)).reshape(-1)
            bg.append(_numpy.where(rows >= 0, base[_numpy.maximum(rows, 0)], full))
        obs = _numpy.stack([self.ux_obs, self.uz_obs], axis=-1)  # shots, nt, rec, 2
        rec_map = -_numpy.ones((cfg.nzc, cfg.nxc), _numpy.int32)
        for r, (x, z) in enumerate(zip(cfg.rec_x, cfg.rec_z)):
            rec_map[z, x] = r
        p = {
            "bg": [_dev.upload(b, "float32") for b in bg],
            "taper": _dev.upload(cfg.taper(), "float32"),
            "rec_map": _dev.upload_int32(rec_map),
            "obs": _dev.upload(obs, "float32"),
            "stf_host": _numpy.ascontiguousarray(cfg.ricker(), dtype=_numpy.float32),
            # per shot: the source records (kept alive beside the wavelets
            # they point to) of configurations with more than one explosion
            "sources": [self._source_array(k) for k in range(cfg.n_shots)],
        }
        if self.use_blob_par:
            Bs = self.blob.simulation_basis()  # [cells][blobs]
            p["B"] = _dev.upload(Bs, "float32")
            p["Bt"] = _dev.upload(_numpy.ascontiguousarray(Bs.T), "float32")
            if self.gradient_projection == "least_squares":
                B = self.blob.B
                p["proj"] = _dev.upload(_numpy.linalg.inv(B.T @ B), "float32")
        else:
            ptr, cells = self.blob.gradient_segments()
            p["map"] = _dev.upload_int32(self.blob.simulation_map())
            p["seg_ptr"] = _dev.upload_int32(ptr)
            p["seg_cells"] = _dev.upload_int32(cells)
        return p

    def _source_array(self, shot):
        """(hmc_fwi_source array, wavelets) of one shot."""
        import ctypes

        srcs = self.config.shots[shot]
        stf = _numpy.ascontiguousarray(self.config.shot_wavelets(shot), dtype=_numpy.float32)
        arr = (_lib.HmcFwiSource * len(srcs))()
        for k, q in enumerate(srcs):
            arr[k].x, arr[k].z = q.x, q.z
            arr[k].mxx, arr[k].mzz, arr[k].mxz = q.mxx, q.mzz, q.mxz
            arr[k].stf_host = stf[k].ctypes.data_as(ctypes.c_void_p).value
        return arr, stf

    def _workspace(self, C, device, with_gradient):
        import torch

        cache = self.__dict__.setdefault("_scratch_cache", {})
        key = ("fwi", int(C))
        ws = cache.get(key)
        cfg = self.config
        cells = cfg.nzc * cfg.nxc
        if ws is None:
            z = lambda *shape: torch.zeros(shape, dtype=torch.float32, device=device)  # noqa: E731
            ws = {name: z(cells, C) for name in ("vp", "vs", "rho", "bx", "bz", "l2m", "lam", "muxz", "vx", "vz",
                                                 "sxx", "szz", "sxz")}
            ws["rec"] = z(cfg.n_shots * cfg.nt * cfg.n_rec * 2 * C)
            ws["partial"] = torch.zeros(64 * C, dtype=torch.float64, device=device)
            ws["status"] = torch.zeros(1, dtype=torch.int32, device=device)
            cache[key] = ws
        if with_gradient and "store" not in ws:
            z = lambda *shape: torch.zeros(shape, dtype=torch.float32, device=device)  # noqa: E731
            for name in ("avx", "avz", "asxx", "aszz", "asxz", "g_bx", "g_bz", "g_l2m", "g_lam", "g_muxz", "g_vp",
                         "g_vs", "g_rho", "t1", "t2", "t3", "t4", "t5"):
                ws[name] = z(cells, C)
            k = max(int(cfg.snapshot_interval), 1)
            planes = 2 * cfg.nt if k == 1 else 4 * (-(-cfg.nt // k))
            ws["store"] = z(planes * cells * C)
            ws["resid"] = z(cfg.nt * cfg.n_rec * 2 * C)
            if self.use_blob_par:
                ws["gtmp"] = z(self.blob.n_blobs, C)
                ws["proj_work"] = z(64 * self.blob.n_blobs * C)  # split-k partial products
        return ws

    def _descriptor(self, ws, C):
        from hmclab_gb300 import _lib as L

        cfg, p = self.config, self._params("float32")
        d = L.HmcFwi()
        d.nx, d.nz, d.nt, d.nrec, d.chains = cfg.nxc, cfg.nzc, cfg.nt, cfg.n_rec, C
        d.h, d.dt, d.w = cfg.h, cfg.dt, self.weight
        d.snapshot_interval = max(int(cfg.snapshot_interval), 1)
        d.taper, d.rec_map, d.obs = p["taper"].data_ptr(), p["rec_map"].data_ptr(), p["obs"].data_ptr()
        d.stf_host = p["stf_host"].ctypes.data
        for name in ("rho", "vp", "vs", "bx", "bz", "l2m", "lam", "muxz", "vx", "vz", "sxx", "szz", "sxz", "rec",
                     "partial", "status"):
            setattr(d, name, ws[name].data_ptr())
        for name in ("store", "resid", "avx", "avz", "asxx", "aszz", "asxz", "g_bx", "g_bz", "g_l2m", "g_lam",
                     "g_muxz", "t1", "t2", "t3", "t4", "t5"):
            if name in ws:
                setattr(d, name, ws[name].data_ptr())
        if not self.staged_tiles:
            d.status = None
        return d

    def _set_model(self, M, ws, stream):
        """Model vectors (3*nb, C) FP32 -> simulation-grid fields."""
        p = self._params("float32")
        nb, C = self.blob.n_blobs, M.shape[1]
        cells = self.config.nzc * self.config.nxc
        for f, name in enumerate(("vp", "vs", "rho")):
            if self.use_blob_par:
                _lib.call("hmc_gemm", _lib.HMC_F32, cells, C, nb, 1.0, p["B"].data_ptr(),
                          M[f * nb:(f + 1) * nb].data_ptr(), p["bg"][f].data_ptr(), ws[name].data_ptr(), 0, stream)
            else:
                _lib.call("hmc_fwi_cell_model", cells, C, p["map"].data_ptr(), M[f * nb:(f + 1) * nb].data_ptr(),
                          p["bg"][f].data_ptr(), ws[name].data_ptr(), stream)

    def _shot_graph(self, ws, C, shot, store_and_adjoint):
        """CUDA graph of one shot's 2*nt half-step launches (and its adjoint),
        captured once per workspace on a private stream and replayed on the
        caller's stream."""
        import ctypes

        import torch

        graphs = ws.setdefault("graphs", {})
        key = (shot, bool(store_and_adjoint), float(self.weight))
        if key not in graphs:
            d = self._descriptor(ws, C)
            ws.setdefault("descriptors", []).append(d)  # keep the struct alive with the graph
            ref = ctypes.byref(d)
            cap = torch.cuda.Stream()
            h = cap.cuda_stream
            _lib.call("hmc_graph_begin", h)
            try:
                if self.config.explosive_shots:
                    sx, sz = self.config.src[shot]
                    _lib.call("hmc_fwi_forward_shot", ref, shot, sx, sz, int(store_and_adjoint), h)
                else:
                    arr, _ = self._params("float32")["sources"][shot]
                    _lib.call("hmc_fwi_forward_shot_sources", ref, shot, arr, len(arr), int(store_and_adjoint), h)
                if store_and_adjoint:
                    _lib.call("hmc_fwi_adjoint_shot", ref, shot, h)
            finally:
                ex = ctypes.c_void_p()
                rc = _lib.load().hmc_graph_end(h, ctypes.byref(ex))
            _lib.check(rc, "hmc_graph_end")
            graphs[key] = ex
        return graphs[key]

    def _forward_all(self, M, ws, stream, store_and_adjoint):
        import ctypes

        cfg = self.config
        C = M.shape[1]
        d = self._descriptor(ws, C)
        ref = ctypes.byref(d)
        self._set_model(M, ws, stream)
        _lib.call("hmc_fwi_prepare", ref, stream)
        if store_and_adjoint:
            _lib.call("hmc_fwi_zero_gradients", ref, stream)
        for k in range(cfg.n_shots):
            _lib.call("hmc_graph_launch", self._shot_graph(ws, C, k, store_and_adjoint), stream)
        return d

    def _check_dtype(self, dtype):
        if dtype != "float32":
            raise NotImplementedError("the elastic finite-difference kernels run in FP32 (float32 chains)")

    def check_device_status(self):
        """The forward stencils stage their tiles through bounded barrier
        waits; a wait that ran out sets the workspace's status word."""
        from hmclab_gb300.Helpers.CustomExceptions import DeviceTimeoutError

        for key, ws in self.__dict__.get("_scratch_cache", {}).items():
            st = ws.get("status") if isinstance(ws, dict) else None
            if st is not None and int(st.cpu()[0]) != 0:
                st.zero_()
                raise DeviceTimeoutError("elastic stencil tile load timed out (bounded wait expired)")

    def _device_misfit(self, M, out, accumulate, dtype, stream):
        import ctypes

        self._check_dtype(dtype)
        ws = self._workspace(M.shape[1], M.device, False)
        d = self._forward_all(M, ws, stream, False)
        _lib.call("hmc_fwi_misfit", ctypes.byref(d), self.config.n_shots, out.data_ptr(), int(accumulate), stream)

    def _device_misfit_after_gradient(self, M, out, accumulate, dtype, stream):
        """The misfit of the records the gradient's forward simulation left
        in the workspace (the reduction only: no second forward)."""
        import ctypes

        self._check_dtype(dtype)
        d = getattr(self, "_last_gradient_descriptor", None)
        if d is None or d.chains != M.shape[1]:
            return self._device_misfit(M, out, accumulate, dtype, stream)
        _lib.call("hmc_fwi_misfit", ctypes.byref(d), self.config.n_shots, out.data_ptr(), int(accumulate), stream)

    def _device_gradient(self, M, out, accumulate, dtype, stream):
        import ctypes

        self._check_dtype(dtype)
        C = M.shape[1]
        ws = self._workspace(C, M.device, True)
        d = self._forward_all(M, ws, stream, True)
        self._last_gradient_descriptor = d
        _lib.call("hmc_fwi_param_gradient", ctypes.byref(d), ws["g_rho"].data_ptr(), ws["g_vp"].data_ptr(),
                  ws["g_vs"].data_ptr(), 0, stream)
        p = self._params("float32")
        nb = self.blob.n_blobs
        cells = self.config.nzc * self.config.nxc
        for f, name in enumerate(("g_vp", "g_vs", "g_rho")):
            dst = out[f * nb:(f + 1) * nb]
            if not self.use_blob_par:
                _lib.call("hmc_fwi_cell_gradient", nb, C, p["seg_ptr"].data_ptr(), p["seg_cells"].data_ptr(),
                          ws[name].data_ptr(), dst.data_ptr(), int(accumulate), stream)
                continue
            work, nwork = ws["proj_work"].data_ptr(), ws["proj_work"].numel()
            if self.gradient_projection == "least_squares":
                _lib.call("hmc_gemm_splitk", _lib.HMC_F32, nb, C, cells, 1.0, p["Bt"].data_ptr(), ws[name].data_ptr(),
                          ws["gtmp"].data_ptr(), 0, work, nwork, stream)
                _lib.call("hmc_gemm", _lib.HMC_F32, nb, C, nb, 1.0, p["proj"].data_ptr(), ws["gtmp"].data_ptr(),
                          None, dst.data_ptr(), int(accumulate), stream)
            else:
                _lib.call("hmc_gemm_splitk", _lib.HMC_F32, nb, C, cells, 1.0, p["Bt"].data_ptr(), ws[name].data_ptr(),
                          dst.data_ptr(), int(accumulate), work, nwork, stream)

    def synthetic_records(self, m):
        """Receiver records (ux, uz), each [shots][nt][receivers], of one blob
        model vector, computed by the device forward (FP32)."""
        import torch

        cfg = self.config
        M = _dev.upload(_numpy.asarray(m, _numpy.float64).reshape(self.dimensions, 1), "float32")
        ws = self._workspace(1, M.device, False)
        s = torch.cuda.current_stream(M.device)
        self._forward_all(M, ws, s.cuda_stream, False)
        s.synchronize()
        r = ws["rec"].double().cpu().numpy().reshape(cfg.n_shots, cfg.nt, cfg.n_rec, 2)
        return r[..., 0].copy(), r[..., 1].copy()

    def last_misfit(self, C, out, stream=None):
        """Misfit of the model of the last gradient call (its forward records
        are still in the workspace)."""
        import ctypes

        ws = self._workspace(C, out.device, False)
        d = self._descriptor(ws, C)
        _lib.call("hmc_fwi_misfit", ctypes.byref(d), self.config.n_shots, out.data_ptr(), 0,
                  _dev.stream_handle(stream))

    def get_model_vector(self):
        """Model vector of the background (reference
        `ElasticFullWaveform2D.py:186-190`): the background's vp, vs, rho per
        free cell, or zero blob amplitudes."""
        return self.blob.background_vector(self.background)[:, None]

    def generate(self, repeat=1, rng=_numpy.random.default_rng()) -> _numpy.ndarray:
        raise _InvalidCaseError("Can't generate samples from non-analytic distributions.")

    @staticmethod
    def create_default(dimensions: int, ini_file=None, omp_threads_override: int = 0) -> "ElasticFullWaveform2D":
        """The reference's default problem (`ElasticFullWaveform2D.py:85-128`):
        the configuration of `ini_file` (a psvWave .ini; default: this
        package's 200 x 100-cell ElasticConfig), a target with a circular
        anomaly of radius 15 (in the grid's length unit) at the middle of
        the model (vp and vs -10 %, rho +10 %) and its noise-free records,
        simulated on the GPU, as observed data.  `dimensions` must equal the
        free parameters of the cell parametrisation (else InvalidCaseError)."""
        from hmclab_gb300 import fwi as _fwi

        cfg = _fwi.ElasticConfig() if ini_file is None else _fwi.ElasticConfig.from_ini(ini_file)
        zeros = _numpy.zeros((cfg.n_shots, cfg.nt, cfg.n_rec))
        model = ElasticFullWaveform2D(cfg, zeros, zeros, omp_threads_override=omp_threads_override)
        if model.dimensions != dimensions:
            raise _InvalidCaseError(f"{model.dimensions} is not equal to {dimensions}")
        X, Z = cfg.cell_centres()
        circle = _numpy.hypot(X - 0.5 * (X.max() + X.min()), Z - 0.5 * (Z.max() + Z.min())) < 15
        vp, vs, rho = (_numpy.asarray(f, _numpy.float64) for f in model.background)
        target = (vp * (1 - 0.1 * circle), vs * (1 - 0.1 * circle), rho * (1 + 0.1 * circle))
        m_target = _numpy.concatenate([model.blob.fit(target[f]) for f in range(3)])
        ux, uz = model.synthetic_records(m_target)
        return ElasticFullWaveform2D(cfg, ux, uz, omp_threads_override=omp_threads_override)
