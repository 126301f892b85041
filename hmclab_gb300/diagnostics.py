"""Mixing diagnostics computed on the device from the sampler's sample ring.

`ess(samples)`: split-chain multi-chain effective sample size per parameter
(Gelman et al., BDA3 section 11.5, Geyer's initial monotone sequence), with
`rank_normalize=True` the rank-normalised bulk-ESS and split-R-hat of
Vehtari et al. (2021, section 4.1), which do not change under monotone
transformations of a parameter and stay finite for heavy-tailed draws;
`moments(samples)`: per-parameter mean and standard deviation over all draws
and chains; `moment_error(...)`: max over parameters of |mean - ref| / ref_std
and |std - ref_std| / ref_std.  Samples are device tensors [N][d][C].
"""
import numpy as _numpy

from hmclab_gb300 import _device as _dev
from hmclab_gb300 import _lib


def rank_normalize(samples, stream=None):
    """Normal scores of the pooled ranks of every parameter's draws (FP64
    device tensor of the samples' shape [N][d][C])."""
    N, d, C = samples.shape
    z = _dev.empty((N, d, C), "float64", samples.device)
    _lib.call("hmc_rank_normalize", _dev.dtype_code(_dev.normalise_dtype(samples.dtype)), N, d, C,
              samples.data_ptr(), z.data_ptr(), _dev.stream_handle(stream))
    return z


_rank_normalize = rank_normalize  # the name ess() can reach under its keyword of the same name


def ess(samples, lags=None, stream=None, return_rhat=False, rank_normalize=False):
    """ESS of every parameter (numpy float64 array of length d).

    Entries whose autocorrelation window `lags` was too short to truncate are
    returned as the (negative, flagged) value computed on that window; callers
    wanting a lower bound take abs().  `rank_normalize=True` computes both
    on the normal scores of the pooled ranks (bulk-ESS, rank split-R-hat)."""
    if rank_normalize:
        samples = _rank_normalize(samples, stream)
    N, d, C = samples.shape
    n = N // 2
    if lags is None:
        lags = min(n, 200)
    lags = max(2, min(int(lags), n))
    work = _dev.empty((_lib.load().hmc_ess_work_size(d, C, lags),), "float64", samples.device)
    out = _dev.empty((d,), "float64", samples.device)
    rh = _dev.empty((d,), "float64", samples.device) if return_rhat else None
    dt = _dev.normalise_dtype(samples.dtype)
    for i0 in range(0, d, 65535):
        i1 = min(d, i0 + 65535)
        # a parameter slice of [N][d][C] is strided; run per slice on a contiguous copy when d is split
        x = samples if (i0 == 0 and i1 == d) else samples[:, i0:i1].contiguous()
        _lib.call("hmc_ess", _dev.dtype_code(dt), N, i1 - i0, C, x.data_ptr(), lags, work.data_ptr(),
                  out[i0:i1].data_ptr(), _dev.ptr(rh[i0:i1]) if rh is not None else None, _dev.stream_handle(stream))
    e = out.cpu().numpy()
    if return_rhat:
        return e, rh.cpu().numpy()
    return e


def moments(samples, stream=None):
    N, d, C = samples.shape
    mean = _dev.empty((d,), "float64", samples.device)
    var = _dev.empty((d,), "float64", samples.device)
    _lib.call("hmc_moments", _dev.dtype_code(_dev.normalise_dtype(samples.dtype)), N, d, C, samples.data_ptr(),
              mean.data_ptr(), var.data_ptr(), _dev.stream_handle(stream))
    return mean.cpu().numpy(), _numpy.sqrt(_numpy.maximum(var.cpu().numpy(), 0.0))


def moment_error(mean, std, ref_mean, ref_std):
    """max_i |mean_i - ref_i| / ref_std_i and max_i |std_i - ref_std_i| / ref_std_i."""
    ref_mean = _numpy.asarray(ref_mean, float).reshape(-1)
    ref_std = _numpy.asarray(ref_std, float).reshape(-1)
    return float(_numpy.max(_numpy.abs(mean - ref_mean) / ref_std)), float(_numpy.max(_numpy.abs(std - ref_std) / ref_std))
