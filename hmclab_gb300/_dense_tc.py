"""Host side of the tensor-core dense contraction (csrc/dense_tc.cu).

`DenseOperands` holds, for one dense LinearMatrix and a chain count C, the
BF16 hi/lo splits of GtG and G (row pitch a multiple of 64), two ping-pong
chain-major operand buffers Q[C][ld] (hi/lo), the per-tile misfit partials
and a device status word.  `FusedDenseStep` drives one proposal of the
sampler with the gradient, the prior and the leapfrog kick/drift fused in
the epilogue of each contraction.
"""
import numpy as _np

from hmclab_gb300 import _device as _dev
from hmclab_gb300 import _lib
from hmclab_gb300.Helpers.CustomExceptions import DeviceTimeoutError

PRIOR_NONE, PRIOR_NORMAL, PRIOR_LAPLACE = 0, 1, 2


def _pad64(n):
    return (int(n) + 63) // 64 * 64


def usable(lik, C):
    """Whether the tensor-core path applies to this LinearMatrix and batch."""
    return lik.dense and lik.dimensions >= 64 and C >= 1


class DenseOperands:
    def __init__(self, lik, C, device):
        import torch

        self.lik = lik
        self.C = int(C)
        self.d = lik.dimensions
        self.n = lik.n_data
        self.ld = _pad64(self.d)
        bf16 = torch.bfloat16
        p = lik._params("float32")
        h = _dev.stream_handle()
        # Centre of the operands: the least-squares point of the likelihood,
        # so that the split products act on q - c, which stays small where
        # the chains live, and G c - d, GtG c - Gtd0 are formed in FP64 once.
        c = _np.linalg.lstsq(lik.G, lik.d, rcond=None)[0]
        c32 = c.astype(_np.float32).astype(_np.float64)
        self.center = _dev.upload(c32[:, 0], "float32", device)
        if lik.premultiplication:
            self.gtg_hi = torch.empty((self.d, self.ld), dtype=bf16, device=device)
            self.gtg_lo = torch.empty_like(self.gtg_hi)
            _lib.call("hmc_split_bf16", self.d, self.d, p["GtG"].data_ptr(), self.ld, self.gtg_hi.data_ptr(),
                      self.gtg_lo.data_ptr(), h)
            # GtG (q - c) - (Gtd0 - GtG c) = GtG q - Gtd0
            self.gtd0 = _dev.upload((lik.Gtd0 - lik.GtG @ c32)[:, 0], "float32", device)
        self.g_hi = torch.empty((self.n, self.ld), dtype=bf16, device=device)
        self.g_lo = torch.empty_like(self.g_hi)
        _lib.call("hmc_split_bf16", self.n, self.d, p["G"].data_ptr(), self.ld, self.g_hi.data_ptr(),
                  self.g_lo.data_ptr(), h)
        # G (q - c) - (d - G c) = G q - d, with G as stored (rounded to the storage dtype)
        self.data = _dev.upload((lik.d - lik.G @ c32)[:, 0], "float32", device)
        self.iv = p["iv"]
        self.q_hi = [torch.zeros((self.C, self.ld), dtype=bf16, device=device) for _ in range(2)]
        self.q_lo = [torch.zeros((self.C, self.ld), dtype=bf16, device=device) for _ in range(2)]
        self.partial = torch.zeros((int(_lib.load().hmc_tc_partials_size(self.n, self.C)),), dtype=torch.float64,
                                   device=device)
        self.status = torch.zeros((1,), dtype=torch.int32, device=device)
        # the splits above ran on the current stream; make them visible to any stream
        torch.cuda.current_stream(device).synchronize()

    def split(self, M, buf, stream):
        _lib.call("hmc_split_bf16_transpose", self.d, self.C, M.data_ptr(), self.center.data_ptr(), self.ld,
                  self.q_hi[buf].data_ptr(), self.q_lo[buf].data_ptr(), stream)

    def gradient(self, M, out, accumulate, stream):
        """out (+)= GtG M - Gtd0 on the tensor cores (premultiplied form)."""
        self.split(M, 0, stream)
        _lib.call("hmc_tc_gradient", self.d, self.d, self.C, self.gtg_hi.data_ptr(), self.gtg_lo.data_ptr(), self.ld,
                  self.q_hi[0].data_ptr(), self.q_lo[0].data_ptr(), self.ld, self.gtd0.data_ptr(), out.data_ptr(),
                  int(accumulate), self.status.data_ptr(), stream)

    def misfit_from(self, buf, out, accumulate, stream):
        _lib.call("hmc_tc_resid_misfit", self.n, self.d, self.C, self.g_hi.data_ptr(), self.g_lo.data_ptr(), self.ld,
                  self.q_hi[buf].data_ptr(), self.q_lo[buf].data_ptr(), self.ld, self.data.data_ptr(),
                  self.iv.data_ptr(), self.partial.data_ptr(), out.data_ptr(), int(accumulate),
                  self.status.data_ptr(), stream)

    def misfit(self, M, out, accumulate, stream):
        """out (+)= 0.5 sum (G M - d)^2 / var with FP64 per-chain sums."""
        self.split(M, 0, stream)
        self.misfit_from(0, out, accumulate, stream)

    def check_status(self):
        s = int(self.status.cpu()[0])
        if s != 0:
            self.status.zero_()
            raise DeviceTimeoutError(f"tensor-core contraction reported status {s} (a bounded wait expired)")


# the fused step and the two-pass step (same arguments, bitwise-equal results)
_STEP_ENTRIES = ("hmc_tc_step", "hmc_tc_step_split")


class FusedDenseStep:
    """One proposal of the sampler for BayesRule([diagonal prior, dense
    premultiplied LinearMatrix]) in FP32 with unit or diagonal mass."""

    def __init__(self, sampler, lik, prior):
        from hmclab_gb300 import Distributions as D

        self.smp = sampler
        self.lik = lik
        self.prior = prior
        self.ops = lik._tc_operands(sampler.chains, sampler.device)
        if prior is None:
            self.kind, self.mean, self.w = PRIOR_NONE, None, None
        elif isinstance(prior, D.Normal):
            pp = prior._params("float32")
            self.kind, self.mean, self.w = PRIOR_NORMAL, pp["mean"], pp["iv"]
        else:
            pp = prior._params("float32")
            self.kind, self.mean, self.w = PRIOR_LAPLACE, pp["mean"], pp["iw"]
        self.cur = 0
        self.entry = self._choose_entry()

    def _call(self, entry, kick, drift, cur, nxt, h):
        o = self.ops
        _lib.call(entry, self.smp._state_ref, o.gtg_hi.data_ptr(), o.gtg_lo.data_ptr(), o.ld,
                  o.q_hi[cur].data_ptr(), o.q_lo[cur].data_ptr(), o.q_hi[nxt].data_ptr(), o.q_lo[nxt].data_ptr(),
                  o.ld, o.center.data_ptr(), o.gtd0.data_ptr(), self.kind, _dev.ptr(self.mean), _dev.ptr(self.w),
                  float(kick), float(drift), o.status.data_ptr(), h)

    def _choose_entry(self):
        """The fused step (contraction with the update in its epilogue) or
        the two-pass step (contraction, then a streaming update), whichever
        the autotuner times faster for this shape; both give bitwise-equal
        results.  Timed with zero kick and drift on the current model, which
        leaves p, q and the flags as they are and only writes the next
        operand buffer, rewritten by the first real step."""
        from hmclab_gb300 import autotune as _autotune

        h = self.smp.stream.cuda_stream
        self.ops.split(self.smp.q_cur, self.cur, h)
        nxt = 1 - self.cur
        shape = {"d": int(self.smp.dimensions), "C": int(self.smp.chains), "prior": int(self.kind),
                 "mass": int(self.smp.mass_matrix.kind)}
        (v,) = _autotune.choose("tc_step", shape, [(0,), (1,)],
                                lambda c: self._call(_STEP_ENTRIES[c[0]], 0.0, 0.0, self.cur, nxt, h),
                                self.smp.device, h)
        return _STEP_ENTRIES[v]

    @staticmethod
    def applies(sampler):
        from hmclab_gb300 import Distributions as D

        dist = sampler.distribution
        if sampler.dtype != "float32" or sampler.mass_matrix.kind == _lib.HMC_MASS_FULL:
            return None
        if getattr(sampler, "beta", None) is not None:  # tempered chains: the fused epilogue kicks at beta = 1
            return None
        parts = dist.separate_distributions if isinstance(dist, D.AdditiveDistribution) else [dist]
        liks = [p for p in parts if isinstance(p, D.LinearMatrix)]
        priors = [p for p in parts if not isinstance(p, D.LinearMatrix)]
        if len(liks) != 1 or len(priors) > 1:
            return None
        lik = liks[0]
        if not (lik.premultiplication and usable(lik, sampler.chains)):
            return None
        if priors:
            pr = priors[0]
            ok = (isinstance(pr, D.Normal) and pr.diagonal) or isinstance(pr, D.Laplace)
            if not ok or type(pr) not in (D.Normal, D.Laplace):
                return None
            return FusedDenseStep(sampler, lik, pr)
        return FusedDenseStep(sampler, lik, None)

    def after_begin(self, h):
        self.ops.split(self.smp.q, self.cur, h)

    def kick_drift(self, kick, drift, h):
        nxt = 1 - self.cur
        self._call(self.entry, kick, drift, self.cur, nxt, h)
        self.cur = nxt

    def drift_only(self, drift, h):
        _lib.call("hmc_kick_drift", self.smp._state_ref, 0.0, float(drift), h)
        self.ops.split(self.smp.q, self.cur, h)

    def misfit(self, h):
        smp = self.smp
        if self.prior is not None:
            self.prior._device_misfit(smp.q, smp.x_prop, False, "float32", h)
        self.ops.misfit_from(self.cur, smp.x_prop, self.prior is not None, h)
