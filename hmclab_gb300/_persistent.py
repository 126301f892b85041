"""Persistent fused proposals (csrc/persistent.cu) for small dense
linear-Gaussian posteriors: whole blocks of proposals in one launch, one warp
per chain, with an autotuner that picks the chains per block.

Applies when the target is a premultiplied dense `LinearMatrix` with
d <= 128, alone or in a `BayesRule` with one diagonal `Normal` or `Laplace`
prior, the mass matrix is unit, diagonal or full (its inverse and Cholesky
factor then share the block's shared memory with GtG), and the run has no
bounds, no autotuning, no temperatures, no surrogate and no training set.
"""
import ctypes as _ct

from hmclab_gb300 import _lib

MAX_D = 128
_WARPS = (1, 2, 4, 8, 16)
_SMEM = 227 * 1024


def _smem(d, full, warps, esize):
    """Shared memory of one block: GtG (and M^-1, L for a full mass) with an
    odd row stride, plus one vector per warp (as in csrc/persistent.cu)."""
    return ((3 if full else 1) * d * (d | 1) + warps * d) * esize
# chosen launch shapes, per (dimension, chains, dtype, mass, prior, schedule length)
_tuned = {}


def _schedule(first, steps):
    s = _lib.HmcSchedule()
    s.first_drift = float(first)
    s.steps = len(steps)
    for k, (needs_grad, kick, drift) in enumerate(steps):
        s.gradient[k] = int(bool(needs_grad))
        s.kick[k] = float(kick)
        s.drift[k] = float(drift)
    return s


class PersistentDense:
    @staticmethod
    def applies(sampler):
        from hmclab_gb300 import Distributions as D

        if getattr(sampler, "use_persistent", None) is False:
            return None
        full = sampler.mass_matrix.kind == _lib.HMC_MASS_FULL
        esize = 8 if sampler.dtype == "float64" else 4
        if sampler.dimensions > MAX_D or _smem(sampler.dimensions, full, 1, esize) > _SMEM:
            return None
        if sampler.autotuning or getattr(sampler, "beta", None) is not None:
            return None
        if sampler.surrogate is not None or sampler.training_set is not None:
            return None
        if sampler.lower is not None or sampler.upper is not None:
            return None
        first, steps = sampler._schedule
        if len(steps) > _lib.HMC_SCHEDULE_MAX:
            return None
        dist = sampler.distribution
        parts = dist.separate_distributions if isinstance(dist, D.AdditiveDistribution) else [dist]
        liks = [p for p in parts if type(p) is D.LinearMatrix]
        others = [p for p in parts if type(p) is not D.LinearMatrix]
        if len(liks) != 1 or len(others) > 1 or len(parts) != len(liks) + len(others):
            return None
        lik = liks[0]
        if not (lik.dense and lik.premultiplication):
            return None
        prior = others[0] if others else None
        if prior is not None:
            if not ((type(prior) is D.Normal and prior.diagonal) or type(prior) is D.Laplace):
                return None
            if prior.lower_bounds is not None or prior.upper_bounds is not None:
                return None
        return PersistentDense(sampler, lik, prior)

    def __init__(self, sampler, lik, prior):
        from hmclab_gb300 import Distributions as D

        self.smp = sampler
        dt = sampler.dtype
        p = lik._params(dt)
        self.GtG, self.Gtd0, self.dtd = p["GtG"], p["Gtd0"], float(lik.dtd)
        self.prior_kind, self.pmean, self.pw = 0, None, None
        if prior is not None:
            pp = prior._params(dt)
            if type(prior) is D.Normal:
                self.prior_kind, self.pmean, self.pw = 1, pp["mean"], pp["iv"]
            else:
                self.prior_kind, self.pmean, self.pw = 2, pp["mean"], pp["iw"]
        first, steps = sampler._schedule
        self.schedule = _schedule(first, steps)
        self._sched_ref = _ct.byref(self.schedule)
        self.key = (sampler.dimensions, sampler.chains, dt, sampler.mass_matrix.kind, self.prior_kind, len(steps))
        self.warps = _tuned.get(self.key)

    def _call(self, n, warps, dry, h):
        _lib.call("hmc_persistent_dense", self.smp._state_ref, self.GtG.data_ptr(), self.Gtd0.data_ptr(), self.dtd,
                  self.prior_kind, self.pmean.data_ptr() if self.pmean is not None else None,
                  self.pw.data_ptr() if self.pw is not None else None, self._sched_ref, n, warps, int(dry), h)

    def autotune(self, h, proposals=4):
        """Time every chains-per-block choice on dry runs (which write no
        state) of the live chains and keep the fastest (cached per problem
        shape by hmclab_gb300.autotune, in memory and on disk)."""
        from hmclab_gb300 import autotune as _autotune

        if self.warps is not None:
            return self.warps
        slen = self.smp._state.stream_len
        if slen > 0:
            proposals = min(proposals, slen)
        full = self.smp.mass_matrix.kind == _lib.HMC_MASS_FULL
        esize = 8 if self.smp.dtype == "float64" else 4
        cands = [(w,) for w in _WARPS if _smem(self.smp.dimensions, full, w, esize) <= _SMEM]
        shape = {"d": self.key[0], "C": self.key[1], "dtype": self.key[2], "mass": int(self.key[3]),
                 "prior": self.key[4], "steps": self.key[5]}
        (self.warps,) = _autotune.choose("persistent_dense", shape, cands,
                                         lambda c: self._call(proposals, c[0], True, h), self.smp.device, h, reps=1)
        _tuned[self.key] = self.warps
        return self.warps

    def run(self, n, h):
        if self.warps is None:
            self.autotune(h)
        self._call(n, self.warps, False, h)


def run_groups(samplers, n_proposals, warps=None):
    """Advance several prepared samplers — different targets, dimensions and
    chain counts, each eligible for the persistent kernel — by n_proposals
    each, with one launch per block of proposals for all of them (the
    sampler of the first target provides the stream).  Returns the chains
    per block used."""
    import torch

    ps = [s._persistent for s in samplers]
    if any(p is None for p in ps):
        raise ValueError("every sampler must run the persistent kernel (small dense linear-Gaussian target)")
    s0 = samplers[0]
    for s in samplers[1:]:
        if (s.dtype, s.mass_matrix.kind, s._persistent.prior_kind) != (s0.dtype, s0.mass_matrix.kind, ps[0].prior_kind):
            raise ValueError("grouped samplers must share dtype, mass kind and prior kind")
        if s._schedule != s0._schedule:
            raise ValueError("grouped samplers must share the integrator and its number of steps")
    st = s0.stream
    h = st.cuda_stream
    for s in samplers[1:]:
        st.wait_stream(s.stream)
    groups = (_lib.HmcDenseGroup * len(samplers))()
    for g, (s, p) in enumerate(zip(samplers, ps)):
        groups[g].chains = _ct.addressof(s._state)
        groups[g].GtG, groups[g].Gtd0, groups[g].dtd = p.GtG.data_ptr(), p.Gtd0.data_ptr(), p.dtd
        groups[g].prior = p.prior_kind
        groups[g].prior_mean = p.pmean.data_ptr() if p.pmean is not None else None
        groups[g].prior_w = p.pw.data_ptr() if p.pw is not None else None
    k = min(s.proposals_per_graph for s in samplers)

    def call(n, w, dry):
        _lib.call("hmc_persistent_dense_groups", groups, len(samplers), ps[0]._sched_ref, n, w, int(dry), h)

    if warps is None:
        full = s0.mass_matrix.kind == _lib.HMC_MASS_FULL
        esize = 8 if s0.dtype == "float64" else 4
        dmax = max(s.dimensions for s in samplers)
        best = None
        for w in _WARPS:
            if _smem(dmax, full, w, esize) > _SMEM:
                continue
            call(1, w, True)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            call(1, w, True)
            e1.record(st)
            st.synchronize()
            if best is None or e0.elapsed_time(e1) < best[0]:
                best = (e0.elapsed_time(e1), w)
        warps = best[1]
    done = 0
    while done < n_proposals:
        n = min(k, n_proposals - done, *(s.proposals - s._done for s in samplers))
        if n <= 0:
            break
        for s in samplers:
            s._load_streams(s._done, n)
        for s in samplers[1:]:
            st.wait_stream(s.stream)
        call(n, warps, False)
        for s in samplers[1:]:
            s.stream.wait_stream(st)
        for s in samplers:
            s._drain(s._done, n)
            s._done += n
        done += n
    return warps
