"""Benchmark of the batched HMC hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload fwi|dense|tomo|srcloc|cfg1]

A "step" is one HMC proposal (a full leapfrog trajectory plus the accept test)
for every chain of the workload.  Prints one JSON line.

Workload `fwi` (default; the metric's configuration): 2-D elastic P-SV
waveform inversion, 200x100 cells plus a 20-cell sponge, 1500 time steps, 4
shots, 20 receivers, 600 blob parameters, Normal prior of 10%, 64 chains.
W exact-gradient burn-in proposals record (position, gradient) pairs; the
surrogate (--surrogate potential: a scalar network whose gradient is used;
gradient: a network that outputs the gradient) is trained on them on the
device; then K surrogate-driven proposals (interior gradients from the
network, exact misfit for the accept test) and --plain-steps plain proposals
(exact gradients) are timed from the same start.  `value` is the surrogate
run's min-ESS/s; `plain` and `speedup_vs_plain` give the comparison, and
`ess_window_not_truncated` the fraction of parameters whose ESS lag window
ended before the autocorrelation sum was truncated (an upper estimate).

Workload `dense`: G 2000x1000 with N(0, 1/1000) entries, m_true ~ N(0, I),
noise sigma 0.05, Normal prior N(0, I), diagonal mass drawn U[0.5, 2], 20
leapfrog steps, 4096 chains, FP32 state, FP64 dH accept.  Chains start at exact
draws of the analytic posterior, so every timed proposal is a post-burn-in
sample.

metric: min over parameters of the multi-chain ESS of the timed proposals'
samples, divided by the device time of those proposals (min-ESS/s).
Synthetic seeded data; the L2 cache is flushed (256 MiB write) between timed
steps, outside the CUDA-event intervals.

--impl reference: the CPU implementation of the same path on the host cores:
for `dense`, the numpy port of the reference algorithm batched over chains on
a bounded sample; for `fwi`, the FP64 C restatement of the stencils timed on
full-size shots, one per core.  Same metric and unit.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "min-ESS/s at fixed moment error: surrogate vs plain batched HMC, 1 GB300"
UNIT = "effective samples/s (min over parameters)"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return p["hbm_gbs"], p["bf16_tflops"], p.get("bf16_tflops_sustained", p["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, 1700.0, "fallback"


# ---------------------------------------------------------------------------
# Workload: dense linear, 4096 chains
# ---------------------------------------------------------------------------
class DenseWorkload:
    name = "dense-linear G2000x1000, Normal prior, diag mass, L=20, 4096 chains, FP32"
    kind = "dense"
    n_data, n_model, chains, L = 2000, 1000, 4096, 20
    noise = 0.05
    default_steps, default_warmup = 100, 5

    def __init__(self, seed=0, chains=None):
        from hmclab_gb300 import problems

        if chains is not None:
            self.chains = chains
        rng = np.random.default_rng(seed + 1)
        self.G, self.d, self.m_true = problems.dense_linear(self.n_data, self.n_model, (1 / self.n_model) ** 0.5,
                                                            self.noise, seed)
        self.diag = rng.uniform(0.5, 2.0, size=(self.n_model, 1))
        self.post_mean, self.post_cov = problems.gaussian_posterior(self.G, self.d, self.noise**2, 0.0, 1.0)
        self.post_std = np.sqrt(np.diag(self.post_cov))
        # largest frequency of the mass-scaled Hessian -> step size
        A = np.linalg.inv(self.post_cov)
        s = 1.0 / np.sqrt(self.diag[:, 0])
        w_max = np.sqrt(np.linalg.eigvalsh(s[:, None] * A * s[None, :]).max())
        self.stepsize = 0.65 / w_max
        Lc = np.linalg.cholesky(self.post_cov)
        self.q0 = self.post_mean + Lc @ rng.normal(size=(self.n_model, self.chains))

    def posterior(self):
        import hmclab_gb300 as H

        prior = H.Distributions.Normal(np.zeros((self.n_model, 1)), np.ones((self.n_model, 1)))
        lik = H.Distributions.LinearMatrix(self.G, self.d, self.noise**2)
        return H.Distributions.BayesRule([prior, lik])

    def mass(self):
        import hmclab_gb300 as H

        return H.MassMatrices.Diagonal(self.diag)

    def sampler_kwargs(self):
        return dict(stepsize=self.stepsize, amount_of_steps=self.L, mass_matrix=self.mass(), chains=self.chains,
                    dtype="float32")

    # algorithmic work of the dominant kernel: the gradient GEMM GtG @ Q
    def gemm_flops(self):
        return 2.0 * self.n_model**2 * self.chains

    def oracle(self):
        from oracle import hmc_oracle as O

        post = O.Sum([O.NormalDiag(np.zeros(self.n_model), np.ones(self.n_model)),
                      O.DensePremul(self.G, self.d, self.noise**2)])
        return post, O.Mass("diag", diag=self.diag)

    def roofline_spec(self, smp):
        fused = smp._fused is not None
        return {"kernel": ("chain_gemm_kernel<EPI_STEP>: tcgen05 BF16 hi/lo GtG@Q + prior + kick + drift"
                           if fused else "dense gradient GEMM"),
                # DRAM read + write of one step launch, ncu capture (54.4 + 2.9 MB)
                "traffic": 57.3e6 if fused else None,
                "bound": "tensor", "unit": "TFLOP/s", "work": self.gemm_flops(),
                "work_name": "algorithmic_flop_per_launch",
                "extra": {"executed_flop_per_launch": 3 * self.gemm_flops() if fused else self.gemm_flops()}}

    def config(self):
        return {"workload": self.name, "n_data": self.n_data, "n_model": self.n_model, "chains": self.chains,
                "leapfrog_steps": self.L, "stepsize": self.stepsize, "prior": "Normal(0, I)",
                "mass": "diagonal U[0.5,2]", "precision": "FP32 state, FP64 dH", "l2": "flushed between timed steps",
                "start": "exact posterior draws"}


# ---------------------------------------------------------------------------
# Workload: the single-chain FP64 configuration the reference runs on a CPU
# ---------------------------------------------------------------------------
class Cfg1Workload:
    name = ("dense-linear G100x50 (N(0,1) entries), noise 0.1, Normal prior N(0, I), unit mass, 10 leapfrog steps "
            "of 0.01, 1 chain, FP64, 10,000 samples")
    kind = "cfg1"
    n_data, n_model, chains, L = 100, 50, 1, 10
    noise, stepsize = 0.1, 0.01
    proposals_per_step = 1000  # a step: 1000 proposals of the single chain
    default_steps, default_warmup = 10, 3
    cpu_sample = (1, 10000)

    def __init__(self, seed=0, chains=None):
        from hmclab_gb300 import problems

        self.G, self.d, self.m_true = problems.dense_linear(self.n_data, self.n_model, 1.0, self.noise, seed)
        self.post_mean, self.post_cov = problems.gaussian_posterior(self.G, self.d, self.noise**2, 0.0, 1.0)
        self.post_std = np.sqrt(np.diag(self.post_cov))
        self.q0 = self.post_mean.copy()

    def posterior(self):
        import hmclab_gb300 as H

        prior = H.Distributions.Normal(np.zeros((self.n_model, 1)), np.ones((self.n_model, 1)))
        lik = H.Distributions.LinearMatrix(self.G, self.d, self.noise**2, dtype=np.float64)
        return H.Distributions.BayesRule([prior, lik])

    def sampler_kwargs(self):
        return dict(stepsize=self.stepsize, amount_of_steps=self.L, chains=1, dtype="float64")

    def oracle(self):
        from oracle import hmc_oracle as O

        post = O.Sum([O.NormalDiag(np.zeros(self.n_model), np.ones(self.n_model)),
                      O.DensePremul(self.G, self.d, self.noise**2)])
        return post, O.Mass("unit")

    # FP64 FLOP of one block of proposals in the persistent kernel: L
    # gradients and one misfit, each a 50 x 50 product
    def roofline_spec(self, smp):
        work = float(self.proposals_per_step) * (self.L + 1) * 2 * self.n_model**2
        return {"kernel": "persistent_dense_kernel (whole proposals, one warp per chain, GtG in shared memory)",
                "bound": "fp64", "unit": "TFLOP/s", "work": work, "work_name": "algorithmic_flop_per_launch",
                "extra": {"proposals_per_launch": self.proposals_per_step, "persistent": smp._persistent is not None}}

    def config(self):
        return {"workload": self.name, "n_data": self.n_data, "n_model": self.n_model, "chains": 1,
                "leapfrog_steps": self.L, "stepsize": self.stepsize, "samples": 10000,
                "step": f"{self.proposals_per_step} proposals of the chain", "precision": "FP64",
                "l2": "flushed between timed steps", "start": "posterior mean"}


# ---------------------------------------------------------------------------
# Workload: straight-ray tomography, CSR ray lengths, 1024 chains
# ---------------------------------------------------------------------------
class TomoWorkload:
    name = ("straight-ray tomography 64x64 slowness cells, 2000 rays (CSR, exact lengths), noise 0.01 s, "
            "Normal prior around the background (sigma 0.05), Jacobi diagonal mass, L=20, 1024 chains, FP32")
    kind = "tomo"
    chains, L = 1024, 20
    noise, prior_std = 0.01, 0.05
    default_steps, default_warmup = 100, 5

    def __init__(self, seed=0, chains=None):
        import scipy.sparse.linalg as spla

        from hmclab_gb300 import problems

        if chains is not None:
            self.chains = chains
        t = problems.tomography(64, 64, 2000, 1.0, self.noise, seed)
        self.G, self.d, self.bg = t["G"], t["d"], t["background"]
        self.n_data, self.n_model = self.G.shape
        self.nnz = self.G.nnz
        self.post_mean, self.post_cov = problems.gaussian_posterior(self.G, self.d, self.noise**2, self.bg,
                                                                    self.prior_std**2)
        self.post_std = np.sqrt(np.diag(self.post_cov))
        A = np.linalg.inv(self.post_cov)
        self.diag = np.diag(A).reshape(-1, 1).copy()
        s = 1.0 / np.sqrt(self.diag[:, 0])
        w_max = np.sqrt(spla.eigsh(s[:, None] * A * s[None, :], k=1, which="LA")[0][0])
        self.stepsize = 0.6 / w_max
        rng = np.random.default_rng(seed + 1)
        self.q0 = self.post_mean + np.linalg.cholesky(self.post_cov) @ rng.normal(size=(self.n_model, self.chains))

    def posterior(self):
        import hmclab_gb300 as H

        prior = H.Distributions.Normal(self.bg, np.full((self.n_model, 1), self.prior_std**2))
        lik = H.Distributions.LinearMatrix(self.G, self.d, self.noise**2)
        return H.Distributions.BayesRule([prior, lik])

    def mass(self):
        import hmclab_gb300 as H

        return H.MassMatrices.Diagonal(self.diag)

    def sampler_kwargs(self):
        return dict(stepsize=self.stepsize, amount_of_steps=self.L, mass_matrix=self.mass(), chains=self.chains,
                    dtype="float32")

    def oracle(self):
        from oracle import hmc_oracle as O

        post = O.Sum([O.NormalDiag(self.bg, np.full(self.n_model, self.prior_std**2)),
                      O.SparseLinear(self.G, self.d, self.noise**2)])
        return post, O.Mass("diag", diag=self.diag)

    # the gradient's two sparse products: G @ Q (minus data, weighted) and
    # G^T @ R, each reading the CSR arrays once (8 B per nonzero: value +
    # column) and streaming the dense operands (4 B per element, FP32)
    def roofline_spec(self, smp):
        C = self.chains
        work = 2 * (8.0 * self.nnz + 4.0 * C * (self.n_data + self.n_model)) + 4.0 * (self.n_data + 1) * 2
        # every nonzero also gathers a row of the dense operand (C values)
        # from L2: the traffic the kernel actually moves
        gather = 2 * 4.0 * self.nnz * C
        return {"kernel": "csr_spmm_kernel x2 (G @ Q - d, G^T @ R)", "bound": "hbm", "unit": "GB/s", "work": work,
                "work_name": "algorithmic_bytes_per_launch",
                "extra": {"nnz": int(self.nnz), "l2_gather_bytes_per_launch": gather}}

    def config(self):
        return {"workload": self.name, "cells": self.n_model, "rays": self.n_data, "nnz": int(self.nnz),
                "chains": self.chains, "leapfrog_steps": self.L, "stepsize": self.stepsize,
                "prior": "Normal(background, 0.05^2)", "mass": "diagonal of the posterior precision",
                "precision": "FP32 state, FP64 dH", "l2": "flushed between timed steps",
                "start": "exact posterior draws"}


# ---------------------------------------------------------------------------
# Workload: 3-D source location, 32 events + velocity, 8192 chains
# ---------------------------------------------------------------------------
class SrclocWorkload:
    name = ("3-D source location: 32 events (x, y, z, t0) + one velocity = 129 params, 200 surface stations, "
            "40x40 km box, depth 0-10 km, v = 5 km/s, noise 0.05 s, full mass = Gauss-Newton Hessian at the truth, "
            "L=5, 8192 chains, FP32")
    kind = "srcloc"
    chains, L = 8192, 5
    noise = 0.05
    default_steps, default_warmup = 100, 10

    def __init__(self, seed=0, chains=None):
        from hmclab_gb300 import problems

        if chains is not None:
            self.chains = chains
        t = problems.source_location(32, 200, 40.0, 10.0, 5.0, self.noise, seed)
        self.t = t
        self.E, self.S = t["obs"].shape
        self.n_model = 4 * self.E + 1
        m = t["m_true"][:, 0]
        # Gauss-Newton Hessian J^T J / sigma^2 of the arrival times at the truth
        J = np.zeros((self.E * self.S, self.n_model))
        v = m[-1]
        for e in range(self.E):
            dx, dy, dz = m[4 * e] - t["rx"][0], m[4 * e + 1] - t["ry"][0], m[4 * e + 2] - t["rz"][0]
            dist = np.sqrt(dx * dx + dy * dy + dz * dz)
            rows = slice(e * self.S, (e + 1) * self.S)
            J[rows, 4 * e] = dx / (v * dist)
            J[rows, 4 * e + 1] = dy / (v * dist)
            J[rows, 4 * e + 2] = dz / (v * dist)
            J[rows, 4 * e + 3] = 1.0
            J[rows, -1] = -dist / v**2
        self.H = J.T @ J / self.noise**2
        self.stepsize = 0.8
        rng = np.random.default_rng(seed + 1)
        Lc = np.linalg.cholesky(np.linalg.inv(self.H))
        self.q0 = t["m_true"] + Lc @ rng.normal(size=(self.n_model, self.chains))
        self.post_mean = self.post_std = None

    def posterior(self):
        import hmclab_gb300 as H

        t = self.t
        return H.Distributions.SourceLocation3D(t["rx"], t["ry"], t["rz"], t["obs"], self.noise)

    def mass(self):
        import hmclab_gb300 as H

        return H.MassMatrices.Full(self.H)

    def sampler_kwargs(self):
        return dict(stepsize=self.stepsize, amount_of_steps=self.L, mass_matrix=self.mass(), chains=self.chains,
                    dtype="float32")

    def oracle(self):
        from oracle import hmc_oracle as O

        t = self.t
        post = O.SourceLocation3D(t["rx"], t["ry"], t["rz"], t["obs"], t["std"])
        return post, O.Mass("full", full=self.H)

    # FP32 operations per (chain, event, station) pair of the gradient: the
    # distance (3 sub, 3 mul/fma, sqrt), travel time and residual (div, add,
    # sub, mul), four partials (mul, div, mul each) and their sums
    FLOP_PER_PAIR = 23

    def roofline_spec(self, smp):
        work = float(self.FLOP_PER_PAIR) * self.chains * self.E * self.S
        return {"kernel": "srcloc_kernel<float, true> (one thread per chain and event lane)", "bound": "fp32",
                "unit": "TFLOP/s", "work": work, "work_name": "algorithmic_flop_per_launch",
                "extra": {"pairs_per_launch": self.chains * self.E * self.S}}

    def config(self):
        return {"workload": self.name, "events": self.E, "stations": self.S, "params": self.n_model,
                "chains": self.chains, "leapfrog_steps": self.L, "stepsize": self.stepsize,
                "mass": "full (Gauss-Newton Hessian at the true model)", "precision": "FP32 state, FP64 dH",
                "l2": "flushed between timed steps", "start": "draws of the Laplace approximation + warm-up"}


# ---------------------------------------------------------------------------
# Workload: 2-D elastic FWI, surrogate-driven vs plain batched HMC, 64 chains
# ---------------------------------------------------------------------------
# Plain-HMC min-ESS per chain-proposal on the FWI workload, measured by this
# bench's GPU arm (the `plain.ess_per_chain_proposal` field of its line); the
# reference arm, which can only afford to time the CPU cost of a proposal,
# converts that cost into min-ESS/s with it.
FWI_PLAIN_ESS_PER_CHAIN_PROPOSAL = 0.203
# DRAM bytes (read + write) of one forward time step at C = 64 from one ncu
# capture of velocity_tma_kernel (60.5 + 0.4 MB) and stress_tma_kernel
# (69.0 + 1.2 MB) on a cold cache; in the time loop the fields stay in L2 and
# DRAM moves less
FWI_STEP_DRAM_BYTES = 131.0e6


class FwiWorkload:
    name = ("elastic P-SV FWI 200x100 cells (+20-cell sponge), h=5 m, dt=0.5 ms, nt=1500, 4 shots x 20 receivers, "
            "25 Hz Ricker, blobs 20x10 x (vp,vs,rho) = 600 params, Normal prior 10%, 64 chains, FP32 stencils, "
            "scalar-potential network surrogate 600-512-512-1 vs plain HMC")
    kind = "fwi"
    chains, L = 64, 10
    stepsize = 0.12  # prior-whitened units: the mass matrix is the prior precision
    noise_fraction = 10.0  # data noise std / RMS of the true records
    hidden = (512, 512)
    # 300 surrogate proposals: the slowest parameters of the surrogate run
    # decorrelate over tens of proposals, and the ESS lag window (K/2) must
    # reach past them
    default_steps, default_warmup = 300, 12

    def __init__(self, seed=0, chains=None):
        from hmclab_gb300 import fwi as F

        if chains is not None:
            self.chains = chains
        self.seed = seed
        self.cfg = F.ElasticConfig()
        self.cells = self.cfg.nxc * self.cfg.nzc
        self.built = False

    def build(self):
        """Synthesise the observed records on the device (forward of the true
        model plus noise) and draw the chains' starting points."""
        from hmclab_gb300 import problems

        pb = problems.elastic_fwi(self.cfg, 20, 10, prior_fraction=0.1, noise_fraction=self.noise_fraction,
                                  seed=self.seed)
        self.pb = pb
        self.d = pb["likelihood"].dimensions
        rng = np.random.default_rng(self.seed + 11)
        self.q0 = pb["m_true"][:, None] + 0.3 * pb["prior_std"][:, None] * rng.normal(size=(self.d, self.chains))
        self.built = True
        return self

    def posterior(self):
        return self.pb["posterior"]

    def mass(self):
        import hmclab_gb300 as H

        return H.MassMatrices.Diagonal(1.0 / self.pb["prior_std"] ** 2)

    def sampler_kwargs(self):
        return dict(stepsize=self.stepsize, amount_of_steps=self.L, mass_matrix=self.mass(), chains=self.chains,
                    dtype="float32")

    # algorithmic HBM bytes of one forward time step (velocity + stress
    # kernels) for all chains: velocity phase reads vx, vz, sxx, szz, sxz, bx,
    # bz and writes vx, vz; stress phase reads vx, vz, sxx, szz, sxz, l2m, lam,
    # muxz and writes sxx, szz, sxz: 20 FP32 words per cell and chain
    def stencil_bytes_per_step(self):
        return 80.0 * self.cells * self.chains

    def config(self):
        return {"workload": self.name, "grid": [self.cfg.nx, self.cfg.nz], "sponge_cells": self.cfg.pad,
                "nt": self.cfg.nt, "shots": self.cfg.n_shots, "receivers": self.cfg.n_rec, "params": 600,
                "chains": self.chains, "leapfrog_steps": self.L, "stepsize": self.stepsize,
                "stepsize_units": "prior-whitened (diagonal mass = prior precision), randomised x U(0.5,1.5)",
                "prior": "Normal(background, (10% of background at blob centre)^2)",
                "noise": f"{self.noise_fraction} x RMS of the true records (seeded Gaussian)",
                "surrogate": ("scalar potential w3 . GELU(W2 GELU(W1 x + b1) + b2) + quadratic, 600-512-512-1, its "
                              "gradient drives the leapfrog; BF16 weights, FP32 accumulate"),
                "precision": "FP32 state and stencils, FP64 dH", "l2": "flushed between timed steps (256 MiB write)",
                "start": "end states of the exact burn-in"}


WORKLOADS = {"cfg1": Cfg1Workload, "dense": DenseWorkload, "tomo": TomoWorkload, "srcloc": SrclocWorkload,
             "fwi": FwiWorkload}


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def cpu_reference_run(wl, chains, warmup, steps, seed=0):
    """The numpy port of the reference path (oracle/hmc_oracle.py) on `chains`
    chains: returns (min-ESS/s, moment errors, seconds, chain-steps/s)."""
    from oracle import hmc_oracle as O

    post, mass = wl.oracle()
    rng = np.random.default_rng(seed + 7)
    q0 = wl.q0[:, :chains]
    P = warmup + steps
    z = rng.normal(size=(P, wl.n_model, chains))
    f = rng.uniform(0.5, 1.5, size=(P, chains))
    u = rng.uniform(size=(P, chains))
    res = O.run_chains(post, mass, q0, wl.stepsize, (z[:warmup], f[:warmup], u[:warmup]), warmup,
                       amount_of_steps=wl.L) if warmup else None
    qs = res["q"] if res is not None else q0
    t0 = time.perf_counter()
    res = O.run_chains(post, mass, qs, wl.stepsize, (z[warmup:], f[warmup:], u[warmup:]), steps, amount_of_steps=wl.L)
    dt = time.perf_counter() - t0
    x = res["samples"][:, :-1, :]  # N, d, C
    ess, _ = O.ess_split(x, lags=max(2, steps // 2))
    ess = np.abs(ess)
    mean, std = x.mean(axis=(0, 2)), x.std(axis=(0, 2))
    if wl.post_mean is not None:
        me = float(np.max(np.abs(mean - wl.post_mean[:, 0]) / wl.post_std))
        se = float(np.max(np.abs(std - wl.post_std) / wl.post_std))
    else:
        me = se = None
    return float(ess.min() / dt), (me, se), dt, chains * steps * wl.L / dt


def run_reference_arm(args, wl):
    B = getattr(wl, "proposals_per_step", 1)
    chains = args.cpu_chains if not hasattr(wl, "cpu_sample") else wl.cpu_sample[0]
    v, (me, se), dt, lps = cpu_reference_run(wl, chains, args.warmup * B, args.steps * B)
    cores = os.cpu_count() if chains > 1 else 1
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "impl": "reference", "config": {**wl.config(), "chains": chains},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{chains} chains x {args.steps * B} proposals of the same workload, numpy port of "
                                   "the reference HMC path batched over chains (BLAS on all host threads)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "leapfrog_steps_per_s": lps, "moment_error": {"mean": me, "std": se},
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------------
def dominant_kernel_timing(post, smp, n_iter=20):
    """Average duration of the dominant kernel with CUDA events on the sampler
    stream, on the live chain state: the persistent kernel running one block
    of proposals (dry: it writes no state) when the sampler uses it, the fused
    tensor-core leapfrog step (GtG @ Q - Gtd0 + prior, kick, drift, operand
    re-split) when it uses that, else the gradient launch of the likelihood."""
    import torch

    st = smp.stream
    h = st.cuda_stream
    lik = post.separate_distributions[1] if hasattr(post, "separate_distributions") else post
    if getattr(smp, "_persistent", None) is not None:
        B = smp.proposals_per_graph
        if smp._persistent.warps is None:
            smp._persistent.autotune(h)

        def launch():  # one block of proposals, writing no state
            smp._persistent._call(B, smp._persistent.warps, True, h)
    elif smp._fused is not None:
        smp._fused.after_begin(h)

        def launch():
            smp._fused.kick_drift(1.0, 1.0, h)
    else:
        def launch():
            lik._device_gradient(smp.q, smp.g, False, smp.dtype, h)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(st):
        for _ in range(3):
            launch()
        ev0.record(st)
        for _ in range(n_iter):
            launch()
        ev1.record(st)
    st.synchronize()
    return ev0.elapsed_time(ev1) / 1e3 / n_iter


def run_gpu_arm(args, wl):
    import torch

    import hmclab_gb300 as H
    from hmclab_gb300 import _lib, diagnostics, sharding

    rank, world, local = sharding.rank_environment()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    post = wl.posterior()
    K, W = args.steps, args.warmup
    B = getattr(wl, "proposals_per_step", 1)  # proposals of every chain in one step
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # ---- device-resident timed run ---------------------------------------
    smp = H.Samplers.HMC(seed=sharding.rank_seed(1000, rank))
    smp.prepare(None, post, initial_model=wl.q0, proposals=(W + K) * B, keep_samples=True, proposals_per_graph=B,
                **wl.sampler_kwargs())
    smp.run(W * B)
    smp.stream.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = _lib.launch_count()
    for k in range(K):
        with torch.cuda.stream(smp.stream):
            flush.fill_(float(k))
            evs[k][0].record(smp.stream)
        smp.run(B)
        evs[k][1].record(smp.stream)
    torch.cuda.synchronize()
    launches = _lib.launch_count() - launches0
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    t_dev = sum(a.elapsed_time(b) for a, b in evs) / 1e3
    t_gemm = dominant_kernel_timing(post, smp)
    smp.finish()
    q, x = smp.samples_device  # [N][d][C]
    timed = q[W * B:]
    ess = np.abs(diagnostics.ess(timed, lags=min(K * B // 2, 100 if B == 1 else 200)))
    mean, std = diagnostics.moments(timed)
    ess, t_dev = sharding.combine_ess(ess, t_dev)
    mean, std = sharding.combine_moments(mean, std, K * B * wl.chains)
    if wl.post_mean is not None:
        me, se = diagnostics.moment_error(mean, std, wl.post_mean, wl.post_std)
    else:
        me = se = None
    value = float(ess.min() / t_dev)
    acc = float(np.mean(smp.accepted_proposals) / ((W + K) * B))

    # ---- end to end through the public API with host buffers -------------
    smp2 = H.Samplers.HMC(seed=sharding.rank_seed(2000, rank))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    smp2.sample(None, post, initial_model=wl.q0, proposals=K * B, keep_samples=True,
                proposals_per_graph=B if B > 1 else min(K, 10), **wl.sampler_kwargs())
    host_q, host_x = smp2.samples_host()  # [N][d][C] and [N][C] on the host
    t_e2e = time.perf_counter() - t0
    ess2 = np.abs(diagnostics.ess(torch.from_numpy(host_q).to("cuda"), lags=min(K * B // 2, 100 if B == 1 else 200)))
    e2e_value = float(ess2.min() / t_e2e)
    esize = 8 if wl.sampler_kwargs().get("dtype") == "float64" else 4
    h2d = wl.q0.size * 8 / K
    d2h = B * (wl.n_model * wl.chains * esize + wl.chains * 8)

    hbm, bf16, bf16s, src = peaks()
    spec = wl.roofline_spec(smp)
    if spec["bound"] == "tensor":
        peak, psrc, scale = bf16, src, 1e12
    elif spec["bound"] == "hbm":
        peak, psrc, scale = hbm, src, 1e9
    elif spec["bound"] == "fp64":  # nominal FP64 rate of the part
        peak, psrc, scale = 1.25, "nominal", 1e12
    else:  # FP32 issue rate: 152 SMs x 128 lanes x 2 (FMA) x 2.07 GHz, nominal
        peak, psrc, scale = 152 * 128 * 2 * 2.07e9 / 1e12, "nominal", 1e12
    achieved = spec["work"] / t_gemm / scale
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": 1e3 * t_dev / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if esize == 8 else "f32", "data": "synthetic (seeded)", "config": wl.config(),
        "leapfrog_steps_per_s": wl.chains * wl.L * K * B / t_dev * world,
        "moment_error": {"mean": me, "std": se}, "acceptance": acc,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "seconds": t_e2e},
        "gpu_launches": int(launches),
        "roofline": {"kernel": spec["kernel"], "bound": spec["bound"], "achieved": achieved, "peak": peak,
                     "unit": spec["unit"], "frac": achieved / peak, "traffic": spec.get("traffic"),
                     "peak_source": psrc,
                     "launch_s": t_gemm, spec["work_name"]: spec["work"], **spec["extra"]},
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        cc, cs = getattr(wl, "cpu_sample", (args.cpu_chains, args.cpu_steps))
        v, (cme, cse), dt, lps = cpu_reference_run(wl, cc, 2, cs)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1 if cc == 1 else os.cpu_count(), "kind": "port",
                                "sample": f"{cc} chains x {cs} proposals, numpy port "
                                          f"batched over chains ({dt:.1f} s, {lps:.0f} leapfrog steps/s)"}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------------------
def fwi_cpu_costs(wl, cores):
    """Seconds of one forward and one forward+adjoint shot of the FP64 C
    restatement (oracle/fwi_oracle.c) on the full grid, `cores` shots at once
    on a spawn process pool (one task per core); returns the medians and the
    wall time."""
    import multiprocessing as mp

    from oracle import build_oracle
    from oracle import fwi as OF
    from hmclab_gb300 import fwi as F

    build_oracle.build()
    cfg = wl.cfg
    bg = F.layered_model(cfg, anomalies=True)
    vp, vs, rho = (cfg.extend(f) for f in bg)
    tasks = [(cfg.nxc, cfg.nzc, cfg.nt, cfg.h, cfg.dt, cfg.taper(), cfg.ricker(), cfg.src[k % cfg.n_shots],
              cfg.rec_x, cfg.rec_z, rho, vp, vs) for k in range(cores)]
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(OF.timed_shot, tasks)
    wall = time.perf_counter() - t0
    return float(np.median([r[0] for r in res])), float(np.median([r[1] for r in res])), wall


def fwi_cpu_rate(wl, cores):
    """CPU chain-proposals/s of plain HMC on the FWI workload: L exact
    gradients (4 shots forward + adjoint) plus one misfit (4 forward shots)
    per chain-proposal, one chain per core."""
    t_fwd, t_grad, wall = fwi_cpu_costs(wl, cores)
    per_chain_proposal = wl.cfg.n_shots * (wl.L * t_grad + t_fwd)
    return cores / per_chain_proposal, t_fwd, t_grad, wall


def run_fwi_reference_arm(args, wl):
    cores = os.cpu_count()
    rate, t_fwd, t_grad, wall = fwi_cpu_rate(wl, cores)
    e = FWI_PLAIN_ESS_PER_CHAIN_PROPOSAL
    value = rate * e if e is not None else None
    sample = (f"{cores} full-size shots (forward {t_fwd:.2f} s, forward+adjoint {t_grad:.2f} s each, FP64 C "
              f"restatement, one per core, {wall:.1f} s wall); chain-proposals/s = cores / (4 shots x (L x "
              f"gradient + misfit)) = {rate:.4g}, times the plain-HMC min-ESS per chain-proposal measured on "
              f"the GPU ({e})")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": 1, "warmup": 0,
        "ms_per_step": 1e3 * wl.chains / rate, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "impl": "reference", "config": wl.config(),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "chain_proposals_per_s": rate,
    }
    print(json.dumps(line))


def timed_proposals(smp, K, flush, evs):
    import torch

    for k in range(K):
        with torch.cuda.stream(smp.stream):
            flush.fill_(float(k))
            evs[k][0].record(smp.stream)
        smp.run(1)
        evs[k][1].record(smp.stream)
    smp.stream.synchronize()
    return sum(a.elapsed_time(b) for a, b in evs) / 1e3


def forward_step_timing(lik, smp, n_iter=2):
    """Seconds of one forward time step (velocity + stress kernel) over all
    chains: the exact misfit (4 shots x nt steps of the two stencil kernels,
    plus the blob-to-grid GEMMs and the misfit reduction) timed with CUDA
    events on the sampler stream, divided by shots x nt."""
    import torch

    st = smp.stream
    h = st.cuda_stream
    out = torch.empty(smp.chains, dtype=torch.float64, device=smp.q.device)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(st):
        lik._device_misfit(smp.q_cur, out, False, "float32", h)
        ev0.record(st)
        for _ in range(n_iter):
            lik._device_misfit(smp.q_cur, out, False, "float32", h)
        ev1.record(st)
    st.synchronize()
    return ev0.elapsed_time(ev1) / 1e3 / n_iter / (lik.config.n_shots * lik.config.nt)


def choose_trajectory(pilot, min_acceptance=0.25):
    """(L, stepsize) of the pilot entry (gain, L, stepsize, acceptance) with
    the largest gain among those that accepted at least `min_acceptance` of
    their proposals (a lower acceptance estimated from a few proposals is too
    noisy to trust); among all entries when none did."""
    usable = [x for x in pilot if x[3] >= min_acceptance] or pilot
    _, L_best, eps_best, _ = max(usable)
    return L_best, eps_best


def run_fwi_arm(args, wl):
    import torch

    import hmclab_gb300 as H
    from hmclab_gb300 import _lib, diagnostics, sharding
    from hmclab_gb300 import surrogate as S

    rank, world, local = sharding.rank_environment()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    t_setup = time.perf_counter()
    wl.build()
    post, lik = wl.posterior(), wl.pb["likelihood"]
    d, C, L = wl.d, wl.chains, wl.L
    K, W, Kp = args.steps, args.warmup, args.plain_steps
    kw = wl.sampler_kwargs()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    t_setup = time.perf_counter() - t_setup

    # ---- exact burn-in, recording (position, gradient) pairs -------------
    data = S.TrainingSet(d, W * L * C)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    burn = H.Samplers.HMC(seed=sharding.rank_seed(100, rank)).sample(None, post, initial_model=wl.q0, proposals=W,
                                                                     training_set=data, **kw)
    t_burn = time.perf_counter() - t0
    q_start = burn.current_model
    acc_burn = float(np.mean(burn.accepted_proposals) / W)

    # ---- surrogate training on the device ---------------------------------
    kind = S.PotentialSurrogate if args.surrogate == "potential" else S.MLPSurrogate
    net = kind(d, hidden=wl.hidden, seed=rank)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fit = net.fit(data, steps=args.train_steps, batch=256, lr=1e-3, holdout_fraction=0.1)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    net.freeze()

    # ---- pilot (untimed): the surrogate run's trajectory ------------------
    # A few proposals per (L, stepsize) from the burn-in end states; the
    # setting with the largest acceptance x (trajectory length)^2 — the
    # diffusive-regime gain per proposal, length capped at the plain run's —
    # is used for the timed run.  --surrogate-L / --surrogate-stepsize fix it.
    pilot = []
    if args.surrogate_L is None or args.surrogate_stepsize is None:
        tau_max = wl.stepsize * wl.L
        for L_s in (2, 4, 8, 16):
            for eps_s in (0.03, 0.06, 0.12):
                if L_s * eps_s > tau_max + 1e-9:
                    continue
                p_smp = H.Samplers.HMC(seed=sharding.rank_seed(150 + 10 * L_s, rank)).sample(
                    None, post, initial_model=q_start, proposals=4, surrogate=net,
                    **dict(kw, amount_of_steps=L_s, stepsize=eps_s))
                a = float(np.mean(p_smp.accepted_proposals) / 4)
                pilot.append((a * (L_s * eps_s) ** 2, L_s, eps_s, a))
        L_best, eps_best = choose_trajectory(pilot)
    else:
        L_best, eps_best = args.surrogate_L, args.surrogate_stepsize

    # ---- timed: surrogate-driven HMC --------------------------------------
    kw_s = dict(kw, amount_of_steps=L_best, stepsize=eps_best)

    def timed_run(seed, n, surrogate):
        smp = H.Samplers.HMC(seed=seed)
        smp.prepare(None, post, initial_model=q_start, proposals=n, keep_samples=True, surrogate=surrogate,
                    **(kw_s if surrogate is not None else kw))
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        torch.cuda.synchronize()
        l0 = _lib.launch_count()
        t = timed_proposals(smp, n, flush, evs)
        launches = _lib.launch_count() - l0
        return smp, t, launches, [a.elapsed_time(b) / 1e3 for a, b in evs]

    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    smp_s, t_s, launches, _ = timed_run(sharding.rank_seed(200, rank), K, net)
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    t_step = forward_step_timing(lik, smp_s)
    smp_s.finish()
    qs = smp_s.samples_device[0]  # [K][d][C]
    ess_s_raw = diagnostics.ess(qs, lags=min(K // 2, 200))
    ess_s = np.abs(ess_s_raw)
    acc_s = float(np.mean(smp_s.accepted_proposals) / K)

    # ---- timed: plain HMC (exact gradients), same start -------------------
    smp_p, t_p, _, per_p = timed_run(sharding.rank_seed(300, rank), Kp, None)
    smp_p.finish()
    qp = smp_p.samples_device[0]
    ess_p_raw = diagnostics.ess(qp, lags=max(2, Kp // 2))
    ess_p = np.abs(ess_p_raw)
    acc_p = float(np.mean(smp_p.accepted_proposals) / Kp)
    # rank-normalised bulk-ESS of the same draws, reported beside the headline
    bulk_s = np.abs(diagnostics.ess(qs, lags=min(K // 2, 200), rank_normalize=True))
    bulk_p = np.abs(diagnostics.ess(qp, lags=max(2, Kp // 2), rank_normalize=True))
    bulk_s, _ = sharding.combine_ess(bulk_s, t_s)
    bulk_p, _ = sharding.combine_ess(bulk_p, t_p)
    ess_s, t_s = sharding.combine_ess(ess_s, t_s)
    ess_p, t_p = sharding.combine_ess(ess_p, t_p)
    value = float(ess_s.min() / t_s)
    plain_value = float(ess_p.min() / t_p)
    mean_s, std_s = sharding.combine_moments(*diagnostics.moments(qs), K * C)
    mean_p, std_p = sharding.combine_moments(*diagnostics.moments(qp), Kp * C)
    me, se = diagnostics.moment_error(mean_s, std_s, mean_p, std_p)
    # the same posterior mean in both runs? z = difference / its Monte Carlo
    # standard error (std / sqrt(ESS) per run); for exact chains |z| ~ N(0, 1)
    se_mean = np.sqrt(std_s**2 / np.maximum(ess_s, 1.0) + std_p**2 / np.maximum(ess_p, 1.0))
    z = np.abs(mean_s - mean_p) / np.maximum(se_mean, 1e-300)
    e_plain = float(ess_p.min() / (C * world * Kp))

    # ---- end to end through the public API with host buffers -------------
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    smp_e = H.Samplers.HMC(seed=sharding.rank_seed(400, rank)).sample(
        None, post, initial_model=q_start, proposals=K, keep_samples=True, surrogate=net, **kw_s)
    host_q, host_x = smp_e.samples_host()
    t_e2e = time.perf_counter() - t0
    ess_e = np.abs(diagnostics.ess(torch.from_numpy(host_q).to("cuda"), lags=min(K // 2, 200)))
    e2e_value = float(ess_e.min() / t_e2e)

    hbm, bf16, bf16s, src = peaks()
    achieved = wl.stencil_bytes_per_step() / t_step / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": 1e3 * t_s / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded; records from the device forward of the true model + noise)",
        "config": wl.config(),
        "speedup_vs_plain": float(value / plain_value),
        "including_burn_in_and_training": {
            "value": float(ess_s.min() / (t_burn + t_train + t_s)),
            "plain_value": float(ess_p.min() / (t_burn + t_p)),
            "note": "min-ESS over (exact burn-in + surrogate training + sampling) seconds; plain over "
                    "(the same burn-in + its sampling)"},
        # parameters whose autocorrelation sum the lag window cut before
        # Geyer's truncation point: their ESS is an upper estimate
        "ess_window_not_truncated": {"surrogate": float(np.mean(ess_s_raw < 0)),
                                     "plain": float(np.mean(ess_p_raw < 0))},
        "rank_normalised_bulk": {"value": float(bulk_s.min() / t_s), "plain_value": float(bulk_p.min() / t_p),
                                 "speedup_vs_plain": float((bulk_s.min() / t_s) / (bulk_p.min() / t_p))},
        "acceptance": acc_s, "surrogate_trajectory": {"leapfrog_steps": L_best, "stepsize": eps_best,
                                                      "pilot": [[L_, e_, round(a_, 4)] for _, L_, e_, a_ in pilot]},
        "plain": {"value": plain_value, "steps": Kp, "ms_per_step": 1e3 * t_p / Kp, "acceptance": acc_p,
                  "ess_per_chain_proposal": e_plain},
        "moment_error_vs_plain": {"mean": me, "std": se,
                                  "mc_floor": float(1.0 / np.sqrt(max(1.0, ess_p.min()))),
                                  "mean_z_max": float(z.max()), "mean_z_frac_above_3": float(np.mean(z > 3.0))},
        "burn_in": {"proposals": W, "seconds": t_burn, "acceptance": acc_burn, "pairs": data.count},
        "surrogate": {"kind": args.surrogate, "train_steps": args.train_steps, "train_seconds": t_train, "train_pairs": fit["train_pairs"],
                      "heldout_pairs": fit["heldout_pairs"], "loss_first": fit["history"][0][1],
                      "loss_last": fit["history"][-1][1], "heldout_rel_error_linear_start": fit["heldout"][0][1],
                      "heldout_rel_error": fit["best_heldout"], "best_step": fit["best_step"],
                      "heldout_curve": [[k, round(e, 5)] for k, e in fit["heldout"]]},
        "setup_seconds": t_setup,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(q_start.size * 8 / K),
                "d2h_bytes_per_step": int(d * C * 4 + C * 8), "seconds": t_e2e},
        "gpu_launches": int(launches),
        "roofline": {"kernel": "fwi forward time step: velocity_tma_kernel + stress_tma_kernel (the exact misfit)",
                     "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": FWI_STEP_DRAM_BYTES, "traffic_source": "ncu capture of one velocity + one stress "
                     "launch at C = 64, default (cold) cache control", "peak_source": src, "step_s": t_step,
                     "algorithmic_bytes_per_step": wl.stencil_bytes_per_step(),
                     "note": "one shot's fields and parameters (86 MB at 64 chains) stay in the 129 MB L2 over the "
                             "time loop, so the algorithmic rate can exceed the HBM copy rate; DRAM traffic per "
                             "step (`traffic`, cold cache) is 0.76 of the algorithmic bytes"},
        "clocks": clk,
    }
    if args.surrogate == "gradient":
        line["config"]["surrogate"] = ("MLP 600-512-512-600 GELU + linear skip (outputs the gradient), BF16 weights, "
                                       "FP32 accumulate")
    if rank == 0 and not args.no_cpu_baseline:
        cores = os.cpu_count()
        rate, t_fwd, t_grad, wall = fwi_cpu_rate(wl, cores)
        line["cpu_baseline"] = {
            "value": rate * e_plain, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": (f"{cores} full-size shots of the FP64 C restatement, one per core ({wall:.1f} s wall; "
                       f"forward {t_fwd:.2f} s, forward+adjoint {t_grad:.2f} s); chain-proposals/s = {rate:.4g} "
                       f"times the plain-HMC min-ESS per chain-proposal of this run ({e_plain:.4g})")}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=None)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="fwi", choices=sorted(WORKLOADS))
    ap.add_argument("--plain-steps", type=int, default=16, help="fwi: timed proposals of plain HMC")
    ap.add_argument("--train-steps", type=int, default=10000, help="fwi: Adam steps of the surrogate")
    ap.add_argument("--surrogate", default="potential", choices=["potential", "gradient"],
                    help="fwi: scalar-potential network (conservative field) or a network that outputs the gradient")
    ap.add_argument("--surrogate-L", type=int, default=None,
                    help="fwi: leapfrog steps of the surrogate-driven run (default: chosen by a pilot)")
    ap.add_argument("--surrogate-stepsize", type=float, default=None,
                    help="fwi: its step size in whitened units (default: chosen by a pilot)")
    ap.add_argument("--cpu-chains", type=int, default=64)
    ap.add_argument("--cpu-steps", type=int, default=300)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]()
    args.steps = wl.default_steps if args.steps is None else args.steps
    args.warmup = wl.default_warmup if args.warmup is None else args.warmup
    assert args.warmup >= 3, "at least 3 warm-up steps"
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        (run_fwi_reference_arm if args.workload == "fwi" else run_reference_arm)(args, wl)
        return
    (run_fwi_arm if args.workload == "fwi" else run_gpu_arm)(args, wl)


if __name__ == "__main__":
    main()
