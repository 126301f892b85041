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


def l2_copy_rate(mbytes=40, reps=50):
    """Read + write bandwidth (GB/s) of a device copy whose source and
    destination (2 x `mbytes` MB) stay resident in the 129 MB L2: the roof of
    kernels whose working set lives in L2 (the elastic stencils of one shot),
    measured in the same process with CUDA events, after warm-up."""
    import torch

    n = mbytes * 1024 * 1024 // 4
    src = torch.ones(n, dtype=torch.float32, device="cuda")
    dst = torch.empty_like(src)
    for _ in range(5):
        dst.copy_(src)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        dst.copy_(src)
    e1.record()
    e1.synchronize()
    return 2.0 * 4 * n * reps / (e0.elapsed_time(e1) / 1e3) / 1e9


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
        two_pass = fused and smp._fused.entry == "hmc_tc_step_split"
        if two_pass:
            kernel = ("leapfrog step in two passes (picked by the autotuner): chain_gemm_kernel<EPI_GRAD> tcgen05 "
                      "BF16 hi/lo GtG@Q - Gtd0, then step_update_kernel (prior + kick + drift + operand split)")
        elif fused:
            kernel = "chain_gemm_kernel<EPI_STEP>: tcgen05 BF16 hi/lo GtG@Q + prior + kick + drift"
        else:
            kernel = "dense gradient GEMM"
        return {"kernel": kernel,
                # DRAM read + write of one fused step launch, ncu capture (54.4 + 2.9 MB)
                "traffic": 57.3e6 if fused and not two_pass else None,
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
        # every nonzero also multiplies a row of the dense operand (C values),
        # gathered from L2 or staged in shared memory: the bytes the kernels
        # actually move through the memory hierarchy
        gather = 2 * 4.0 * self.nnz * C
        names = {0: "csr_gather_kernel<1>", 1: "csr_gather_kernel<4>", 2: "csr_slab_kernel"}
        lik = smp.distribution.separate_distributions[1]
        plan = lik.__dict__.get("_scratch_cache", {}).get(("csr_slab", C))
        shapes = (plan.shape_g, plan.shape_gt) if plan is not None else None
        kern = (f"{names[shapes[0][0]]} (G @ (Q - c) - d_c) + {names[shapes[1][0]]} (G^T @ R), shapes picked by "
                f"the autotuner {list(shapes[0])} / {list(shapes[1])}" if shapes else "CSR products G @ Q, G^T @ R")
        return {"kernel": kern, "bound": "hbm", "unit": "GB/s", "work": work,
                "work_name": "algorithmic_bytes_per_launch",
                "extra": {"nnz": int(self.nnz), "gather_bytes_per_launch": gather}}

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
        return {"kernel": "srcloc_f32_kernel<true> (one thread per chain and event lane, pair data in shared memory)",
                "bound": "fp32",
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
# The FWI workload's reference run: one long plain-HMC run on the GPU
# (tests/golden/make_fwi_reference.py) gives the posterior moments the
# surrogate-driven run is judged against, plain HMC's ESS per chain-proposal
# with lag windows that truncate, and posterior draws the chains start from.
FWI_REFERENCE = os.path.join(ROOT, "tests", "golden", "fwi_reference.npz")
# Validity of the headline: at least this fraction of the parameters' ESS lag
# windows must truncate (Geyer), and the surrogate run's posterior means and
# standard deviations must agree with the reference run's within their joint
# Monte Carlo error (|z| at most this, over all 600 parameters)
FWI_MIN_TRUNCATED = 0.95
FWI_MAX_Z = 4.5
# DRAM bytes (read + write) of one forward time step at C = 64 from one ncu
# capture of velocity_tma_kernel (60.5 + 0.4 MB) and stress_tma_kernel
# (69.0 + 1.2 MB) on a cold cache; in the time loop the fields stay in L2 and
# DRAM moves less
FWI_STEP_DRAM_BYTES = 131.0e6
# DRAM bytes of one time step of an exact gradient at C = 64 (ncu, cold cache):
# forward with the velocity store 131 MB + adjoint velocity pass 195.6 MB +
# adjoint stress pass 70.7 MB
FWI_GRADIENT_STEP_DRAM_BYTES = 397.3e6


class FwiWorkload:
    name = ("elastic P-SV FWI 200x100 cells (+20-cell sponge), h=5 m, dt=0.5 ms, nt=1500, 4 shots x 20 receivers, "
            "25 Hz Ricker, blobs 20x10 x (vp,vs,rho) = 600 params, Normal prior 10%, 64 chains, FP32 stencils, "
            "scalar-potential network surrogate 600-512-512-1 vs plain HMC")
    kind = "fwi"
    chains, L = 64, 10
    stepsize = 0.12  # prior-whitened units: the mass matrix is the prior precision
    noise_fraction = 10.0  # data noise std / RMS of the true records
    hidden = (512, 512)
    # a step is one block of proposals of every chain: `block` surrogate-
    # driven ones (20 steps = 2000 proposals), or, when the screen falls back
    # to plain HMC, enough exact ones for 100 timed proposals in all
    default_steps, default_warmup = 20, 3
    block = 100
    burn_in = 12  # exact proposals recording (position, gradient) training pairs
    # gradient correlation at every k-th time step (psvWave's snapshot_interval)
    snapshot_interval = 1

    def __init__(self, seed=0, chains=None, snapshot_interval=None):
        from hmclab_gb300 import fwi as F

        if chains is not None:
            self.chains = chains
        if snapshot_interval is not None:
            self.snapshot_interval = int(snapshot_interval)
        self.seed = seed
        self.cfg = F.ElasticConfig(snapshot_interval=self.snapshot_interval)
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

    # algorithmic HBM bytes of one time step of an exact gradient: the forward
    # step with the velocity store (80 + 8 B) plus the adjoint velocity pass
    # (112 B: adjoint fields, temporaries, stored velocities of two steps,
    # read-modify-write of five gradient accumulators) and stress pass (56 B)
    def gradient_bytes_per_step(self):
        return 256.0 * self.cells * self.chains

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
                "snapshot_interval": self.snapshot_interval,
                "start": "posterior draws: final states of the reference plain-HMC run"}


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
def load_fwi_reference(wl, path=None):
    """The FWI reference run's fixture as a dict, or None (with the reason)
    when it is missing or was made for other workload settings."""
    path = path or FWI_REFERENCE
    if not os.path.exists(path):
        return None, f"no reference fixture ({os.path.relpath(path, ROOT)})"
    ref = dict(np.load(path))
    want = {"chains": wl.chains, "leapfrog_steps": wl.L, "stepsize": wl.stepsize,
            "noise_fraction": wl.noise_fraction, "seed": wl.seed}
    for k, v in want.items():
        if not np.isclose(float(ref[k]), float(v)):
            return None, f"reference fixture made for {k} = {float(ref[k])}, workload has {v}"
    return ref, None


def moment_check(mean, std, ess, ref):
    """Posterior moments of a run against the reference run's: the largest
    differences in units of the reference std, and z-scores against the
    joint Monte Carlo error (std^2 / ESS of each run for means; std^2 / (2 ESS)
    for standard deviations).  For unbiased chains |z| ~ N(0, 1)."""
    rm, rs, re = ref["mean"], ref["std"], np.maximum(np.abs(ref["ess"]), 1.0)
    e = np.maximum(np.abs(ess), 1.0)
    z_mean = (mean - rm) / np.sqrt(std**2 / e + rs**2 / re)
    z_std = (std - rs) / np.sqrt(std**2 / (2 * e) + rs**2 / (2 * re))
    return {"mean": float(np.max(np.abs(mean - rm) / rs)), "std": float(np.max(np.abs(std - rs) / rs)),
            "mc_floor": float(1.0 / np.sqrt(e.min())), "mean_z_max": float(np.abs(z_mean).max()),
            "std_z_max": float(np.abs(z_std).max()), "mean_z_frac_above_3": float(np.mean(np.abs(z_mean) > 3)),
            "within_2pct_of_reference_std": bool(np.max(np.abs(mean - rm) / rs) <= 0.02
                                                 and np.max(np.abs(std - rs) / rs) <= 0.02)}


def fwi_validity(ess_raw, mc):
    """Reasons the surrogate run's min-ESS/s is not a valid headline (empty
    when it is): lag windows that did not truncate, or moments inconsistent
    with the reference run."""
    reasons = []
    truncated = float(np.mean(np.asarray(ess_raw) >= 0))
    if truncated < FWI_MIN_TRUNCATED:
        reasons.append(f"only {truncated:.2f} of the parameters' ESS lag windows truncated (need "
                       f"{FWI_MIN_TRUNCATED}): the run is too short for its autocorrelation")
    if mc is None:
        reasons.append("no reference moments to check the run against")
    elif max(mc["mean_z_max"], mc["std_z_max"]) > FWI_MAX_Z:
        reasons.append(f"moments disagree with the reference run beyond Monte Carlo error (max |z| "
                       f"{max(mc['mean_z_max'], mc['std_z_max']):.1f} > {FWI_MAX_Z})")
    return reasons


def _fwi_shot_task(task):
    """One full-size shot of the FP64 C restatement: (forward seconds,
    forward + adjoint seconds); a process-pool task."""
    from oracle import fwi as OF

    return OF.timed_shot(task)


def fwi_cpu_shots(wl, cores, shots_per_core=1):
    """Run `shots_per_core` forward + adjoint shots of the FP64 C restatement
    (oracle/fwi_oracle.c) on every host core at once (spawn pool, one shot
    per task, each on its own chain's model); returns per-shot forward and
    forward + adjoint seconds (medians) and the wall time."""
    import multiprocessing as mp

    from oracle import build_oracle
    from hmclab_gb300 import fwi as F

    build_oracle.build()
    cfg = wl.cfg
    bg = F.layered_model(cfg, anomalies=True)
    vp, vs, rho = (cfg.extend(f) for f in bg)
    tasks = [(cfg.nxc, cfg.nzc, cfg.nt, cfg.h, cfg.dt, cfg.taper(), cfg.ricker(), cfg.src[k % cfg.n_shots],
              cfg.rec_x, cfg.rec_z, rho, vp, vs) for k in range(cores * shots_per_core)]
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(_fwi_shot_task, tasks, chunksize=1)
    wall = time.perf_counter() - t0
    return float(np.median([r[0] for r in res])), float(np.median([r[1] for r in res])), wall


def fwi_cpu_rate(wl, t_fwd, t_grad, cores):
    """Plain-HMC chain-proposals/s of the CPU path, one chain per core: a
    proposal is L exact gradients (4 shots forward + adjoint) and one misfit
    (4 forward shots)."""
    return cores / (wl.cfg.n_shots * (wl.L * t_grad + t_fwd))


def run_fwi_reference_arm(args, wl):
    """Plain HMC's hot path on the host cores: the FP64 C restatement of the
    elastic stencils, one chain per core.  A step is one forward + adjoint
    shot of every core's chain (a bounded sample of a proposal, which is
    4 shots x (10 gradients + 1 misfit)); min-ESS/s converts the measured
    chain-proposals/s with plain HMC's ESS per chain-proposal from the
    reference run (the same algorithm on the GPU; a CPU run long enough to
    estimate it takes hours)."""
    cores = os.cpu_count()
    ref, why = load_fwi_reference(wl)
    t_fwd, _, _ = fwi_cpu_shots(wl, cores)  # warm-up step, also gives the forward cost
    for _ in range(args.warmup - 1):
        fwi_cpu_shots(wl, cores)
    per_step, grads = [], []
    for _ in range(args.steps):
        _, tg, wall = fwi_cpu_shots(wl, cores)
        per_step.append(wall)
        grads.append(tg)
    t_grad = float(np.median(grads))
    rate = fwi_cpu_rate(wl, t_fwd, t_grad, cores)
    e = float(ref["ess_per_chain_proposal"]) if ref is not None else None
    value = rate * e if e is not None else None
    sample = (f"{args.steps} steps of one full-size forward + adjoint shot per core ({cores} cores, FP64 C "
              f"restatement; forward {t_fwd:.2f} s, forward + adjoint {t_grad:.2f} s per shot); chain-proposals/s "
              f"= cores / (4 shots x (L x gradient + misfit)) = {rate:.4g}, times plain HMC's min-ESS per "
              f"chain-proposal from the reference run ({e})")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(per_step)), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": wl.config(),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "chain_proposals_per_s": rate, "ess_per_chain_proposal": e,
    }
    if why:
        line["reason"] = why
    print(json.dumps(line))


def gradient_step_timing(lik, smp, n_iter=2):
    """Seconds of one time step of an exact gradient (forward with store,
    adjoint velocity and stress passes) over all chains: a 4-shot gradient
    timed with CUDA events on the sampler stream, divided by shots x nt."""
    import torch

    st = smp.stream
    h = st.cuda_stream
    g = torch.empty_like(smp.q_cur)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(st):
        lik._device_gradient(smp.q_cur, g, False, "float32", h)
        ev0.record(st)
        for _ in range(n_iter):
            lik._device_gradient(smp.q_cur, g, False, "float32", h)
        ev1.record(st)
    st.synchronize()
    return ev0.elapsed_time(ev1) / 1e3 / n_iter / (lik.config.n_shots * lik.config.nt)


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


def variogram_min(q, std, lag=1):
    """Smallest per-parameter mean squared displacement over `lag` draws, in
    units of the posterior variance: min_i mean_(t,c) (q[t+lag,i,c] -
    q[t,i,c])^2 / (2 std_i^2), for draws q [N][d][C] (device) and the
    posterior std from a long reference run.  It equals 1 - rho_i(lag) (the
    autocorrelation at that lag) without estimating the variance from the
    short run itself, so a short run that has not yet decorrelated reads low
    instead of looking converged."""
    import torch

    s = torch.as_tensor(np.asarray(std, np.float64), device=q.device)[:, None]
    dq = (q[lag:].double() - q[:-lag].double()) / s
    return float((dq * dq).mean(dim=(0, 2)).min() / 2.0)


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
    K, W, Nb = args.steps, args.warmup, args.burn_in
    ref, ref_why = load_fwi_reference(wl)
    # chains start at the reference run's final states (posterior draws): a
    # converged exact burn-in, which this bench cannot afford to repeat
    q_init = ref["q_final"] if ref is not None else wl.q0
    post_std = ref["std"] if ref is not None else wl.pb["prior_std"]
    kw = wl.sampler_kwargs()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    t_setup = time.perf_counter() - t_setup

    # ---- exact proposals from the start states, recording training pairs --
    R = args.refresh_interval if args.refresh_interval > 0 else None
    B_s = args.block
    extra = (W + K) * B_s // R * C if R else 0  # rows the refreshes of a surrogate run append
    data = S.TrainingSet(d, Nb * L * C + extra + 4 * C, values=args.value_weight > 0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    burn = H.Samplers.HMC(seed=sharding.rank_seed(100, rank)).sample(None, post, initial_model=q_init, proposals=Nb,
                                                                     training_set=data, keep_samples=True, **kw)
    t_burn = time.perf_counter() - t0
    q_start = burn.current_model
    acc_burn = float(np.mean(burn.accepted_proposals) / Nb)
    decor_plain = variogram_min(burn.samples_device[0], post_std, 1)

    # ---- surrogate training on the device ---------------------------------
    kind = S.PotentialSurrogate if args.surrogate == "potential" else S.MLPSurrogate
    net = kind(d, hidden=wl.hidden, seed=rank)
    if args.surrogate == "potential":
        net.value_weight = args.value_weight
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fit = net.fit(data, steps=args.train_steps, batch=256, lr=1e-3, holdout_fraction=0.1)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    net.freeze()

    # ---- pilot (untimed): the surrogate run's trajectory ------------------
    # A few proposals per (L, stepsize) from the start states; the setting
    # with the largest acceptance x (trajectory length)^2 — the diffusive-
    # regime gain per proposal, length capped at the plain run's — is used.
    # --surrogate-L / --surrogate-stepsize fix it.
    pilot = []
    if args.surrogate_L is None or args.surrogate_stepsize is None:
        tau_max = args.pilot_max_length * wl.stepsize * wl.L
        for L_s in (2, 4, 8, 16, 32):
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
    kw_s = dict(kw, amount_of_steps=L_best, stepsize=eps_best)
    refresh_kw = dict(training_set=data, refresh_interval=R, refresh_steps=args.refresh_steps) if R else {}

    # ---- screen (untimed): surrogate against plain HMC ---------------------
    # A short surrogate run (with its refreshes) measures its cost per
    # proposal; with it, the number of surrogate proposals `lag` that cost
    # one plain proposal.  How far each sampler decorrelates its slowest
    # parameter in that time (variogram_min: plain HMC over one proposal of
    # the exact burn-in, the surrogate over `lag` proposals) decides: plain
    # HMC is the fallback, and with --sampler auto the timed run uses the
    # surrogate only when it decorrelates further.  (The jump of a single
    # surrogate proposal over-predicts: its successive jumps partly undo each
    # other, and a short run's ESS windows end long before its chains
    # decorrelate.)
    screen = H.Samplers.HMC(seed=sharding.rank_seed(170, rank))
    n_screen = args.screen_proposals
    screen.prepare(None, post, initial_model=q_start, proposals=n_screen, keep_samples=True, surrogate=net,
                   **dict(refresh_kw, refresh_interval=min(R, n_screen // 2) if R else None), **kw_s)
    ev_a, ev_b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev_a.record(screen.stream)
    screen.run(n_screen)
    ev_b.record(screen.stream)
    screen.stream.synchronize()
    t_screen = ev_a.elapsed_time(ev_b) / 1e3 / n_screen
    screen.finish()
    t_plain_burn = t_burn / Nb  # wall seconds per exact proposal (recording included)
    lag = int(min(max(round(t_plain_burn / t_screen), 1), n_screen // 2))
    q_screen = screen.samples_device[0]
    decor_sur = variogram_min(q_screen, post_std, lag)
    acc_screen = float(np.mean(screen.accepted_proposals) / n_screen)
    if args.sampler == "auto":
        sampler = "surrogate" if decor_sur > decor_plain * (lag * t_screen / t_plain_burn) else "plain"
    else:
        sampler = args.sampler
    choice = {"rule": "surrogate when, per second, it decorrelates its slowest parameter further than plain HMC "
                      "(1 - autocorrelation over the surrogate proposals that cost one plain proposal, against plain "
                      "HMC's over one proposal; posterior std from the reference run)",
              "sampler": sampler, "forced": args.sampler != "auto",
              "surrogate": {"proposals": n_screen, "ms_per_proposal": 1e3 * t_screen, "acceptance": acc_screen,
                            "lag": lag, "decorrelation_over_lag": decor_sur,
                            "single_proposal_decorrelation": variogram_min(q_screen, post_std, 1)},
              "plain": {"proposals": Nb, "ms_per_proposal": 1e3 * t_plain_burn, "acceptance": acc_burn,
                        "decorrelation_over_one_proposal": decor_plain,
                        "note": "from the exact burn-in (wall time, pair recording included)"},
              "estimated_speedup_of_surrogate": (decor_sur / (lag * t_screen)) / (decor_plain / t_plain_burn)
              if decor_plain > 0 else None}

    # ---- the timed run: W untimed blocks, then K timed blocks --------------
    # The run goes through the public API from host arrays to host arrays:
    # `e2e` is its wall time from the upload of the start states (prepare) to
    # the samples back on the host; `value` uses the device time of the K
    # timed blocks (CUDA events on the sampler's stream).
    if sampler == "surrogate":
        B = B_s
        run_kw = dict(kw_s, surrogate=net, **refresh_kw)
    else:
        # at least 100 timed proposals: the split-chain ESS windows (half the
        # run) then reach 50 lags, where plain HMC's autocorrelation (about 4
        # proposals) has died out for nearly every parameter; 40 proposals
        # truncated only 29 % of them
        B = args.plain_block if args.plain_block else max(2, -(-100 // K))
        run_kw = dict(kw)
    torch.cuda.synchronize()
    t_e2e0 = time.perf_counter()
    smp_s = H.Samplers.HMC(seed=sharding.rank_seed(200, rank))
    smp_s.prepare(None, post, initial_model=q_start, proposals=(W + K) * B, keep_samples=True, **run_kw)
    smp_s.run(W * B)
    smp_s.stream.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    l0 = _lib.launch_count()
    for k in range(K):
        with torch.cuda.stream(smp_s.stream):
            flush.fill_(float(k))
            evs[k][0].record(smp_s.stream)
        smp_s.run(B)
        evs[k][1].record(smp_s.stream)
    torch.cuda.synchronize()
    launches = _lib.launch_count() - l0
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    t_s = sum(a.elapsed_time(b) for a, b in evs) / 1e3
    smp_s.finish()
    host_q, host_x = smp_s.samples_host()
    t_e2e = time.perf_counter() - t_e2e0
    t_step = forward_step_timing(lik, smp_s)
    t_gstep = gradient_step_timing(lik, smp_s) if sampler == "plain" else None
    qall = smp_s.samples_device[0]  # [(W+K)*B][d][C]
    qs = qall[W * B:]
    N = qs.shape[0]
    # acceptance per block, read from the samples (a chain accepted when its position changed)
    moved = (qall[1:] != qall[:-1]).any(dim=1).double().mean(dim=1).cpu().numpy()
    acc_blocks = [round(float(moved[max(0, k * B - 1):(k + 1) * B - 1].mean()), 4) for k in range(W + K)]
    # lag windows up to half the run
    ess_s_raw = diagnostics.ess(qs, lags=min(N // 2, 1000))
    acc_s = float(np.mean(smp_s.accepted_proposals) / ((W + K) * B))
    # rank normalisation compares every pooled draw with every other (S^2 per
    # parameter); reported when that stays below the library's limit
    S_pool = N * C
    bulk_s = (np.abs(diagnostics.ess(qs, lags=min(N // 2, 1000), rank_normalize=True))
              if S_pool * S_pool * d <= 1.0e12 else None)
    ess_s, t_s = sharding.combine_ess(np.abs(ess_s_raw), t_s)
    if bulk_s is not None:
        bulk_s, _ = sharding.combine_ess(bulk_s, t_s)
    mean_s, std_s = sharding.combine_moments(*diagnostics.moments(qs), N * C)
    mc = moment_check(mean_s, std_s, ess_s, ref) if ref is not None else None
    reasons = fwi_validity(ess_s_raw, mc)
    if ref_why:
        reasons.insert(0, ref_why)
    value_measured = float(ess_s.min() / t_s)
    value = value_measured if not reasons else None
    e_plain = float(ref["ess_per_chain_proposal"]) if ref is not None else None
    if sampler == "plain":
        plain = {"value": value_measured, "source": "the timed run itself", "ms_per_proposal": 1e3 * t_s / (K * B),
                 "acceptance": acc_s, "ess_per_chain_proposal": float(ess_s.min()) / (N * C * world)}
    else:
        # plain HMC's cost per proposal timed here; its ESS per chain-proposal
        # from the reference run
        Kp = args.plain_steps
        smp_p = H.Samplers.HMC(seed=sharding.rank_seed(300, rank))
        smp_p.prepare(None, post, initial_model=q_start, proposals=Kp, keep_samples=False, **kw)
        evp = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(Kp)]
        for k in range(Kp):
            with torch.cuda.stream(smp_p.stream):
                flush.fill_(float(k))
                evp[k][0].record(smp_p.stream)
            smp_p.run(1)
            evp[k][1].record(smp_p.stream)
        smp_p.stream.synchronize()
        t_p = sum(a.elapsed_time(b) for a, b in evp) / 1e3
        smp_p.finish()
        plain = {"value": e_plain * C * world * Kp / t_p if e_plain is not None else None,
                 "source": f"{Kp} timed proposals x the reference run's ESS per chain-proposal",
                 "ms_per_proposal": 1e3 * t_p / Kp, "acceptance": float(np.mean(smp_p.accepted_proposals) / Kp),
                 "ess_per_chain_proposal": e_plain}

    # ---- end to end: the same run, wall clock, host arrays in and out ------
    refreshes_timed = getattr(smp_s, "refreshes", 0)
    ess_e = np.abs(diagnostics.ess(torch.from_numpy(host_q).to("cuda"), lags=min(host_q.shape[0] // 2, 1000)))
    e2e_measured = float(ess_e.min() / t_e2e)
    step_text = (f"{B} surrogate-driven proposals of every chain" if sampler == "surrogate" else
                 f"{B} plain HMC proposals of every chain (the fallback the screen chose)")

    hbm, bf16, bf16s, src = peaks()
    achieved = wl.stencil_bytes_per_step() / t_step / 1e9
    l2 = l2_copy_rate()
    forward_roof = {
        "kernel": "fwi forward time step: velocity_tma_kernel + stress_tma_kernel (the exact misfit)",
        "bound": "l2", "achieved": achieved, "peak": l2, "unit": "GB/s", "frac": achieved / l2,
        "peak_source": "measured in this run: read + write rate of a copy over a 2 x 40 MB L2-resident buffer",
        "hbm_peak": hbm, "hbm_peak_source": src, "frac_of_hbm": achieved / hbm,
        "traffic": FWI_STEP_DRAM_BYTES, "traffic_source": "ncu capture of one velocity + one stress launch at "
                                                          "C = 64, default (cold) cache control",
        "step_s": t_step, "algorithmic_bytes_per_step": wl.stencil_bytes_per_step(),
        "note": "one shot's fields and parameters (86 MB at 64 chains) stay in the 129 MB L2 over the time loop, so "
                "the binding roof is the L2 rate, not HBM; DRAM traffic per step (`traffic`, cold cache) is 0.76 "
                "of the algorithmic bytes"}
    if t_gstep is not None:
        # plain HMC spends its time in exact gradients: forward with store and
        # the adjoint passes, whose fields, temporaries and accumulators
        # (20 fields, 172 MB at 64 chains) exceed the L2
        g_ach = wl.gradient_bytes_per_step() / t_gstep / 1e9
        roof = {"kernel": "fwi exact-gradient time step: velocity_tma_kernel + stress_tma_kernel (with store), then "
                          "adj_velocity_tma_kernel<1, true> + adj_stress_tma_kernel<4>",
                "bound": "hbm", "achieved": g_ach, "peak": hbm, "unit": "GB/s", "frac": g_ach / hbm,
                "peak_source": src, "traffic": FWI_GRADIENT_STEP_DRAM_BYTES,
                "traffic_source": "ncu captures of the forward, adjoint velocity and adjoint stress launches at "
                                  "C = 64, default (cold) cache control",
                "step_s": t_gstep, "algorithmic_bytes_per_step": wl.gradient_bytes_per_step(),
                "l2_peak": l2, "frac_of_l2": g_ach / l2,
                "note": "part of the working set stays in L2, so the algorithmic rate can exceed the HBM copy rate; "
                        "DRAM traffic per step (cold cache) is 0.72 of the algorithmic bytes",
                "forward_stencil": forward_roof}
    else:
        roof = forward_roof
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": 1e3 * t_s / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded; records from the device forward of the true model + noise)",
        "config": {**wl.config(), "step": step_text, "sampler": sampler,
                   "start": "posterior draws: final states of the reference plain-HMC run"
                            if ref is not None else "m_true + 0.3 prior std (no reference run)"},
        "valid": not reasons, "invalid_reasons": reasons, "value_measured": value_measured,
        "sampler": sampler, "sampler_choice": choice,
        "speedup_vs_plain": (float(value_measured / plain["value"]) if sampler == "surrogate" and plain["value"]
                             else 1.0 if sampler == "plain" else None),
        "including_burn_in_and_training": {
            "value": float(ess_s.min() / (t_burn + t_train + t_s)),
            "note": "min-ESS over (exact training-pair proposals + surrogate training + sampling) seconds"},
        "ess_window_truncated": float(np.mean(ess_s_raw >= 0)), "proposals_per_chain": N,
        "rank_normalised_bulk": ({"value": float(bulk_s.min() / t_s)} if bulk_s is not None else
                                 {"value": None, "note": "skipped: pooled rank normalisation of this many draws "
                                                         "exceeds the library's comparison limit"}),
        "refresh": {"interval": R if sampler == "surrogate" else None,
                    "adam_steps": args.refresh_steps if R and sampler == "surrogate" else 0,
                    "refreshes": refreshes_timed,
                    "note": "after every block: exact gradient and misfit at the chains' current positions appended "
                            "to the training set, then more training; inside the timed region"},
        "acceptance": acc_s, "acceptance_per_block": acc_blocks,
        "surrogate_trajectory": {"leapfrog_steps": L_best, "stepsize": eps_best,
                                                      "pilot": [[L_, e_, round(a_, 4)] for _, L_, e_, a_ in pilot]},
        "plain": plain,
        "reference_run": {"ess_per_chain_proposal": e_plain,
                          "source": "reference plain-HMC run (tests/golden/fwi_reference.npz): "
                                    f"{int(ref['proposals']) if ref is not None else 0} proposals x {C} chains, "
                                    "lag windows truncated"},
        "moment_error_vs_reference": mc,
        "training_proposals": {"proposals": Nb, "seconds": t_burn, "acceptance": acc_burn, "pairs": data.count},
        "surrogate": {"kind": args.surrogate, "train_steps": args.train_steps, "train_seconds": t_train,
                      "train_pairs": fit["train_pairs"], "heldout_pairs": fit["heldout_pairs"],
                      "heldout_rel_error_linear_start": fit["heldout"][0][1], "heldout_rel_error": fit["best_heldout"],
                      "value_weight": args.value_weight if args.surrogate == "potential" else None,
                      "heldout_value_error": fit.get("best_heldout_value"),
                      "heldout_value_error_start": (fit.get("heldout_value") or [(0, None)])[0][1],
                      "best_step": fit["best_step"]},
        "setup_seconds": t_setup,
        "e2e": {"value": e2e_measured if not reasons else None, "value_measured": e2e_measured, "unit": UNIT,
                "h2d_bytes_per_step": int(q_start.size * 8 / (W + K)),
                "d2h_bytes_per_step": int(B * (d * C * 4 + C * 8)),
                "seconds": t_e2e, "note": "wall time of the timed run itself through the public API (prepare from "
                                          "host start states, W + K blocks, samples back to the host); ESS over "
                                          "all its draws"},
        "gpu_launches": int(launches),
        "roofline": roof,
        "clocks": clk,
    }
    if args.surrogate == "gradient":
        line["config"]["surrogate"] = ("MLP 600-512-512-600 GELU + linear skip (outputs the gradient), BF16 weights, "
                                       "FP32 accumulate")
    if rank == 0 and not args.no_cpu_baseline:
        cores = os.cpu_count()
        t_fwd, t_grad, wall = fwi_cpu_shots(wl, cores)
        rate = fwi_cpu_rate(wl, t_fwd, t_grad, cores)
        line["cpu_baseline"] = {
            "value": rate * e_plain if e_plain is not None else None, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": (f"one full-size forward + adjoint shot of the FP64 C restatement per core ({wall:.1f} s wall; "
                       f"forward {t_fwd:.2f} s, forward + adjoint {t_grad:.2f} s per shot); chain-proposals/s = "
                       f"{rate:.4g} times plain HMC's min-ESS per chain-proposal from the reference run ({e_plain})")}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------------------
# Profiling cases: small, self-contained runs of the hot-path kernels
#
#   python bench.py --profile-case fwi-gradient [--nt 100] [--chains 64] [--repeat 2]
#   python bench.py --profile-case fwi-misfit   [--nt 100] [--chains 64] [--repeat 2]
#   python bench.py --profile-case mlp          [--chains 64] [--repeat 3]
#   python bench.py --profile-case potential    [--chains 64] [--repeat 3]
#   python bench.py --profile-case persistent   [--chains 4096] [--repeat 2]
#   python bench.py --profile-case tomo         [--chains 1024] [--repeat 2]
#   python bench.py --profile-case srcloc       [--chains 8192] [--repeat 2]
#
# The FWI cases build the workload's full spatial grid (200x100 cells plus
# the 20-cell sponge, 4 shots, 600 blob parameters) with a shortened record
# (`--nt` time steps) so that a profiler capture of every launch of one
# gradient stays small, run the evaluation `--repeat` times and synchronise.
# `mlp` runs the surrogate's training step (batch 256) and its sampler-side
# prediction for 600 parameters; `potential` the same for the scalar-potential
# surrogate (gradient pass and double backpropagation).  `persistent` runs
# blocks of 10 proposals of a d = 50 dense linear-Gaussian posterior (FP32,
# 10 leapfrog steps) through the persistent kernel; `tomo` and `srcloc`
# evaluate the gradient of the tomography (64 x 64 cells, 2000 rays) and
# source-location (32 events, 200 stations) posteriors.
# ---------------------------------------------------------------------------
PROFILE_CASES = ("fwi-gradient", "fwi-misfit", "mlp", "potential", "persistent", "tomo", "srcloc")


def _profile_fwi(nt, chains, snapshot_interval=1):
    import numpy as np
    import torch

    from hmclab_gb300 import fwi as F
    from hmclab_gb300 import problems

    cfg = F.ElasticConfig(nt=nt, snapshot_interval=snapshot_interval)
    pb = problems.elastic_fwi(cfg, 20, 10, prior_fraction=0.1, noise_fraction=10.0, seed=0)
    rng = np.random.default_rng(1)
    q = pb["m_true"][:, None] + 0.3 * pb["prior_std"][:, None] * rng.normal(size=(pb["m_true"].size, chains))
    return pb["posterior"], torch.from_numpy(q).float().cuda().contiguous()


def run_profile_case(a):
    """--profile-case: a small, self-contained run of one hot-path kernel for
    an ncu capture (see PROFILE_CASES); prints one status line, no JSON."""
    import torch

    torch.cuda.set_device(0)
    a.chains = a.chains or (4096 if a.profile_case == "persistent" else 1024 if a.profile_case == "tomo"
                            else 8192 if a.profile_case == "srcloc" else 64)
    a.case = a.profile_case
    if a.case.startswith("fwi"):
        post, q = _profile_fwi(a.nt, a.chains, a.snapshot_interval or 1)
        out = torch.empty_like(q)
        x = torch.empty(a.chains, dtype=torch.float64, device="cuda")
        t0 = time.perf_counter()
        for _ in range(a.repeat):
            if a.case == "fwi-gradient":
                post.gradient_batch(q, out=out)
            else:
                post.misfit_batch(q, out=x)
        torch.cuda.synchronize()
        print(f"{a.case}: nt={a.nt} chains={a.chains} repeat={a.repeat} {time.perf_counter() - t0:.3f} s")
    elif a.case == "persistent":
        import numpy as np

        import hmclab_gb300 as H

        d = 50
        rng = np.random.default_rng(0)
        G = rng.normal(size=(2 * d, d)) / np.sqrt(d)
        dat = G @ rng.normal(size=(d, 1)) + 0.1 * rng.normal(size=(2 * d, 1))
        post = H.Distributions.BayesRule([H.Distributions.Normal(np.zeros((d, 1)), np.ones((d, 1))),
                                          H.Distributions.LinearMatrix(G, dat, 0.01, dtype=np.float64)])
        w = np.sqrt(np.linalg.eigvalsh(G.T @ G / 0.01).max())
        smp = H.Samplers.HMC(seed=1).prepare(None, post, stepsize=0.5 / w, amount_of_steps=10,
                                            proposals=10 * (a.repeat + 1), chains=a.chains, dtype="float32",
                                            proposals_per_graph=10, persistent=True)
        smp.run(10 * (a.repeat + 1))
        smp.finish()
        print(f"persistent: d={d} chains={a.chains} warps={smp._persistent.warps} ok")
    elif a.case in ("tomo", "srcloc"):
        import numpy as np

        import hmclab_gb300 as H
        from hmclab_gb300 import problems

        rng = np.random.default_rng(0)
        if a.case == "tomo":
            t = problems.tomography(64, 64, 2000, 1.0, 0.01, 0)
            post = H.Distributions.BayesRule([H.Distributions.Normal(t["background"], np.full((4096, 1), 0.0025)),
                                              H.Distributions.LinearMatrix(t["G"], t["d"], 1e-4)])
            q = t["m_true"] + 0.01 * rng.normal(size=(4096, a.chains))
        else:
            t = problems.source_location(32, 200, 40.0, 10.0, 5.0, 0.05, 0)
            post = H.Distributions.SourceLocation3D(t["rx"], t["ry"], t["rz"], t["obs"], 0.05)
            q = t["m_true"] + 0.01 * rng.normal(size=(t["m_true"].size, a.chains))
        M = torch.from_numpy(q).float().cuda().contiguous()
        out = torch.empty_like(M)
        for _ in range(a.repeat):
            post.gradient_batch(M, out=out)
        torch.cuda.synchronize()
        print(f"{a.case}: chains={a.chains} repeat={a.repeat} ok")
    else:
        import numpy as np

        from hmclab_gb300 import surrogate as S

        d = 600
        kind = S.PotentialSurrogate if a.case == "potential" else S.MLPSurrogate
        net = kind(d, hidden=(512, 512), seed=0)
        data = S.TrainingSet(d, 4096)
        rng = np.random.default_rng(0)
        st = torch.cuda.current_stream().cuda_stream
        for k in range(4):
            qb = torch.from_numpy(rng.normal(size=(d, 1024))).float().cuda()
            data.record(qb, 2.0 * qb + torch.tanh(qb), st)
        net.fit_normalization(data)
        for _ in range(a.repeat):
            net.train_step(data, rng.integers(0, 4096, size=256), lr=1e-3)
        torch.cuda.synchronize()
        net.freeze()
        q = torch.from_numpy(rng.normal(size=(d, a.chains))).float().cuda()
        g = torch.empty_like(q)
        for _ in range(a.repeat):
            net.predict_into(q, g, st)
        torch.cuda.synchronize()
        net.check_status()
        print(f"{a.case}: d={d} hidden=512x512 batch=256 chains={a.chains} repeat={a.repeat} ok")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=None)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="fwi", choices=sorted(WORKLOADS))
    ap.add_argument("--sampler", default="auto", choices=["auto", "surrogate", "plain"],
                    help="fwi: sampler of the timed run; auto: the surrogate when the screen finds that it "
                         "decorrelates faster per second than plain HMC, else plain HMC (the fallback)")
    ap.add_argument("--screen-proposals", type=int, default=96,
                    help="fwi: surrogate proposals of the untimed screen against plain HMC")
    ap.add_argument("--plain-steps", type=int, default=3,
                    help="fwi: timed plain proposals giving plain HMC's cost when the surrogate runs")
    ap.add_argument("--block", type=int, default=None, help="fwi: surrogate-driven proposals per step")
    ap.add_argument("--plain-block", type=int, default=None,
                    help="fwi: plain proposals per step when plain HMC runs (default: at least 100 timed proposals)")
    ap.add_argument("--value-weight", type=float, default=1.0,
                    help="fwi: weight of the misfit-value matching loss of the potential surrogate (0: gradients only)")
    ap.add_argument("--refresh-interval", type=int, default=32,
                    help="fwi: surrogate proposals between refreshes of the network on exact gradients at the chains' "
                         "positions (0: never)")
    ap.add_argument("--refresh-steps", type=int, default=300, help="fwi: Adam steps per refresh")
    ap.add_argument("--pilot-max-length", type=float, default=2.0,
                    help="fwi: longest surrogate trajectory the pilot tries, in units of plain HMC's")
    ap.add_argument("--snapshot-interval", type=int, default=None,
                    help="fwi and the FWI profiling cases: the gradient correlates forward and adjoint fields at every "
                         "k-th time step (psvWave's snapshot_interval; 1: every step, the exact discrete gradient)")
    ap.add_argument("--burn-in", type=int, default=None,
                    help="fwi: exact proposals recording the surrogate's training pairs (independent of --warmup)")
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
    ap.add_argument("--profile-case", default=None, choices=PROFILE_CASES,
                    help="run one small profiling case instead of a benchmark (no JSON line)")
    ap.add_argument("--nt", type=int, default=100, help="profiling: time steps of the FWI cases")
    ap.add_argument("--chains", type=int, default=None, help="profiling: chains of the case")
    ap.add_argument("--repeat", type=int, default=2, help="profiling: evaluations of the case")
    args = ap.parse_args()
    if args.profile_case:
        run_profile_case(args)
        return
    wl = (WORKLOADS[args.workload](snapshot_interval=args.snapshot_interval) if args.workload == "fwi"
          else WORKLOADS[args.workload]())
    args.steps = wl.default_steps if args.steps is None else args.steps
    args.warmup = wl.default_warmup if args.warmup is None else args.warmup
    if args.workload == "fwi":
        args.block = wl.block if args.block is None else args.block
        args.burn_in = wl.burn_in if args.burn_in is None else args.burn_in
    assert args.warmup >= 3, "at least 3 warm-up steps"
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        (run_fwi_reference_arm if args.workload == "fwi" else run_reference_arm)(args, wl)
        return
    (run_fwi_arm if args.workload == "fwi" else run_gpu_arm)(args, wl)


if __name__ == "__main__":
    main()
