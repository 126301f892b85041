"""Benchmark of the batched HMC hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload dense]

A "step" is one HMC proposal (a full leapfrog trajectory plus the accept test)
for every chain of the workload.  Prints one JSON line.

Workload `dense` (the batched dense linear configuration): G 2000x1000 with
N(0, 1/1000) entries, m_true ~ N(0, I), noise sigma 0.05, Normal prior N(0, I),
diagonal mass drawn U[0.5, 2], 20 leapfrog steps, 4096 chains, FP32 state,
FP64 dH accept.  Chains start at exact draws of the analytic posterior, so
every timed proposal is a post-burn-in sample.

metric: min over parameters of the multi-chain ESS of the timed proposals'
samples, divided by the device time of those proposals (min-ESS/s).
Synthetic seeded data; the L2 cache is flushed (256 MiB write) between timed
steps, outside the CUDA-event intervals.

--impl reference: the CPU implementation of the same path (the numpy port of
the reference algorithm, batched over chains, all host BLAS threads) on a
bounded sample of the workload, same metric and unit.
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
    n_data, n_model, chains, L = 2000, 1000, 4096, 20
    noise = 0.05

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

    def config(self):
        return {"workload": self.name, "n_data": self.n_data, "n_model": self.n_model, "chains": self.chains,
                "leapfrog_steps": self.L, "stepsize": self.stepsize, "prior": "Normal(0, I)",
                "mass": "diagonal U[0.5,2]", "precision": "FP32 state, FP64 dH", "l2": "flushed between timed steps",
                "start": "exact posterior draws"}


WORKLOADS = {"dense": DenseWorkload}


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

    lik = O.DensePremul(wl.G, wl.d, wl.noise**2)
    post = O.Sum([O.NormalDiag(np.zeros(wl.n_model), np.ones(wl.n_model)), lik])
    mass = O.Mass("diag", diag=wl.diag)
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
    me = float(np.max(np.abs(mean - wl.post_mean[:, 0]) / wl.post_std))
    se = float(np.max(np.abs(std - wl.post_std) / wl.post_std))
    return float(ess.min() / dt), (me, se), dt, chains * steps * wl.L / dt


def run_reference_arm(args, wl):
    chains = args.cpu_chains
    v, (me, se), dt, lps = cpu_reference_run(wl, chains, args.warmup, args.steps)
    cores = os.cpu_count()
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "impl": "reference", "config": {**wl.config(), "chains": chains},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{chains} chains x {args.steps} proposals of the same workload, numpy port of "
                                   "the reference HMC path batched over chains (BLAS on all host threads)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "leapfrog_steps_per_s": lps, "moment_error": {"mean": me, "std": se},
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------------
def dominant_kernel_timing(post, smp, n_iter=20):
    """Average duration of the dominant kernel with CUDA events on the sampler
    stream, on the live chain state: the fused tensor-core leapfrog step
    (GtG @ Q - Gtd0 + prior, kick, drift, operand re-split) when the sampler
    uses it, else the gradient launch of the likelihood."""
    import torch

    st = smp.stream
    h = st.cuda_stream
    lik = post.separate_distributions[1]
    if smp._fused is not None:
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
    from hmclab_gb300 import _lib, diagnostics

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    post = wl.posterior()
    K, W = args.steps, args.warmup
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # ---- device-resident timed run ---------------------------------------
    smp = H.Samplers.HMC(seed=1000 + rank)
    smp.prepare(None, post, initial_model=wl.q0, proposals=W + K, keep_samples=True, proposals_per_graph=1,
                **wl.sampler_kwargs())
    smp.run(W)
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
        smp.run(1)
        evs[k][1].record(smp.stream)
    torch.cuda.synchronize()
    launches = _lib.launch_count() - launches0 - 0
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    t_dev = sum(a.elapsed_time(b) for a, b in evs) / 1e3
    t_gemm = dominant_kernel_timing(post, smp)
    smp.finish()
    q, x = smp.samples_device  # [N][d][C]
    timed = q[W:]
    ess = np.abs(diagnostics.ess(timed, lags=min(K // 2, 100)))
    mean, std = diagnostics.moments(timed)
    if world > 1:
        t = torch.tensor(np.concatenate([ess, [t_dev]]), dtype=torch.float64)
        parts = [torch.zeros_like(t) for _ in range(world)]
        torch.distributed.all_gather(parts, t)
        ess = sum(p[:-1].numpy() for p in parts)
        t_dev = max(float(p[-1]) for p in parts)
    me, se = diagnostics.moment_error(mean, std, wl.post_mean, wl.post_std)
    value = float(ess.min() / t_dev)
    acc = float(np.mean(smp.accepted_proposals) / (W + K))

    # ---- end to end through the public API with host buffers -------------
    smp2 = H.Samplers.HMC(seed=2000 + rank)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    smp2.sample(None, post, initial_model=wl.q0, proposals=K, keep_samples=True, proposals_per_graph=min(K, 10),
                **wl.sampler_kwargs())
    host_q, host_x = smp2.samples_host()  # [N][d][C] and [N][C] on the host
    t_e2e = time.perf_counter() - t0
    ess2 = np.abs(diagnostics.ess(torch.from_numpy(host_q).to("cuda"), lags=min(K // 2, 100)))
    e2e_value = float(ess2.min() / t_e2e)
    h2d = wl.q0.size * 8 / K
    d2h = (wl.n_model * wl.chains * 4 + wl.chains * 8)

    hbm, bf16, bf16s, src = peaks()
    achieved = wl.gemm_flops() / t_gemm / 1e12
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": 1e3 * t_dev / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded)", "config": wl.config(),
        "leapfrog_steps_per_s": wl.chains * wl.L * K / t_dev * world,
        "moment_error": {"mean": me, "std": se}, "acceptance": acc,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "seconds": t_e2e},
        "gpu_launches": int(launches),
        "roofline": {"kernel": ("chain_gemm_kernel<EPI_STEP>: tcgen05 BF16 hi/lo GtG@Q + prior + kick + drift"
                                if smp._fused is not None else "dense gradient GEMM"),
                     "bound": "tensor", "achieved": achieved, "peak": bf16, "unit": "TFLOP/s",
                     "frac": achieved / bf16, "traffic": None, "peak_source": src, "launch_s": t_gemm,
                     "algorithmic_flop_per_launch": wl.gemm_flops(),
                     "executed_flop_per_launch": 3 * wl.gemm_flops() if smp._fused is not None else wl.gemm_flops()},
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu_baseline:
        v, (cme, cse), dt, lps = cpu_reference_run(wl, args.cpu_chains, 2, args.cpu_steps)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                "sample": f"{args.cpu_chains} chains x {args.cpu_steps} proposals, numpy port "
                                          f"batched over chains ({dt:.1f} s, {lps:.0f} leapfrog steps/s)"}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="dense", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-chains", type=int, default=64)
    ap.add_argument("--cpu-steps", type=int, default=300)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    assert args.warmup >= 3, "at least 3 warm-up steps"
    wl = WORKLOADS[args.workload]()
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        run_reference_arm(args, wl)
        return
    run_gpu_arm(args, wl)


if __name__ == "__main__":
    main()
