"""Reference moments of the FWI benchmark posterior from one long plain-HMC
run on the GPU (exact gradients at every leapfrog step), written to
tests/golden/fwi_reference.npz.

The benchmark's surrogate-driven sampler is judged against these moments:
its posterior mean and standard deviation must agree with them within their
joint Monte Carlo error.  The same run gives plain HMC's effective sample
size per chain-proposal with lag windows long enough to truncate (the short
plain run a benchmark can afford cannot resolve it), and posterior draws
(the run's final states) from which the benchmark's chains start.

Run on a GPU (about 20 minutes):
    python tests/golden/make_fwi_reference.py OUT.npz [--burn-in 40] [--proposals 200]

Stored: mean, std, ess (per parameter; negative where the window did not
truncate), rhat, ess_per_chain_proposal (min over parameters), acceptance,
final states q_final [d][C], and the workload's settings for a consistency
check (chains, leapfrog steps, step size, noise, seed)."""
import argparse
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("out")
    ap.add_argument("--burn-in", type=int, default=40)
    ap.add_argument("--proposals", type=int, default=200)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args()

    import torch

    import bench
    import hmclab_gb300 as H
    from hmclab_gb300 import diagnostics

    torch.cuda.set_device(0)
    wl = bench.FwiWorkload(seed=args.seed).build()
    post = wl.posterior()
    kw = wl.sampler_kwargs()
    t0 = time.perf_counter()
    burn = H.Samplers.HMC(seed=7001).sample(None, post, initial_model=wl.q0, proposals=args.burn_in, **kw)
    t_burn = time.perf_counter() - t0
    q_start = burn.current_model
    t0 = time.perf_counter()
    smp = H.Samplers.HMC(seed=7002).sample(None, post, initial_model=q_start, proposals=args.proposals,
                                           keep_samples=True, **kw)
    t_run = time.perf_counter() - t0
    q = smp.samples_device[0]  # [N][d][C]
    N = q.shape[0]
    ess, rhat = diagnostics.ess(q, lags=N // 2, return_rhat=True)
    mean, std = diagnostics.moments(q)
    acc = float(np.mean(smp.accepted_proposals) / args.proposals)
    C = wl.chains
    per = float(np.abs(ess).min() / (N * C))
    np.savez(args.out, mean=mean, std=std, ess=ess, rhat=rhat, ess_per_chain_proposal=per, acceptance=acc,
             q_final=smp.current_model.astype(np.float64), chains=C, leapfrog_steps=wl.L, stepsize=wl.stepsize,
             noise_fraction=wl.noise_fraction, seed=args.seed, burn_in=args.burn_in, proposals=N,
             seconds_per_proposal=t_run / N, burn_in_acceptance=float(np.mean(burn.accepted_proposals) / args.burn_in))
    print(f"burn-in {args.burn_in} proposals in {t_burn:.0f} s; {N} proposals x {C} chains in {t_run:.0f} s "
          f"({t_run / N:.2f} s each), acceptance {acc:.3f}; min ESS {np.abs(ess).min():.0f} "
          f"({per:.4f} per chain-proposal), windows not truncated {np.mean(ess < 0):.3f}, max R-hat {rhat.max():.3f}")


if __name__ == "__main__":
    main()
