"""Small, self-contained runs of the hot-path kernels for profiling.

    python -m hmclab_gb300.profile_cases fwi-gradient [--nt 100] [--chains 64] [--repeat 2]
    python -m hmclab_gb300.profile_cases fwi-misfit   [--nt 100] [--chains 64] [--repeat 2]
    python -m hmclab_gb300.profile_cases mlp          [--chains 64] [--repeat 3]
    python -m hmclab_gb300.profile_cases potential    [--chains 64] [--repeat 3]
    python -m hmclab_gb300.profile_cases persistent   [--chains 4096] [--repeat 2]
    python -m hmclab_gb300.profile_cases tomo         [--chains 1024] [--repeat 2]
    python -m hmclab_gb300.profile_cases srcloc       [--chains 8192] [--repeat 2]

Each case builds the workload's full spatial grid (200x100 cells plus the
20-cell sponge, 4 shots, 600 blob parameters, 64 chains) with a shortened
record (`--nt` time steps) so that a profiler capture of every launch of one
gradient stays small, runs the evaluation `--repeat` times on the current
stream and synchronises.  `mlp` runs the surrogate's training step (batch
256) and its sampler-side prediction for 600 parameters; `potential` the same
for the scalar-potential surrogate (gradient pass and double
backpropagation).  `persistent` runs
blocks of 10 proposals of a d = 50 dense linear-Gaussian posterior (FP32,
10 leapfrog steps) through the persistent kernel; `tomo` and `srcloc` evaluate
the gradient of the tomography (64 x 64 cells, 2000 rays) and source-location
(32 events, 200 stations) posteriors.
"""
import argparse
import time


def _fwi(nt, chains):
    import numpy as np
    import torch

    from hmclab_gb300 import fwi as F
    from hmclab_gb300 import problems

    cfg = F.ElasticConfig(nt=nt)
    pb = problems.elastic_fwi(cfg, 20, 10, prior_fraction=0.1, noise_fraction=10.0, seed=0)
    rng = np.random.default_rng(1)
    q = pb["m_true"][:, None] + 0.3 * pb["prior_std"][:, None] * rng.normal(size=(pb["m_true"].size, chains))
    return pb["posterior"], torch.from_numpy(q).float().cuda().contiguous()


def main(argv=None):
    import torch

    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["fwi-gradient", "fwi-misfit", "mlp", "potential", "persistent", "tomo", "srcloc"])
    ap.add_argument("--nt", type=int, default=100)
    ap.add_argument("--chains", type=int, default=64)
    ap.add_argument("--repeat", type=int, default=2)
    a = ap.parse_args(argv)
    torch.cuda.set_device(0)
    if a.case.startswith("fwi"):
        post, q = _fwi(a.nt, a.chains)
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


if __name__ == "__main__":
    main()
