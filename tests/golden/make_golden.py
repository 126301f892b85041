"""Generate the golden fixtures under tests/golden/ by running the reference
(larsgeb/hmclab, imported through oracle/ref_shim.py) on seeded inputs.

Run from the repository root, in a container that has the reference sources:

    python tests/golden/make_golden.py

Each fixture stores the inputs, the injected random streams (replayed from
`numpy.random.default_rng(seed)` in the reference's draw order) and the
reference's own outputs: the samples file content (d+1, N), accepted counts,
per-proposal step sizes / acceptance rates when autotuning, misfit and
gradient values at probe points, and the positions/gradients of the first
trajectory.
"""
import os
import sys
import tempfile
import warnings

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref_shim  # noqa: E402
from oracle.hmc_oracle import reference_streams  # noqa: E402
from hmclab_gb300 import problems  # noqa: E402

warnings.simplefilter("ignore")
hmclab = ref_shim.load()
if hmclab is None:
    raise SystemExit("reference sources not found; set HMCLAB_REFERENCE_ROOT")
D = hmclab.Distributions
MM = hmclab.MassMatrices
from hmclab.Distributions.LinearMatrix import (  # noqa: E402
    _LinearMatrix_dense_forward_simple_covariance as DenseSimple,
)


def run_reference(posterior, seed, q0, proposals, record_first=False, **kw):
    """HMC(seed).sample on `posterior` from q0 (d,1); returns samples (d+1,N),
    accepted count, sampler, and (q, g) pairs of the first trajectory."""
    rec = []
    if record_first:
        orig = posterior.gradient

        def wrapped(m):
            g = orig(m)
            if len(rec) < kw.get("amount_of_steps", 10) * 4:
                rec.append((m.copy(), g.copy()))
            return g

        posterior.gradient = wrapped
    with tempfile.TemporaryDirectory() as tmp:
        fn = os.path.join(tmp, "s.npy")
        smp = hmclab.Samplers.HMC(seed=seed)
        smp.sample(
            fn,
            posterior,
            initial_model=q0.copy(),
            proposals=proposals,
            overwrite_existing_file=True,
            disable_progressbar=True,
            **kw,
        )
        samples = np.array(smp.load_results())
    if record_first:
        posterior.gradient = orig
    return samples, smp.accepted_proposals, smp, rec


def probes(dist, d, n=4, scale=1.0, center=None, seed=1234):
    rng = np.random.default_rng(seed)
    c = np.zeros((d, 1)) if center is None else center
    pts = [c + scale * rng.normal(size=(d, 1)) for _ in range(n)]
    mis = np.array([dist.misfit(p) for p in pts])
    grads = np.stack([dist.gradient(p)[:, 0] for p in pts], axis=1)
    return np.concatenate(pts, axis=1), mis, grads


def multi_chain(posterior_factory, seeds, q0s, proposals, randomize=True, **kw):
    outs, accs, extras = [], [], []
    for s, q0 in zip(seeds, q0s.T):
        post = posterior_factory()
        samples, acc, smp, _ = run_reference(post, s, q0[:, None], proposals, randomize_stepsize=randomize, **kw)
        outs.append(samples)
        accs.append(acc)
        extras.append(smp)
    return np.stack(outs, axis=-1), np.array(accs), extras


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print(f"wrote {name}: {os.path.getsize(path) / 1024:.1f} KiB")


def streams_for(seeds, d, proposals, randomize=True):
    zs, fs, us = zip(*(reference_streams(s, d, proposals, randomize) for s in seeds))
    return np.stack(zs, -1), np.stack(fs, -1), np.stack(us, -1)


def case_cfg1():
    """G 100x50 N(0,1), noise 0.1, prior N(0,I), unit mass, L=10, eps=0.01, seed 0,
    started at the analytic posterior mean; FP64 (dense premultiplied)."""
    G, d, m_true = problems.dense_linear(100, 50, 1.0, 0.1, seed=0)
    mean, cov = problems.gaussian_posterior(G, d, 0.01, 0.0, 1.0)
    lik = DenseSimple(G, d, 0.01, dtype=np.float64)
    prior = D.Normal(np.zeros((50, 1)), np.ones((50, 1)))
    post = D.BayesRule([prior, lik])
    P = 400
    samples, acc, smp, rec = run_reference(post, 0, mean, P, record_first=True, stepsize=0.01, amount_of_steps=10)
    z, f, u = streams_for([0], 50, P)
    pts, mis, grads = probes(post, 50, center=mean, scale=0.05)
    save(
        "cfg1_dense_lf.npz",
        G=G,
        d=d,
        m_true=m_true,
        q0=mean,
        post_mean=mean,
        post_cov=cov,
        z=z,
        f=f,
        u=u,
        samples=samples[..., None],
        accepted=np.array([acc]),
        traj_q=np.stack([r[0][:, 0] for r in rec[:10]], 0),
        traj_g=np.stack([r[1][:, 0] for r in rec[:10]], 0),
        probe_m=pts,
        probe_misfit=mis,
        probe_grad=grads,
        stepsize=0.01,
        amount_of_steps=10,
    )


def case_public_linearmatrix():
    """The public LinearMatrix (default dtype single: G rounded to FP32 while
    GtG is FP64 and Gtd0 uses the unrounded G) on a 30x12 problem."""
    G, d, _ = problems.dense_linear(30, 12, 1.0, 0.2, seed=7)
    lik = D.LinearMatrix(G.copy(), d.copy(), 0.04)
    pts, mis, grads = probes(lik, 12, scale=1.0)
    save("linearmatrix_public.npz", G=G, d=d, var=0.04, probe_m=pts, probe_misfit=mis, probe_grad=grads)


def case_cfg2_small(prior_kind):
    """Small dense problem with cfg2's structure: G 240x120 N(0,1/120), noise
    0.05, Normal N(0,I) or Laplace(0,1) prior, diagonal mass U[0.5,2], L=20."""
    G, d, m_true = problems.dense_linear(240, 120, (1 / 120) ** 0.5, 0.05, seed=2)
    rng = np.random.default_rng(22)
    diag = rng.uniform(0.5, 2.0, size=(120, 1))
    mean, _ = problems.gaussian_posterior(G, d, 0.0025, 0.0, 1.0)
    C = 3
    seeds = [100 + c for c in range(C)]
    q0 = mean + 0.01 * rng.normal(size=(120, C))

    def factory():
        lik = DenseSimple(G, d, 0.0025, dtype=np.float64)
        if prior_kind == "normal":
            prior = D.Normal(np.zeros((120, 1)), np.ones((120, 1)))
        else:
            prior = D.Laplace(np.zeros((120, 1)), np.ones((120, 1)))
        return D.BayesRule([prior, lik])

    P = 40
    mm = MM.Diagonal(diag.copy())
    samples, accs, _ = multi_chain(factory, seeds, q0, P, stepsize=0.008, amount_of_steps=20, mass_matrix=mm)
    z, f, u = streams_for(seeds, 120, P)
    pts, mis, grads = probes(factory(), 120, center=mean, scale=0.05)
    save(
        f"cfg2_small_{prior_kind}.npz",
        G=G,
        d=d,
        diag=diag,
        q0=q0,
        z=z,
        f=f,
        u=u,
        samples=samples,
        accepted=accs,
        probe_m=pts,
        probe_misfit=mis,
        probe_grad=grads,
        stepsize=0.008,
        amount_of_steps=20,
    )


def case_tomography_small():
    """16x16 straight-ray tomography, 60 rays, sparse LinearMatrix (n < d, no
    premultiplication), Normal prior around the background (sigma 0.05)."""
    tomo = problems.tomography(nx=16, ny=16, n_rays=60, h=1.0, noise_std=0.01, seed=3, anomalies=2)
    G, d, bg = tomo["G"], tomo["d"], tomo["background"]
    n = G.shape[1]
    C = 2
    seeds = [200, 201]
    rng = np.random.default_rng(33)
    q0 = bg + 0.01 * rng.normal(size=(n, C))

    def factory():
        lik = D.LinearMatrix(G.copy(), d.copy(), 1e-4)
        prior = D.Normal(bg.copy(), np.full((n, 1), 0.05**2))
        return D.BayesRule([prior, lik])

    P = 30
    samples, accs, _ = multi_chain(factory, seeds, q0, P, stepsize=0.004, amount_of_steps=10)
    z, f, u = streams_for(seeds, n, P)
    pts, mis, grads = probes(factory(), n, center=bg, scale=0.02)
    save(
        "tomo_small.npz",
        indptr=G.indptr,
        indices=G.indices,
        data=G.data,
        shape=np.array(G.shape),
        d=d,
        background=bg,
        q0=q0,
        z=z,
        f=f,
        u=u,
        samples=samples,
        accepted=accs,
        probe_m=pts,
        probe_misfit=mis,
        probe_grad=grads,
        stepsize=0.004,
        amount_of_steps=10,
    )


def case_srcloc_small():
    """SourceLocation3D, 4 events, 12 stations, inferred velocity, one NaN
    observation (skipped by nansum), unit mass."""
    sl = problems.source_location(n_events=4, n_stations=12, seed=4)
    obs = sl["obs"].copy()
    obs[1, 3] = np.nan
    dist = D.SourceLocation3D(sl["rx"], sl["ry"], sl["rz"], obs, sl["std"].copy(), infer_velocity=True)
    m0 = sl["m_true"]
    C = 2
    seeds = [300, 301]
    rng = np.random.default_rng(44)
    q0 = m0 + 0.01 * rng.normal(size=(17, C))
    P = 30

    def factory():
        return D.SourceLocation3D(sl["rx"], sl["ry"], sl["rz"], obs, sl["std"].copy(), infer_velocity=True)

    samples, accs, _ = multi_chain(factory, seeds, q0, P, stepsize=0.002, amount_of_steps=10)
    z, f, u = streams_for(seeds, 17, P)
    pts, mis, grads = probes(dist, 17, center=m0, scale=0.3)
    # Fixed-velocity variant: misfit/gradient probes only.
    dist_fixed = D.SourceLocation3D(
        sl["rx"], sl["ry"], sl["rz"], obs, sl["std"].copy(), infer_velocity=False, medium_velocity=5.0
    )
    pts_f, mis_f, grads_f = probes(dist_fixed, 16, center=m0[:-1], scale=0.3)
    save(
        "srcloc_small.npz",
        rx=sl["rx"],
        ry=sl["ry"],
        rz=sl["rz"],
        obs=obs,
        std=sl["std"],
        m_true=m0,
        q0=q0,
        z=z,
        f=f,
        u=u,
        samples=samples,
        accepted=accs,
        probe_m=pts,
        probe_misfit=mis,
        probe_grad=grads,
        probe_fixed_m=pts_f,
        probe_fixed_misfit=mis_f,
        probe_fixed_grad=grads_f,
        stepsize=0.002,
        amount_of_steps=10,
    )


def case_full_mass_bounds():
    """6-D correlated Normal with bounds (reflection at base.py:239-270), full
    mass matrix, no step randomisation, plus a Laplace prior term."""
    rng = np.random.default_rng(5)
    A = rng.normal(size=(6, 6))
    cov = A @ A.T / 6 + 0.5 * np.eye(6)
    mean = rng.normal(size=(6, 1))
    lower = mean - 0.8
    upper = mean + 1.2
    mass = np.eye(6) + 0.1 * np.eye(6, k=1) + 0.1 * np.eye(6, k=-1)
    C = 2
    seeds = [400, 401]
    q0 = mean + 0.1 * rng.normal(size=(6, C))
    P = 60

    def factory():
        nrm = D.Normal(mean.copy(), cov.copy(), lower_bounds=lower.copy(), upper_bounds=upper.copy())
        lap = D.Laplace(mean.copy(), np.full((6, 1), 2.0))
        return D.BayesRule([nrm, lap])

    samples, accs, _ = multi_chain(
        factory,
        seeds,
        q0,
        P,
        randomize=False,
        stepsize=0.3,
        amount_of_steps=8,
        mass_matrix=MM.Full(mass.copy()),
    )
    z, f, u = streams_for(seeds, 6, P, randomize=False)
    pts, mis, grads = probes(factory(), 6, center=mean, scale=0.3)
    save(
        "fullmass_bounds.npz",
        cov=cov,
        mean=mean,
        lower=lower,
        upper=upper,
        mass=mass,
        q0=q0,
        z=z,
        f=f,
        u=u,
        samples=samples,
        accepted=accs,
        probe_m=pts,
        probe_misfit=mis,
        probe_grad=grads,
        stepsize=0.3,
        amount_of_steps=8,
    )


def case_integrators_autotune():
    """3-stage and 4-stage integrators, and leapfrog with autotuning and
    online thinning, on a 5-D diagonal Normal."""
    mean = np.arange(5, dtype=float).reshape(5, 1)
    var = np.array([1.0, 2.0, 0.5, 3.0, 1.5]).reshape(5, 1)
    q0 = mean.copy()
    out = {}
    for integ in ("3s", "4s"):
        P = 50
        post = D.Normal(mean.copy(), var.copy())
        samples, acc, _, _ = run_reference(post, 500, q0, P, stepsize=0.4, amount_of_steps=4, integrator=integ)
        out[f"samples_{integ}"] = samples[..., None]
        out[f"accepted_{integ}"] = np.array([acc])
    P = 60
    post = D.Normal(mean.copy(), var.copy())
    samples, acc, smp, _ = run_reference(
        post,
        501,
        q0,
        P,
        stepsize=1.5,
        amount_of_steps=3,
        autotuning=True,
        online_thinning=3,
        target_acceptance_rate=0.7,
        learning_rate=0.6,
    )
    out["samples_auto"] = samples[..., None]
    out["accepted_auto"] = np.array([acc])
    out["auto_stepsizes"] = np.array(smp.stepsizes)[:, 0]
    out["auto_rates"] = np.array(smp.acceptance_rates)[:, 0]
    out["auto_final_stepsize"] = np.array(smp.stepsize)
    z, f, u = streams_for([500], 5, 50)
    za, fa, ua = streams_for([501], 5, 60)
    save("integrators_autotune.npz", mean=mean, var=var, q0=q0, z=z, f=f, u=u, za=za, fa=fa, ua=ua, **out)


class _GridModel:
    """Stands in for the psvWave fdModel that the reference's
    BlobParametrization (ElasticFullWaveform2D.py:229-341) reads: cell-centre
    coordinates of the whole grid as [x][z] arrays, the boundary widths, the
    free-parameter count and a background model vector (vp | vs | rho over
    the physical cells, x fastest).  psvWave itself is not installed."""

    def __init__(self, nx, nz, pad, h, background):
        self.np_boundary, self.nx_inner_boundary, self.nz_inner_boundary = pad, 0, 0
        self.free_parameters = 3 * nx * nz
        self._bg = background
        ix = (np.arange(nx + 2 * pad) - pad + 0.5) * h
        iz = (np.arange(nz + 2 * pad) - pad + 0.5) * h
        self._x, self._z = np.meshgrid(ix, iz, indexing="ij")

    def get_coordinates(self, _all):
        return self._x.copy(), self._z.copy()

    def get_model_vector(self):
        return self._bg.copy()


def case_blob_projection():
    """The reference's Gaussian-blob collocation matrix, its (C^T C)^-1 C^T
    map applied to grid gradients, and the forward map of a blob vector, on a
    12 x 8-cell grid with 4 x 3 blobs per field."""
    import importlib
    import types

    stub = types.ModuleType("psvWave")
    stub.fdModel = _GridModel  # only named in a class annotation at import
    sys.modules.setdefault("psvWave", stub)

    efwi = importlib.import_module("hmclab.Distributions.ElasticFullWaveform2D")
    nx, nz, pad, h, nbx, nbz = 12, 8, 4, 5.0, 4, 3
    rng = np.random.default_rng(17)
    bg = np.concatenate([np.full(nx * nz, 2000.0), np.full(nx * nz, 1100.0), np.full(nx * nz, 2100.0)])
    blob = efwi.BlobParametrization(_GridModel(nx, nz, pad, h, bg), nbx, nbz)
    g = rng.normal(size=(3 * nx * nz, 3))
    m = rng.normal(size=(3 * nbx * nbz, 1)) * 50.0
    save("blob_projection.npz", nx=nx, nz=nz, pad=pad, h=h, nbx=nbx, nbz=nbz, background=bg,
         collocation=blob.collocation_matrix, confusion=blob.confusion_matrix, grid_gradients=g,
         projected=np.stack([blob.inverse_transform(g[:, k]) for k in range(3)], axis=1), blob_model=m,
         fine_model=blob.forward_transform_background(m))


def case_replica_exchange():
    """Parallel tempering through the reference's own ParallelSampleSMP
    (Samplers.py:1807-1977, forked chains exchanging over pipes,
    Samplers.py:589-669): four chains on Normal posteriors tempered by
    T = 1, 2, 4, 8, exchanges after proposals 0, 2, 4, ...  Stored: the
    exchange schedule, every chain's samples file, and the random streams
    each chain's generator produced in the reference's draw order, with the
    exchange uniform the pair's second ("master") chain draws after its
    accept draw."""
    d, C, P, interval = 3, 4, 20, 2
    temps = np.array([1.0, 2.0, 4.0, 8.0])
    mean = np.arange(d, dtype=float).reshape(d, 1)
    var = np.array([1.0, 2.0, 0.5]).reshape(d, 1)
    seeds = [100 + i for i in range(C)]
    with tempfile.TemporaryDirectory() as tmp:
        fns = [os.path.join(tmp, f"chain{i}.npy") for i in range(C)]
        psmp = hmclab.Samplers.ParallelSampleSMP(seed=7)
        psmp.sample([hmclab.Samplers.HMC(seed=s) for s in seeds], fns, [D.Normal(mean.copy(), var * T) for T in temps],
                    overwrite_existing_files=True, proposals=P, exchange=True, exchange_interval=interval,
                    initial_model=[mean.copy() for _ in range(C)],
                    kwargs={"stepsize": 0.5, "amount_of_steps": 3, "disable_progressbar": True})
        samples = np.stack([np.load(fn).T for fn in fns], axis=-1)  # (d+1, N, C)
    sched = np.asarray(psmp.exchange_schedule)
    npairs = C // 2
    z = np.empty((P, d, C))
    f = np.empty((P, C))
    u = np.empty((P, C))
    uex = np.full((sched.shape[0], npairs), np.nan)
    for c, seed in enumerate(seeds):
        rng = np.random.default_rng(seed)
        for n in range(P):
            z[n, :, c] = rng.normal(size=(d, 1))[:, 0]
            f[n, c] = rng.uniform(0.5, 1.5)
            u[n, c] = rng.uniform(0, 1)
            if n % interval == 0:
                row = sched[n // interval]
                pos = int(np.where(row == c)[0][0]) if c in row else -1
                if pos >= 0 and pos % 2 == 1:  # odd position: the pair's master draws the uniform
                    uex[n // interval, pos // 2] = rng.uniform(0, 1)
    save("replica_exchange.npz", mean=mean, var=var, temps=temps, interval=interval, stepsize=0.5, amount_of_steps=3,
         schedule=sched, samples=samples, z=z, f=f, u=u, exchange_u=uex)


if __name__ == "__main__":
    case_cfg1()
    case_public_linearmatrix()
    case_cfg2_small("normal")
    case_cfg2_small("laplace")
    case_tomography_small()
    case_srcloc_small()
    case_full_mass_bounds()
    case_integrators_autotune()
    case_blob_projection()
    case_replica_exchange()
