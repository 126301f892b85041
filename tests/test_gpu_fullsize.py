"""Parity at the benchmark sizes: the dense (G 2000 x 1000, 4096 chains,
Normal and Laplace priors), tomography (64 x 64 cells, 2000 rays, 1024
chains) and source-location (32 events x 200 stations, 8192 chains)
workloads run through the FP32 device sampler for a few proposals under
injected random streams, and a subset of their chains is replayed by the FP64
oracle with the same streams.  The FWI workload's full grid (240 x 140 cells
with the sponge, nt = 1500, 4 shots) is compared with the FP64 C oracle for
misfits and blob gradients.

Tolerances: positions within 1e-5 of the largest |coordinate| of the chain
(FP32 relative); the misfits the device recorded within 1e-5 relative of
the FP64 misfits of the positions it recorded; accept decisions identical
except where |dH - log u| < 1e-3 in the oracle (the FP32 states' dH error
scale; chains with such a decision are not compared further).  The chains the oracle replays are
spread over the whole batch (first, last and evenly spaced ones), so every
block of the device launch is covered."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bench  # noqa: E402
import hmclab_gb300 as H  # noqa: E402
from hmclab_gb300 import _lib  # noqa: E402
from oracle import hmc_oracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

FP32_RTOL = 1e-5
# Accept-decision tie band of the FP32 chains: the decision compares dH with
# log u, and an FP32 state carries dH to about 1e-6 of the Hamiltonian
# (misfits of 1e3 here), so decisions within 1e-3 of the threshold may part
# legitimately; the FP64 path's band is 1e-9 (tests/test_gpu_parity.py).
TIE = 1e-3


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _lib.load()


def _streams(P, d, C, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(P, d, C)), rng.uniform(0.5, 1.5, size=(P, C)), rng.uniform(size=(P, C))


def _compare(wl, P, n_check, seed, post=None, opost=None):
    """Run every chain of workload `wl` on the device for P proposals under
    injected streams, replay n_check of them with the oracle, compare."""
    d, C = wl.q0.shape
    q0 = wl.q0.astype(np.float32).astype(np.float64)  # the device starts from the FP32-rounded positions
    z, f, u = _streams(P, d, C, seed)
    kw = wl.sampler_kwargs()
    smp = H.Samplers.HMC(seed=0).sample(None, post or wl.posterior(), initial_model=q0, proposals=P,
                                        rng_streams=(z, f, u), keep_samples=True, proposals_per_graph=P, **kw)
    got = smp.samples_numpy()  # C, d+1, P
    acc = np.atleast_1d(smp.accepted_proposals)
    S = np.unique(np.r_[0, C - 1, np.linspace(0, C - 1, n_check - 2).astype(int)])
    o_post, o_mass = wl.oracle()
    res = O.run_chains(opost or o_post, o_mass, q0[:, S], kw["stepsize"], (z[:, :, S], f[:, S], u[:, S]), P,
                       amount_of_steps=kw["amount_of_steps"])
    ref = np.transpose(res["samples"], (2, 1, 0))  # n_check, d+1, P
    dh_gap = np.abs((res["H0"] - res["H1"]) - np.log(u[:P, S]))
    checked, worst, worst_x = 0, 0.0, 0.0
    for k, c in enumerate(S):
        if np.any(dh_gap[:, k] < TIE):
            continue  # an accept decision within the tie band: the chains may part legitimately
        assert acc[c] == res["accepted"][k], f"chain {c}: accepted {acc[c]} vs oracle {res['accepted'][k]}"
        scale = np.abs(ref[k, :-1]).max()
        err = np.abs(got[c, :-1] - ref[k, :-1]).max() / scale
        # the misfit the device recorded, against the FP64 misfit of the
        # positions it recorded (the trajectories' own drift is bounded above)
        x64 = (opost or o_post).misfit(got[c, :-1])
        xerr = np.max(np.abs(got[c, -1] - x64) / np.abs(x64))
        worst, worst_x = max(worst, err), max(worst_x, xerr)
        checked += 1
    assert checked >= n_check // 2
    rate = float(np.mean(acc) / P)
    print(f"{wl.kind}: C={C} d={d} P={P}: {checked} chains checked, max position error {worst:.2e} of max |q|, "
          f"max misfit rel error {worst_x:.2e}, acceptance {rate:.2f}, min |dH - log u| {dh_gap.min():.2e}")
    assert worst < FP32_RTOL, worst
    assert worst_x < FP32_RTOL, worst_x
    return smp


def test_dense_2000x1000_4096_chains_normal_prior():
    wl = bench.DenseWorkload(seed=0)
    smp = _compare(wl, P=3, n_check=16, seed=5)
    assert smp._fused is not None  # the tcgen05 fused step ran


def test_dense_2000x1000_4096_chains_laplace_prior():
    wl = bench.DenseWorkload(seed=0)
    n = wl.n_model
    post = H.Distributions.BayesRule([H.Distributions.Laplace(np.zeros((n, 1)), np.ones((n, 1))),
                                      H.Distributions.LinearMatrix(wl.G, wl.d, wl.noise**2)])
    opost = O.Sum([O.Laplace(np.zeros(n), np.ones(n)), O.DensePremul(wl.G, wl.d, wl.noise**2)])
    smp = _compare(wl, P=3, n_check=16, seed=6, post=post, opost=opost)
    assert smp._fused is not None


def test_tomography_64x64_2000_rays_1024_chains():
    wl = bench.TomoWorkload(seed=0)
    assert wl.n_model == 4096 and wl.n_data == 2000
    _compare(wl, P=3, n_check=32, seed=7)


def test_source_location_32x200_8192_chains():
    wl = bench.SrclocWorkload(seed=0)
    assert wl.n_model == 129 and wl.S == 200
    _compare(wl, P=3, n_check=24, seed=8)


def test_fwi_full_grid_matches_oracle():
    """The benchmark's FWI configuration (240 x 140 simulation cells, 1500
    time steps, 4 shots x 20 receivers, 600 blob parameters) for 32 chains
    on the staged-tile kernels: misfits and blob gradients of two chains
    against the FP64 C oracle."""
    from hmclab_gb300 import fwi as FW
    from oracle import fwi as OF

    cfg = FW.ElasticConfig()
    shots = [OF.Shot(cfg.nxc, cfg.nzc, cfg.nt, cfg.h, cfg.dt, cfg.taper(), cfg.ricker(), src, cfg.rec_x, cfg.rec_z)
             for src in cfg.src]
    bg = FW.layered_model(cfg, anomalies=False)
    blob = FW.BlobBasis(cfg, 20, 10)
    truth = FW.layered_model(cfg, anomalies=True)
    m_true = np.concatenate([blob.fit(truth[f] - bg[f]) for f in range(3)])
    fine_true = [(blob.B @ m_true.reshape(3, -1)[f]).reshape(cfg.nz, cfg.nx) + bg[f] for f in range(3)]
    obs = [s.forward(*(cfg.extend(fine_true[f]) for f in (2, 0, 1))) for s in shots]
    ux = np.stack([o[0] for o in obs])
    uz = np.stack([o[1] for o in obs])
    std = 0.05 * float(np.sqrt(np.mean(ux**2 + uz**2)))
    dist = H.Distributions.ElasticFullWaveform2D(cfg, ux, uz, data_std=std, free_parameter_grid=[20, 10],
                                                 background=bg)
    assert dist.dimensions == 600
    centre = np.argmax(blob.B, axis=0)
    prior_std = np.concatenate([0.1 * bg[f].reshape(-1)[centre] for f in range(3)])
    rng = np.random.default_rng(4)
    C = 32
    M = m_true[:, None] + 0.3 * prior_std[:, None] * rng.normal(size=(600, C))
    Md = torch.from_numpy(M).to("cuda", torch.float32)
    x = dist.misfit_batch(Md).cpu().numpy()
    g = dist.gradient_batch(Md).double().cpu().numpy()
    dist.check_device_status()
    Bs = blob.simulation_basis()
    for c in (0, C - 1):
        m32 = Md[:, c].double().cpu().numpy()
        vp, vs, rho = (cfg.extend(f) for f in dist.fine_model(m32))
        chi, gv = 0.0, [np.zeros_like(vp) for _ in range(3)]
        for k, s in enumerate(shots):
            ch, gk = s.gradient(rho, vp, vs, ux[k], uz[k], dist.weight)
            chi += ch
            for f in range(3):
                gv[f] += gk[f]
        g_ref = np.concatenate([Bs.T @ gv[1].reshape(-1), Bs.T @ gv[2].reshape(-1), Bs.T @ gv[0].reshape(-1)])
        xerr = abs(x[c] / chi - 1)
        gerr = np.abs(g[:, c] - g_ref).max() / np.abs(g_ref).max()
        print(f"FWI full grid, chain {c}: misfit {x[c]:.6e} vs oracle {chi:.6e} (rel {xerr:.2e}); gradient max "
              f"error {gerr:.2e} of max |g|")
        assert xerr < FP32_RTOL
        assert gerr < FP32_RTOL
