"""2-D elastic P-SV FWI: the FP64 oracle's adjoint against finite differences
(CPU), and the CUDA forward records and blob-space gradients against the
oracle (GPU).

Tolerances: oracle gradient vs central differences 1e-6 relative (FP64);
FP32 device misfits vs the FP64 oracle 1e-5 relative; FP32 device gradients
vs the FP64 oracle 1e-5 of the gradient scale (measured ~2e-6 here and at
the full 240 x 140-cell, 1500-step grid, tests/test_gpu_fullsize.py)."""
import numpy as np
import pytest

from hmclab_gb300 import fwi as FW
from oracle import fwi as OF


def small_config(nt=300):
    return FW.ElasticConfig(nx=40, nz=24, pad=8, h=5.0, dt=5e-4, nt=nt, f0=25.0, sponge=0.05,
                            src_x=(60.0, 140.0), src_z=20.0, rec_x=np.linspace(15.0, 185.0, 9), rec_z=20.0)


def oracle_shots(cfg):
    return [OF.Shot(cfg.nxc, cfg.nzc, cfg.nt, cfg.h, cfg.dt, cfg.taper(), cfg.ricker(), src, cfg.rec_x, cfg.rec_z)
            for src in cfg.src]


def test_config_geometry():
    cfg = FW.ElasticConfig()
    assert (cfg.nxc, cfg.nzc) == (240, 140)
    assert cfg.n_shots == 4 and cfg.n_rec == 20
    t = cfg.taper()
    assert t.shape == (140, 240) and t[70, 120] == 1.0 and t[0, 0] < 1.0
    vp, vs, rho = FW.layered_model(cfg)
    assert vp.shape == (100, 200) and 1600 < vp.min() and vp.max() < 2900
    b = FW.BlobBasis(cfg)
    assert b.B.shape == (20000, 200) and b.free_parameters == 600
    assert b.simulation_basis().shape == (33600, 200)


def test_oracle_adjoint_matches_finite_differences():
    cfg = small_config(nt=250)
    shot = oracle_shots(cfg)[0]
    vp, vs, rho = (cfg.extend(f) for f in FW.layered_model(cfg))
    ovx, ovz = shot.forward(rho, vp * 1.02, vs * 0.99)
    w = 1.0 / np.mean(ovx**2 + ovz**2)
    chi, grads = shot.gradient(rho, vp, vs, ovx, ovz, w)
    rng = np.random.default_rng(3)
    for k in range(3):
        dm = rng.normal(size=vp.shape) * [rho, vp, vs][k] * 1e-5
        args = [rho, vp, vs]

        def mis(sign):
            a = list(args)
            a[k] = a[k] + sign * dm
            rvx, rvz = shot.forward(*a)
            return 0.5 * w * np.sum((rvx - ovx) ** 2 + (rvz - ovz) ** 2)

        fd = (mis(1) - mis(-1)) / 2
        an = np.sum(grads[k] * dm)
        assert abs(fd - an) <= 1e-6 * abs(fd), (k, fd, an)


# ---------------------------------------------------------------------------
@pytest.mark.gpu
def test_device_fwi_matches_oracle():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import hmclab_gb300 as H

    cfg = small_config(nt=300)
    shots = oracle_shots(cfg)
    bg = FW.layered_model(cfg, anomalies=False)
    truth = FW.layered_model(cfg, anomalies=True)
    obs = [s.forward(*(cfg.extend(f) for f in (truth[2], truth[0], truth[1]))) for s in shots]
    ux = np.stack([o[0] for o in obs])
    uz = np.stack([o[1] for o in obs])
    std = float(np.sqrt(np.mean(ux**2 + uz**2))) * 0.1
    dist = H.Distributions.ElasticFullWaveform2D(cfg, ux, uz, data_std=std, free_parameter_grid=[5, 3],
                                                 background=bg)
    assert dist.dimensions == 45
    rng = np.random.default_rng(0)
    C = 3
    M = np.stack([rng.normal(size=45) * np.repeat([40.0, 20.0, 15.0], 15) for _ in range(C)], axis=1)
    Md = torch.from_numpy(M).to("cuda", torch.float32)
    x = dist.misfit_batch(Md).cpu().numpy()
    g = dist.gradient_batch(Md).double().cpu().numpy()
    torch.cuda.synchronize()
    Bs = dist.blob.simulation_basis()
    w = dist.weight
    for c in range(C):
        m32 = Md[:, c].double().cpu().numpy()
        vp, vs, rho = (cfg.extend(f) for f in dist.fine_model(m32))
        chi = 0.0
        gv = [np.zeros_like(vp) for _ in range(3)]
        for k, s in enumerate(shots):
            ch, gk = s.gradient(rho, vp, vs, obs[k][0], obs[k][1], w)
            chi += ch
            for f in range(3):
                gv[f] += gk[f]
        # device records of chain c agree with the oracle's
        np.testing.assert_allclose(x[c], chi, rtol=1e-5)
        g_ref = np.concatenate([Bs.T @ gv[1].reshape(-1), Bs.T @ gv[2].reshape(-1), Bs.T @ gv[0].reshape(-1)])
        scale = np.abs(g_ref).max()
        err = np.abs(g[:, c] - g_ref).max() / scale
        print(f"chain {c}: misfit {x[c]:.6e} vs oracle {chi:.6e}; gradient max rel err {err:.2e}")
        assert err < 1e-5


@pytest.mark.gpu
def test_device_fwi_staged_tiles_match_direct_loads():
    """64 chains on a ragged grid (57 x 41 cells: neither a multiple of the
    8 x 4-cell tile): the forward and adjoint stencils reading shared-memory
    tiles staged by the tensor memory accelerator give the same misfits and
    gradients as the direct-load kernels, and chain 0 agrees with the FP64
    oracle."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import hmclab_gb300 as H

    cfg = FW.ElasticConfig(nx=41, nz=25, pad=8, h=5.0, dt=5e-4, nt=200, f0=25.0, sponge=0.05,
                           src_x=(60.0, 140.0), src_z=20.0, rec_x=np.linspace(15.0, 185.0, 9), rec_z=20.0)
    assert (cfg.nxc % 8, cfg.nzc % 4) != (0, 0)
    shots = oracle_shots(cfg)
    bg = FW.layered_model(cfg, anomalies=False)
    truth = FW.layered_model(cfg, anomalies=True)
    obs = [s.forward(*(cfg.extend(f) for f in (truth[2], truth[0], truth[1]))) for s in shots]
    ux = np.stack([o[0] for o in obs])
    uz = np.stack([o[1] for o in obs])
    std = float(np.sqrt(np.mean(ux**2 + uz**2))) * 0.1
    dists = [H.Distributions.ElasticFullWaveform2D(cfg, ux, uz, data_std=std, free_parameter_grid=[5, 3],
                                                   background=bg) for _ in range(2)]
    dists[1].staged_tiles = False
    rng = np.random.default_rng(2)
    C = 64
    M = np.stack([rng.normal(size=45) * np.repeat([40.0, 20.0, 15.0], 15) for _ in range(C)], axis=1)
    Md = torch.from_numpy(M).to("cuda", torch.float32)
    x = [d.misfit_batch(Md).cpu().numpy() for d in dists]
    g = [d.gradient_batch(Md).double().cpu().numpy() for d in dists]
    for d in dists:
        d.check_device_status()
    # the staged kernels evaluate the same expressions: equal bit for bit
    np.testing.assert_array_equal(x[0], x[1])
    np.testing.assert_array_equal(g[0], g[1])
    print(f"staged vs direct: misfit max rel {np.max(np.abs(x[0] / x[1] - 1)):.2e}, "
          f"gradient max abs {np.abs(g[0] - g[1]).max():.2e} (bitwise equal: {np.array_equal(g[0], g[1])})")
    m32 = Md[:, 0].double().cpu().numpy()
    vp, vs, rho = (cfg.extend(f) for f in dists[0].fine_model(m32))
    chi = sum(s.gradient(rho, vp, vs, obs[k][0], obs[k][1], dists[0].weight)[0] for k, s in enumerate(shots))
    np.testing.assert_allclose(x[0][0], chi, rtol=1e-5)


def _blob_case(golden):
    g = golden("blob_projection.npz")
    cfg = FW.ElasticConfig(nx=int(g["nx"]), nz=int(g["nz"]), pad=int(g["pad"]), h=float(g["h"]), dt=5e-4, nt=10,
                           src_x=(20.0,), src_z=10.0, rec_x=np.array([10.0, 50.0]), rec_z=10.0)
    return g, cfg, FW.BlobBasis(cfg, int(g["nbx"]), int(g["nbz"]))


def test_blob_basis_and_projection_match_the_reference(golden):
    """BlobBasis against the reference's BlobParametrization
    (ElasticFullWaveform2D.py:229-341, golden fixture from the reference
    itself): the same collocation matrix, the same (C^T C)^-1 C^T map that
    the reference applies to grid gradients (`gradient_projection=
    "least_squares"`), and the same forward map of a blob vector."""
    g, cfg, blob = _blob_case(golden)
    n, nb = cfg.nx * cfg.nz, blob.n_blobs
    Cref = g["collocation"]
    for f in range(3):
        np.testing.assert_allclose(Cref[f * n:(f + 1) * n, f * nb:(f + 1) * nb], blob.B, rtol=1e-12, atol=1e-15)
        off = np.delete(Cref[f * n:(f + 1) * n], np.s_[f * nb:(f + 1) * nb], axis=1)
        assert not off.any()
    proj = np.linalg.inv(blob.B.T @ blob.B)
    for k in range(3):
        gg = g["grid_gradients"][:, k].reshape(3, n)
        mine = np.concatenate([proj @ (blob.B.T @ gg[f]) for f in range(3)])
        np.testing.assert_allclose(mine, g["projected"][:, k], rtol=1e-9, atol=1e-9 * np.abs(mine).max())
    m = g["blob_model"][:, 0].reshape(3, nb)
    bg = g["background"].reshape(3, n)
    fine = np.concatenate([blob.B @ m[f] + bg[f] for f in range(3)])
    np.testing.assert_allclose(fine, g["fine_model"], rtol=1e-12)


@pytest.mark.gpu
def test_device_least_squares_projection_is_the_reference_map():
    """`gradient_projection="least_squares"` on the device returns the
    reference's (C^T C)^-1 C^T map of the grid gradient: per field,
    (B^T B)^-1 times the chain-rule blob gradient (which the oracle pins)."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import hmclab_gb300 as H

    cfg = small_config(nt=200)
    shots = oracle_shots(cfg)
    truth = FW.layered_model(cfg, anomalies=True)
    obs = [s.forward(*(cfg.extend(f) for f in (truth[2], truth[0], truth[1]))) for s in shots]
    ux, uz = np.stack([o[0] for o in obs]), np.stack([o[1] for o in obs])
    std = float(np.sqrt(np.mean(ux**2 + uz**2))) * 0.1
    bg = FW.layered_model(cfg, anomalies=False)
    kw = dict(data_std=std, free_parameter_grid=[5, 3], background=bg)
    chain = H.Distributions.ElasticFullWaveform2D(cfg, ux, uz, **kw)
    ls = H.Distributions.ElasticFullWaveform2D(cfg, ux, uz, gradient_projection="least_squares", **kw)
    rng = np.random.default_rng(6)
    M = torch.from_numpy(rng.normal(size=(45, 32)) * np.repeat([40.0, 20.0, 15.0], 15)[:, None]).to("cuda",
                                                                                                 torch.float32)
    g_cr = chain.gradient_batch(M).double().cpu().numpy()
    g_ls = ls.gradient_batch(M).double().cpu().numpy()
    proj = np.linalg.inv(chain.blob.B.T @ chain.blob.B)
    nb = chain.blob.n_blobs
    want = np.concatenate([proj @ g_cr[f * nb:(f + 1) * nb] for f in range(3)])
    err = np.abs(g_ls - want).max() / np.abs(want).max()
    print(f"least-squares projection on the device vs (B^T B)^-1 chain-rule gradient: {err:.2e}")
    assert err < 1e-5  # FP32 products; cond(B^T B) is 14 here
