"""psvWave-configured elastic problems: the .ini reader, moment-tensor and
multi-source shots, the cell parametrisation (psvWave's own model vector)
and the Uniform prior the reference's FWI sampling test uses.

CPU: the reader against the file's values; the oracle's adjoint with
moment-tensor sources against finite differences (1e-6, FP64); the gradient
correlated at every k-th step (psvWave's snapshot_interval) against the
exact one; cell-basis ordering and segments; the constructor's error paths (reference
tests/test_elasticFWI.py:18-52).  GPU: records and cell-space gradients of a
multi-source moment-tensor configuration with snapshot interval 5 against
the FP64 oracle (1e-5);
create_default on the .ini, a gradient step that lowers the misfit, and a
short HMC run under a Uniform prior (reference tests/test_elasticFWI.py:
55-122)."""
import os

import numpy as np
import pytest

import hmclab_gb300 as H
from hmclab_gb300 import fwi as FW
from hmclab_gb300.Helpers.CustomExceptions import InvalidCaseError
from oracle import fwi as OF

INI = os.path.join(os.path.dirname(__file__), "configurations", "elastic_psv_small.ini")


def ini_config():
    return FW.ElasticConfig.from_ini(INI)


def oracle_shots(cfg, snapshot_interval=None):
    k = cfg.snapshot_interval if snapshot_interval is None else snapshot_interval
    return [OF.Shot(cfg.nxc, cfg.nzc, cfg.nt, cfg.h, cfg.dt, cfg.taper(), cfg.shot_wavelets(s), None, cfg.rec_x,
                    cfg.rec_z, sources=[(q.x, q.z, q.mxx, q.mzz, q.mxz) for q in cfg.shots[s]], snapshot_interval=k)
            for s in range(cfg.n_shots)]


def test_ini_reader_values():
    cfg = ini_config()
    assert (cfg.nx, cfg.nz, cfg.pad, cfg.h, cfg.dt, cfg.nt) == (36, 30, 10, 2.0, 3e-4, 600)
    assert (cfg.nxc, cfg.nzc) == (56, 50)
    assert cfg.f0 == 40.0 and cfg.t0 == 0.03 and cfg.sponge == 0.05
    assert cfg.medium == (2000.0, 900.0, 1600.0)
    assert cfg.kernel_region == (2, 34, 6, 24) and cfg.cell_block == (2, 2) and cfg.snapshot_interval == 5
    assert not cfg.extend_parameters and not cfg.explosive_shots
    # shot 0 fires sources 0 and 2, the second delayed by 3 cycles of 40 Hz
    s0, s1 = cfg.shots
    assert [(q.x, q.z) for q in s0] == [(16, 14), (40, 14)] and [(q.x, q.z) for q in s1] == [(28, 14)]
    assert s0[0].delay == 0.0 and s0[1].delay == pytest.approx(0.075)
    for q, angle in ((s0[0], 30), (s0[1], 75), (s1[0], 110)):
        assert (q.mxx, q.mzz, q.mxz) == pytest.approx(FW.moment_tensor(angle))
    assert list(cfg.rec_x) == [13, 19, 25, 31, 37, 43] and set(cfg.rec_z) == {35}
    w = cfg.shot_wavelets(0)
    assert w.shape == (2, 600)
    assert np.argmax(w[0]) == round(0.03 / 3e-4) and np.argmax(w[1]) == round(0.105 / 3e-4)


def test_moment_tensor_is_a_unit_double_couple():
    for a in (0.0, 30.0, 47.0, 134.0):
        mxx, mzz, mxz = FW.moment_tensor(a)
        M = np.array([[mxx, mxz], [mxz, mzz]])
        assert abs(np.trace(M)) < 1e-15  # no volume change
        assert np.allclose(sorted(np.linalg.eigvalsh(M)), [-1.0, 1.0])


def test_ini_reader_rejects_inconsistent_files(tmp_path):
    text = open(INI).read()
    bad = tmp_path / "bad.ini"
    bad.write_text(text.replace("dz = 2.0;", "dz = 2.5;"))
    with pytest.raises(ValueError, match="square cells"):
        FW.read_ini(str(bad))
    bad.write_text(text.replace("nr = 6;", "nr = 7;"))
    with pytest.raises(ValueError, match="nr"):
        FW.read_ini(str(bad))
    bad.write_text(text.replace("{{0, 2}, {1}}", "{{0, 3}, {1}}"))
    with pytest.raises(ValueError, match="does not exist"):
        FW.read_ini(str(bad))
    bad.write_text(text.replace("dt = 0.0003;", "dt = 0.003;"))
    with pytest.raises(ValueError, match="CFL"):
        FW.ElasticConfig.from_ini(str(bad))


def test_cell_basis_order_and_segments():
    cfg = ini_config()
    cb = FW.CellBasis(cfg, *cfg.cell_block)
    assert (cb.nbx, cb.nbz, cb.free_parameters) == (16, 9, 432)
    P = cb.param_of.reshape(cfg.nz, cfg.nx)
    i0, i1, j0, j1 = cfg.kernel_region
    assert np.all(P[:j0] == -1) and np.all(P[j1:] == -1) and np.all(P[:, :i0] == -1) and np.all(P[:, i1:] == -1)
    # blocks of 2 x 2 cells, x fastest (column-major over [x][z])
    assert P[j0, i0] == 0 and P[j0, i0 + 1] == 0 and P[j0 + 1, i0 + 1] == 0 and P[j0, i0 + 2] == 1
    assert P[j0 + 2, i0] == cb.nbx
    ptr, cells = cb.gradient_segments()
    assert ptr[0] == 0 and ptr[-1] == len(cells) == 4 * cb.n_blobs  # no padding copies: the sponge keeps the medium
    m = cb.simulation_map()
    for p in (0, 17, cb.n_blobs - 1):
        assert np.all(m[cells[ptr[p]:ptr[p + 1]]] == p)
    bg = FW.background_model(cfg)
    v = cb.background_vector(bg)
    assert np.allclose(v.reshape(3, -1), np.array(cfg.medium)[:, None])
    assert np.allclose(cb.fit(bg[0]), 2000.0)


def test_oracle_adjoint_with_moment_tensor_sources_matches_finite_differences():
    cfg = ini_config()
    shot = oracle_shots(cfg, snapshot_interval=1)[0]
    vp, vs, rho = (cfg.extend(f) for f in FW.background_model(cfg))
    X, Z = np.meshgrid(np.arange(cfg.nxc), np.arange(cfg.nzc))
    bump = np.exp(-((X - 28) ** 2 + (Z - 25) ** 2) / 20.0)
    ovx, ovz = shot.forward(rho * (1 + 0.05 * bump), vp * (1 - 0.05 * bump), vs * (1 - 0.05 * bump))
    assert np.abs(ovx).max() > 0 and np.abs(ovz).max() > 0
    w = 1.0 / np.mean(ovx**2 + ovz**2)
    chi, grads = shot.gradient(rho, vp, vs, ovx, ovz, w)
    assert chi > 0
    rng = np.random.default_rng(5)
    for k in range(3):
        dm = rng.normal(size=vp.shape) * [rho, vp, vs][k] * 1e-5

        def mis(sign):
            a = [rho, vp, vs]
            a[k] = a[k] + sign * dm
            rvx, rvz = shot.forward(*a)
            return 0.5 * w * np.sum((rvx - ovx) ** 2 + (rvz - ovz) ** 2)

        fd = (mis(1) - mis(-1)) / 2
        an = np.sum(grads[k] * dm)
        assert abs(fd - an) <= 1e-6 * abs(fd), (k, fd, an)


def test_snapshot_correlation_approximates_the_exact_gradient():
    """Correlating forward and adjoint fields at every k-th step only (weight
    k) leaves the misfit unchanged and, for k well below the wavelet's
    period (83 steps here), the gradient within a few 1e-3 of the exact one
    (aliasing of the correlation's spectrum above 1 / (2 k dt))."""
    cfg = ini_config()
    vp, vs, rho = (cfg.extend(f) for f in FW.background_model(cfg))
    X, Z = np.meshgrid(np.arange(cfg.nxc), np.arange(cfg.nzc))
    bump = np.exp(-((X - 28) ** 2 + (Z - 25) ** 2) / 20.0)
    exact = oracle_shots(cfg, 1)[0]
    ovx, ovz = exact.forward(rho * (1 + 0.05 * bump), vp * (1 - 0.05 * bump), vs * (1 - 0.05 * bump))
    w = 1.0 / np.mean(ovx**2 + ovz**2)
    c1, g1 = exact.gradient(rho, vp, vs, ovx, ovz, w)
    for k, tol in ((2, 1e-3), (5, 5e-3)):
        ck, gk = oracle_shots(cfg, k)[0].gradient(rho, vp, vs, ovx, ovz, w)
        assert ck == c1
        errs = [np.abs(gk[f] - g1[f]).max() / np.abs(g1[f]).max() for f in range(3)]
        print(f"snapshot interval {k}: max relative gradient error (rho, vp, vs) {np.round(errs, 5)}")
        assert max(errs) < tol


def test_explosive_sources_are_the_single_source_special_case():
    """The multi-source path of the oracle with one (1, 1, 0) source gives the
    explosive path's records exactly."""
    cfg = FW.ElasticConfig(nx=30, nz=20, pad=8, h=5.0, dt=5e-4, nt=150, f0=25.0, sponge=0.05, src_x=(70.0,),
                           src_z=20.0, rec_x=np.linspace(15.0, 135.0, 5), rec_z=20.0)
    vp, vs, rho = (cfg.extend(f) for f in FW.layered_model(cfg))
    a = OF.Shot(cfg.nxc, cfg.nzc, cfg.nt, cfg.h, cfg.dt, cfg.taper(), cfg.ricker(), cfg.src[0], cfg.rec_x, cfg.rec_z)
    b = OF.Shot(cfg.nxc, cfg.nzc, cfg.nt, cfg.h, cfg.dt, cfg.taper(), cfg.ricker()[None], None, cfg.rec_x, cfg.rec_z,
                sources=[(*cfg.src[0], 1.0, 1.0, 0.0)])
    ra, rb = a.forward(rho, vp, vs), b.forward(rho, vp, vs)
    assert np.array_equal(ra[0], rb[0]) and np.array_equal(ra[1], rb[1])


def test_constructor_paths_follow_the_reference():
    cfg = ini_config()
    zeros = np.zeros((cfg.n_shots, cfg.nt, cfg.n_rec))
    d = H.Distributions.ElasticFullWaveform2D(INI, ux_obs=zeros, uz_obs=zeros)
    assert d.dimensions == 432 and not d.use_blob_par
    assert d.get_model_vector().shape == (432, 1)
    assert np.allclose(d.get_model_vector().reshape(3, -1), np.array(cfg.medium)[:, None])
    with pytest.raises(ValueError):
        H.Distributions.ElasticFullWaveform2D(42)
    with pytest.raises(ValueError):
        H.Distributions.ElasticFullWaveform2D(INI)
    with pytest.raises(InvalidCaseError):
        d.generate()
    c = H.Distributions.ElasticFullWaveform2D(d, temperature=2)
    assert c.temperature == 2 and c.dimensions == 432
    d.make_blob(4, 3)
    assert d.dimensions == 36 and d.use_blob_par and np.all(d.get_model_vector() == 0)
    # the blobs live inside the free-parameter region only
    B = d.blob.B.reshape(cfg.nz, cfg.nx, -1)
    i0, i1, j0, j1 = cfg.kernel_region
    assert np.all(B[:j0] == 0) and np.all(B[:, i1:] == 0) and B[j0:j1, i0:i1].max() > 0.9


def test_uniform_host_contract():
    lo, hi = np.full((4, 1), -1.0), np.array([[1.0], [2.0], [3.0], [4.0]])
    u = H.Distributions.Uniform(lo, hi)
    assert u.dimensions == 4
    assert u.misfit_bounds(np.zeros((4, 1))) == 0.0
    assert u.misfit_bounds(np.full((4, 1), 5.0)) == np.inf
    s = u.generate(1000, np.random.default_rng(0))
    assert s.shape == (4, 1000) and np.all(s >= lo) and np.all(s <= hi)
    with pytest.raises(ValueError):
        H.Distributions.Uniform(hi, lo)  # upper below lower
    assert H.Distributions.Uniform.create_default(7).dimensions == 7


# ---------------------------------------------------------------------------
@pytest.fixture
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _oracle_cell_problem(cfg, d, m):
    """FP64 oracle misfit and cell-space gradient of model vector m."""
    cb = d.blob
    fine = d.fine_model(m)  # vp, vs, rho physical
    rows = cfg.extension_matrix_rows()
    ext = [np.where(rows >= 0, fine[f].reshape(-1)[np.maximum(rows, 0)],
                    cfg.extend(d.background[f]).reshape(-1)).reshape(cfg.nzc, cfg.nxc) for f in range(3)]
    chi, g = 0.0, [np.zeros((cfg.nzc, cfg.nxc)) for _ in range(3)]
    for k, shot in enumerate(oracle_shots(cfg)):
        c, gs = shot.gradient(ext[2], ext[0], ext[1], d.ux_obs[k], d.uz_obs[k], d.weight)
        chi += c
        for f, src in zip((2, 0, 1), gs):
            g[f] += src
    ptr, cells = cb.gradient_segments()
    gm = np.concatenate([np.add.reduceat(g[f].reshape(-1)[cells], ptr[:-1]) for f in range(3)])
    return chi, gm


@pytest.mark.gpu
@pytest.mark.parametrize("staged", [True, False])
def test_moment_tensor_shots_match_oracle(cuda, staged):
    torch = cuda
    cfg = ini_config()
    rng = np.random.default_rng(2)
    shots = oracle_shots(cfg)
    bg = FW.background_model(cfg)
    X, Z = cfg.cell_centres()
    bump = np.exp(-((X - 40.0) ** 2 + (Z - 30.0) ** 2) / 80.0)
    truth = [bg[0] * (1 - 0.06 * bump), bg[1] * (1 - 0.06 * bump), bg[2] * (1 + 0.04 * bump)]
    obs = [s.forward(*(cfg.extend(truth[f]) for f in (2, 0, 1))) for s in shots]
    ux, uz = np.stack([o[0] for o in obs]), np.stack([o[1] for o in obs])
    std = 0.05 * float(np.sqrt(np.mean(ux**2 + uz**2)))
    d = H.Distributions.ElasticFullWaveform2D(INI, ux, uz, data_std=std)
    d.staged_tiles = staged
    m0 = d.get_model_vector()[:, 0]
    C = 32
    M = m0[:, None] * (1 + 0.02 * rng.normal(size=(d.dimensions, C)))
    Mt = torch.from_numpy(M).to("cuda", torch.float32).contiguous()
    x = d.misfit_batch(Mt).cpu().numpy()
    g = d.gradient_batch(Mt).double().cpu().numpy()
    d.check_device_status()
    # records of chain 0 against the oracle's forward
    ux0, uz0 = d.synthetic_records(M[:, 0])
    for k, s in enumerate(shots):
        fine = d.fine_model(M[:, 0])
        rows = cfg.extension_matrix_rows()
        ext = [np.where(rows >= 0, fine[f].reshape(-1)[np.maximum(rows, 0)], cfg.extend(bg[f]).reshape(-1))
               .reshape(cfg.nzc, cfg.nxc) for f in range(3)]
        rvx, rvz = s.forward(ext[2], ext[0], ext[1])
        scale = max(np.abs(rvx).max(), np.abs(rvz).max())
        assert np.abs(ux0[k] - rvx).max() <= 1e-5 * scale and np.abs(uz0[k] - rvz).max() <= 1e-5 * scale
    for c in (0, 13):
        chi, gm = _oracle_cell_problem(cfg, d, M[:, c])
        assert abs(x[c] - chi) <= 1e-5 * chi, (c, x[c], chi)
        err = np.abs(g[:, c] - gm).max() / np.abs(gm).max()
        print(f"chain {c}: misfit {x[c]:.6e} vs {chi:.6e}, gradient error {err:.2e}")
        assert err <= 1e-5


@pytest.mark.gpu
def test_create_default_gradient_step_and_uniform_sampling(cuda):
    """The reference's FWI tests on this package's .ini: create_default,
    a gradient step from the background lowers the misfit, and ten HMC
    proposals of two steps under a Uniform prior stay inside its bounds."""
    with pytest.raises(InvalidCaseError):
        H.Distributions.ElasticFullWaveform2D.create_default(4800, INI)
    lik = H.Distributions.ElasticFullWaveform2D.create_default(432, INI)
    m = lik.get_model_vector()
    x1 = lik.misfit(m)
    g = lik.gradient(m)
    assert x1 > 0 and np.all(np.isfinite(g)) and np.abs(g).max() > 0
    step = 0.02 * np.abs(m).max() / np.abs(g).max()
    x2 = lik.misfit(m - step * g)
    assert x2 < x1, (x1, x2)
    lik.temperature = 100.0
    t = np.ones((lik.dimensions // 3, 1))
    lower = np.vstack((t * 1800, t * 800, t * 1400))
    upper = np.vstack((t * 2200, t * 1000, t * 1800))
    post = H.Distributions.BayesRule([H.Distributions.Uniform(lower, upper), lik])
    smp = H.Samplers.HMC(seed=3).sample(None, post, proposals=10, amount_of_steps=2, stepsize=0.03,
                                        initial_model=(upper + lower) / 2.0, keep_samples=True)
    q = smp.samples_numpy()[0, :-1, :]
    assert q.shape == (lik.dimensions, 10)
    assert np.all(q >= lower - 1e-3) and np.all(q <= upper + 1e-3)
    assert np.all(np.isfinite(smp.samples_numpy()[0, -1, :]))


def test_reader_opens_the_reference_configuration_file():
    """The reference's own psvWave configuration
    (tests/configurations/default_testing_configuration.ini of the reference)
    parses, and its cell parametrisation has the 4800 free parameters the
    reference's FWI tests ask create_default for (test_elasticFWI.py:20)."""
    from oracle import ref_shim

    path = os.path.join(ref_shim.REFERENCE_ROOT, "tests", "configurations", "default_testing_configuration.ini")
    if not os.path.exists(path):
        pytest.skip("the reference checkout is not on this machine")
    cfg = FW.ElasticConfig.from_ini(path)
    assert (cfg.nx, cfg.nz, cfg.pad, cfg.nt) == (40, 60, 25, 3000)
    assert cfg.n_shots == 1 and len(cfg.shots[0]) == 4 and cfg.n_rec == 9
    assert cfg.kernel_region == (0, 40, 10, 50)
    zeros = np.zeros((cfg.n_shots, cfg.nt, cfg.n_rec))
    d = H.Distributions.ElasticFullWaveform2D(path, ux_obs=zeros, uz_obs=zeros)
    assert d.dimensions == 4800
    with pytest.raises(InvalidCaseError):
        H.Distributions.ElasticFullWaveform2D.create_default(4801, path)
