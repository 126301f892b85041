"""Seeded synthetic inverse problems for the five benchmark workloads.

These build host-side numpy inputs (matrices, data, stations) with the shapes,
sizes and value distributions of the workloads; they are set-up code, not part
of the sampling hot path.

  dense_linear   dense linear Gaussian problem (G entries N(0, s^2), d = G m + noise)
  tomography     straight-ray travel-time tomography on a square grid, CSR ray
                 lengths from exact ray/cell intersections (Siddon 1985)
  source_loc     3-D earthquake location with surface stations (homogeneous v)
  elastic_fwi    2-D elastic P-SV waveform inversion in Gaussian-blob
                 parameters (data from the device forward of the true model)
"""
import numpy as _np
import scipy.sparse as _sparse


# ---------------------------------------------------------------------------
# Dense linear problems (G 100x50 N(0,1) single chain; G 2000x1000 N(0,1/1000))
# ---------------------------------------------------------------------------
def dense_linear(n_data, n_model, g_std, noise_std, seed):
    """G ~ N(0, g_std^2), m_true ~ N(0, I), d = G m_true + N(0, noise_std^2)."""
    rng = _np.random.default_rng(seed)
    G = rng.normal(size=(n_data, n_model)) * g_std
    m_true = rng.normal(size=(n_model, 1))
    d = G @ m_true + noise_std * rng.normal(size=(n_data, 1))
    return G, d, m_true


def gaussian_posterior(G, d, noise_var, prior_mean, prior_var):
    """Analytic posterior of a linear Gaussian problem with a diagonal prior:
    Sigma = (G^T G / s^2 + P^-1)^-1, mu = Sigma (G^T d / s^2 + P^-1 mu_p)."""
    G = G.toarray() if _sparse.issparse(G) else _np.asarray(G, float)
    pm = _np.broadcast_to(_np.asarray(prior_mean, float).reshape(-1, 1), (G.shape[1], 1))
    piv = 1.0 / _np.broadcast_to(_np.asarray(prior_var, float).reshape(-1), (G.shape[1],))
    A = G.T @ G / noise_var + _np.diag(piv)
    cov = _np.linalg.inv(A)
    mean = cov @ (G.T @ d / noise_var + piv[:, None] * pm)
    return mean, cov


# ---------------------------------------------------------------------------
# Straight-ray tomography
# ---------------------------------------------------------------------------
def ray_cell_lengths(x0, y0, x1, y1, nx, ny, h):
    """Exact intersection lengths of the segment (x0,y0)-(x1,y1) with the cells
    of an nx-by-ny grid of spacing h whose corner is at the origin (Siddon 1985:
    parametric crossings of the grid lines, merged and sorted).

    Returns (cell_indices, lengths) with cell index ix * ny + iy."""
    dx, dy = x1 - x0, y1 - y0
    length = float(_np.hypot(dx, dy))
    if length == 0.0:
        return _np.zeros(0, _np.int64), _np.zeros(0)
    alphas = [_np.array([0.0, 1.0])]
    if dx != 0.0:
        a = (_np.arange(nx + 1) * h - x0) / dx
        alphas.append(a[(a > 0.0) & (a < 1.0)])
    if dy != 0.0:
        a = (_np.arange(ny + 1) * h - y0) / dy
        alphas.append(a[(a > 0.0) & (a < 1.0)])
    a = _np.unique(_np.concatenate(alphas))
    seg = _np.diff(a) * length
    mid = 0.5 * (a[1:] + a[:-1])
    ix = _np.floor((x0 + mid * dx) / h).astype(_np.int64)
    iy = _np.floor((y0 + mid * dy) / h).astype(_np.int64)
    keep = (seg > 0) & (ix >= 0) & (ix < nx) & (iy >= 0) & (iy < ny)
    idx = ix[keep] * ny + iy[keep]
    # Merge repeated cells (a crossing exactly through a corner).
    uniq, inv = _np.unique(idx, return_inverse=True)
    lens = _np.zeros(len(uniq))
    _np.add.at(lens, inv, seg[keep])
    return uniq, lens


def _boundary_point(rng, L):
    side = rng.integers(4)
    t = rng.uniform(0, L)
    return [(t, 0.0), (t, L), (0.0, t), (L, t)][side]


def smooth_random_field(nx, ny, corr, rng):
    """Gaussian random field with a Gaussian covariance of length `corr` cells,
    normalised to zero mean and unit standard deviation (FFT filtering)."""
    white = rng.normal(size=(nx, ny))
    kx = _np.fft.fftfreq(nx)[:, None]
    ky = _np.fft.fftfreq(ny)[None, :]
    filt = _np.exp(-2 * (_np.pi * corr) ** 2 * (kx**2 + ky**2))
    f = _np.real(_np.fft.ifft2(_np.fft.fft2(white) * filt))
    return (f - f.mean()) / f.std()


def tomography(nx=64, ny=64, n_rays=2000, h=1.0, noise_std=0.01, seed=0, anomalies=3):
    """Slowness in 0.2-0.5 s/km: smooth Gaussian random field background plus
    `anomalies` circular +-15% anomalies; rays between random boundary points;
    CSR matrix of exact ray lengths.  Returns dict with G (CSR, n_rays x nx*ny),
    d (n_rays,1), background, m_true (nx*ny,1)."""
    rng = _np.random.default_rng(seed)
    field = smooth_random_field(nx, ny, corr=8.0, rng=rng)
    field = (field - field.min()) / (field.max() - field.min())
    background = 0.2 + 0.3 * field
    X, Y = _np.meshgrid((_np.arange(nx) + 0.5) * h, (_np.arange(ny) + 0.5) * h, indexing="ij")
    true = background.copy()
    for k in range(anomalies):
        cx, cy = rng.uniform(0.2, 0.8, size=2) * nx * h
        r = rng.uniform(0.06, 0.12) * nx * h
        sign = 1.0 if k % 2 == 0 else -1.0
        mask = (X - cx) ** 2 + (Y - cy) ** 2 < r * r
        true[mask] *= 1.0 + sign * 0.15
    L = nx * h
    rows, cols, vals = [], [], []
    r = 0
    while r < n_rays:
        x0, y0 = _boundary_point(rng, L)
        x1, y1 = _boundary_point(rng, L)
        if _np.hypot(x1 - x0, y1 - y0) < 0.25 * L:
            continue
        idx, lens = ray_cell_lengths(x0, y0, x1, y1, nx, ny, h)
        if len(idx) == 0:
            continue
        rows.append(_np.full(len(idx), r))
        cols.append(idx)
        vals.append(lens)
        r += 1
    G = _sparse.csr_matrix(
        (_np.concatenate(vals), (_np.concatenate(rows), _np.concatenate(cols))), shape=(n_rays, nx * ny)
    )
    m_true = true.reshape(-1, 1)
    d = G @ m_true + noise_std * rng.normal(size=(n_rays, 1))
    return dict(G=G, d=d, background=background.reshape(-1, 1), m_true=m_true, nx=nx, ny=ny, h=h)


# ---------------------------------------------------------------------------
# 3-D source location
# ---------------------------------------------------------------------------
def source_location(n_events=32, n_stations=200, box=40.0, depth=10.0, v=5.0, noise_std=0.05, seed=0):
    """Events ~ U([0,box]^2 x [0,depth]) with origin times ~ U(0,1) s, stations
    ~ U on the z = 0 surface, straight rays in a homogeneous medium of velocity
    v.  Returns dict with stations (1,S) arrays, obs (E,S), std (E,S) and the
    true model in the interleaved [x,y,z,T]*E + [v] layout."""
    rng = _np.random.default_rng(seed)
    sx = rng.uniform(0, box, size=(1, n_stations))
    sy = rng.uniform(0, box, size=(1, n_stations))
    sz = _np.zeros((1, n_stations))
    ex = rng.uniform(0, box, size=(n_events, 1))
    ey = rng.uniform(0, box, size=(n_events, 1))
    ez = rng.uniform(0, depth, size=(n_events, 1))
    et = rng.uniform(0, 1, size=(n_events, 1))
    dist = _np.sqrt((ex - sx) ** 2 + (ey - sy) ** 2 + (ez - sz) ** 2)
    obs = et + dist / v + noise_std * rng.normal(size=dist.shape)
    m = _np.zeros((4 * n_events + 1, 1))
    m[0:-1:4, 0] = ex[:, 0]
    m[1:-1:4, 0] = ey[:, 0]
    m[2:-1:4, 0] = ez[:, 0]
    m[3:-1:4, 0] = et[:, 0]
    m[-1, 0] = v
    return dict(rx=sx, ry=sy, rz=sz, obs=obs, std=_np.full_like(obs, noise_std), m_true=m)


# ---------------------------------------------------------------------------
# 2-D elastic full-waveform inversion
# ---------------------------------------------------------------------------
def elastic_fwi(cfg=None, nbx=20, nbz=10, prior_fraction=0.1, noise_fraction=0.5, seed=0):
    """Blob-parametrised elastic FWI posterior (needs the CUDA device: the
    observed records are the device forward of the true model plus noise).

    Model vector m = [vp | vs | rho] blob amplitudes (m/s, m/s, kg/m^3) added
    to the layered background.  The true model is the least-squares blob fit
    of the layered model with its two Gaussian anomalies.  Prior: Normal with
    mean 0 (the background) and standard deviation `prior_fraction` times the
    background value at each blob centre.  Data noise: Gaussian with standard
    deviation `noise_fraction` times the RMS of the true records.

    Returns a dict with the posterior (BayesRule of prior and likelihood), the
    likelihood, the prior, m_true, prior_std and data_std."""
    from hmclab_gb300 import Distributions as D
    from hmclab_gb300 import fwi as F

    cfg = cfg or F.ElasticConfig()
    rng = _np.random.default_rng(seed)
    bg = F.layered_model(cfg, anomalies=False)
    truth = F.layered_model(cfg, anomalies=True)
    blob = F.BlobBasis(cfg, nbx, nbz)
    m_true = _np.concatenate([blob.fit(truth[f] - bg[f]) for f in range(3)])
    zeros = _np.zeros((cfg.n_shots, cfg.nt, cfg.n_rec))
    fwd = D.ElasticFullWaveform2D(cfg, zeros, zeros, free_parameter_grid=[nbx, nbz], background=bg)
    ux, uz = fwd.synthetic_records(m_true)
    rms = float(_np.sqrt(_np.mean(ux**2 + uz**2) / 2.0))
    data_std = noise_fraction * rms
    ux = ux + data_std * rng.normal(size=ux.shape)
    uz = uz + data_std * rng.normal(size=uz.shape)
    lik = D.ElasticFullWaveform2D(cfg, ux, uz, data_std=data_std, free_parameter_grid=[nbx, nbz], background=bg)
    # background value at each blob centre (blob index = ibx * nbz + ibz)
    X, Z = cfg.cell_centres()
    centre = _np.argmax(blob.B, axis=0)
    prior_std = _np.concatenate([prior_fraction * bg[f].reshape(-1)[centre] for f in range(3)])
    prior = D.Normal(_np.zeros((lik.dimensions, 1)), (prior_std**2).reshape(-1, 1))
    post = D.BayesRule([prior, lik])
    return dict(posterior=post, likelihood=lik, prior=prior, m_true=m_true, prior_std=prior_std, data_std=data_std,
                config=cfg)
