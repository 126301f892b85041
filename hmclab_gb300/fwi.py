"""Set-up of the 2-D elastic P-SV full-waveform problem (host side, numpy).

ElasticConfig       grid, time stepping, sponge, Ricker wavelet, shots, receivers
layered_model       layered vp/vs/rho with Gaussian anomalies
BlobBasis           Gaussian-blob parametrisation of (vp, vs, rho)
                    (reference: hmclab/Distributions/ElasticFullWaveform2D.py:229-341)

The physical model is nx x nz cells of size h; the simulation grid adds `pad`
absorbing cells (Cerjan et al. 1985 sponge) on every side, and the parameters
of a padding cell are those of the nearest physical cell.
"""
import numpy as _np


class ElasticConfig:
    def __init__(self, nx=200, nz=100, pad=20, h=5.0, dt=5e-4, nt=1500, f0=25.0, sponge=0.015, amplitude=1e9,
                 src_x=(125.0, 375.0, 625.0, 875.0), src_z=10.0, rec_x=None, rec_z=10.0):
        self.nx, self.nz, self.pad, self.h, self.dt, self.nt = int(nx), int(nz), int(pad), float(h), float(dt), int(nt)
        self.f0, self.sponge, self.amplitude = float(f0), float(sponge), float(amplitude)
        self.nxc, self.nzc = self.nx + 2 * self.pad, self.nz + 2 * self.pad
        if rec_x is None:
            rec_x = _np.linspace(25.0, self.nx * self.h - 25.0, 20)
        self.src = [(self._ix(x), self._iz(src_z)) for x in src_x]
        self.rec_x = _np.array([self._ix(x) for x in rec_x], _np.int32)
        self.rec_z = _np.full(len(rec_x), self._iz(rec_z), _np.int32)
        self.n_shots = len(self.src)
        self.n_rec = len(rec_x)
        cfl = self.dt * 4000.0 / self.h * _np.sqrt(2.0) * (9.0 / 8.0 + 1.0 / 24.0)
        assert cfl < 1.0, "time step too large for the grid (4th-order staggered CFL)"

    def _ix(self, x):
        return self.pad + int(round(x / self.h - 0.5))

    def _iz(self, z):
        return self.pad + int(round(z / self.h - 0.5))

    def taper(self):
        """Cerjan sponge factors on the simulation grid [nzc][nxc]."""
        i = _np.arange(self.nxc)
        j = _np.arange(self.nzc)
        di = _np.minimum(i, self.nxc - 1 - i)[None, :]
        dj = _np.minimum(j, self.nzc - 1 - j)[:, None]
        d = _np.minimum(di, dj).astype(float)
        t = _np.exp(-((self.sponge * (self.pad - d)) ** 2))
        t[d >= self.pad] = 1.0
        return t

    def ricker(self):
        t = _np.arange(self.nt) * self.dt
        t0 = 1.2 / self.f0
        a = (_np.pi * self.f0 * (t - t0)) ** 2
        return self.amplitude * (1.0 - 2.0 * a) * _np.exp(-a)

    def extend(self, phys):
        """Physical field [nz][nx] -> simulation grid [nzc][nxc] (edge values
        repeated into the padding)."""
        jj = _np.clip(_np.arange(self.nzc) - self.pad, 0, self.nz - 1)
        ii = _np.clip(_np.arange(self.nxc) - self.pad, 0, self.nx - 1)
        return phys[jj][:, ii]

    def extension_matrix_rows(self):
        """For each simulation cell, the index of the physical cell it copies."""
        jj = _np.clip(_np.arange(self.nzc) - self.pad, 0, self.nz - 1)
        ii = _np.clip(_np.arange(self.nxc) - self.pad, 0, self.nx - 1)
        return (jj[:, None] * self.nx + ii[None, :]).reshape(-1)

    def cell_centres(self):
        x = (_np.arange(self.nx) + 0.5) * self.h
        z = (_np.arange(self.nz) + 0.5) * self.h
        return _np.meshgrid(x, z)  # X[z][x], Z[z][x]


def layered_model(cfg, anomalies=True):
    """vp, vs, rho on the physical grid [nz][nx]: three layers (interfaces at
    30% and 60% of the depth) plus, optionally, two Gaussian anomalies of
    +-8% (vp, vs) and +-4% (rho)."""
    X, Z = cfg.cell_centres()
    depth = cfg.nz * cfg.h
    vp = _np.where(Z < 0.3 * depth, 1800.0, _np.where(Z < 0.6 * depth, 2200.0, 2600.0))
    vs = vp / 1.8
    rho = 310.0 * vp**0.25
    if anomalies:
        L = cfg.nx * cfg.h
        for cx, cz, amp in ((0.35 * L, 0.4 * depth, 1.0), (0.65 * L, 0.65 * depth, -1.0)):
            g = _np.exp(-((X - cx) ** 2 + (Z - cz) ** 2) / (2 * (0.06 * L) ** 2))
            vp = vp * (1 + 0.08 * amp * g)
            vs = vs * (1 + 0.08 * amp * g)
            rho = rho * (1 + 0.04 * amp * g)
    return vp, vs, rho


class BlobBasis:
    """Gaussian blobs on an nbx x nbz grid of centres over the physical model,
    one set per field (vp, vs, rho): fine = B m_field + background_field.
    Blob index = ibx * nbz + ibz and widths sqrt(0.5) * spacing, as in the
    reference's BlobParametrization (ElasticFullWaveform2D.py:256-313)."""

    def __init__(self, cfg, nbx=20, nbz=10):
        self.cfg, self.nbx, self.nbz = cfg, int(nbx), int(nbz)
        X, Z = cfg.cell_centres()
        Lx = X.max() - X.min()
        Lz = Z.max() - Z.min()
        dx, dz = Lx / nbx, Lz / nbz
        px = dx * 0.5 + _np.arange(nbx) * dx + X.min()
        pz = dz * 0.5 + _np.arange(nbz) * dz + Z.min()
        B = _np.zeros((cfg.nz * cfg.nx, nbx * nbz))
        for ix, xc in enumerate(px):
            for iz, zc in enumerate(pz):
                g = _np.exp(-(((X - xc) / (0.5**0.5 * dx)) ** 2 + ((Z - zc) / (0.5**0.5 * dz)) ** 2))
                B[:, ix * nbz + iz] = g.reshape(-1)
        self.B = B  # physical cells x blobs
        self.n_blobs = nbx * nbz
        self.free_parameters = 3 * self.n_blobs

    def simulation_basis(self):
        """Basis rows for every simulation cell (padding copies the nearest
        physical cell): [nzc*nxc][n_blobs]."""
        return self.B[self.cfg.extension_matrix_rows()]

    def fit(self, fine_phys):
        """Least-squares blob amplitudes of a physical field [nz][nx]."""
        return _np.linalg.lstsq(self.B, fine_phys.reshape(-1), rcond=None)[0]
