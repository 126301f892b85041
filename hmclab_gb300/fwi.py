"""Set-up of the 2-D elastic P-SV full-waveform problem (host side, numpy).

ElasticConfig       grid, time stepping, sponge, Ricker wavelets, shots of one
                    or more point sources (explosions or moment tensors),
                    receivers, the region of free parameters
read_ini            the psvWave configuration file the reference constructs
                    its model from (tests/configurations/
                    default_testing_configuration.ini of the reference)
layered_model       layered vp/vs/rho with Gaussian anomalies
BlobBasis           Gaussian-blob parametrisation of (vp, vs, rho)
                    (reference: hmclab/Distributions/ElasticFullWaveform2D.py:229-341)
CellBasis           one parameter per cell (or per npx x npz block of cells)
                    of the free-parameter region: psvWave's own model vector

The physical model is nx x nz cells of size h; the simulation grid adds `pad`
absorbing cells (Cerjan et al. 1985 sponge) on every side.  With
`extend_parameters` (the default) the parameters of a padding cell are those
of the nearest physical cell; configurations read from a psvWave file keep the
background medium in the padding instead (its free parameters exclude the
boundary).
"""
import numpy as _np


class PointSource:
    """A point source on the simulation grid: the sxx/szz node (x, z), its
    moment tensor (mxx, mzz, mxz) and the delay (s) of its wavelet."""

    __slots__ = ("x", "z", "mxx", "mzz", "mxz", "delay")

    def __init__(self, x, z, mxx=1.0, mzz=1.0, mxz=0.0, delay=0.0):
        self.x, self.z = int(x), int(z)
        self.mxx, self.mzz, self.mxz, self.delay = float(mxx), float(mzz), float(mxz), float(delay)

    @property
    def explosive(self):
        return self.mxx == 1.0 and self.mzz == 1.0 and self.mxz == 0.0

    def __repr__(self):
        return (f"PointSource(x={self.x}, z={self.z}, mxx={self.mxx:g}, mzz={self.mzz:g}, mxz={self.mxz:g}, "
                f"delay={self.delay:g})")


def moment_tensor(angle_degrees):
    """(Mxx, Mzz, Mxz) of a unit double couple on a fault at `angle_degrees`
    from the x axis in the x-z plane: M = [[-sin 2a, cos 2a], [cos 2a, sin 2a]].
    This is how this package reads psvWave's `moment_angles`; psvWave itself
    is not available to confirm its convention."""
    a = _np.deg2rad(float(angle_degrees))
    return -_np.sin(2.0 * a), _np.sin(2.0 * a), _np.cos(2.0 * a)


class ElasticConfig:
    """Grid, time stepping and acquisition of the elastic problem.

    The keyword form builds one explosive source per shot at depth `src_z`
    below each `src_x`, receivers at `rec_z`, a Ricker wavelet of peak
    frequency f0 centred at 1.2 / f0 (`t0`), and the whole physical model as
    the free-parameter region.  `shots` (a list per shot of PointSource on
    the simulation grid) replaces the src_x / src_z form; `kernel_region` =
    (i0, i1, j0, j1) limits the free parameters to physical cells
    i0 <= i < i1, j0 <= j < j1 (psvWave's nx/nz_inner_boundary) and
    `cell_block` = (npx, npz) groups its cells for the cell parametrisation;
    `medium` = (vp, vs, rho) makes the background homogeneous (default: the
    layered model); `snapshot_interval` k > 1 makes the gradient correlate
    the forward and adjoint fields at every k-th time step only, weighted by
    k (psvWave's; 1, the default, is the exact discrete adjoint); `vmax` is
    the fastest P velocity the time step must be stable for."""

    def __init__(self, nx=200, nz=100, pad=20, h=5.0, dt=5e-4, nt=1500, f0=25.0, sponge=0.015, amplitude=1e9,
                 src_x=(125.0, 375.0, 625.0, 875.0), src_z=10.0, rec_x=None, rec_z=10.0, shots=None, t0=None,
                 kernel_region=None, extend_parameters=True, medium=None, snapshot_interval=1, vmax=4000.0,
                 rec_cells=None, cell_block=(1, 1)):
        self.nx, self.nz, self.pad, self.h, self.dt, self.nt = int(nx), int(nz), int(pad), float(h), float(dt), int(nt)
        self.f0, self.sponge, self.amplitude = float(f0), float(sponge), float(amplitude)
        self.t0 = 1.2 / self.f0 if t0 is None else float(t0)
        self.nxc, self.nzc = self.nx + 2 * self.pad, self.nz + 2 * self.pad
        if shots is None:
            shots = [[PointSource(self._ix(x), self._iz(src_z))] for x in src_x]
        self.shots = [list(s) for s in shots]
        for shot in self.shots:
            if not shot:
                raise ValueError("a shot needs at least one source")
            for q in shot:
                if not (1 <= q.x < self.nxc and 1 <= q.z < self.nzc):
                    raise ValueError(f"{q} is outside the simulation grid's interior")
        # first source of every shot (the explosive form's single source)
        self.src = [(s[0].x, s[0].z) for s in self.shots]
        if rec_cells is not None:
            self.rec_x = _np.asarray(rec_cells[0], _np.int32)
            self.rec_z = _np.asarray(rec_cells[1], _np.int32)
        else:
            if rec_x is None:
                rec_x = _np.linspace(25.0, self.nx * self.h - 25.0, 20)
            self.rec_x = _np.array([self._ix(x) for x in rec_x], _np.int32)
            self.rec_z = _np.full(len(rec_x), self._iz(rec_z), _np.int32)
        if not (_np.all((self.rec_x >= 0) & (self.rec_x < self.nxc)) and
                _np.all((self.rec_z >= 0) & (self.rec_z < self.nzc))):
            raise ValueError("a receiver is outside the simulation grid")
        self.n_shots = len(self.shots)
        self.n_rec = len(self.rec_x)
        self.kernel_region = (0, self.nx, 0, self.nz) if kernel_region is None else tuple(int(v) for v in kernel_region)
        i0, i1, j0, j1 = self.kernel_region
        if not (0 <= i0 < i1 <= self.nx and 0 <= j0 < j1 <= self.nz):
            raise ValueError(f"kernel region {self.kernel_region} is not inside the {self.nx} x {self.nz} model")
        self.extend_parameters = bool(extend_parameters)
        self.medium = None if medium is None else tuple(float(v) for v in medium)  # (vp, vs, rho)
        self.snapshot_interval = int(snapshot_interval)
        self.cell_block = tuple(int(v) for v in cell_block)  # (npx, npz) of the cell parametrisation
        cfl = self.dt * float(vmax) / self.h * _np.sqrt(2.0) * (9.0 / 8.0 + 1.0 / 24.0)
        if not cfl < 1.0:
            raise ValueError(f"time step too large for the grid (4th-order staggered CFL number {cfl:.2f} at "
                             f"vp {vmax:g})")

    @property
    def explosive_shots(self):
        """Every shot is one explosion fed by the undelayed wavelet."""
        return all(len(s) == 1 and s[0].explosive and s[0].delay == 0.0 for s in self.shots)

    def shot_wavelets(self, shot):
        """[sources][nt] wavelets of the shot's sources (delayed Rickers)."""
        return _np.stack([self.ricker(q.delay) for q in self.shots[shot]])

    @classmethod
    def from_ini(cls, path, **overrides):
        """The configuration of a psvWave .ini file (see read_ini)."""
        kw = read_ini(path)
        kw.update(overrides)
        return cls(**kw)

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

    def ricker(self, delay=0.0):
        """Ricker wavelet of peak frequency f0 centred at t0 + delay."""
        t = _np.arange(self.nt) * self.dt
        a = (_np.pi * self.f0 * (t - self.t0 - float(delay))) ** 2
        return self.amplitude * (1.0 - 2.0 * a) * _np.exp(-a)

    def extend(self, phys):
        """Physical field [nz][nx] -> simulation grid [nzc][nxc] (edge values
        repeated into the padding)."""
        jj = _np.clip(_np.arange(self.nzc) - self.pad, 0, self.nz - 1)
        ii = _np.clip(_np.arange(self.nxc) - self.pad, 0, self.nx - 1)
        return phys[jj][:, ii]

    def extension_matrix_rows(self):
        """For each simulation cell, the index of the physical cell whose
        parameters it takes (-1: a padding cell that keeps the background,
        when `extend_parameters` is off)."""
        jj = _np.clip(_np.arange(self.nzc) - self.pad, 0, self.nz - 1)
        ii = _np.clip(_np.arange(self.nxc) - self.pad, 0, self.nx - 1)
        rows = (jj[:, None] * self.nx + ii[None, :]).reshape(-1)
        if not self.extend_parameters:
            jr, ir = _np.arange(self.nzc) - self.pad, _np.arange(self.nxc) - self.pad
            inside = ((jr >= 0) & (jr < self.nz))[:, None] & ((ir >= 0) & (ir < self.nx))[None, :]
            rows = _np.where(inside.reshape(-1), rows, -1)
        return rows

    def region_mask(self):
        """Physical cells [nz][nx] of the free-parameter region."""
        i0, i1, j0, j1 = self.kernel_region
        m = _np.zeros((self.nz, self.nx), bool)
        m[j0:j1, i0:i1] = True
        return m

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


def background_model(cfg):
    """Background (vp, vs, rho) on the physical grid [nz][nx]: the
    configuration's homogeneous medium, else the layered model without
    anomalies."""
    if cfg.medium is not None:
        return tuple(_np.full((cfg.nz, cfg.nx), v) for v in cfg.medium)
    return layered_model(cfg, anomalies=False)


class BlobBasis:
    """Gaussian blobs on an nbx x nbz grid of centres over the free-parameter
    region, one set per field (vp, vs, rho): fine = B m_field +
    background_field, B zero outside the region.  Blob index = ibx * nbz +
    ibz, centres at the middle of nbx x nbz equal spans of the region's cell
    centres, widths sqrt(0.5) * spacing, as in the reference's
    BlobParametrization (ElasticFullWaveform2D.py:256-313).  Model vectors
    are amplitudes relative to the background."""

    absolute = False

    def __init__(self, cfg, nbx=20, nbz=10):
        self.cfg, self.nbx, self.nbz = cfg, int(nbx), int(nbz)
        X, Z = cfg.cell_centres()
        mask = cfg.region_mask()
        Xr, Zr = X[mask], Z[mask]
        Lx = Xr.max() - Xr.min()
        Lz = Zr.max() - Zr.min()
        dx, dz = Lx / nbx, Lz / nbz
        px = dx * 0.5 + _np.arange(nbx) * dx + Xr.min()
        pz = dz * 0.5 + _np.arange(nbz) * dz + Zr.min()
        B = _np.zeros((cfg.nz * cfg.nx, nbx * nbz))
        for ix, xc in enumerate(px):
            for iz, zc in enumerate(pz):
                g = _np.exp(-(((X - xc) / (0.5**0.5 * dx)) ** 2 + ((Z - zc) / (0.5**0.5 * dz)) ** 2))
                B[:, ix * nbz + iz] = _np.where(mask, g, 0.0).reshape(-1)
        self.B = B  # physical cells x blobs
        self.n_blobs = nbx * nbz  # parameters per field
        self.free_parameters = 3 * self.n_blobs

    def simulation_basis(self):
        """Basis rows for every simulation cell (padding cells take the row
        of the physical cell they copy, or zeros): [nzc*nxc][n_blobs]."""
        rows = self.cfg.extension_matrix_rows()
        out = self.B[_np.maximum(rows, 0)]
        out[rows < 0] = 0.0
        return out

    def to_physical(self, m_field):
        """Contribution of one field's parameters to the physical cells [nz*nx]."""
        return self.B @ _np.asarray(m_field, _np.float64)

    def base_field(self, background_field):
        """The field of the physical cells that the parameters are added to."""
        return _np.asarray(background_field, _np.float64)

    def background_vector(self, background):
        """Model vector of the background fields: zero amplitudes."""
        return _np.zeros(self.free_parameters)

    def fit(self, fine_phys):
        """Least-squares blob amplitudes of a physical field [nz][nx]."""
        return _np.linalg.lstsq(self.B, fine_phys.reshape(-1), rcond=None)[0]


class CellBasis:
    """One free parameter per npx x npz block of cells of the free-parameter
    region, per field: psvWave's own model vector, which the reference
    samples when no blob grid is given (ElasticFullWaveform2D.py:57, 194-210).
    Parameters are absolute values (vp, vs, rho), blocks ordered with x
    fastest (the column-major flattening of the reference's [x][z] fields,
    ElasticFullWaveform2D.py:297-311); cells outside the region keep the
    background.  Applied on the device by a gather (model) and a segmented
    sum (gradient) instead of a dense basis matrix."""

    absolute = True

    def __init__(self, cfg, npx=1, npz=1):
        self.cfg, self.npx, self.npz = cfg, int(npx), int(npz)
        i0, i1, j0, j1 = cfg.kernel_region
        if (i1 - i0) % self.npx or (j1 - j0) % self.npz:
            raise ValueError(f"the {i1 - i0} x {j1 - j0} free-parameter region does not split into "
                             f"{self.npx} x {self.npz} blocks")
        self.nbx, self.nbz = (i1 - i0) // self.npx, (j1 - j0) // self.npz
        self.n_blobs = self.nbx * self.nbz  # parameters per field
        self.free_parameters = 3 * self.n_blobs
        jj, ii = _np.meshgrid(_np.arange(cfg.nz), _np.arange(cfg.nx), indexing="ij")
        inside = cfg.region_mask()
        par = ((jj - j0) // self.npz) * self.nbx + (ii - i0) // self.npx
        self.param_of = _np.where(inside, par, -1).reshape(-1).astype(_np.int32)  # physical cell -> parameter

    def simulation_map(self):
        """Parameter of every simulation cell (-1: none) [nzc*nxc]."""
        rows = self.cfg.extension_matrix_rows()
        return _np.where(rows >= 0, self.param_of[_np.maximum(rows, 0)], -1).astype(_np.int32)

    def gradient_segments(self):
        """CSR of parameter -> simulation cells (pointer [n_blobs+1], cells),
        for the gradient's segmented sum."""
        m = self.simulation_map()
        cells = _np.nonzero(m >= 0)[0]
        order = _np.argsort(m[cells], kind="stable")
        cells = cells[order].astype(_np.int32)
        ptr = _np.zeros(self.n_blobs + 1, _np.int64)
        _np.add.at(ptr, m[cells] + 1, 1)
        return _np.cumsum(ptr).astype(_np.int32), cells

    def to_physical(self, m_field):
        m = _np.asarray(m_field, _np.float64)
        return _np.where(self.param_of >= 0, m[_np.maximum(self.param_of, 0)], 0.0)

    def base_field(self, background_field):
        return _np.where(self.param_of >= 0, 0.0, _np.asarray(background_field, _np.float64).reshape(-1))

    def background_vector(self, background):
        """Model vector of the background fields (vp, vs, rho): block means."""
        out = []
        for f in range(3):
            b = _np.asarray(background[f], _np.float64).reshape(-1)
            sel = self.param_of >= 0
            out.append(_np.bincount(self.param_of[sel], b[sel], self.n_blobs) /
                       _np.bincount(self.param_of[sel], None, self.n_blobs))
        return _np.concatenate(out)

    def fit(self, fine_phys):
        """Block means of a physical field [nz][nx] (its least-squares fit)."""
        b = _np.asarray(fine_phys, _np.float64).reshape(-1)
        sel = self.param_of >= 0
        return _np.bincount(self.param_of[sel], b[sel], self.n_blobs) / _np.bincount(self.param_of[sel], None,
                                                                                      self.n_blobs)


def _ini_value(text):
    text = text.strip()
    if text.startswith("{"):
        depth, end = 0, None
        for k, ch in enumerate(text):
            depth += ch == "{"
            depth -= ch == "}"
            if depth == 0:
                end = k
                break
        if end is None:
            raise ValueError(f"unbalanced braces in {text!r}")
        body = text[: end + 1].replace("{", "[").replace("}", "]")
        import ast

        return ast.literal_eval(body)
    words = text.split(";")[0].split("//")[0].split()
    token = words[0] if words else ""
    for conv in (int, float):
        try:
            return conv(token)
        except ValueError:
            pass
    return token


def read_ini(path):
    """ElasticConfig keywords of a psvWave configuration file: the sections
    [domain] (nt, nx_inner, nz_inner, nx/nz_inner_boundary, dx, dz, dt),
    [boundary] (np_boundary, np_factor), [medium] (scalar_vp/vs/rho),
    [sources] (peak_frequency, source_timeshift, delay_cycles_per_shot,
    moment_angles, ix/iz_sources, which_source_to_fire_in_which_shot),
    [receivers] (nr, ix/iz_receivers), [inversion] (snapshot_interval) and
    [basis] (npx, npz) that the reference's configuration carries
    (tests/configurations/default_testing_configuration.ini:1-52 of the
    reference).  Values end at ';' or '//'; lists are in braces.

    Read as: cell indices of sources and receivers count from the physical
    model's corner (the simulation grid adds np_boundary sponge cells on
    every side); the k-th source fired in a shot starts its Ricker wavelet
    k * delay_cycles_per_shot / peak_frequency after the first, which is
    centred at source_timeshift; the free parameters are the cells at least
    nx/nz_inner_boundary cells inside the physical model, npx x npz cells per
    parameter; the sponge keeps the background medium.  The [output] folders
    are not used: observed data are passed to the distribution."""
    sec, raw = None, {}
    with open(path) as fh:
        for line in fh:
            line = line.strip()
            if not line or line.startswith(("#", ";")):
                continue
            if line.startswith("[") and "]" in line:
                sec = line[1:line.index("]")].strip()
                continue
            if "=" not in line:
                continue
            key, val = line.split("=", 1)
            raw[(sec, key.strip())] = _ini_value(val)

    def get(section, key, default=None):
        if (section, key) in raw:
            return raw[(section, key)]
        if default is None:
            raise ValueError(f"{path}: missing [{section}] {key}")
        return default

    nx, nz = int(get("domain", "nx_inner")), int(get("domain", "nz_inner"))
    dx, dz = float(get("domain", "dx")), float(get("domain", "dz"))
    if abs(dx - dz) > 1e-9 * max(dx, dz):
        raise ValueError(f"{path}: dx = {dx} and dz = {dz}; the stencils here use square cells")
    pad = int(get("boundary", "np_boundary"))
    f0 = float(get("sources", "peak_frequency"))
    ix_s, iz_s = list(get("sources", "ix_sources")), list(get("sources", "iz_sources"))
    angles = list(get("sources", "moment_angles"))
    n_src = int(get("sources", "n_sources", len(ix_s)))
    if not (len(ix_s) == len(iz_s) == len(angles) == n_src):
        raise ValueError(f"{path}: n_sources, ix_sources, iz_sources and moment_angles disagree")
    fire = get("sources", "which_source_to_fire_in_which_shot")
    n_shots = int(get("sources", "n_shots", len(fire)))
    if len(fire) != n_shots:
        raise ValueError(f"{path}: n_shots = {n_shots} but {len(fire)} firing lists")
    delay = float(get("sources", "delay_cycles_per_shot", 0.0)) / f0
    shots = []
    for lst in fire:
        shot = []
        for k, q in enumerate(lst):
            if not 0 <= int(q) < n_src:
                raise ValueError(f"{path}: source {q} of a firing list does not exist")
            shot.append(PointSource(pad + int(ix_s[q]), pad + int(iz_s[q]), *moment_tensor(angles[q]), delay=k * delay))
        shots.append(shot)
    ix_r, iz_r = list(get("receivers", "ix_receivers")), list(get("receivers", "iz_receivers"))
    nr = int(get("receivers", "nr", len(ix_r)))
    if not len(ix_r) == len(iz_r) == nr:
        raise ValueError(f"{path}: nr, ix_receivers and iz_receivers disagree")
    nxb, nzb = int(get("domain", "nx_inner_boundary", 0)), int(get("domain", "nz_inner_boundary", 0))
    vp = float(get("medium", "scalar_vp"))
    return dict(nx=nx, nz=nz, pad=pad, h=dx, dt=float(get("domain", "dt")), nt=int(get("domain", "nt")), f0=f0,
                sponge=float(get("boundary", "np_factor")), t0=float(get("sources", "source_timeshift", 1.2 / f0)),
                shots=shots, rec_cells=(pad + _np.asarray(ix_r, int), pad + _np.asarray(iz_r, int)),
                kernel_region=(nxb, nx - nxb, nzb, nz - nzb), extend_parameters=False,
                medium=(vp, float(get("medium", "scalar_vs")), float(get("medium", "scalar_rho"))),
                snapshot_interval=int(get("inversion", "snapshot_interval", 1)), vmax=1.25 * vp,
                cell_block=(int(get("basis", "npx", 1)), int(get("basis", "npz", 1))))
