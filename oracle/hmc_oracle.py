"""CPU oracle of the HMC hot path — TEST INFRASTRUCTURE ONLY.

A numpy (FP64) restatement of the reference algorithm, batched over chains in
the [d][C] layout the GPU library uses.  Only `tests/`, `__graft_entry__.smoke()`
and `bench.py`'s CPU-baseline leg may import this module; the product package
never does.

Pinning: every function here is checked against outputs of the reference
itself (larsgeb/hmclab imported through `oracle/ref_shim.py`), stored as golden
fixtures under `tests/golden/` by `tests/golden/make_golden.py`.  The Philox
restatement is pinned against the Random123 known-answer vectors.

Reference functions restated (file:line in larsgeb/hmclab):
  draw order of the random streams  MassMatrices.py:142,227,314; Samplers.py:1534,1486
  leapfrog (position Verlet)         Samplers.py:1524-1584
  3-stage / 4-stage integrators      Samplers.py:1586-1726
  accept / autotune                  Samplers.py:1471-1522
  thinned append                     Samplers.py:675-678
  corrector                          Distributions/base.py:239-270
  Normal / Laplace                   Distributions/base.py:539-574, 689-710
  LinearMatrix dense / sparse        Distributions/LinearMatrix.py:139-222, 309-440
  SourceLocation3D                   Distributions/SourceLocation.py:482-540, 697-713
  kinetic energy (Unit/Diag/Full)    MassMatrices.py:100-142, 185-227, 270-314
"""
import numpy as np

# ---------------------------------------------------------------------------
# Philox4x32-10 (Salmon et al. 2011), vectorised over numpy uint32 arrays.
# ---------------------------------------------------------------------------
_M0, _M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
_W0, _W1 = 0x9E3779B9, 0xBB67AE85
_MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(ctr, key):
    """ctr: uint32 array (..., 4); key: uint32 array (..., 2). Returns (..., 4)."""
    c = [np.asarray(ctr[..., j], dtype=np.uint64) for j in range(4)]
    k0 = np.asarray(key[..., 0], dtype=np.uint64)
    k1 = np.asarray(key[..., 1], dtype=np.uint64)
    for r in range(10):
        if r > 0:
            k0 = (k0 + np.uint64(_W0)) & _MASK
            k1 = (k1 + np.uint64(_W1)) & _MASK
        p0 = _M0 * c[0]
        p1 = _M1 * c[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & _MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & _MASK
        c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
    return np.stack([x.astype(np.uint32) for x in c], axis=-1)


# Random123 known-answer vectors for philox4x32-10 (counter, key, result).
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    (
        (0xFFFFFFFF,) * 4,
        (0xFFFFFFFF,) * 2,
        (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD),
    ),
    (
        (0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344),
        (0xA4093822, 0x299F31D0),
        (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1),
    ),
]


def philox_normal_f64(seed, rows, chains, proposal, purpose=0):
    """Standard normals of the FP64 device mode (two Philox blocks per quad)."""
    quads = (rows + 3) // 4
    qi, ci = np.meshgrid(np.arange(quads, dtype=np.uint64), np.arange(chains, dtype=np.uint64), indexing="ij")
    w = np.uint64(((proposal >> 32) & 0x07FFFFFF) | (purpose << 28))
    ctr0 = np.stack([qi, ci, np.full_like(qi, proposal & 0xFFFFFFFF), np.full_like(qi, w)], -1).astype(np.uint32)
    ctr1 = ctr0.copy()
    ctr1[..., 3] |= np.uint32(0x08000000)
    key = np.broadcast_to(np.array([seed & 0xFFFFFFFF, seed >> 32], dtype=np.uint32), ctr0.shape[:-1] + (2,))
    r0 = philox4x32_10(ctr0, key).astype(np.uint64)
    r1 = philox4x32_10(ctr1, key).astype(np.uint64)

    def u01d(a, b):
        v = (a << np.uint64(21)) ^ (b >> np.uint64(11))
        return (v.astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)

    u1, u2 = u01d(r0[..., 0], r0[..., 1]), u01d(r0[..., 2], r0[..., 3])
    u3, u4 = u01d(r1[..., 0], r1[..., 1]), u01d(r1[..., 2], r1[..., 3])
    a, b = np.sqrt(-2.0 * np.log(u1)), np.sqrt(-2.0 * np.log(u3))
    t1, t2 = 2 * np.pi * u2, 2 * np.pi * u4
    z = np.stack([a * np.cos(t1), a * np.sin(t1), b * np.cos(t2), b * np.sin(t2)], axis=1)  # quads,4,C
    return z.reshape(quads * 4, chains)[:rows]


def philox_normal_f32(seed, rows, chains, proposal, purpose=0):
    """Standard normals of the FP32 device mode (one Philox block per quad), FP64 math."""
    quads = (rows + 3) // 4
    qi, ci = np.meshgrid(np.arange(quads, dtype=np.uint64), np.arange(chains, dtype=np.uint64), indexing="ij")
    w = np.uint64(((proposal >> 32) & 0x0FFFFFFF) | (purpose << 28))
    ctr = np.stack([qi, ci, np.full_like(qi, proposal & 0xFFFFFFFF), np.full_like(qi, w)], -1).astype(np.uint32)
    key = np.broadcast_to(np.array([seed & 0xFFFFFFFF, seed >> 32], dtype=np.uint32), ctr.shape[:-1] + (2,))
    r = philox4x32_10(ctr, key)
    u = ((r >> np.uint32(8)).astype(np.float64) + 0.5) / 16777216.0
    a, b = np.sqrt(-2.0 * np.log(u[..., 0])), np.sqrt(-2.0 * np.log(u[..., 2]))
    t1, t2 = 2 * np.pi * u[..., 1], 2 * np.pi * u[..., 3]
    z = np.stack([a * np.cos(t1), a * np.sin(t1), b * np.cos(t2), b * np.sin(t2)], axis=1)
    return z.reshape(quads * 4, chains)[:rows]


# ---------------------------------------------------------------------------
# Random streams in the reference's draw order.
# ---------------------------------------------------------------------------
def reference_streams(seed, dims, proposals, randomize_stepsize=True):
    """Replay `numpy.random.default_rng(seed)` in the order the reference HMC
    draws: normal(d,1) (momentum) -> uniform(0.5,1.5) (step factor, if
    randomised) -> uniform(0,1) (accept).  Returns z[P][d], f[P], u[P]."""
    rng = np.random.default_rng(seed)
    z = np.empty((proposals, dims))
    f = np.ones(proposals)
    u = np.empty(proposals)
    for n in range(proposals):
        z[n] = rng.normal(size=(dims, 1))[:, 0]
        if randomize_stepsize:
            f[n] = rng.uniform(0.5, 1.5)
        u[n] = rng.uniform(0, 1)
    return z, f, u


def batched_streams(seeds, dims, proposals, randomize_stepsize=True):
    """Per-chain reference streams stacked to the device layout:
    z[P][d][C], f[P][C], u[P][C]."""
    zs, fs, us = zip(*(reference_streams(s, dims, proposals, randomize_stepsize) for s in seeds))
    return np.stack(zs, axis=-1), np.stack(fs, axis=-1), np.stack(us, axis=-1)


# ---------------------------------------------------------------------------
# Target distributions, batched: M is (d, C) float64.
# ---------------------------------------------------------------------------
class NormalDiag:
    def __init__(self, mean, var):
        self.mean = np.asarray(mean, float).reshape(-1, 1)
        self.iv = 1.0 / np.asarray(var, float).reshape(-1, 1) * np.ones_like(self.mean)

    def misfit(self, M):
        r = self.mean - M
        return 0.5 * np.sum(r * (self.iv * r), axis=0)

    def gradient(self, M):
        return -self.iv * (self.mean - M)


class NormalFull:
    def __init__(self, mean, cov):
        self.mean = np.asarray(mean, float).reshape(-1, 1)
        self.icov = np.linalg.inv(np.asarray(cov, float))

    def misfit(self, M):
        r = self.mean - M
        return 0.5 * np.sum(r * (self.icov @ r), axis=0)

    def gradient(self, M):
        return -self.icov @ (self.mean - M)


class Laplace:
    def __init__(self, mean, disp):
        self.mean = np.asarray(mean, float).reshape(-1, 1)
        self.idisp = 1.0 / np.asarray(disp, float).reshape(-1, 1) * np.ones_like(self.mean)

    def misfit(self, M):
        return np.sum(np.abs(M - self.mean) * self.idisp, axis=0)

    def gradient(self, M):
        return np.sign(M - self.mean) * self.idisp


class DensePremul:
    """LinearMatrix.py:164-208 with premultiplication (n > d)."""

    def __init__(self, G, d, var):
        G = np.asarray(G, float)
        d = np.asarray(d, float).reshape(-1, 1)
        iv = (1.0 / np.asarray(var, float)).reshape(-1, 1) * np.ones_like(d)
        self.GtG = G.T @ (iv * G)
        self.Gtd0 = G.T @ (iv * d)
        self.dtd = (d.T @ (iv * d)).item()

    def misfit(self, M):
        return 0.5 * (np.sum(M * (self.GtG @ M - 2 * self.Gtd0), axis=0) + self.dtd)

    def gradient(self, M):
        return self.GtG @ M - self.Gtd0


class DenseResid:
    """LinearMatrix.py:193-208 without premultiplication (residual form)."""

    def __init__(self, G, d, var):
        self.G = np.asarray(G, float)
        self.d = np.asarray(d, float).reshape(-1, 1)
        self.iv = (1.0 / np.asarray(var, float)).reshape(-1, 1) * np.ones_like(self.d)

    def misfit(self, M):
        r = self.G @ M - self.d
        return 0.5 * np.sum(r * r * self.iv, axis=0)

    def gradient(self, M):
        return self.G.T @ ((self.G @ M - self.d) * self.iv)


class SparseLinear(DenseResid):
    """LinearMatrix.py:389-426: G is a scipy CSR matrix (restated with its dense product)."""

    def __init__(self, G_csr, d, var):
        self.Gs = G_csr
        self.d = np.asarray(d, float).reshape(-1, 1)
        self.iv = (1.0 / np.asarray(var, float)).reshape(-1, 1) * np.ones_like(self.d)

    def misfit(self, M):
        r = self.Gs @ M - self.d
        return 0.5 * np.sum(r * r * self.iv, axis=0)

    def gradient(self, M):
        return self.Gs.T @ ((self.Gs @ M - self.d) * self.iv)


class SourceLocation3D:
    """SourceLocation.py:482-540 with the interleaved [x,y,z,T]*E (+v) layout."""

    def __init__(self, rx, ry, rz, obs, std, infer_velocity=True, medium_velocity=None):
        self.rx = np.asarray(rx, float).reshape(1, 1, -1)
        self.ry = np.asarray(ry, float).reshape(1, 1, -1)
        self.rz = np.asarray(rz, float).reshape(1, 1, -1)
        self.obs = np.asarray(obs, float)[:, None, :]  # E,1,S
        self.iv = 1.0 / np.asarray(std, float)[:, None, :] ** 2
        self.infer_velocity = infer_velocity
        self.v = medium_velocity
        self.E = self.obs.shape[0]

    def _split(self, M):
        E = self.E
        x, y, z, T = (M[k : 4 * E : 4][:, :, None] for k in range(4))  # E,C,1
        v = M[4 * E][None, :, None] if self.infer_velocity else self.v
        return x, y, z, T, v

    def misfit(self, M):
        x, y, z, T, v = self._split(M)
        dist = np.sqrt((x - self.rx) ** 2 + (y - self.ry) ** 2 + (z - self.rz) ** 2)
        r = (self.obs - (T + dist / v)) ** 2 * self.iv
        return 0.5 * np.nansum(r, axis=(0, 2))

    def gradient(self, M):
        x, y, z, T, v = self._split(M)
        dx, dy, dz = x - self.rx, y - self.ry, z - self.rz
        dist = np.sqrt(dx * dx + dy * dy + dz * dz)
        with np.errstate(divide="ignore", invalid="ignore"):
            mg = (T + dist / v - self.obs) * self.iv
            out = np.zeros_like(M)
            out[0 : 4 * self.E : 4] = np.nansum(mg * dx / (v * dist), axis=2)
            out[1 : 4 * self.E : 4] = np.nansum(mg * dy / (v * dist), axis=2)
            out[2 : 4 * self.E : 4] = np.nansum(mg * dz / (v * dist), axis=2)
            out[3 : 4 * self.E : 4] = np.nansum(mg, axis=2)
            if self.infer_velocity:
                out[4 * self.E] = np.nansum(mg * (-dist / (v * v)), axis=(0, 2))
        return out


class Tempered:
    """Per-chain tempered target: chain c has misfit beta[c] * U and gradient
    beta[c] * grad U (the reference tempers by giving each parallel chain its
    own distribution with the misfit divided by the temperature)."""

    def __init__(self, dist, beta):
        self.dist = dist
        self.beta = np.asarray(beta, float).reshape(-1)

    def misfit(self, M):
        return self.beta * self.dist.misfit(M)

    def gradient(self, M):
        return self.beta[None, :] * self.dist.gradient(M)


def run_tempered_exchange(dist, beta, mass, q0, eps0, streams, proposals, interval, schedule, exchange_u,
                          amount_of_steps=10):
    """Parallel tempering as the reference's ParallelSampleSMP runs it
    (Samplers.py:529-704 with the exchange section 589-669 and the schedule
    of 1872-1885): every chain makes one proposal on its tempered target;
    after proposals n with n % interval == 0 the pairs of schedule row
    n // interval (entries 2j, 2j+1) swap models iff
    exp(improvement_a + improvement_b) > u; then the sample is recorded.
    The recorded misfit is the chain's current misfit, which the reference's
    exchange leaves unchanged, so a swapped chain records its pre-swap value.
    Returns samples [N][d+1][C] and the swap decisions [E][pairs]."""
    z, f, u = streams
    beta = np.asarray(beta, float)
    tdist = Tempered(dist, beta)
    q = np.array(q0, float, copy=True)
    out, decisions = [], []
    for n in range(proposals):
        res = run_chains(tdist, mass, q, eps0, (z[n:n + 1], f[n:n + 1], u[n:n + 1]), 1,
                         amount_of_steps=amount_of_steps)
        q, x = res["q"], res["x"]
        if n % interval == 0 and n // interval < len(schedule):
            pairs = np.asarray(schedule[n // interval]).reshape(-1, 2)
            q, _, sw = exchange(q, x / beta, beta, pairs, exchange_u[n // interval])
            decisions.append(sw)
        out.append(np.vstack([q, x[None, :]]))
    return np.array(out), np.array(decisions)


class Sum:
    """BayesRule / AdditiveDistribution (base.py:1036-1054): sum in list order."""

    def __init__(self, parts):
        self.parts = list(parts)

    def misfit(self, M):
        return sum(p.misfit(M) for p in self.parts)

    def gradient(self, M):
        g = np.zeros_like(M)
        for p in self.parts:
            g = g + p.gradient(M)
        return g


# ---------------------------------------------------------------------------
# Mass matrices.
# ---------------------------------------------------------------------------
class Mass:
    def __init__(self, kind="unit", diag=None, full=None, dims=None):
        self.kind = kind
        if kind == "diag":
            self.diag = np.asarray(diag, float).reshape(-1, 1)
            self.inv_diag = 1.0 / self.diag
        elif kind == "full":
            self.full = np.asarray(full, float)
            self.L = np.linalg.cholesky(self.full)
            self.inv = np.linalg.inv(self.full)

    def momentum(self, z):
        if self.kind == "unit":
            return z.copy()
        if self.kind == "diag":
            return np.sqrt(self.diag) * z
        return self.L @ z

    def grad(self, p):
        if self.kind == "unit":
            return p
        if self.kind == "diag":
            return self.inv_diag * p
        return self.inv @ p

    def energy(self, p):
        return 0.5 * np.sum(p * self.grad(p), axis=0)


# ---------------------------------------------------------------------------
# Integrators and the sampler loop.
# ---------------------------------------------------------------------------
LF = "lf"
THREE_STAGE = (0.11888010966548, 0.29619504261126)  # a1, b1 (Samplers.py:1666-1669)
FOUR_STAGE = (0.071353913450279725904, 0.268548791161230105820, 0.191667800000000000000)  # a1, a2, b1


def integrator_schedule(integrator, amount_of_steps):
    """List of ('d', coeff) drift and ('k', coeff) kick operations, in order."""
    ops = []
    if integrator == "lf":
        ops.append(("d", 0.5))
        for _ in range(amount_of_steps - 1):
            ops += [("k", 1.0), ("d", 1.0)]
        ops += [("k", 1.0), ("d", 0.5)]
    elif integrator == "3s":
        a1, b1 = THREE_STAGE
        a2, b2 = 0.5 - a1, 1.0 - 2.0 * b1
        for _ in range(amount_of_steps):
            ops += [("d", a1), ("k", b1), ("d", a2), ("k", b2), ("d", a2), ("k", b1), ("d", a1)]
    elif integrator == "4s":
        a1, a2, b1 = FOUR_STAGE
        a3 = 1.0 - 2.0 * a1 - 2.0 * a2
        b2 = 0.5 - b1
        for _ in range(amount_of_steps):
            ops += [("d", a1), ("k", b1), ("d", a2), ("k", b2), ("d", a3), ("k", b2), ("d", a2), ("k", b1), ("d", a1)]
    else:
        raise ValueError(integrator)
    return ops


def reflect(q, p, lower, upper):
    """base.py:239-270, vectorised; returns a per-chain still-outside mask."""
    if lower is not None:
        lo = q < lower
        q[lo] += 2 * (np.broadcast_to(lower, q.shape)[lo] - q[lo])
        p[lo] *= -1.0
    if upper is not None:
        hi = q > upper
        q[hi] += 2 * (np.broadcast_to(upper, q.shape)[hi] - q[hi])
        p[hi] *= -1.0
    out = np.zeros(q.shape[1], bool)
    if lower is not None:
        out |= np.any(q < lower, axis=0)
    if upper is not None:
        out |= np.any(q > upper, axis=0)
    return out


def trajectory(dist, mass, q0, p0, eps, integrator="lf", amount_of_steps=10, lower=None, upper=None, record=None):
    """One trajectory for every chain; eps is (C,).  Mirrors Samplers.py:1524-1726:
    the coefficient is multiplied by the step size first, then by the vector."""
    q, p = q0.copy(), p0.copy()
    oob = np.zeros(q.shape[1], bool)
    eps = np.asarray(eps, float).reshape(1, -1)
    for op, coeff in integrator_schedule(integrator, amount_of_steps):
        if op == "d":
            q += (coeff * eps) * mass.grad(p)
            oob |= reflect(q, p, lower, upper)
        else:
            g = dist.gradient(q)
            if record is not None:
                record.append((q.copy(), g.copy()))
            p -= (coeff * eps) * g
    return q, p, oob


def run_chains(
    dist,
    mass,
    q0,
    eps0,
    streams,
    proposals,
    integrator="lf",
    amount_of_steps=10,
    randomize_stepsize=True,
    online_thinning=1,
    lower=None,
    upper=None,
    autotuning=False,
    target_acceptance_rate=0.65,
    learning_rate=0.75,
    minimal_stepsize=1e-18,
):
    """The reference proposal loop (Samplers.py:529-704 + 1463-1522) for C chains
    driven by injected streams (z[P][d][C], f[P][C], u[P][C]).

    Returns dict with samples [N][d+1][C] (the reference's vstack([q, x])),
    accepted counts, final stepsizes, per-proposal H0/H1/u and accept flags."""
    z, f, u = streams
    q = np.array(q0, float, copy=True)
    C = q.shape[1]
    eps = np.full(C, float(eps0)) if np.ndim(eps0) == 0 else np.array(eps0, float)
    x = dist.misfit(q)
    out_s, H0s, H1s, acc, stepsizes, rates = [], [], [], [], [], []
    accepted = np.zeros(C, int)
    for n in range(proposals):
        p0 = mass.momentum(z[n])
        le = f[n] * eps if randomize_stepsize else eps.copy()
        q1, p1, oob = trajectory(dist, mass, q, p0, le, integrator, amount_of_steps, lower, upper)
        x0 = x
        k0 = mass.energy(p0)
        x1 = dist.misfit(q1)
        x1 = np.where(oob, np.inf, x1)
        k1 = mass.energy(p1)
        h0, h1 = x0 + k0, x1 + k1
        with np.errstate(over="ignore", invalid="ignore"):
            alpha = np.exp(h0 - h1)
        if autotuning:
            stepsizes.append(eps.copy())
            rates.append(alpha.copy())
            w = (n + 1) ** (-learning_rate)
            a = np.where(np.isnan(alpha), 0.0, alpha)
            eps = eps - w * (target_acceptance_rate - np.minimum(a, 1.0))
            eps = np.where(eps <= 0, np.maximum(eps, minimal_stepsize), eps)
        a_mask = alpha > u[n]
        q = np.where(a_mask[None, :], q1, q)
        x = np.where(a_mask, x1, x)
        accepted += a_mask
        H0s.append(h0)
        H1s.append(h1)
        acc.append(a_mask)
        if n % online_thinning == 0:
            out_s.append(np.vstack([q, x[None, :]]))
    res = dict(
        samples=np.array(out_s),
        accepted=accepted,
        stepsize=eps,
        H0=np.array(H0s),
        H1=np.array(H1s),
        accept=np.array(acc),
        q=q,
        x=x,
    )
    if autotuning:
        res["stepsizes"] = np.array(stepsizes)
        res["acceptance_rates"] = np.array(rates)
    return res


# ---------------------------------------------------------------------------
# Effective sample size (the reference has none; BDA3 section 11.5 split-chain
# multi-chain estimator with Geyer's initial monotone sequence).
# ---------------------------------------------------------------------------
def exchange(q, x, beta, pairs, u):
    """Replica exchange of the reference's parallel sampler
    (Samplers.py:589-669): chains a, b with tempered misfits beta * x swap
    their models iff exp(improvement_a + improvement_b) > u, where
    improvement_a = beta_a (x_a - x_b) and improvement_b = beta_b (x_b - x_a).
    q is [d][C] (columns are chains), x and beta are [C]; pairs is [P][2].
    Returns the new (q, x) and the decisions."""
    q = np.array(q, copy=True)
    x = np.array(x, copy=True)
    swapped = np.zeros(len(pairs), bool)
    for k, (a, b) in enumerate(pairs):
        improvement = beta[a] * (x[a] - x[b]) + beta[b] * (x[b] - x[a])
        with np.errstate(over="ignore"):
            if np.exp(improvement) > u[k]:
                swapped[k] = True
                q[:, [a, b]] = q[:, [b, a]]
                x[[a, b]] = x[[b, a]]
    return q, x, swapped


def ess_split(x, lags):
    """x: [N][d][C] samples.  Returns (ess[d], rhat[d]); ess is negated where
    the lag window was too short to truncate (same convention as hmc_ess)."""
    N, d, C = x.shape
    n = N // 2
    h = np.concatenate([x[:n], x[n : 2 * n]], axis=2)  # n, d, M
    M = 2 * C
    mu_m = h.mean(axis=0)  # d, M
    var_m = h.var(axis=0, ddof=1)
    W = var_m.mean(axis=1)
    mu = mu_m.mean(axis=1)
    B = n / (M - 1) * np.sum((mu_m - mu[:, None]) ** 2, axis=1)
    varp = (n - 1) / n * W + B / n
    hc = h - mu_m[None]
    out = np.empty(d)
    for i in range(d):
        def rho(t):
            g = np.sum(hc[: n - t, i] * hc[t:, i], axis=0) / n  # M
            return 1.0 - (W[i] - g.mean()) / varp[i]

        s, prev, trunc = 0.0, np.inf, False
        t = 0
        while t + 1 < lags:
            P = rho(t) + rho(t + 1)
            if P < 0:
                trunc = True
                break
            P = min(P, prev)
            prev = P
            s += P
            t += 2
        e = M * n / (-1.0 + 2.0 * s)
        out[i] = e if trunc else -e
    return out, np.sqrt(varp / W)


def rank_normalize(x):
    """Normal scores of pooled ranks per parameter (Vehtari, Gelman, Simpson,
    Carpenter & Buerkner 2021, section 4.1): x [N][d][C] -> z of the same
    shape, z = Phi^-1((r - 3/8) / (S + 1/4)) with r the average rank of a draw
    among the S = N C draws of its parameter.  (No counterpart in the
    reference, whose only mixing diagnostic is Helpers/Processing.py:6-13.)"""
    from scipy.special import ndtri
    from scipy.stats import rankdata

    N, d, C = x.shape
    S = N * C
    z = np.empty((N, d, C))
    for i in range(d):
        r = rankdata(x[:, i, :].reshape(-1), method="average")
        z[:, i, :] = ndtri((r - 0.375) / (S + 0.25)).reshape(N, C)
    return z


def ar1_ess(phi, n_total):
    """Asymptotic ESS of a stationary AR(1) chain: N (1 - phi) / (1 + phi)."""
    return n_total * (1 - phi) / (1 + phi)
