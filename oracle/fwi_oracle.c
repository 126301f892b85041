/*
 * FP64 CPU oracle of the 2-D elastic P-SV finite-difference forward model and
 * its exact discrete adjoint — TEST INFRASTRUCTURE ONLY (tests, smoke() and
 * the CPU leg of bench.py load it; the product never does).
 *
 * The reference wraps the third-party package psvWave 0.2.1 (pinned in the
 * reference's Dockerfile:10; not vendored and not installed here), called at
 * hmclab/Distributions/ElasticFullWaveform2D.py:150-184.  Its arithmetic is
 * restated from the published methods it names: Virieux (1986) velocity-stress
 * staggered grid, Levander (1988) fourth-order differences (9/8, -1/24),
 * Cerjan et al. (1985) sponge, explosive or moment-tensor point sources (a
 * stress glut) with Ricker wavelets,
 * an L2 waveform misfit and the gradient by the exact transpose (reverse mode)
 * of the discrete time stepping, optionally with the forward/adjoint
 * correlation taken at every k-th step only and weighted by k (psvWave's
 * snapshot_interval).  No reference numbers exist for this path
 * (the reference's FWI test is skipped without psvWave), so parity is pinned
 * by finite differences and by the CUDA implementation agreeing with this one.
 *
 * Grid: fields on an nz x nx grid (x fastest), spacing h, time step dt.
 *   vx at (i+1/2, j), vz at (i, j+1/2), sxx/szz at (i, j), sxz at (i+1/2, j+1/2)
 *   b = 1/rho, lambda = rho (vp^2 - 2 vs^2), mu = rho vs^2,
 *   bx = (b[i] + b[i+1]) / 2, bz = (b[j] + b[j+1]) / 2,
 *   muxz = (mu[i,j] + mu[i+1,j] + mu[i,j+1] + mu[i+1,j+1]) / 4.
 * Every field is updated on 2 <= i < nx-2, 2 <= j < nz-2 and is zero outside.
 * One time step n:
 *   1. vx += dt bx (Dx+ sxx + Dz- sxz),  vz += dt bz (Dx- sxz + Dz+ szz)
 *   2. vx, vz *= taper
 *   3. record vx, vz at the receivers
 *   4. sxx += dt ((l+2m) Dx- vx + l Dz- vz), szz += dt (l Dx- vx + (l+2m) Dz- vz),
 *      sxz += dt muxz (Dz+ vx + Dx+ vz)
 *   5. sxx, szz at the source += stf[n] * dt / h^2 (an explosion); for a
 *      moment tensor M: sxx += Mxx s, szz += Mzz s at the source node and
 *      each of the four surrounding sxz nodes += Mxz s / 4, s = stf[n] dt / h^2
 *   6. sxx, szz, sxz *= taper
 * with Dx+ f[i] = (c1 (f[i+1] - f[i]) + c2 (f[i+2] - f[i-1])) / h and
 *      Dx- f[i] = (c1 (f[i] - f[i-1]) + c2 (f[i+1] - f[i-2])) / h, c1 = 9/8, c2 = -1/24.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define C1 (9.0 / 8.0)
#define C2 (-1.0 / 24.0)

typedef struct {
  int nx, nz, nt;
  double h, dt;
  const double* taper; /* [nz][nx] */
  const double* stf;   /* [nt] */
  int src_x, src_z;
  int nrec;
  const int* rec_x;
  const int* rec_z;
  /* nsrc > 0: the shot is fired by nsrc moment-tensor point sources instead
   * of the explosive source above (src_x, src_z, stf unused) */
  int nsrc;
  const int* msrc_x;
  const int* msrc_z;
  const double* moment; /* [nsrc][3]: Mxx, Mzz, Mxz */
  const double* mstf;   /* [nsrc][nt] wavelets */
  /* k > 1: the gradient correlates forward and adjoint fields at the steps
   * n = 0, k, 2k, ... only, each weighted by k (psvWave's snapshot_interval);
   * 0 or 1: at every step (the exact discrete gradient) */
  int snapshot_interval;
} fwi_shot;

#define IDX(j, i) ((size_t)(j) * (size_t)nx + (size_t)(i))

static inline int valid(int i, int j, int nx, int nz) { return i >= 2 && i < nx - 2 && j >= 2 && j < nz - 2; }

static void derived(int nx, int nz, const double* rho, const double* vp, const double* vs, double* bx, double* bz,
                    double* l2m, double* lam, double* muxz) {
  for (int j = 0; j < nz; ++j)
    for (int i = 0; i < nx; ++i) {
      const size_t k = IDX(j, i);
      const double mu = rho[k] * vs[k] * vs[k];
      lam[k] = rho[k] * (vp[k] * vp[k] - 2.0 * vs[k] * vs[k]);
      l2m[k] = lam[k] + 2.0 * mu;
      const int i1 = i + 1 < nx ? i + 1 : i, j1 = j + 1 < nz ? j + 1 : j;
      bx[k] = 0.5 * (1.0 / rho[k] + 1.0 / rho[IDX(j, i1)]);
      bz[k] = 0.5 * (1.0 / rho[k] + 1.0 / rho[IDX(j1, i)]);
      const double m00 = mu, m10 = rho[IDX(j, i1)] * vs[IDX(j, i1)] * vs[IDX(j, i1)];
      const double m01 = rho[IDX(j1, i)] * vs[IDX(j1, i)] * vs[IDX(j1, i)];
      const double m11 = rho[IDX(j1, i1)] * vs[IDX(j1, i1)] * vs[IDX(j1, i1)];
      muxz[k] = 0.25 * (m00 + m10 + m01 + m11);
    }
}

static inline double dxp(const double* f, int nx, int j, int i, double h) {
  return (C1 * (f[IDX(j, i + 1)] - f[IDX(j, i)]) + C2 * (f[IDX(j, i + 2)] - f[IDX(j, i - 1)])) / h;
}
static inline double dxm(const double* f, int nx, int j, int i, double h) {
  return (C1 * (f[IDX(j, i)] - f[IDX(j, i - 1)]) + C2 * (f[IDX(j, i + 1)] - f[IDX(j, i - 2)])) / h;
}
static inline double dzp(const double* f, int nx, int j, int i, double h) {
  return (C1 * (f[IDX(j + 1, i)] - f[IDX(j, i)]) + C2 * (f[IDX(j + 2, i)] - f[IDX(j - 1, i)])) / h;
}
static inline double dzm(const double* f, int nx, int j, int i, double h) {
  return (C1 * (f[IDX(j, i)] - f[IDX(j - 1, i)]) + C2 * (f[IDX(j + 1, i)] - f[IDX(j - 2, i)])) / h;
}

/* Forward simulation of one shot.  rec_vx/rec_vz: [nt][nrec].  store_vx/vz
 * ([nt][nz][nx], nullable) receive the velocities after step 2 of every n. */
int fwi_forward(const fwi_shot* s, const double* rho, const double* vp, const double* vs, double* rec_vx,
                double* rec_vz, double* store_vx, double* store_vz) {
  const int nx = s->nx, nz = s->nz;
  const size_t N = (size_t)nx * nz;
  double* buf = (double*)calloc(10 * N, sizeof(double));
  if (!buf) return 1;
  double *vx = buf, *vz = buf + N, *sxx = buf + 2 * N, *szz = buf + 3 * N, *sxz = buf + 4 * N;
  double *bx = buf + 5 * N, *bz = buf + 6 * N, *l2m = buf + 7 * N, *lam = buf + 8 * N, *muxz = buf + 9 * N;
  derived(nx, nz, rho, vp, vs, bx, bz, l2m, lam, muxz);
  const double dt = s->dt, h = s->h;
  for (int n = 0; n < s->nt; ++n) {
    for (int j = 2; j < nz - 2; ++j)
      for (int i = 2; i < nx - 2; ++i) {
        const size_t k = IDX(j, i);
        vx[k] += dt * bx[k] * (dxp(sxx, nx, j, i, h) + dzm(sxz, nx, j, i, h));
        vz[k] += dt * bz[k] * (dxm(sxz, nx, j, i, h) + dzp(szz, nx, j, i, h));
      }
    for (size_t k = 0; k < N; ++k) {
      vx[k] *= s->taper[k];
      vz[k] *= s->taper[k];
    }
    for (int r = 0; r < s->nrec; ++r) {
      rec_vx[(size_t)n * s->nrec + r] = vx[IDX(s->rec_z[r], s->rec_x[r])];
      rec_vz[(size_t)n * s->nrec + r] = vz[IDX(s->rec_z[r], s->rec_x[r])];
    }
    if (store_vx) {
      memcpy(store_vx + (size_t)n * N, vx, N * sizeof(double));
      memcpy(store_vz + (size_t)n * N, vz, N * sizeof(double));
    }
    for (int j = 2; j < nz - 2; ++j)
      for (int i = 2; i < nx - 2; ++i) {
        const size_t k = IDX(j, i);
        const double exx = dxm(vx, nx, j, i, h), ezz = dzm(vz, nx, j, i, h);
        sxx[k] += dt * (l2m[k] * exx + lam[k] * ezz);
        szz[k] += dt * (lam[k] * exx + l2m[k] * ezz);
        sxz[k] += dt * muxz[k] * (dzp(vx, nx, j, i, h) + dxp(vz, nx, j, i, h));
      }
    if (s->nsrc > 0) {
      /* stress glut of a moment tensor M at the sxx/szz node (i, j): Mxx and
       * Mzz there, Mxz shared by the four sxz nodes (i -/+ 1/2, j -/+ 1/2) */
      for (int q = 0; q < s->nsrc; ++q) {
        const int i = s->msrc_x[q], j = s->msrc_z[q];
        const double v = s->mstf[(size_t)q * s->nt + n] * dt / (h * h);
        const double* M = s->moment + 3 * q;
        sxx[IDX(j, i)] += M[0] * v;
        szz[IDX(j, i)] += M[1] * v;
        sxz[IDX(j - 1, i - 1)] += 0.25 * M[2] * v;
        sxz[IDX(j - 1, i)] += 0.25 * M[2] * v;
        sxz[IDX(j, i - 1)] += 0.25 * M[2] * v;
        sxz[IDX(j, i)] += 0.25 * M[2] * v;
      }
    } else {
      const size_t ks = IDX(s->src_z, s->src_x);
      sxx[ks] += s->stf[n] * dt / (h * h);
      szz[ks] += s->stf[n] * dt / (h * h);
    }
    for (size_t k = 0; k < N; ++k) {
      sxx[k] *= s->taper[k];
      szz[k] *= s->taper[k];
      sxz[k] *= s->taper[k];
    }
  }
  free(buf);
  return 0;
}

/* Misfit 0.5 * w * sum (rec - obs)^2 of one shot and the gradient of that
 * misfit with respect to rho, vp, vs on the whole grid (accumulated into
 * g_rho/g_vp/g_vs), by the exact reverse of fwi_forward.  obs: [nt][nrec]. */
double fwi_gradient(const fwi_shot* s, const double* rho, const double* vp, const double* vs, const double* obs_vx,
                    const double* obs_vz, double w, double* g_rho, double* g_vp, double* g_vs) {
  const int nx = s->nx, nz = s->nz, nt = s->nt, nr = s->nrec;
  const size_t N = (size_t)nx * nz;
  double* rvx = (double*)malloc((size_t)nt * nr * sizeof(double));
  double* rvz = (double*)malloc((size_t)nt * nr * sizeof(double));
  double* svx = (double*)malloc((size_t)nt * N * sizeof(double));
  double* svz = (double*)malloc((size_t)nt * N * sizeof(double));
  double* buf = (double*)calloc(18 * N, sizeof(double));
  if (!rvx || !rvz || !svx || !svz || !buf) return NAN;
  fwi_forward(s, rho, vp, vs, rvx, rvz, svx, svz);
  double chi = 0.0;
  for (size_t t = 0; t < (size_t)nt * nr; ++t) {
    const double a = rvx[t] - obs_vx[t], b = rvz[t] - obs_vz[t];
    chi += 0.5 * w * (a * a + b * b);
  }
  double *ax = buf, *az = buf + N, *asxx = buf + 2 * N, *aszz = buf + 3 * N, *asxz = buf + 4 * N;
  double *bx = buf + 5 * N, *bz = buf + 6 * N, *l2m = buf + 7 * N, *lam = buf + 8 * N, *muxz = buf + 9 * N;
  double *g_bx = buf + 10 * N, *g_bz = buf + 11 * N, *g_l2m = buf + 12 * N, *g_lam = buf + 13 * N;
  double *g_muxz = buf + 14 * N, *t1 = buf + 15 * N, *t2 = buf + 16 * N, *t3 = buf + 17 * N;
  derived(nx, nz, rho, vp, vs, bx, bz, l2m, lam, muxz);
  const double dt = s->dt, h = s->h;
  const int ksnap = s->snapshot_interval > 1 ? s->snapshot_interval : 1;
  for (int n = nt - 1; n >= 0; --n) {
    const double* vxn = svx + (size_t)n * N;
    const double* vzn = svz + (size_t)n * N;
    /* weight of this step's correlation: k at snapshot steps, else none */
    const double wk = n % ksnap == 0 ? (double)ksnap : 0.0;
    /* reverse of 6 */
    for (size_t k = 0; k < N; ++k) {
      asxx[k] *= s->taper[k];
      aszz[k] *= s->taper[k];
      asxz[k] *= s->taper[k];
    }
    /* reverse of 4: parameter gradients and adjoint velocities */
    memset(t1, 0, N * sizeof(double));
    memset(t2, 0, N * sizeof(double));
    memset(t3, 0, N * sizeof(double));
    for (int j = 2; j < nz - 2; ++j)
      for (int i = 2; i < nx - 2; ++i) {
        const size_t k = IDX(j, i);
        const double exx = dxm(vxn, nx, j, i, h), ezz = dzm(vzn, nx, j, i, h);
        const double exz = dzp(vxn, nx, j, i, h) + dxp(vzn, nx, j, i, h);
        g_l2m[k] += wk * dt * (exx * asxx[k] + ezz * aszz[k]);
        g_lam[k] += wk * dt * (ezz * asxx[k] + exx * aszz[k]);
        g_muxz[k] += wk * dt * exz * asxz[k];
        t1[k] = dt * (l2m[k] * asxx[k] + lam[k] * aszz[k]); /* pairs with Dx- vx */
        t2[k] = dt * (lam[k] * asxx[k] + l2m[k] * aszz[k]); /* pairs with Dz- vz */
        t3[k] = dt * muxz[k] * asxz[k];                      /* pairs with Dz+ vx, Dx+ vz */
      }
    /* transposes: (Dx-)^T = -Dx+, (Dz-)^T = -Dz+, (Dz+)^T = -Dz-, (Dx+)^T = -Dx- */
    for (int j = 2; j < nz - 2; ++j)
      for (int i = 2; i < nx - 2; ++i) {
        const size_t k = IDX(j, i);
        ax[k] += -dxp(t1, nx, j, i, h) - dzm(t3, nx, j, i, h);
        az[k] += -dzp(t2, nx, j, i, h) - dxm(t3, nx, j, i, h);
      }
    /* reverse of 3: adjoint sources */
    for (int r = 0; r < nr; ++r) {
      const size_t t = (size_t)n * nr + r;
      ax[IDX(s->rec_z[r], s->rec_x[r])] += w * (rvx[t] - obs_vx[t]);
      az[IDX(s->rec_z[r], s->rec_x[r])] += w * (rvz[t] - obs_vz[t]);
    }
    /* reverse of 2 */
    for (size_t k = 0; k < N; ++k) {
      ax[k] *= s->taper[k];
      az[k] *= s->taper[k];
    }
    /* reverse of 1: buoyancy gradients (acceleration from the stored
     * velocities) and adjoint stresses */
    const double* vxp = n > 0 ? svx + (size_t)(n - 1) * N : NULL;
    const double* vzp = n > 0 ? svz + (size_t)(n - 1) * N : NULL;
    memset(t1, 0, N * sizeof(double));
    memset(t2, 0, N * sizeof(double));
    for (int j = 2; j < nz - 2; ++j)
      for (int i = 2; i < nx - 2; ++i) {
        const size_t k = IDX(j, i);
        /* velocity before the taper of step n minus the velocity after step n-1 */
        const double dvx = vxn[k] / s->taper[k] - (vxp ? vxp[k] : 0.0);
        const double dvz = vzn[k] / s->taper[k] - (vzp ? vzp[k] : 0.0);
        g_bx[k] += wk * dvx / bx[k] * ax[k];
        g_bz[k] += wk * dvz / bz[k] * az[k];
        t1[k] = dt * bx[k] * ax[k];
        t2[k] = dt * bz[k] * az[k];
      }
    for (int j = 2; j < nz - 2; ++j)
      for (int i = 2; i < nx - 2; ++i) {
        const size_t k = IDX(j, i);
        asxx[k] += -dxm(t1, nx, j, i, h);
        asxz[k] += -dzp(t1, nx, j, i, h) - dxp(t2, nx, j, i, h);
        aszz[k] += -dzm(t2, nx, j, i, h);
      }
  }
  /* (bx, bz, l2m, lam, muxz) -> (b, lambda, mu) -> (rho, vp, vs) */
  for (int j = 0; j < nz; ++j)
    for (int i = 0; i < nx; ++i) {
      const size_t k = IDX(j, i);
      double gl = g_lam[k] + g_l2m[k];
      double gm = 2.0 * g_l2m[k];
      /* the averaged parameters are only used (and only have gradients) on
       * valid cells, which never touch the grid edge */
      double gb = 0.5 * g_bx[k] + 0.5 * g_bz[k];
      if (i > 0) gb += 0.5 * g_bx[IDX(j, i - 1)];
      if (j > 0) gb += 0.5 * g_bz[IDX(j - 1, i)];
      double gmu = 0.25 * g_muxz[k];
      if (i > 0) gmu += 0.25 * g_muxz[IDX(j, i - 1)];
      if (j > 0) gmu += 0.25 * g_muxz[IDX(j - 1, i)];
      if (i > 0 && j > 0) gmu += 0.25 * g_muxz[IDX(j - 1, i - 1)];
      gm += gmu;
      const double r = rho[k], p = vp[k], v = vs[k];
      g_vp[k] += gl * 2.0 * r * p;
      g_vs[k] += gl * (-4.0 * r * v) + gm * 2.0 * r * v;
      g_rho[k] += gl * (p * p - 2.0 * v * v) + gm * v * v + gb * (-1.0 / (r * r));
    }
  free(rvx);
  free(rvz);
  free(svx);
  free(svz);
  free(buf);
  return chi;
}
