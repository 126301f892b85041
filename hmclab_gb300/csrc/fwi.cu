// 2-D elastic P-SV finite differences for many chains at once, FP32: forward
// simulation, L2 waveform misfit, exact discrete adjoint and parameter
// gradients.  Replaces the psvWave calls of the reference
// (hmclab/Distributions/ElasticFullWaveform2D.py:138-184: forward_simulate,
// calculate_l2_misfit, calculate_l2_adjoint_sources, adjoint_simulate,
// map_kernels_to_velocity), restated from Virieux (1986) / Levander (1988)
// with a Cerjan et al. (1985) sponge.
//
// Layout: every field is [nz][nx][C] (chain fastest), so each warp reads 32
// chains of one cell in one 128-byte transaction and the stencil neighbours
// of a block stay in L1/L2; one shot is simulated at a time so that the
// fields and parameters of all chains (about 86 MB at 240 x 140 x 64) stay in
// L2 for the 2 x nt half-step launches.
//
// Scheme (identical to the FP64 oracle): on the cells 2 <= i < nx-2,
// 2 <= j < nz-2 of a zero-padded grid,
//   velocity:  vx += dt bx (Dx+ sxx + Dz- sxz),  vz += dt bz (Dx- sxz + Dz+ szz),
//              then taper, record receivers, store (vx, vz) for the adjoint;
//   stress:    sxx += dt ((l+2m) Dx- vx + l Dz- vz), szz += dt (l Dx- vx + (l+2m) Dz- vz),
//              sxz += dt muxz (Dz+ vx + Dx+ vz), the sources' stress terms
//              (an explosion into sxx and szz, a moment tensor also into the
//              four sxz nodes around its cell), taper.
// The adjoint runs the transpose of these maps backwards in time
// ((Dx+)^T = -Dx-, (Dx-)^T = -Dx+, same in z), accumulating gradients with
// respect to bx, bz, l+2m, l, muxz, which are then mapped to rho, vp, vs;
// with a snapshot interval k > 1 it accumulates at every k-th step only
// (weight k) and otherwise just propagates the adjoint fields.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "common.cuh"

namespace hmc {
namespace fwi {

constexpr float C1 = 9.0f / 8.0f;
constexpr float C2 = -1.0f / 24.0f;

struct Grid {
  int nx, nz;
  int C;
  float inv_h;
  float dt;
  uint64_t wait_ns;  // limit of the tile-barrier waits (2 s in production)
  int withhold;      // test hook: block (0, 0) of the staged kernels never arms its barrier
  __device__ __forceinline__ int at(int j, int i) const { return (j * nx + i) * C; }
  __device__ __forceinline__ bool valid(int i, int j) const { return i >= 2 && i < nx - 2 && j >= 2 && j < nz - 2; }
};

// Fourth-order staggered differences of field f around flat index k with
// stride s (C along x, nx*C along z).
__device__ __forceinline__ float dxp(const float* __restrict__ f, int k, int s, float ih) {
  return (C1 * (f[k + s] - f[k]) + C2 * (f[k + 2 * s] - f[k - s])) * ih;
}
__device__ __forceinline__ float dxm(const float* __restrict__ f, int k, int s, float ih) {
  return (C1 * (f[k] - f[k - s]) + C2 * (f[k + s] - f[k - 2 * s])) * ih;
}

// Programmatic dependent launch: the stencil kernels of a time loop are
// launched with programmatic stream serialisation, so the next step's CTAs
// are scheduled while this step's last wave runs; every such kernel waits
// for its predecessor grid (completion and memory visibility) before its
// first memory access.  Without the launch attribute both are no-ops.
__device__ __forceinline__ void step_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void step_dependents_go() { asm volatile("griddepcontrol.launch_dependents;" :::); }

template <typename... KArgs, typename... Args>
cudaError_t launch_step(bool overlap, void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st,
                        Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = overlap ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Thread mapping: block (32 chains, 8 cells along x, TZ rows along z), grid.x
// over (x tiles, chain tiles), grid.y over row tiles.  No integer division
// per thread.  Blocks of 4 rows (more stencil neighbours shared in L1) and a
// 12-row march per thread with register windows both ran 7-12 % slower than
// one-row blocks at 240 x 140 cells x 64 chains.
constexpr int TX = 32, TY = 8, TZ = 1;
struct Cell {
  int i, j, c, k;
  bool in;
};
__device__ __forceinline__ Cell cell_of(const Grid& g) {
  const int ctiles = (g.C + TX - 1) / TX;
  const int it = blockIdx.x / ctiles, ct = blockIdx.x - it * ctiles;
  Cell e;
  e.c = ct * TX + threadIdx.x;
  e.i = it * TY + threadIdx.y;
  e.j = blockIdx.y * TZ + threadIdx.z;
  e.in = e.c < g.C && e.i < g.nx && e.j < g.nz;
  e.k = e.in ? g.at(e.j, e.i) + e.c : 0;
  return e;
}
inline dim3 cell_grid(int nx, int nz, int64_t C) {
  return dim3((unsigned)(((nx + TY - 1) / TY) * ((C + TX - 1) / TX)), (unsigned)((nz + TZ - 1) / TZ));
}
inline dim3 cell_block() { return dim3(TX, TY, TZ); }

// Source injection of one time step: up to MAX_SRC_TERMS stress increments
// (cell index j * nx + i, and the amounts added to sxx, szz and sxz there),
// passed by value with every stress launch, and their bounding box so that
// cells away from the sources test four integers only.  A moment-tensor point
// source at cell (i, j) adds Mxx s and Mzz s to sxx and szz of that cell and
// Mxz s / 4 to each of the four sxz nodes around it ((i -/+ 1/2, j -/+ 1/2):
// flat cells (j-1, i-1), (j-1, i), (j, i-1), (j, i)), s = stf[n] dt / h^2.
constexpr int MAX_SRC_TERMS = 32;
struct SourceStep {
  int n, i0, i1, j0, j1;
  int cell[MAX_SRC_TERMS];
  float a_xx[MAX_SRC_TERMS], a_zz[MAX_SRC_TERMS], a_xz[MAX_SRC_TERMS];
};
__device__ __forceinline__ void add_sources(const SourceStep& s, int nx, int i, int j, float& sxx, float& szz,
                                            float& sxz) {
  if (i < s.i0 || i > s.i1 || j < s.j0 || j > s.j1) return;
  const int cell = j * nx + i;
  for (int t = 0; t < s.n; ++t)
    if (s.cell[t] == cell) {
      sxx += s.a_xx[t];
      szz += s.a_zz[t];
      sxz += s.a_xz[t];
    }
}

__global__ void derive_params_kernel(Grid g, const float* __restrict__ rho, const float* __restrict__ vp,
                                     const float* __restrict__ vs, float* bx, float* bz, float* l2m, float* lam,
                                     float* muxz) {
  const Cell e = cell_of(g);
  if (!e.in) return;
  const int i1 = e.i + 1 < g.nx ? e.i + 1 : e.i, j1 = e.j + 1 < g.nz ? e.j + 1 : e.j;
  const int k = e.k, kx = g.at(e.j, i1) + e.c, kz = g.at(j1, e.i) + e.c, kxz = g.at(j1, i1) + e.c;
  const float r = rho[k], p = vp[k], s = vs[k];
  const float mu = r * s * s;
  lam[k] = r * (p * p - 2.f * s * s);
  l2m[k] = lam[k] + 2.f * mu;
  bx[k] = 0.5f * (1.f / r + 1.f / rho[kx]);
  bz[k] = 0.5f * (1.f / r + 1.f / rho[kz]);
  muxz[k] = 0.25f * (mu + rho[kx] * vs[kx] * vs[kx] + rho[kz] * vs[kz] * vs[kz] + rho[kxz] * vs[kxz] * vs[kxz]);
}

struct Fields {
  float *vx, *vz, *sxx, *szz, *sxz;
};
struct Params {
  const float *bx, *bz, *l2m, *lam, *muxz;
};

__global__ void __launch_bounds__(TX* TY* TZ) velocity_kernel(Grid g, Fields f, Params p, const float* __restrict__ taper,
                                                            const int32_t* __restrict__ rec_map, float* rec_n,
                                                            float* store_n, float* store_p) {
  step_dependency_wait();
  step_dependents_go();
  const Cell e = cell_of(g);
  if (!e.in) return;
  const int k = e.k, sx = g.C, sz = g.nx * g.C;
  float vx = f.vx[k], vz = f.vz[k];
  if (store_p) {  // a snapshot keeps the velocities of the step before too
    store_p[k] = vx;
    store_p[g.nx * g.nz * g.C + k] = vz;
  }
  if (g.valid(e.i, e.j)) {
    vx += g.dt * p.bx[k] * (dxp(f.sxx, k, sx, g.inv_h) + dxm(f.sxz, k, sz, g.inv_h));
    vz += g.dt * p.bz[k] * (dxm(f.sxz, k, sx, g.inv_h) + dxp(f.szz, k, sz, g.inv_h));
  }
  const int cell = e.j * g.nx + e.i;
  const float t = taper[cell];
  vx *= t;
  vz *= t;
  f.vx[k] = vx;
  f.vz[k] = vz;
  const int r = rec_map[cell];
  if (r >= 0) {
    rec_n[(r * 2 + 0) * g.C + e.c] = vx;
    rec_n[(r * 2 + 1) * g.C + e.c] = vz;
  }
  if (store_n) {
    store_n[k] = vx;
    store_n[g.nx * g.nz * g.C + k] = vz;
  }
}

__global__ void __launch_bounds__(TX* TY* TZ) stress_kernel(Grid g, Fields f, Params p, const float* __restrict__ taper,
                                                          const __grid_constant__ SourceStep src) {
  step_dependency_wait();
  step_dependents_go();
  const Cell e = cell_of(g);
  if (!e.in) return;
  const int k = e.k, sx = g.C, sz = g.nx * g.C;
  float sxx = f.sxx[k], szz = f.szz[k], sxz = f.sxz[k];
  if (g.valid(e.i, e.j)) {
    const float exx = dxm(f.vx, k, sx, g.inv_h), ezz = dxm(f.vz, k, sz, g.inv_h);
    sxx += g.dt * (p.l2m[k] * exx + p.lam[k] * ezz);
    szz += g.dt * (p.lam[k] * exx + p.l2m[k] * ezz);
    sxz += g.dt * p.muxz[k] * (dxp(f.vx, k, sz, g.inv_h) + dxp(f.vz, k, sx, g.inv_h));
  }
  add_sources(src, g.nx, e.i, e.j, sxx, szz, sxz);
  const float t = taper[e.j * g.nx + e.i];
  f.sxx[k] = sxx * t;
  f.szz[k] = szz * t;
  f.sxz[k] = sxz * t;
}

// ---- forward step with TMA-staged tiles --------------------------------------
// A block owns 32 chains x TT_X cells along x x TT_Z rows.  The fields it
// differentiates are copied into shared memory with their stencil halos by
// three (velocity) or two (stress) tensor-memory-accelerator loads that
// complete on one mbarrier; out-of-grid parts of a halo read as zero and are
// never used (stencils are applied on interior cells only).  The block's own
// fields and parameters are read directly.  The arithmetic is the same
// expression for expression as velocity_kernel / stress_kernel.
// Tile shape (overridable at build time): 8 x 4 measured fastest at 240 x 140
// cells x 64 chains against 8 x 2, 8 x 8, 16 x 2 and 16 x 4 (117 ms per
// 4-shot misfit against 120-128 ms).
#ifndef HMC_FWI_TILE_X
#define HMC_FWI_TILE_X 8
#endif
#ifndef HMC_FWI_TILE_Z
#define HMC_FWI_TILE_Z 4
#endif
constexpr int TT_X = HMC_FWI_TILE_X, TT_Z = HMC_FWI_TILE_Z;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool tile_barrier_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred P;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, P;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// One tile load (32 chains x cells x rows) that completes on `bar`.
__device__ __forceinline__ void tile_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::
          "r"(smem_addr(dst)),
      "l"((uint64_t)map), "r"(smem_addr(bar)), "r"(x), "r"(y), "r"(z)
      : "memory");
}

// Thread 0 arms the barrier and issues the tile loads; every thread then
// waits (at most g.wait_ns, 2 s in production).  Returns false when the wait
// expired.
__device__ __forceinline__ bool tile_wait(uint64_t* bar, uint64_t limit_ns) {
  if (tile_barrier_try(bar, 0)) return true;
  const uint64_t t0 = now_ns();
  while (!tile_barrier_try(bar, 0))
    if (now_ns() - t0 > limit_ns) return false;
  return true;
}

// Initialises the barrier and announces `bytes` of tile copies.  Returns
// false, with the barrier initialised but never armed, in block (0, 0) when
// the wait-limit test hook withholds its arrival: the caller then issues no
// copies, so nothing is in flight when the block's wait runs out.
__device__ __forceinline__ bool tile_barrier_arm(uint64_t* bar, uint32_t bytes, const Grid& g) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(1u) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  if (g.withhold && blockIdx.x == 0 && blockIdx.y == 0) return false;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
  return true;
}

struct TileOrigin {
  int c0, i0, j0;
  int tx, lane;
};
__device__ __forceinline__ TileOrigin tile_of(const Grid& g, int rows = TT_Z) {
  const int ctiles = (g.C + 31) / 32;
  const int it = blockIdx.x / ctiles, ct = blockIdx.x - it * ctiles;
  TileOrigin o;
  o.c0 = ct * 32;
  o.i0 = it * TT_X;
  o.j0 = blockIdx.y * rows;
  o.tx = threadIdx.y;
  o.lane = threadIdx.x;
  return o;
}
inline dim3 tile_grid(int nx, int nz, int64_t C, int rows = TT_Z) {
  return dim3((unsigned)(((nx + TT_X - 1) / TT_X) * ((C + 31) / 32)), (unsigned)((nz + rows - 1) / rows));
}

// staged differences: the same expressions as dxp / dxm on the tile
#define HMC_DP(a, b, c, d) ((C1 * ((a) - (b)) + C2 * ((c) - (d))) * g.inv_h)

__global__ void __launch_bounds__(32 * TT_X) velocity_tma_kernel(
    const __grid_constant__ CUtensorMap m_sxx, const __grid_constant__ CUtensorMap m_sxz,
    const __grid_constant__ CUtensorMap m_szz, Grid g, Fields f, Params p, const float* __restrict__ taper,
    const int32_t* __restrict__ rec_map, float* rec_n, float* store_n, float* store_p, int* status) {
  __shared__ __align__(128) float t_sxx[TT_Z][TT_X + 3][32];      // rows j0.., cells i0-1..
  __shared__ __align__(128) float t_sxz[TT_Z + 3][TT_X + 3][32];  // rows j0-2.., cells i0-2..
  __shared__ __align__(128) float t_szz[TT_Z + 3][TT_X][32];      // rows j0-1.., cells i0..
  __shared__ __align__(8) uint64_t bar;
  step_dependency_wait();
  step_dependents_go();
  const TileOrigin o = tile_of(g);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    if (tile_barrier_arm(&bar, (uint32_t)(sizeof(t_sxx) + sizeof(t_sxz) + sizeof(t_szz)), g)) {
      tile_load_3d(t_sxx, &m_sxx, &bar, o.c0, o.i0 - 1, o.j0);
      tile_load_3d(t_sxz, &m_sxz, &bar, o.c0, o.i0 - 2, o.j0 - 2);
      tile_load_3d(t_szz, &m_szz, &bar, o.c0, o.i0, o.j0 - 1);
    }
  }
  // the block's own cells do not depend on the tiles: their loads are in
  // flight while the tensor copies land
  const int c = o.c0 + o.lane, i = o.i0 + o.tx, tx = o.tx, l = o.lane;
  const bool active = c < g.C && i < g.nx;
  float r_vx[TT_Z], r_vz[TT_Z], r_bx[TT_Z], r_bz[TT_Z], r_tp[TT_Z];
  int r_rec[TT_Z];
#pragma unroll
  for (int zz = 0; zz < TT_Z; ++zz) {
    const int j = o.j0 + zz;
    if (active && j < g.nz) {
      const int k = g.at(j, i) + c, cell = j * g.nx + i;
      r_vx[zz] = f.vx[k];
      r_vz[zz] = f.vz[k];
      r_bx[zz] = p.bx[k];
      r_bz[zz] = p.bz[k];
      r_tp[zz] = taper[cell];
      r_rec[zz] = rec_map[cell];
    }
  }
  __syncthreads();
  if (!tile_wait(&bar, g.wait_ns)) {
    // record the failure, give the copies in flight one more bounded wait
    // so that none lands in a retired block's shared memory, and leave
    if (threadIdx.x == 0 && threadIdx.y == 0) atomicExch(status, 1);
    tile_wait(&bar, g.wait_ns);
    return;
  }
  if (!active) return;
  const bool xin = i >= 2 && i < g.nx - 2;
#pragma unroll
  for (int zz = 0; zz < TT_Z; ++zz) {
    const int j = o.j0 + zz;
    if (j >= g.nz) break;
    const int k = g.at(j, i) + c;
    float vx = r_vx[zz], vz = r_vz[zz];
    if (store_p) {  // a snapshot keeps the velocities of the step before too
      store_p[k] = vx;
      store_p[g.nx * g.nz * g.C + k] = vz;
    }
    if (xin && j >= 2 && j < g.nz - 2) {
      const float dsxx = HMC_DP(t_sxx[zz][tx + 2][l], t_sxx[zz][tx + 1][l], t_sxx[zz][tx + 3][l], t_sxx[zz][tx][l]);
      const float dsxz_z =
          HMC_DP(t_sxz[zz + 2][tx + 2][l], t_sxz[zz + 1][tx + 2][l], t_sxz[zz + 3][tx + 2][l], t_sxz[zz][tx + 2][l]);
      vx += g.dt * r_bx[zz] * (dsxx + dsxz_z);
      const float dsxz_x =
          HMC_DP(t_sxz[zz + 2][tx + 2][l], t_sxz[zz + 2][tx + 1][l], t_sxz[zz + 2][tx + 3][l], t_sxz[zz + 2][tx][l]);
      const float dszz = HMC_DP(t_szz[zz + 2][tx][l], t_szz[zz + 1][tx][l], t_szz[zz + 3][tx][l], t_szz[zz][tx][l]);
      vz += g.dt * r_bz[zz] * (dsxz_x + dszz);
    }
    const float t = r_tp[zz];
    vx *= t;
    vz *= t;
    f.vx[k] = vx;
    f.vz[k] = vz;
    const int r = r_rec[zz];
    if (r >= 0) {
      rec_n[(r * 2 + 0) * g.C + c] = vx;
      rec_n[(r * 2 + 1) * g.C + c] = vz;
    }
    if (store_n) {
      store_n[k] = vx;
      store_n[g.nx * g.nz * g.C + k] = vz;
    }
  }
}

__global__ void __launch_bounds__(32 * TT_X) stress_tma_kernel(const __grid_constant__ CUtensorMap m_vx,
                                                               const __grid_constant__ CUtensorMap m_vz, Grid g,
                                                               Fields f, Params p, const float* __restrict__ taper,
                                                               const __grid_constant__ SourceStep src,
                                                               int* status) {
  __shared__ __align__(128) float t_vx[TT_Z + 3][TT_X + 3][32];  // rows j0-1.., cells i0-2..
  __shared__ __align__(128) float t_vz[TT_Z + 3][TT_X + 3][32];  // rows j0-2.., cells i0-1..
  __shared__ __align__(8) uint64_t bar;
  step_dependency_wait();
  step_dependents_go();
  const TileOrigin o = tile_of(g);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    if (tile_barrier_arm(&bar, (uint32_t)(sizeof(t_vx) + sizeof(t_vz)), g)) {
      tile_load_3d(t_vx, &m_vx, &bar, o.c0, o.i0 - 2, o.j0 - 1);
      tile_load_3d(t_vz, &m_vz, &bar, o.c0, o.i0 - 1, o.j0 - 2);
    }
  }
  const int c = o.c0 + o.lane, i = o.i0 + o.tx, tx = o.tx, l = o.lane;
  const bool active = c < g.C && i < g.nx;
  float r_sxx[TT_Z], r_szz[TT_Z], r_sxz[TT_Z], r_l2m[TT_Z], r_lam[TT_Z], r_mu[TT_Z], r_tp[TT_Z];
#pragma unroll
  for (int zz = 0; zz < TT_Z; ++zz) {
    const int j = o.j0 + zz;
    if (active && j < g.nz) {
      const int k = g.at(j, i) + c;
      r_sxx[zz] = f.sxx[k];
      r_szz[zz] = f.szz[k];
      r_sxz[zz] = f.sxz[k];
      r_l2m[zz] = p.l2m[k];
      r_lam[zz] = p.lam[k];
      r_mu[zz] = p.muxz[k];
      r_tp[zz] = taper[j * g.nx + i];
    }
  }
  __syncthreads();
  if (!tile_wait(&bar, g.wait_ns)) {
    // record the failure, give the copies in flight one more bounded wait
    // so that none lands in a retired block's shared memory, and leave
    if (threadIdx.x == 0 && threadIdx.y == 0) atomicExch(status, 1);
    tile_wait(&bar, g.wait_ns);
    return;
  }
  if (!active) return;
  const bool xin = i >= 2 && i < g.nx - 2;
#pragma unroll
  for (int zz = 0; zz < TT_Z; ++zz) {
    const int j = o.j0 + zz;
    if (j >= g.nz) break;
    const int k = g.at(j, i) + c;
    float sxx = r_sxx[zz], szz = r_szz[zz], sxz = r_sxz[zz];
    if (xin && j >= 2 && j < g.nz - 2) {
      const float exx = HMC_DP(t_vx[zz + 1][tx + 2][l], t_vx[zz + 1][tx + 1][l], t_vx[zz + 1][tx + 3][l],
                               t_vx[zz + 1][tx][l]);
      const float ezz = HMC_DP(t_vz[zz + 2][tx + 1][l], t_vz[zz + 1][tx + 1][l], t_vz[zz + 3][tx + 1][l],
                               t_vz[zz][tx + 1][l]);
      sxx += g.dt * (r_l2m[zz] * exx + r_lam[zz] * ezz);
      szz += g.dt * (r_lam[zz] * exx + r_l2m[zz] * ezz);
      const float dvx = HMC_DP(t_vx[zz + 2][tx + 2][l], t_vx[zz + 1][tx + 2][l], t_vx[zz + 3][tx + 2][l],
                               t_vx[zz][tx + 2][l]);
      const float dvz = HMC_DP(t_vz[zz + 2][tx + 2][l], t_vz[zz + 2][tx + 1][l], t_vz[zz + 2][tx + 3][l],
                               t_vz[zz + 2][tx][l]);
      sxz += g.dt * r_mu[zz] * (dvx + dvz);
    }
    add_sources(src, g.nx, i, j, sxx, szz, sxz);
    const float t = r_tp[zz];
    f.sxx[k] = sxx * t;
    f.szz[k] = szz * t;
    f.sxz[k] = sxz * t;
  }
}
#undef HMC_DP

// ---- adjoint ---------------------------------------------------------------
struct Grads {
  float *bx, *bz, *l2m, *lam, *muxz;
};
// Inputs of the transposed difference operators, zero outside valid cells:
// t1 = dt (l2m asxx + lam aszz), t2 = dt (lam asxx + l2m aszz), t3 = dt muxz asxz
// (velocity pass), t4 = dt bx avx, t5 = dt bz avz (stress pass).
struct Temps {
  float *t1, *t2, *t3, *t4, *t5;
};

// Adjoint velocity pass of step n: reverse of stress step 4 (adjoint
// velocities and stiffness gradients), receivers 3, taper 2, and the
// buoyancy gradients of velocity step 1; writes t4, t5 for the stress pass.
// CORR: the step correlates the forward and adjoint fields into the gradient
// accumulators, each contribution weighted by w (the snapshot interval; 1
// at every step); without it the pass only propagates the adjoint fields.
template <bool CORR>
__global__ void __launch_bounds__(TX* TY* TZ) adj_velocity_kernel(Grid g, Fields a, Params p, Grads gr, Temps tm,
                                                                const float* __restrict__ taper,
                                                                const int32_t* __restrict__ rec_map,
                                                                const float* __restrict__ resid_n,
                                                                const float* __restrict__ vn,
                                                                const float* __restrict__ vprev, float w) {
  step_dependency_wait();
  step_dependents_go();
  const Cell e = cell_of(g);
  if (!e.in || !g.valid(e.i, e.j)) return;
  const int k = e.k, sx = g.C, sz = g.nx * g.C, plane = g.nx * g.nz * g.C;
  const float ih = g.inv_h;
  const int cell = e.j * g.nx + e.i;
  // every load first: the stores below may alias them as far as the
  // compiler knows, and would otherwise hold later loads back
  const float avx = a.vx[k], avz = a.vz[k];
  const float bx = p.bx[k], bz = p.bz[k];
  const float tp = taper[cell];
  const int r = rec_map[cell];
  // (Dx+)^T = -Dx-, etc.: -Dx+ t1 - Dz- t3 and -Dz+ t2 - Dx- t3
  float ax = avx - dxp(tm.t1, k, sx, ih) - dxm(tm.t3, k, sz, ih);
  float az = avz - dxp(tm.t2, k, sz, ih) - dxm(tm.t3, k, sx, ih);
  if (r >= 0) {
    ax += resid_n[(r * 2 + 0) * g.C + e.c];
    az += resid_n[(r * 2 + 1) * g.C + e.c];
  }
  ax *= tp;
  az *= tp;
  if constexpr (CORR) {
    const float* vxn = vn;
    const float* vzn = vn + plane;
    const float asxx = a.sxx[k], aszz = a.szz[k], asxz = a.sxz[k];
    const float g_l2m = gr.l2m[k], g_lam = gr.lam[k], g_mu = gr.muxz[k], g_bx = gr.bx[k], g_bz = gr.bz[k];
    const float vxk = vxn[k], vzk = vzn[k];
    const float vxp = vprev ? vprev[k] : 0.f, vzp = vprev ? vprev[plane + k] : 0.f;
    const float exx = dxm(vxn, k, sx, ih), ezz = dxm(vzn, k, sz, ih);
    const float exz = dxp(vxn, k, sz, ih) + dxp(vzn, k, sx, ih);
    const float wdt = w * g.dt;
    gr.l2m[k] = g_l2m + wdt * (exx * asxx + ezz * aszz);
    gr.lam[k] = g_lam + wdt * (ezz * asxx + exx * aszz);
    gr.muxz[k] = g_mu + wdt * exz * asxz;
    const float dvx = (vxk / tp - vxp) * w;
    const float dvz = (vzk / tp - vzp) * w;
    gr.bx[k] = g_bx + dvx / bx * ax;
    gr.bz[k] = g_bz + dvz / bz * az;
  }
  a.vx[k] = ax;
  a.vz[k] = az;
  tm.t4[k] = g.dt * bx * ax;
  tm.t5[k] = g.dt * bz * az;
}

// Adjoint stress pass of step n (reverse of velocity step 1), then the taper
// of step n-1 (reverse of its stress taper); writes t1..t3 for step n-1.
__global__ void __launch_bounds__(TX* TY* TZ) adj_stress_kernel(Grid g, Fields a, Params p, Temps tm,
                                                              const float* __restrict__ taper) {
  step_dependency_wait();
  step_dependents_go();
  const Cell e = cell_of(g);
  if (!e.in || !g.valid(e.i, e.j)) return;
  const int k = e.k, sx = g.C, sz = g.nx * g.C;
  const float ih = g.inv_h;
  const float tp = taper[e.j * g.nx + e.i];
  const float l2m = p.l2m[k], lam = p.lam[k], mu = p.muxz[k];
  const float asxx = (a.sxx[k] - dxm(tm.t4, k, sx, ih)) * tp;
  const float asxz = (a.sxz[k] - dxp(tm.t4, k, sz, ih) - dxp(tm.t5, k, sx, ih)) * tp;
  const float aszz = (a.szz[k] - dxm(tm.t5, k, sz, ih)) * tp;
  a.sxx[k] = asxx;
  a.sxz[k] = asxz;
  a.szz[k] = aszz;
  tm.t1[k] = g.dt * (l2m * asxx + lam * aszz);
  tm.t2[k] = g.dt * (lam * asxx + l2m * aszz);
  tm.t3[k] = g.dt * mu * asxz;
}

// ---- adjoint passes with TMA-staged tiles ----------------------------------
// Same tiling, barrier and bounded wait as the forward pair, R rows per
// thread, every own-cell operand loaded before the wait; the arithmetic is
// the same expression for expression as adj_velocity_kernel /
// adj_stress_kernel.  The stored forward velocities of step n come through
// one map over all stored planes ([2 nt x nz] rows of nx cells): halo rows
// that fall into a neighbouring plane are never used, because only interior
// cells are updated.
// Rows per thread (overridable at build time): velocity 1 / stress 4 measured
// fastest at 240 x 140 cells x 64 chains (gradient 454 ms against 455-470 ms
// for 2 / 4, 2 / 2 and 4 / 4, and 535 ms with direct loads); it is also the
// variant whose results are bitwise equal to the direct-load kernels.
#ifndef HMC_FWI_ADJ_ROWS_V
#define HMC_FWI_ADJ_ROWS_V 1
#endif
#ifndef HMC_FWI_ADJ_ROWS_S
#define HMC_FWI_ADJ_ROWS_S 4
#endif
constexpr int AR_V = HMC_FWI_ADJ_ROWS_V, AR_S = HMC_FWI_ADJ_ROWS_S;
#define HMC_DP(a, b, c, d) ((C1 * ((a) - (b)) + C2 * ((c) - (d))) * g.inv_h)

template <int R, bool CORR>
__global__ void __launch_bounds__(32 * TT_X) adj_velocity_tma_kernel(
    const __grid_constant__ CUtensorMap m_t1, const __grid_constant__ CUtensorMap m_t2,
    const __grid_constant__ CUtensorMap m_t3, const __grid_constant__ CUtensorMap m_store, int row_vx, int row_vz,
    Grid g, Fields a, Params p, Grads gr, Temps tm, const float* __restrict__ taper,
    const int32_t* __restrict__ rec_map, const float* __restrict__ resid_n, const float* __restrict__ vprev, float w,
    int* status) {
  // the stored forward velocities are staged only when the step correlates
  constexpr int SR = CORR ? R + 3 : 1;
  __shared__ __align__(128) float t_t1[R][TT_X + 3][32];      // rows j0.., cells i0-1..
  __shared__ __align__(128) float t_t3[R + 3][TT_X + 3][32];  // rows j0-2.., cells i0-2..
  __shared__ __align__(128) float t_t2[R + 3][TT_X][32];      // rows j0-1.., cells i0..
  __shared__ __align__(128) float t_vx[SR][TT_X + 3][32];     // rows j0-1.., cells i0-2..
  __shared__ __align__(128) float t_vz[SR][TT_X + 3][32];     // rows j0-2.., cells i0-1..
  __shared__ __align__(8) uint64_t bar;
  step_dependency_wait();
  step_dependents_go();
  const TileOrigin o = tile_of(g, R);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    const uint32_t bytes =
        (uint32_t)(sizeof(t_t1) + sizeof(t_t3) + sizeof(t_t2) + (CORR ? sizeof(t_vx) + sizeof(t_vz) : 0));
    if (tile_barrier_arm(&bar, bytes, g)) {
      tile_load_3d(t_t1, &m_t1, &bar, o.c0, o.i0 - 1, o.j0);
      tile_load_3d(t_t3, &m_t3, &bar, o.c0, o.i0 - 2, o.j0 - 2);
      tile_load_3d(t_t2, &m_t2, &bar, o.c0, o.i0, o.j0 - 1);
      if constexpr (CORR) {
        tile_load_3d(t_vx, &m_store, &bar, o.c0, o.i0 - 2, row_vx + o.j0 - 1);
        tile_load_3d(t_vz, &m_store, &bar, o.c0, o.i0 - 1, row_vz + o.j0 - 2);
      }
    }
  }
  const int c = o.c0 + o.lane, i = o.i0 + o.tx, tx = o.tx, l = o.lane;
  const bool active = c < g.C && i >= 2 && i < g.nx - 2;
  const int plane = g.nx * g.nz * g.C;
  float r_avx[R], r_avz[R], r_sxx[R], r_szz[R], r_sxz[R], r_gl2m[R], r_glam[R], r_gmu[R], r_gbx[R], r_gbz[R];
  float r_bx[R], r_bz[R], r_tp[R], r_vxp[R], r_vzp[R];
  int r_rec[R];
#pragma unroll
  for (int zz = 0; zz < R; ++zz) {
    const int j = o.j0 + zz;
    if (active && j >= 2 && j < g.nz - 2) {
      const int k = g.at(j, i) + c, cell = j * g.nx + i;
      r_avx[zz] = a.vx[k];
      r_avz[zz] = a.vz[k];
      r_bx[zz] = p.bx[k];
      r_bz[zz] = p.bz[k];
      r_tp[zz] = taper[cell];
      r_rec[zz] = rec_map[cell];
      if constexpr (CORR) {
        r_sxx[zz] = a.sxx[k];
        r_szz[zz] = a.szz[k];
        r_sxz[zz] = a.sxz[k];
        r_gl2m[zz] = gr.l2m[k];
        r_glam[zz] = gr.lam[k];
        r_gmu[zz] = gr.muxz[k];
        r_gbx[zz] = gr.bx[k];
        r_gbz[zz] = gr.bz[k];
        r_vxp[zz] = vprev ? vprev[k] : 0.f;
        r_vzp[zz] = vprev ? vprev[plane + k] : 0.f;
      }
    }
  }
  __syncthreads();
  if (!tile_wait(&bar, g.wait_ns)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) atomicExch(status, 1);
    tile_wait(&bar, g.wait_ns);
    return;
  }
  if (!active) return;
#pragma unroll
  for (int zz = 0; zz < R; ++zz) {
    const int j = o.j0 + zz;
    if (j < 2 || j >= g.nz - 2) continue;
    const int k = g.at(j, i) + c;
    float ax = r_avx[zz] -
               HMC_DP(t_t1[zz][tx + 2][l], t_t1[zz][tx + 1][l], t_t1[zz][tx + 3][l], t_t1[zz][tx][l]) -
               HMC_DP(t_t3[zz + 2][tx + 2][l], t_t3[zz + 1][tx + 2][l], t_t3[zz + 3][tx + 2][l], t_t3[zz][tx + 2][l]);
    float az = r_avz[zz] -
               HMC_DP(t_t2[zz + 2][tx][l], t_t2[zz + 1][tx][l], t_t2[zz + 3][tx][l], t_t2[zz][tx][l]) -
               HMC_DP(t_t3[zz + 2][tx + 2][l], t_t3[zz + 2][tx + 1][l], t_t3[zz + 2][tx + 3][l], t_t3[zz + 2][tx][l]);
    const int r = r_rec[zz];
    if (r >= 0) {
      ax += resid_n[(r * 2 + 0) * g.C + c];
      az += resid_n[(r * 2 + 1) * g.C + c];
    }
    const float tp = r_tp[zz];
    ax *= tp;
    az *= tp;
    const float bx = r_bx[zz], bz = r_bz[zz];
    if constexpr (CORR) {
      const float exx = HMC_DP(t_vx[zz + 1][tx + 2][l], t_vx[zz + 1][tx + 1][l], t_vx[zz + 1][tx + 3][l],
                               t_vx[zz + 1][tx][l]);
      const float ezz = HMC_DP(t_vz[zz + 2][tx + 1][l], t_vz[zz + 1][tx + 1][l], t_vz[zz + 3][tx + 1][l],
                               t_vz[zz][tx + 1][l]);
      const float exz = HMC_DP(t_vx[zz + 2][tx + 2][l], t_vx[zz + 1][tx + 2][l], t_vx[zz + 3][tx + 2][l],
                               t_vx[zz][tx + 2][l]) +
                        HMC_DP(t_vz[zz + 2][tx + 2][l], t_vz[zz + 2][tx + 1][l], t_vz[zz + 2][tx + 3][l],
                               t_vz[zz + 2][tx][l]);
      const float asxx = r_sxx[zz], aszz = r_szz[zz], asxz = r_sxz[zz];
      const float wdt = w * g.dt;
      gr.l2m[k] = r_gl2m[zz] + wdt * (exx * asxx + ezz * aszz);
      gr.lam[k] = r_glam[zz] + wdt * (ezz * asxx + exx * aszz);
      gr.muxz[k] = r_gmu[zz] + wdt * exz * asxz;
      const float dvx = (t_vx[zz + 1][tx + 2][l] / tp - r_vxp[zz]) * w;
      const float dvz = (t_vz[zz + 2][tx + 1][l] / tp - r_vzp[zz]) * w;
      gr.bx[k] = r_gbx[zz] + dvx / bx * ax;
      gr.bz[k] = r_gbz[zz] + dvz / bz * az;
    }
    a.vx[k] = ax;
    a.vz[k] = az;
    tm.t4[k] = g.dt * bx * ax;
    tm.t5[k] = g.dt * bz * az;
  }
}

template <int R>
__global__ void __launch_bounds__(32 * TT_X) adj_stress_tma_kernel(const __grid_constant__ CUtensorMap m_t4,
                                                                   const __grid_constant__ CUtensorMap m_t5, Grid g,
                                                                   Fields a, Params p, Temps tm,
                                                                   const float* __restrict__ taper, int* status) {
  __shared__ __align__(128) float t_t4[R + 3][TT_X + 3][32];  // rows j0-1.., cells i0-2..
  __shared__ __align__(128) float t_t5[R + 3][TT_X + 3][32];  // rows j0-2.., cells i0-1..
  __shared__ __align__(8) uint64_t bar;
  step_dependency_wait();
  step_dependents_go();
  const TileOrigin o = tile_of(g, R);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    if (tile_barrier_arm(&bar, (uint32_t)(sizeof(t_t4) + sizeof(t_t5)), g)) {
      tile_load_3d(t_t4, &m_t4, &bar, o.c0, o.i0 - 2, o.j0 - 1);
      tile_load_3d(t_t5, &m_t5, &bar, o.c0, o.i0 - 1, o.j0 - 2);
    }
  }
  const int c = o.c0 + o.lane, i = o.i0 + o.tx, tx = o.tx, l = o.lane;
  const bool active = c < g.C && i >= 2 && i < g.nx - 2;
  float r_sxx[R], r_sxz[R], r_szz[R], r_l2m[R], r_lam[R], r_mu[R], r_tp[R];
#pragma unroll
  for (int zz = 0; zz < R; ++zz) {
    const int j = o.j0 + zz;
    if (active && j >= 2 && j < g.nz - 2) {
      const int k = g.at(j, i) + c;
      r_sxx[zz] = a.sxx[k];
      r_sxz[zz] = a.sxz[k];
      r_szz[zz] = a.szz[k];
      r_l2m[zz] = p.l2m[k];
      r_lam[zz] = p.lam[k];
      r_mu[zz] = p.muxz[k];
      r_tp[zz] = taper[j * g.nx + i];
    }
  }
  __syncthreads();
  if (!tile_wait(&bar, g.wait_ns)) {
    if (threadIdx.x == 0 && threadIdx.y == 0) atomicExch(status, 1);
    tile_wait(&bar, g.wait_ns);
    return;
  }
  if (!active) return;
#pragma unroll
  for (int zz = 0; zz < R; ++zz) {
    const int j = o.j0 + zz;
    if (j < 2 || j >= g.nz - 2) continue;
    const int k = g.at(j, i) + c;
    const float tp = r_tp[zz];
    const float asxx =
        (r_sxx[zz] - HMC_DP(t_t4[zz + 1][tx + 2][l], t_t4[zz + 1][tx + 1][l], t_t4[zz + 1][tx + 3][l],
                            t_t4[zz + 1][tx][l])) *
        tp;
    const float asxz =
        (r_sxz[zz] -
         HMC_DP(t_t4[zz + 2][tx + 2][l], t_t4[zz + 1][tx + 2][l], t_t4[zz + 3][tx + 2][l], t_t4[zz][tx + 2][l]) -
         HMC_DP(t_t5[zz + 2][tx + 2][l], t_t5[zz + 2][tx + 1][l], t_t5[zz + 2][tx + 3][l], t_t5[zz + 2][tx][l])) *
        tp;
    const float aszz =
        (r_szz[zz] -
         HMC_DP(t_t5[zz + 2][tx + 1][l], t_t5[zz + 1][tx + 1][l], t_t5[zz + 3][tx + 1][l], t_t5[zz][tx + 1][l])) *
        tp;
    a.sxx[k] = asxx;
    a.sxz[k] = asxz;
    a.szz[k] = aszz;
    tm.t1[k] = g.dt * (r_l2m[zz] * asxx + r_lam[zz] * aszz);
    tm.t2[k] = g.dt * (r_lam[zz] * asxx + r_l2m[zz] * aszz);
    tm.t3[k] = g.dt * r_mu[zz] * asxz;
  }
}
#undef HMC_DP

// Weighted residuals w (rec - obs) of one shot, all steps: [nt][nrec][2][C];
// obs is shared by all chains: [nt][nrec][2].
__global__ void residual_kernel(int64_t n_rows, int64_t C, const float* __restrict__ rec,
                                const float* __restrict__ obs, float w, float* resid) {
  const int64_t total = n_rows * C;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
    resid[t] = w * (rec[t] - obs[t / C]);
}

// Misfit in two deterministic passes: blockIdx.y takes one of MISFIT_SPLITS
// contiguous row ranges and writes its sum per chain to partial[y][c]; the
// second kernel adds the ranges in order.
constexpr int MISFIT_SPLITS = 64;
__global__ void misfit_partial_kernel(int64_t n_rows, int64_t C, const float* __restrict__ rec,
                                      const float* __restrict__ obs, double* partial) {
  __shared__ double sh[RED_Y][RED_X + 1];
  const int64_t c = blockIdx.x * (int64_t)RED_X + threadIdx.x;
  const int64_t per = (n_rows + MISFIT_SPLITS - 1) / MISFIT_SPLITS;
  const int64_t r0 = (int64_t)blockIdx.y * per, r1 = r0 + per < n_rows ? r0 + per : n_rows;
  double acc = 0.0;
  if (c < C) {
    for (int64_t r = r0 + threadIdx.y; r < r1; r += RED_Y) {
      const double d = (double)rec[r * C + c] - (double)obs[r];
      acc += d * d;
    }
  }
  const double s = block_chain_sum(acc, sh);
  if (c < C && threadIdx.y == 0) partial[blockIdx.y * C + c] = s;
}

__global__ void misfit_final_kernel(int64_t C, const double* __restrict__ partial, double w, double* out,
                                    int accumulate) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= C) return;
  double s = 0.0;
  for (int y = 0; y < MISFIT_SPLITS; ++y) s += partial[y * C + c];
  const double v = 0.5 * w * s;
  out[c] = accumulate ? out[c] + v : v;
}

// Cell parametrisation.  Model: out[cell][c] = base[cell] + M[map[cell]][c]
// (map -1: base only), one thread per (cell, chain), chains fastest.
__global__ void cell_model_kernel(int64_t cells, int64_t C, const int32_t* __restrict__ map,
                                  const float* __restrict__ M, const float* __restrict__ base, float* __restrict__ out) {
  const int64_t n = cells * C;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = t / C, c = t - cell * C;
    const int32_t p = map[cell];
    out[t] = base[cell] + (p >= 0 ? M[(int64_t)p * C + c] : 0.f);
  }
}
// Gradient: out[p][c] (+)= sum over the cells ptr[p] <= k < ptr[p+1] of
// g[cells[k]][c], in segment order; one thread per (parameter, chain).
__global__ void cell_gradient_kernel(int64_t P, int64_t C, const int32_t* __restrict__ ptr,
                                     const int32_t* __restrict__ cells, const float* __restrict__ g,
                                     float* __restrict__ out, int accumulate) {
  const int64_t n = P * C;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = t / C, c = t - p * C;
    float acc = 0.f;
    for (int32_t k = ptr[p]; k < ptr[p + 1]; ++k) acc += g[(int64_t)cells[k] * C + c];
    out[t] = accumulate ? out[t] + acc : acc;
  }
}

// (bx, bz, l+2m, l, muxz) gradients -> (rho, vp, vs) gradients, all cells.
__global__ void param_gradient_kernel(Grid g, Grads gr, const float* __restrict__ rho, const float* __restrict__ vp,
                                      const float* __restrict__ vs, float* g_rho, float* g_vp, float* g_vs,
                                      int accumulate) {
  const Cell e = cell_of(g);
  if (!e.in) return;
  const int k = e.k, i = e.i, j = e.j, c = e.c;
  float gl = gr.lam[k] + gr.l2m[k];
  float gm = 2.f * gr.l2m[k];
  float gb = 0.5f * gr.bx[k] + 0.5f * gr.bz[k];
  if (i > 0) gb += 0.5f * gr.bx[g.at(j, i - 1) + c];
  if (j > 0) gb += 0.5f * gr.bz[g.at(j - 1, i) + c];
  float gmu = 0.25f * gr.muxz[k];
  if (i > 0) gmu += 0.25f * gr.muxz[g.at(j, i - 1) + c];
  if (j > 0) gmu += 0.25f * gr.muxz[g.at(j - 1, i) + c];
  if (i > 0 && j > 0) gmu += 0.25f * gr.muxz[g.at(j - 1, i - 1) + c];
  gm += gmu;
  const float r = rho[k], pv = vp[k], s = vs[k];
  const float vgp = gl * 2.f * r * pv;
  const float vgs = gl * (-4.f * r * s) + gm * 2.f * r * s;
  const float vgr = gl * (pv * pv - 2.f * s * s) + gm * s * s - gb / (r * r);
  if (accumulate) {
    g_vp[k] += vgp;
    g_vs[k] += vgs;
    g_rho[k] += vgr;
  } else {
    g_vp[k] = vgp;
    g_vs[k] = vgs;
    g_rho[k] = vgr;
  }
}

inline unsigned grid_for(int64_t n) {
  const unsigned b = blocks_for(n, 256);
  return b > 152u * 64u ? 152u * 64u : b;
}

PFN_cuTensorMapEncodeTiled_v12000 tile_encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  });
  return fn;
}

// 3-D FP32 map of a [nz][nx][C] field with a box of 32 chains x bx cells x bz
// rows; out-of-grid elements of a box read as zero.
int field_map(CUtensorMap* m, const float* base, int nx, int nz, int64_t C, int bx, int bz) {
  auto fn = tile_encode_fn();
  if (!fn) return fail(HMC_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
  cuuint64_t dims[3] = {(cuuint64_t)C, (cuuint64_t)nx, (cuuint64_t)nz};
  cuuint64_t strides[2] = {(cuuint64_t)C * 4, (cuuint64_t)nx * C * 4};
  cuuint32_t box[3] = {32u, (cuuint32_t)bx, (cuuint32_t)bz};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(HMC_ERR_INVALID_ARG, "cuTensorMapEncodeTiled(field) failed (%d)", (int)r);
  return HMC_OK;
}

}  // namespace fwi
}  // namespace hmc

using namespace hmc;
using namespace hmc::fwi;

static int check_fwi(const hmc_fwi* s, const char* who) {
  HMC_REQUIRE(s != nullptr, "%s: null descriptor", who);
  HMC_REQUIRE(s->nx >= 5 && s->nz >= 5 && s->nt > 0 && s->chains > 0 && s->nrec > 0, "%s: bad sizes", who);
  HMC_REQUIRE(s->taper && s->stf_host && s->rec_map && s->rho && s->vp && s->vs, "%s: missing model buffer", who);
  HMC_REQUIRE(s->bx && s->bz && s->l2m && s->lam && s->muxz, "%s: missing parameter work buffer", who);
  HMC_REQUIRE(s->vx && s->vz && s->sxx && s->szz && s->sxz && s->rec, "%s: missing wavefield buffer", who);
  HMC_REQUIRE((int64_t)s->nx * s->nz * s->chains * 2 < (1ll << 31), "%s: grid x chains too large for 32-bit indexing",
              who);
  return HMC_OK;
}

static Grid grid_of(const hmc_fwi* s) {
  Grid g;
  g.nx = s->nx;
  g.nz = s->nz;
  g.C = (int)s->chains;
  g.inv_h = 1.f / s->h;
  g.dt = s->dt;
  const WaitLimits wl = wait_limits();
  g.wait_ns = wl.ns;
  g.withhold = wl.withhold;
  return g;
}

// Where the forward pass stores step n's velocities for the adjoint: every
// step ([nt][2] planes) at snapshot interval 1; else only at the snapshot
// steps n = 0, k, 2k, ..., which keep the velocities after step n - 1 too
// ([ceil(nt / k)][4] planes).
struct StoreSlot {
  float* now;   // vx, vz after step n (nullptr: not stored)
  float* prev;  // vx, vz after step n - 1 (nullptr: the plane before `now`)
  int64_t row;  // first row of `now` in the [planes x nz] view of the store
};
static int snapshot_interval(const hmc_fwi* s) { return s->snapshot_interval > 1 ? s->snapshot_interval : 1; }
static int64_t stored_planes(const hmc_fwi* s) {
  const int k = snapshot_interval(s);
  return k == 1 ? 2ll * s->nt : 4ll * ((s->nt + k - 1) / k);
}
static StoreSlot store_slot(const hmc_fwi* s, int n) {
  const int64_t cells = (int64_t)s->nx * s->nz * s->chains;
  const int k = snapshot_interval(s);
  if (k == 1) return {s->store + (int64_t)n * 2 * cells, nullptr, 2ll * n * s->nz};
  if (n % k != 0) return {nullptr, nullptr, 0};
  float* base = s->store + (int64_t)(n / k) * 4 * cells;
  return {base, base + 2 * cells, 4ll * (n / k) * s->nz};
}

extern "C" {

HMC_API int hmc_fwi_prepare(const hmc_fwi* s, void* stream) {
  HMC_TRY(check_fwi(s, "hmc_fwi_prepare"));
  const Grid g = grid_of(s);
  derive_params_kernel<<<cell_grid(s->nx, s->nz, s->chains), cell_block(), 0, as_stream(stream)>>>(
      g, s->rho, s->vp, s->vs, s->bx, s->bz, s->l2m, s->lam, s->muxz);
  return check_launch("derive_params_kernel");
}

HMC_API int hmc_fwi_forward_shot(const hmc_fwi* s, int shot, int src_x, int src_z, int store, void* stream) {
  HMC_REQUIRE(s != nullptr, "hmc_fwi_forward_shot: null descriptor");
  const hmc_fwi_source explosive{src_x, src_z, 1.f, 1.f, 0.f, s->stf_host};
  return hmc_fwi_forward_shot_sources(s, shot, &explosive, 1, store, stream);
}

HMC_API int hmc_fwi_forward_shot_sources(const hmc_fwi* s, int shot, const hmc_fwi_source* src, int n_src,
                                         int store, void* stream) {
  HMC_TRY(check_fwi(s, "hmc_fwi_forward_shot_sources"));
  HMC_REQUIRE(src != nullptr && n_src >= 1, "hmc_fwi_forward_shot_sources: no source");
  int n_terms = 0;
  for (int q = 0; q < n_src; ++q) {
    HMC_REQUIRE(src[q].x >= 1 && src[q].x < s->nx && src[q].z >= 1 && src[q].z < s->nz,
                "hmc_fwi_forward_shot_sources: source %d off the grid's interior", q);
    HMC_REQUIRE(src[q].stf_host != nullptr, "hmc_fwi_forward_shot_sources: source %d has no wavelet", q);
    n_terms += src[q].mxz != 0.f ? 4 : 1;
  }
  HMC_REQUIRE(n_terms <= MAX_SRC_TERMS,
              "hmc_fwi_forward_shot_sources: %d stress terms (a moment tensor with Mxz takes 4), at most %d", n_terms,
              MAX_SRC_TERMS);
  HMC_REQUIRE(!store || s->store, "hmc_fwi_forward_shot_sources: storing needs the store buffer");
  // the stress increments of step n; the wavelets are read on the host (a
  // handful of floats per step)
  const float src_scale = s->dt / (s->h * s->h);
  auto source_step = [&](int n) {
    SourceStep ss{};
    ss.i0 = s->nx;
    ss.j0 = s->nz;
    ss.i1 = ss.j1 = -1;
    auto term = [&](int i, int j, float axx, float azz, float axz) {
      ss.cell[ss.n] = j * s->nx + i;
      ss.a_xx[ss.n] = axx;
      ss.a_zz[ss.n] = azz;
      ss.a_xz[ss.n] = axz;
      ++ss.n;
      ss.i0 = i < ss.i0 ? i : ss.i0;
      ss.i1 = i > ss.i1 ? i : ss.i1;
      ss.j0 = j < ss.j0 ? j : ss.j0;
      ss.j1 = j > ss.j1 ? j : ss.j1;
    };
    for (int q = 0; q < n_src; ++q) {
      const float v = src[q].stf_host[n] * src_scale;
      const int i = src[q].x, j = src[q].z;
      const float xz = 0.25f * src[q].mxz * v;
      term(i, j, src[q].mxx * v, src[q].mzz * v, xz);
      if (src[q].mxz != 0.f) {
        term(i - 1, j - 1, 0.f, 0.f, xz);
        term(i, j - 1, 0.f, 0.f, xz);
        term(i - 1, j, 0.f, 0.f, xz);
      }
    }
    return ss;
  };
  cudaStream_t st = as_stream(stream);
  const Grid g = grid_of(s);
  const int64_t cells = (int64_t)s->nx * s->nz * s->chains;
  const size_t fb = (size_t)cells * sizeof(float);
  // zero the wavefields
  for (float* f : {s->vx, s->vz, s->sxx, s->szz, s->sxz}) {
    cudaError_t e = cudaMemsetAsync(f, 0, fb, st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(fwi fields)");
  }
  Fields f{s->vx, s->vz, s->sxx, s->szz, s->sxz};
  Params p{s->bx, s->bz, s->l2m, s->lam, s->muxz};
  const dim3 grid = cell_grid(s->nx, s->nz, s->chains), block = cell_block();
  float* rec_shot = s->rec + (int64_t)shot * s->nt * s->nrec * 2 * s->chains;
  // tiles staged by the tensor memory accelerator: whole 32-chain tiles and
  // 16-byte row pitches (C a multiple of 32), and a status word for the
  // bounded barrier wait
  if (s->chains % 32 == 0 && s->status) {
    CUtensorMap m_sxx, m_sxz, m_szz, m_vx, m_vz;
    HMC_TRY(field_map(&m_sxx, s->sxx, s->nx, s->nz, s->chains, TT_X + 3, TT_Z));
    HMC_TRY(field_map(&m_sxz, s->sxz, s->nx, s->nz, s->chains, TT_X + 3, TT_Z + 3));
    HMC_TRY(field_map(&m_szz, s->szz, s->nx, s->nz, s->chains, TT_X, TT_Z + 3));
    HMC_TRY(field_map(&m_vx, s->vx, s->nx, s->nz, s->chains, TT_X + 3, TT_Z + 3));
    HMC_TRY(field_map(&m_vz, s->vz, s->nx, s->nz, s->chains, TT_X + 3, TT_Z + 3));
    const dim3 tgrid = tile_grid(s->nx, s->nz, s->chains), tblock(32, TT_X);
    for (int n = 0; n < s->nt; ++n) {
      float* rec_n = rec_shot + (int64_t)n * s->nrec * 2 * s->chains;
      const StoreSlot slot = store ? store_slot(s, n) : StoreSlot{nullptr, nullptr, 0};
      cudaError_t e = launch_step(n > 0, velocity_tma_kernel, tgrid, tblock, st, m_sxx, m_sxz, m_szz, g, f, p,
                                  s->taper, s->rec_map, rec_n, slot.now, slot.prev, s->status);
      if (e != cudaSuccess) return cuda_fail(e, "launch velocity_tma_kernel");
      HMC_TRY(check_launch("velocity_tma_kernel"));
      e = launch_step(true, stress_tma_kernel, tgrid, tblock, st, m_vx, m_vz, g, f, p, s->taper, source_step(n),
                      s->status);
      if (e != cudaSuccess) return cuda_fail(e, "launch stress_tma_kernel");
      HMC_TRY(check_launch("stress_tma_kernel"));
    }
    return HMC_OK;
  }
  for (int n = 0; n < s->nt; ++n) {
    float* rec_n = rec_shot + (int64_t)n * s->nrec * 2 * s->chains;
    const StoreSlot slot = store ? store_slot(s, n) : StoreSlot{nullptr, nullptr, 0};
    // the first launch follows the memsets: ordinary stream order
    cudaError_t e = launch_step(n > 0, velocity_kernel, grid, block, st, g, f, p, s->taper, s->rec_map, rec_n,
                                slot.now, slot.prev);
    if (e != cudaSuccess) return cuda_fail(e, "launch velocity_kernel");
    HMC_TRY(check_launch("velocity_kernel"));
    e = launch_step(true, stress_kernel, grid, block, st, g, f, p, s->taper, source_step(n));
    if (e != cudaSuccess) return cuda_fail(e, "launch stress_kernel");
    HMC_TRY(check_launch("stress_kernel"));
  }
  return HMC_OK;
}

HMC_API int hmc_fwi_misfit(const hmc_fwi* s, int nshots, double* out_x, int accumulate, void* stream) {
  HMC_TRY(check_fwi(s, "hmc_fwi_misfit"));
  HMC_REQUIRE(s->obs && out_x && s->partial, "hmc_fwi_misfit: missing observations, output or partial buffer");
  const int64_t rows = (int64_t)nshots * s->nt * s->nrec * 2;
  cudaStream_t st = as_stream(stream);
  const dim3 grid(red_grid(s->chains).x, MISFIT_SPLITS);
  misfit_partial_kernel<<<grid, red_block(), 0, st>>>(rows, s->chains, s->rec, s->obs, s->partial);
  HMC_TRY(check_launch("fwi misfit_partial_kernel"));
  misfit_final_kernel<<<blocks_for(s->chains, 128), 128, 0, st>>>(s->chains, s->partial, (double)s->w, out_x,
                                                                   accumulate);
  return check_launch("fwi misfit_final_kernel");
}

HMC_API int hmc_fwi_adjoint_shot(const hmc_fwi* s, int shot, void* stream) {
  HMC_TRY(check_fwi(s, "hmc_fwi_adjoint_shot"));
  HMC_REQUIRE(s->store && s->obs && s->resid && s->avx && s->avz && s->asxx && s->aszz && s->asxz,
              "hmc_fwi_adjoint_shot: missing adjoint buffer");
  HMC_REQUIRE(s->g_bx && s->g_bz && s->g_l2m && s->g_lam && s->g_muxz, "hmc_fwi_adjoint_shot: missing gradients");
  HMC_REQUIRE(s->t1 && s->t2 && s->t3 && s->t4 && s->t5, "hmc_fwi_adjoint_shot: missing adjoint temporaries");
  cudaStream_t st = as_stream(stream);
  const Grid g = grid_of(s);
  const int64_t cells = (int64_t)s->nx * s->nz * s->chains;
  const size_t fb = (size_t)cells * sizeof(float);
  for (float* f : {s->avx, s->avz, s->asxx, s->aszz, s->asxz, s->t1, s->t2, s->t3, s->t4, s->t5}) {
    cudaError_t e = cudaMemsetAsync(f, 0, fb, st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(fwi adjoint)");
  }
  const int64_t rows = (int64_t)s->nt * s->nrec * 2;
  const int64_t shot_off = (int64_t)shot * rows;
  residual_kernel<<<grid_for(rows * s->chains), 256, 0, st>>>(rows, s->chains, s->rec + shot_off * s->chains,
                                                              s->obs + shot_off, s->w, s->resid);
  HMC_TRY(check_launch("residual_kernel"));
  Fields a{s->avx, s->avz, s->asxx, s->aszz, s->asxz};
  Params p{s->bx, s->bz, s->l2m, s->lam, s->muxz};
  Grads gr{s->g_bx, s->g_bz, s->g_l2m, s->g_lam, s->g_muxz};
  Temps tm{s->t1, s->t2, s->t3, s->t4, s->t5};
  // staged tiles, as in the forward pass (C a multiple of 32, a status word)
  const int k = snapshot_interval(s);
  const float w = (float)k;  // weight of a correlating step
  // the velocities after step n - 1 (nullptr before the first step)
  auto prev_of = [&](int n, const StoreSlot& slot) -> const float* {
    if (slot.prev) return slot.prev;
    return n > 0 ? s->store + (int64_t)(n - 1) * 2 * cells : nullptr;
  };
  if (s->chains % 32 == 0 && s->status) {
    HMC_REQUIRE(stored_planes(s) * s->nz < INT32_MAX, "hmc_fwi_adjoint_shot: too many stored rows");
    CUtensorMap m_t1, m_t2, m_t3, m_t4, m_t5, m_store;
    HMC_TRY(field_map(&m_t1, s->t1, s->nx, s->nz, s->chains, TT_X + 3, AR_V));
    HMC_TRY(field_map(&m_t2, s->t2, s->nx, s->nz, s->chains, TT_X, AR_V + 3));
    HMC_TRY(field_map(&m_t3, s->t3, s->nx, s->nz, s->chains, TT_X + 3, AR_V + 3));
    HMC_TRY(field_map(&m_store, s->store, s->nx, (int)(stored_planes(s) * s->nz), s->chains, TT_X + 3, AR_V + 3));
    HMC_TRY(field_map(&m_t4, s->t4, s->nx, s->nz, s->chains, TT_X + 3, AR_S + 3));
    HMC_TRY(field_map(&m_t5, s->t5, s->nx, s->nz, s->chains, TT_X + 3, AR_S + 3));
    const dim3 gv = tile_grid(s->nx, s->nz, s->chains, AR_V), gs = tile_grid(s->nx, s->nz, s->chains, AR_S);
    const dim3 tblock(32, TT_X);
    for (int n = s->nt - 1; n >= 0; --n) {
      const StoreSlot slot = store_slot(s, n);
      const float* resid_n = s->resid + (int64_t)n * s->nrec * 2 * s->chains;
      // the first launch follows the residual kernel and memsets: ordinary stream order
      cudaError_t e;
      if (slot.now)
        e = launch_step(n < s->nt - 1, adj_velocity_tma_kernel<AR_V, true>, gv, tblock, st, m_t1, m_t2, m_t3,
                        m_store, (int)slot.row, (int)(slot.row + s->nz), g, a, p, gr, tm, s->taper, s->rec_map,
                        resid_n, prev_of(n, slot), w, s->status);
      else
        e = launch_step(n < s->nt - 1, adj_velocity_tma_kernel<AR_V, false>, gv, tblock, st, m_t1, m_t2, m_t3,
                        m_store, 0, 0, g, a, p, gr, tm, s->taper, s->rec_map, resid_n, (const float*)nullptr, w,
                        s->status);
      if (e != cudaSuccess) return cuda_fail(e, "launch adj_velocity_tma_kernel");
      HMC_TRY(check_launch("adj_velocity_tma_kernel"));
      e = launch_step(true, adj_stress_tma_kernel<AR_S>, gs, tblock, st, m_t4, m_t5, g, a, p, tm, s->taper,
                      s->status);
      if (e != cudaSuccess) return cuda_fail(e, "launch adj_stress_tma_kernel");
      HMC_TRY(check_launch("adj_stress_tma_kernel"));
    }
    return HMC_OK;
  }
  const dim3 grid = cell_grid(s->nx, s->nz, s->chains), block = cell_block();
  for (int n = s->nt - 1; n >= 0; --n) {
    const StoreSlot slot = store_slot(s, n);
    const float* resid_n = s->resid + (int64_t)n * s->nrec * 2 * s->chains;
    // the first launch follows the residual kernel and memsets: ordinary stream order
    cudaError_t e;
    if (slot.now)
      e = launch_step(n < s->nt - 1, adj_velocity_kernel<true>, grid, block, st, g, a, p, gr, tm, s->taper,
                      s->rec_map, resid_n, (const float*)slot.now, prev_of(n, slot), w);
    else
      e = launch_step(n < s->nt - 1, adj_velocity_kernel<false>, grid, block, st, g, a, p, gr, tm, s->taper,
                      s->rec_map, resid_n, (const float*)nullptr, (const float*)nullptr, w);
    if (e != cudaSuccess) return cuda_fail(e, "launch adj_velocity_kernel");
    HMC_TRY(check_launch("adj_velocity_kernel"));
    e = launch_step(true, adj_stress_kernel, grid, block, st, g, a, p, tm, s->taper);
    if (e != cudaSuccess) return cuda_fail(e, "launch adj_stress_kernel");
    HMC_TRY(check_launch("adj_stress_kernel"));
  }
  return HMC_OK;
}

HMC_API int hmc_fwi_zero_gradients(const hmc_fwi* s, void* stream) {
  HMC_REQUIRE(s && s->g_bx && s->g_bz && s->g_l2m && s->g_lam && s->g_muxz, "hmc_fwi_zero_gradients: missing buffer");
  const size_t fb = (size_t)s->nx * s->nz * s->chains * sizeof(float);
  for (float* f : {s->g_bx, s->g_bz, s->g_l2m, s->g_lam, s->g_muxz}) {
    cudaError_t e = cudaMemsetAsync(f, 0, fb, as_stream(stream));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync(fwi gradients)");
  }
  return HMC_OK;
}

HMC_API int hmc_fwi_param_gradient(const hmc_fwi* s, float* g_rho, float* g_vp, float* g_vs, int accumulate,
                                   void* stream) {
  HMC_TRY(check_fwi(s, "hmc_fwi_param_gradient"));
  HMC_REQUIRE(g_rho && g_vp && g_vs, "hmc_fwi_param_gradient: null output");
  const Grid g = grid_of(s);
  Grads gr{s->g_bx, s->g_bz, s->g_l2m, s->g_lam, s->g_muxz};
  param_gradient_kernel<<<cell_grid(s->nx, s->nz, s->chains), cell_block(), 0, as_stream(stream)>>>(
      g, gr, s->rho, s->vp, s->vs, g_rho, g_vp, g_vs, accumulate);
  return check_launch("param_gradient_kernel");
}

HMC_API int hmc_fwi_cell_model(int64_t cells, int64_t C, const int32_t* map, const float* M, const float* base,
                               float* out, void* stream) {
  HMC_REQUIRE(cells > 0 && C > 0, "hmc_fwi_cell_model: bad sizes");
  HMC_REQUIRE(map && M && base && out, "hmc_fwi_cell_model: null buffer");
  cell_model_kernel<<<blocks_for(cells * C, 256), 256, 0, as_stream(stream)>>>(cells, C, map, M, base, out);
  return check_launch("cell_model_kernel");
}

HMC_API int hmc_fwi_cell_gradient(int64_t P, int64_t C, const int32_t* ptr, const int32_t* cells, const float* g,
                                  float* out, int accumulate, void* stream) {
  HMC_REQUIRE(P > 0 && C > 0, "hmc_fwi_cell_gradient: bad sizes");
  HMC_REQUIRE(ptr && cells && g && out, "hmc_fwi_cell_gradient: null buffer");
  cell_gradient_kernel<<<blocks_for(P * C, 256), 256, 0, as_stream(stream)>>>(P, C, ptr, cells, g, out, accumulate);
  return check_launch("cell_gradient_kernel");
}

}  // extern "C"
