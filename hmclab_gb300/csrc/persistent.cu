// Persistent fused proposals for small dense linear-Gaussian targets: one
// launch runs many whole HMC proposals for every chain, one warp per chain,
// with the d x d GtG of the premultiplied LinearMatrix in shared memory.
// Everything a proposal needs — Philox momenta (or injected streams), every
// kick and drift of the integrator, the misfit at the end point, the FP64
// accept test, the thinned sample record — happens in registers and shared
// memory, so a chain of d <= 128 costs a handful of microseconds per
// proposal instead of four launches per leapfrog step.
//
// Each lane owns the rows lane, lane + 32, ... of the chain's state.  The
// arithmetic follows the launch-per-step path operation by operation (same
// random draws, the same (GtG q - Gtd0) + prior-gradient composition, the
// same casts); the sums of the products and of the energies are taken in a
// different order, so the two paths agree to rounding of those sums.
#include "common.cuh"

namespace hmc {
namespace pers {

constexpr int MAX_D = 128;
enum PriorKind { PRIOR_NONE = 0, PRIOR_NORMAL = 1, PRIOR_LAPLACE = 2 };

template <typename T>
struct Target {
  int d, ld;  // dimension, odd row stride of GtG in shared memory
  int prior;  // PriorKind
  const T* GtG;
  const T* Gtd0;
  double dtd;
  const T* pmean;
  const T* pw;
};

template <typename T>
struct State {
  int64_t C;
  int mass;  // HMC_MASS_*
  T* q_cur;
  double* x_cur;
  const T* eps;
  int64_t* accepted;
  const int64_t* control;
  uint64_t seed;
  int randomize;
  const T* mdiag;
  const T* minv;
  const T* mchol;      // FULL: lower Cholesky factor of M, [d][d]
  const T* mfull_inv;  // FULL: M^-1, [d][d]
  const T* sz;
  const T* seps;
  const double* su;
  int64_t slen;
  T* ring_q;
  double* ring_x;
  int64_t ring_slots, thin;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <typename T>
__device__ __forceinline__ T sign_of(T x) {
  return x > (T)0 ? (T)1 : (x < (T)0 ? (T)-1 : (T)0);
}

// Standard normal for row i of chain c at proposal n: the injected stream or
// the Philox quad (i / 4) that the launch-per-step path draws.
template <typename T>
__device__ __forceinline__ T momentum_draw(const State<T>& s, int d, int i, int64_t c, int64_t n) {
  if (s.sz) return s.sz[((n % s.slen) * d + i) * s.C + c];
  T z[4];
  philox_normal4<T>(s.seed, (uint32_t)(i >> 2), (uint32_t)c, (uint64_t)n, PURPOSE_MOMENTUM, z);
  const int j = i & 3;  // select without a local-memory array index
  return j == 0 ? z[0] : (j == 1 ? z[1] : (j == 2 ? z[2] : z[3]));
}

// out[k] = sum_j GtG[row][j] q[j] for the lane's rows (q published in qw).
// Four partial sums per row (j mod 4) keep four independent FMA chains in
// flight; they are combined as (s0 + s1) + (s2 + s3).
template <typename T, int E>
__device__ __forceinline__ void matvec(const T* A, int ld, int d, const T* qw, int lane, T out[E]) {
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = lane + 32 * k;
    T s0 = (T)0, s1 = (T)0, s2 = (T)0, s3 = (T)0;
    if (i < d) {
      const T* row = A + i * ld;
      int j = 0;
      for (; j + 4 <= d; j += 4) {
        s0 += row[j] * qw[j];
        s1 += row[j + 1] * qw[j + 1];
        s2 += row[j + 2] * qw[j + 2];
        s3 += row[j + 3] * qw[j + 3];
      }
      for (; j < d; ++j) s0 += row[j] * qw[j];
    }
    out[k] = (s0 + s1) + (s2 + s3);
  }
}

// mp = M^-1 p for the lane's rows: unit, diagonal, or (FULL) the product
// with the explicit inverse held in shared memory (p published in qw).
template <typename T, int E>
__device__ __forceinline__ void apply_minv(int mass, const T* Mi, int ld, int d, T* qw, int lane, const bool live[E],
                                           const T minv[E], const T p[E], T mp[E]) {
  if (mass == HMC_MASS_FULL) {
#pragma unroll
    for (int k = 0; k < E; ++k)
      if (live[k]) qw[lane + 32 * k] = p[k];
    __syncwarp();
    matvec<T, E>(Mi, ld, d, qw, lane, mp);
    __syncwarp();
  } else {
#pragma unroll
    for (int k = 0; k < E; ++k) mp[k] = mass == HMC_MASS_DIAG ? minv[k] * p[k] : p[k];
  }
}

// Shared-memory matrices of one block: GtG, and for a full mass its
// inverse and Cholesky factor, each [d][ld]; then one q vector per warp.
template <typename T>
__device__ __forceinline__ void load_matrix(T* dst, const T* src, int d, int ld) {
  for (int e = threadIdx.x; e < d * d; e += blockDim.x) {
    const int r = e / d;
    dst[r * ld + (e - r * d)] = src[e];
  }
}

// One block of chains of one target: `block` numbers the block within the
// target's chains (warps of 32 lanes, one chain per warp).
template <typename T, int E>
__device__ __forceinline__ void run_block(const State<T>& s, const Target<T>& tg, const hmc_schedule& sch,
                                          int64_t nprop, int dry, int64_t block) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int d = tg.d, ld = tg.ld;
  const int MASS = s.mass, PRIOR = tg.prior;  // uniform over the block
  T* A = (T*)smem_raw;                                  // GtG [d][ld]
  T* Mi = A + d * ld;                                   // M^-1 [d][ld] (FULL)
  T* Lc = Mi + (MASS == HMC_MASS_FULL ? d * ld : 0);    // Cholesky factor [d][ld] (FULL)
  T* qbuf = Lc + (MASS == HMC_MASS_FULL ? d * ld : 0);  // [warps][d]
  load_matrix(A, tg.GtG, d, ld);
  if (MASS == HMC_MASS_FULL) {
    load_matrix(Mi, s.mfull_inv, d, ld);
    load_matrix(Lc, s.mchol, d, ld);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t c = block * (blockDim.x >> 5) + warp;
  if (c >= s.C) return;  // whole warps only; no block barrier follows
  T* qw = qbuf + warp * d;
  const int64_t n0 = s.control[0];

  // per-row constants of the lane's rows
  T minv[E], msq[E], gtd[E], pm[E], pw[E], qc[E];
  bool live[E];
#pragma unroll
  for (int k = 0; k < E; ++k) {
    const int i = lane + 32 * k;
    live[k] = i < d;
    minv[k] = (MASS == HMC_MASS_DIAG && live[k]) ? s.minv[i] : (T)1;
    msq[k] = (MASS == HMC_MASS_DIAG && live[k]) ? (T)sqrt((double)s.mdiag[i]) : (T)1;
    gtd[k] = live[k] ? tg.Gtd0[i] : (T)0;
    pm[k] = (PRIOR != PRIOR_NONE && live[k]) ? tg.pmean[i] : (T)0;
    pw[k] = (PRIOR != PRIOR_NONE && live[k]) ? tg.pw[i] : (T)0;
    qc[k] = live[k] ? s.q_cur[(int64_t)i * s.C + c] : (T)0;
  }
  double xc = s.x_cur[c];
  const T eps0 = s.eps[c];
  int64_t n_acc = 0;
  // which steps drift (the schedule's drift coefficient is nonzero)
  const unsigned drift_lo = __ballot_sync(0xffffffffu, lane < sch.steps && sch.drift[lane] != 0.0);
  const unsigned drift_hi = __ballot_sync(0xffffffffu, lane + 32 < sch.steps && sch.drift[lane + 32] != 0.0);

  for (int64_t t = 0; t < nprop; ++t) {
    const int64_t n = n0 + t;
    // Scalars of the proposal, each formed once per warp (FP64 issues at a
    // small fraction of the FP32 rate, so lanes split this work and share
    // the results by shuffles): the step size and accept uniform in lane 0,
    // the kick / drift coefficients of step l in lane l % 32.
    T e = eps0, ce = (T)0;
    double u = 0.0;
    if (lane == 0) {
      double ue = 0.0, ua = 0.0;
      if (!s.seps || !s.su) philox_scalars(s.seed, (uint32_t)c, (uint64_t)n, &ue, &ua);
      if (s.randomize) {
        const T f = s.seps ? s.seps[(n % s.slen) * s.C + c] : (T)(0.5 + ue);
        e = (T)((double)f * (double)e);
      }
      u = s.su ? s.su[(n % s.slen) * s.C + c] : ua;
      ce = (T)(sch.first_drift * (double)e);
    }
    e = __shfl_sync(0xffffffffu, e, 0);
    ce = __shfl_sync(0xffffffffu, ce, 0);
    T ck_lo = (T)0, cd_lo = (T)0, ck_hi = (T)0, cd_hi = (T)0;
    if (lane < sch.steps) {
      ck_lo = (T)(sch.kick[lane] * (double)e);
      cd_lo = (T)(sch.drift[lane] * (double)e);
    }
    if (lane + 32 < sch.steps) {
      ck_hi = (T)(sch.kick[lane + 32] * (double)e);
      cd_hi = (T)(sch.drift[lane + 32] * (double)e);
    }

    // momenta, K0, first drift
    T p[E], q[E];
    double k0 = 0.0;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      p[k] = (T)0;
      if (live[k]) {
        const T z = momentum_draw(s, d, lane + 32 * k, c, n);
        p[k] = MASS == HMC_MASS_DIAG ? msq[k] * z : z;
      }
    }
    if (MASS == HMC_MASS_FULL) {  // p = L z
#pragma unroll
      for (int k = 0; k < E; ++k)
        if (live[k]) qw[lane + 32 * k] = p[k];
      __syncwarp();
      matvec<T, E>(Lc, ld, d, qw, lane, p);
      __syncwarp();
    }
    T mp[E];
    apply_minv<T, E>(MASS, Mi, ld, d, qw, lane, live, minv, p, mp);
#pragma unroll
    for (int k = 0; k < E; ++k) {
      q[k] = qc[k];
      if (live[k]) {
        k0 += (double)p[k] * (double)mp[k];
        q[k] = qc[k] + ce * mp[k];
      }
    }
    k0 = 0.5 * warp_sum(k0);

    // kicks and drifts
    for (int st = 0; st < sch.steps; ++st) {
      if (sch.gradient[st]) {
#pragma unroll
        for (int k = 0; k < E; ++k)
          if (live[k]) qw[lane + 32 * k] = q[k];
        __syncwarp();
        T g[E];
        matvec<T, E>(A, ld, d, qw, lane, g);
        __syncwarp();
        const T ck = __shfl_sync(0xffffffffu, st < 32 ? ck_lo : ck_hi, st & 31);
#pragma unroll
        for (int k = 0; k < E; ++k) {
          T gk = g[k] - gtd[k];
          if (PRIOR == PRIOR_NORMAL) gk = gk + -(pw[k] * (pm[k] - q[k]));
          if (PRIOR == PRIOR_LAPLACE) gk = gk + sign_of(q[k] - pm[k]) * pw[k];
          p[k] -= ck * gk;
        }
      }
      if ((st < 32 ? drift_lo : drift_hi) >> (st & 31) & 1u) {
        const T cd = __shfl_sync(0xffffffffu, st < 32 ? cd_lo : cd_hi, st & 31);
        apply_minv<T, E>(MASS, Mi, ld, d, qw, lane, live, minv, p, mp);
#pragma unroll
        for (int k = 0; k < E; ++k) q[k] = q[k] + cd * mp[k];
      }
    }

    // misfit at the end point, K1 and the accept test (FP64)
#pragma unroll
    for (int k = 0; k < E; ++k)
      if (live[k]) qw[lane + 32 * k] = q[k];
    __syncwarp();
    T aq[E];
    matvec<T, E>(A, ld, d, qw, lane, aq);
    __syncwarp();
    apply_minv<T, E>(MASS, Mi, ld, d, qw, lane, live, minv, p, mp);
    double lik = 0.0, pri = 0.0, k1 = 0.0;
#pragma unroll
    for (int k = 0; k < E; ++k) {
      if (!live[k]) continue;
      const T w = aq[k] + (T)-2 * gtd[k];
      lik += (double)q[k] * (double)w;
      if (PRIOR == PRIOR_NORMAL) {
        const T r = pm[k] - q[k];
        pri += (double)r * (double)(pw[k] * r);
      }
      if (PRIOR == PRIOR_LAPLACE) pri += (double)(fabs(q[k] - pm[k]) * pw[k]);
      k1 += (double)p[k] * (double)mp[k];
    }
    lik = 0.5 * (warp_sum(lik) + tg.dtd);
    k1 = 0.5 * warp_sum(k1);
    double x1 = lik;
    if (PRIOR == PRIOR_NORMAL) x1 = 0.5 * warp_sum(pri) + lik;
    if (PRIOR == PRIOR_LAPLACE) x1 = warp_sum(pri) + lik;
    int accept = 0;
    if (lane == 0) accept = exp((xc + k0) - (x1 + k1)) > u ? 1 : 0;  // strict; NaN compares false
    if (__shfl_sync(0xffffffffu, accept, 0)) {
#pragma unroll
      for (int k = 0; k < E; ++k) qc[k] = q[k];
      xc = x1;
      ++n_acc;
    }
    if (!dry && s.ring_q && (n % s.thin) == 0) {
      const int64_t slot = (n / s.thin) % s.ring_slots;
#pragma unroll
      for (int k = 0; k < E; ++k)
        if (live[k]) s.ring_q[(slot * d + lane + 32 * k) * s.C + c] = qc[k];
      if (lane == 0) s.ring_x[slot * s.C + c] = xc;
    }
  }
  if (dry) return;
#pragma unroll
  for (int k = 0; k < E; ++k)
    if (live[k]) s.q_cur[(int64_t)(lane + 32 * k) * s.C + c] = qc[k];
  if (lane == 0) {
    s.x_cur[c] = xc;
    s.accepted[c] += n_acc;
  }
}

template <typename T, int E>
__global__ void __launch_bounds__(512) persistent_dense_kernel(State<T> s, Target<T> tg, hmc_schedule sch,
                                                               int64_t nprop, int dry) {
  run_block<T, E>(s, tg, sch, nprop, dry, blockIdx.x);
}

// Several targets of different dimensions (and chain counts) in one launch:
// group g owns the blocks [block0, next group's block0).
constexpr int MAX_GROUPS = 48;
template <typename T>
struct GroupTable {
  int n;
  int block0[MAX_GROUPS];
  State<T> s[MAX_GROUPS];
  Target<T> tg[MAX_GROUPS];
};

template <typename T, int E>
__global__ void __launch_bounds__(512) persistent_groups_kernel(GroupTable<T> tab, hmc_schedule sch, int64_t nprop,
                                                                int dry) {
  int g = 0;
  while (g + 1 < tab.n && tab.block0[g + 1] <= (int)blockIdx.x) ++g;
  run_block<T, E>(tab.s[g], tab.tg[g], sch, nprop, dry, (int64_t)blockIdx.x - tab.block0[g]);
}

__global__ void advance_counter_kernel(int64_t* control, int64_t n) { control[0] += n; }

}  // namespace pers
}  // namespace hmc

using namespace hmc;
using namespace hmc::pers;

namespace {

template <typename T>
size_t persistent_smem(int d, int mass_kind, int warps) {
  const size_t ld = (size_t)(d | 1);
  return ((mass_kind == HMC_MASS_FULL ? 3 : 1) * (size_t)d * ld + (size_t)warps * d) * sizeof(T);
}

template <typename T, int E>
int launch_single(const State<T>& st, const Target<T>& tg, const hmc_schedule& sch, int64_t nprop, int dry,
                  int warps, cudaStream_t stream) {
  const size_t smem = persistent_smem<T>(tg.d, st.mass, warps);
  auto kern = persistent_dense_kernel<T, E>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(persistent_dense_kernel)");
  }
  const unsigned blocks = (unsigned)((st.C + warps - 1) / warps);
  kern<<<blocks, 32 * warps, smem, stream>>>(st, tg, sch, nprop, dry);
  return check_launch("persistent_dense_kernel");
}

// Checks one target's state and fills the kernel's views of it.
template <typename T>
int fill_target(const char* who, const hmc_chains* s, const void* GtG, const void* Gtd0, double dtd, int prior,
                const void* pmean, const void* pw, int64_t nprop, int warps, State<T>& st, Target<T>& tg) {
  HMC_REQUIRE(s != nullptr, "%s: null state", who);
  HMC_REQUIRE(s->dims > 0 && s->dims <= MAX_D, "%s: dimension %lld outside 1..%d", who, (long long)s->dims, MAX_D);
  HMC_REQUIRE(s->chains > 0 && s->chains <= 0x7FFFFFFFll, "%s: bad number of chains", who);
  HMC_REQUIRE(s->q_cur && s->x_cur && s->eps && s->accepted && s->proposal, "%s: missing state buffer", who);
  HMC_REQUIRE(s->mass_kind >= HMC_MASS_UNIT && s->mass_kind <= HMC_MASS_FULL, "%s: bad mass kind", who);
  if (s->mass_kind == HMC_MASS_DIAG) HMC_REQUIRE(s->mass_diag && s->mass_inv_diag, "%s: diagonal mass buffers", who);
  if (s->mass_kind == HMC_MASS_FULL) HMC_REQUIRE(s->mass_chol && s->mass_inv, "%s: full mass buffers", who);
  HMC_REQUIRE(!s->lower && !s->upper, "%s: bounded targets use the launch-per-step path", who);
  HMC_REQUIRE(!s->autotune, "%s: autotuning uses the launch-per-step path", who);
  HMC_REQUIRE(!s->beta, "%s: tempered chains use the launch-per-step path", who);
  HMC_REQUIRE(GtG && Gtd0, "%s: null GtG or Gtd0", who);
  HMC_REQUIRE(prior >= PRIOR_NONE && prior <= PRIOR_LAPLACE, "%s: unknown prior kind %d", who, prior);
  HMC_REQUIRE(prior == PRIOR_NONE || (pmean && pw), "%s: prior parameters missing", who);
  if (s->stream_z || s->stream_eps || s->stream_u)
    HMC_REQUIRE(s->stream_z && s->stream_u && s->stream_len >= nprop && (s->stream_eps || !s->randomize_stepsize),
                "%s: injected streams shorter than the launch", who);
  if (s->ring_q) HMC_REQUIRE(s->ring_x && s->ring_slots > 0 && s->thinning > 0, "%s: bad sample ring", who);
  HMC_REQUIRE(persistent_smem<T>((int)s->dims, s->mass_kind, warps) <= 227 * 1024,
              "%s: the matrices of d = %lld do not fit in shared memory", who, (long long)s->dims);
  st.C = s->chains;
  st.mass = s->mass_kind;
  st.q_cur = (T*)s->q_cur;
  st.x_cur = s->x_cur;
  st.eps = (const T*)s->eps;
  st.accepted = s->accepted;
  st.control = s->proposal;
  st.seed = s->seed;
  st.randomize = s->randomize_stepsize;
  st.mdiag = (const T*)s->mass_diag;
  st.minv = (const T*)s->mass_inv_diag;
  st.mchol = (const T*)s->mass_chol;
  st.mfull_inv = (const T*)s->mass_inv;
  st.sz = (const T*)s->stream_z;
  st.seps = (const T*)s->stream_eps;
  st.su = s->stream_u;
  st.slen = s->stream_len;
  st.ring_q = (T*)s->ring_q;
  st.ring_x = s->ring_x;
  st.ring_slots = s->ring_slots;
  st.thin = s->thinning;
  tg.d = (int)s->dims;
  tg.ld = tg.d | 1;
  tg.prior = prior;
  tg.GtG = (const T*)GtG;
  tg.Gtd0 = (const T*)Gtd0;
  tg.dtd = dtd;
  tg.pmean = (const T*)pmean;
  tg.pw = (const T*)pw;
  return HMC_OK;
}

int check_common(const char* who, const hmc_schedule* sch, int64_t nprop, int warps) {
  HMC_REQUIRE(sch && sch->steps >= 1 && sch->steps <= HMC_SCHEDULE_MAX, "%s: bad schedule", who);
  HMC_REQUIRE(warps == 1 || warps == 2 || warps == 4 || warps == 8 || warps == 16, "%s: warps_per_block %d", who,
              warps);
  HMC_REQUIRE(nprop >= 0, "%s: negative proposal count", who);
  return HMC_OK;
}

template <typename T>
int persistent_impl(const hmc_chains* s, const void* GtG, const void* Gtd0, double dtd, int prior,
                    const void* pmean, const void* pw, const hmc_schedule* sch, int64_t nprop, int warps, int dry,
                    cudaStream_t stream) {
  const char* who = "hmc_persistent_dense";
  HMC_TRY(check_common(who, sch, nprop, warps));
  State<T> st;
  Target<T> tg;
  HMC_TRY(fill_target<T>(who, s, GtG, Gtd0, dtd, prior, pmean, pw, nprop, warps, st, tg));
  if (nprop == 0) return HMC_OK;
  const int E = (tg.d + 31) / 32;
  int rc;
  switch (E) {
    case 1: rc = launch_single<T, 1>(st, tg, *sch, nprop, dry, warps, stream); break;
    case 2: rc = launch_single<T, 2>(st, tg, *sch, nprop, dry, warps, stream); break;
    case 3: rc = launch_single<T, 3>(st, tg, *sch, nprop, dry, warps, stream); break;
    default: rc = launch_single<T, 4>(st, tg, *sch, nprop, dry, warps, stream); break;
  }
  HMC_TRY(rc);
  if (dry) return HMC_OK;
  advance_counter_kernel<<<1, 1, 0, stream>>>(s->proposal, nprop);
  return check_launch("advance_counter_kernel");
}

template <typename T, int E>
int launch_groups(const GroupTable<T>& tab, int blocks, size_t smem, const hmc_schedule& sch, int64_t nprop, int dry,
                  int warps, cudaStream_t stream) {
  auto kern = persistent_groups_kernel<T, E>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(persistent_groups_kernel)");
  }
  kern<<<(unsigned)blocks, 32 * warps, smem, stream>>>(tab, sch, nprop, dry);
  return check_launch("persistent_groups_kernel");
}

template <typename T>
int groups_impl(const hmc_dense_group* groups, int ngroups, const hmc_schedule* sch, int64_t nprop, int warps,
                int dry, cudaStream_t stream) {
  const char* who = "hmc_persistent_dense_groups";
  HMC_TRY(check_common(who, sch, nprop, warps));
  HMC_REQUIRE(groups && ngroups >= 1 && ngroups <= MAX_GROUPS, "%s: 1..%d groups", who, MAX_GROUPS);
  GroupTable<T> tab;
  tab.n = ngroups;
  const int mk = groups[0].chains ? groups[0].chains->mass_kind : -1;
  const int prior = groups[0].prior;
  int64_t blocks = 0;
  int dmax = 0;
  size_t smem = 0;
  for (int g = 0; g < ngroups; ++g) {
    const hmc_dense_group& G = groups[g];
    HMC_REQUIRE(G.chains && G.chains->dtype == groups[0].chains->dtype, "%s: group %d has another dtype", who, g);
    HMC_REQUIRE(G.chains->mass_kind == mk && G.prior == prior, "%s: group %d differs in mass or prior kind", who, g);
    HMC_TRY(fill_target<T>(who, G.chains, G.GtG, G.Gtd0, G.dtd, G.prior, G.prior_mean, G.prior_w, nprop, warps,
                           tab.s[g], tab.tg[g]));
    tab.block0[g] = (int)blocks;
    blocks += (G.chains->chains + warps - 1) / warps;
    dmax = tab.tg[g].d > dmax ? tab.tg[g].d : dmax;
    const size_t sm = persistent_smem<T>(tab.tg[g].d, mk, warps);
    smem = sm > smem ? sm : smem;
  }
  HMC_REQUIRE(blocks <= 0x7FFFFFFF, "%s: too many blocks", who);
  if (nprop == 0) return HMC_OK;
  const int E = (dmax + 31) / 32;
  int rc;
  switch (E) {
    case 1: rc = launch_groups<T, 1>(tab, (int)blocks, smem, *sch, nprop, dry, warps, stream); break;
    case 2: rc = launch_groups<T, 2>(tab, (int)blocks, smem, *sch, nprop, dry, warps, stream); break;
    case 3: rc = launch_groups<T, 3>(tab, (int)blocks, smem, *sch, nprop, dry, warps, stream); break;
    default: rc = launch_groups<T, 4>(tab, (int)blocks, smem, *sch, nprop, dry, warps, stream); break;
  }
  HMC_TRY(rc);
  if (dry) return HMC_OK;
  for (int g = 0; g < ngroups; ++g) {
    advance_counter_kernel<<<1, 1, 0, stream>>>(groups[g].chains->proposal, nprop);
    HMC_TRY(check_launch("advance_counter_kernel"));
  }
  return HMC_OK;
}

}  // namespace

extern "C" HMC_API int hmc_persistent_dense(const hmc_chains* s, const void* GtG, const void* Gtd0, double dtd,
                                            int prior, const void* prior_mean, const void* prior_w,
                                            const hmc_schedule* schedule, int64_t proposals, int warps_per_block,
                                            int dry, void* stream) {
  if (!s) return fail(HMC_ERR_INVALID_ARG, "hmc_persistent_dense: null state");
  return HMC_DISPATCH(s->dtype, T, [&] {
    return persistent_impl<T>(s, GtG, Gtd0, dtd, prior, prior_mean, prior_w, schedule, proposals, warps_per_block,
                              dry, as_stream(stream));
  });
}

extern "C" HMC_API int hmc_persistent_dense_groups(const hmc_dense_group* groups, int ngroups,
                                                   const hmc_schedule* schedule, int64_t proposals,
                                                   int warps_per_block, int dry, void* stream) {
  if (!groups || ngroups < 1 || !groups[0].chains)
    return fail(HMC_ERR_INVALID_ARG, "hmc_persistent_dense_groups: no groups");
  return HMC_DISPATCH(groups[0].chains->dtype, T, [&] {
    return groups_impl<T>(groups, ngroups, schedule, proposals, warps_per_block, dry, as_stream(stream));
  });
}
