// Batched HMC trajectory kernels: momentum draw + first drift, kick/drift
// steps, and the FP64 Metropolis accept with thinned sample recording.
//
// Semantics follow the reference sampler (larsgeb/hmclab):
//   momentum   MassMatrices.py:135-142 (Unit), 220-227 (Diagonal), 307-314 (Full)
//   K, dK/dp   MassMatrices.py:100-133, 185-218, 270-305
//   leapfrog   Samplers.py:1524-1584 (position Verlet: drift-kick-drift)
//   corrector  Distributions/base.py:239-270 (reflect at bounds, flip p)
//   accept     Samplers.py:1471-1492 (exp(H0 - H1) > u, strict, NaN rejects)
//   autotune   Samplers.py:1494-1522
//   append     Samplers.py:675-678 (thinned vstack([q, x]))
#include <math.h>

#include <type_traits>

#include "common.cuh"

namespace hmc {
int gemm_dispatch(int dtype, int64_t m, int64_t n, int64_t k, double alpha, const void* A, const void* B,
                  const void* bias, void* out, int accumulate, cudaStream_t stream);
}

namespace hmc {
namespace {

template <typename T>
struct ChainView {
  int64_t d, C;
  T* q_cur;
  T* q;
  T* p;
  const T* g;
  T* v;
  const T* mdiag;
  const T* minv;
  const T* lo;
  const T* hi;
  T* eps;
  T* eps_local;
  double* x_cur;
  double* x_prop;
  double* k_cur;
  double* k_prop;
  int64_t* accepted;
  int32_t* flags;
  int64_t* control;  // [0] proposal counter, [1] block arrival counter
  uint64_t seed;
  int randomize;
  int autotune;
  double target, kappa, min_eps;
  const T* sz;
  const T* seps;
  const double* su;
  int64_t slen;
  T* ring_q;
  double* ring_x;
  int64_t ring_slots, thin;
  double* rec_eps;
  double* rec_acc;
  int64_t rec_len;
  const double* beta;  // per-chain inverse temperature, nullptr = 1
};

template <typename T>
ChainView<T> view(const hmc_chains* s) {
  ChainView<T> v;
  v.d = s->dims;
  v.C = s->chains;
  v.q_cur = (T*)s->q_cur;
  v.q = (T*)s->q;
  v.p = (T*)s->p;
  v.g = (const T*)s->g;
  v.v = (T*)s->v;
  v.mdiag = (const T*)s->mass_diag;
  v.minv = (const T*)s->mass_inv_diag;
  v.lo = (const T*)s->lower;
  v.hi = (const T*)s->upper;
  v.eps = (T*)s->eps;
  v.eps_local = (T*)s->eps_local;
  v.x_cur = s->x_cur;
  v.x_prop = s->x_prop;
  v.k_cur = s->k_cur;
  v.k_prop = s->k_prop;
  v.accepted = s->accepted;
  v.flags = s->flags;
  v.control = s->proposal;
  v.seed = s->seed;
  v.randomize = s->randomize_stepsize;
  v.autotune = s->autotune;
  v.target = s->target_acceptance;
  v.kappa = s->learning_rate;
  v.min_eps = s->minimal_stepsize;
  v.sz = (const T*)s->stream_z;
  v.seps = (const T*)s->stream_eps;
  v.su = s->stream_u;
  v.slen = s->stream_len;
  v.ring_q = (T*)s->ring_q;
  v.ring_x = s->ring_x;
  v.ring_slots = s->ring_slots;
  v.thin = s->thinning;
  v.rec_eps = s->rec_stepsize;
  v.rec_acc = s->rec_acceptance;
  v.rec_len = s->rec_len;
  v.beta = s->beta;
  return v;
}

// M^-1 p for one element; FULL reads the precomputed product from v.
template <typename T, int MASS>
__device__ __forceinline__ T minv_p(const ChainView<T>& s, int64_t i, int64_t idx, T p) {
  if (MASS == HMC_MASS_UNIT) return p;
  if (MASS == HMC_MASS_DIAG) return s.minv[i] * p;
  return s.v[idx];
}

// Reflection of base.py:239-270 (lower bound first, then upper); returns
// true when the position is still outside after the reflection.
template <typename T>
__device__ __forceinline__ bool reflect(const ChainView<T>& s, int64_t i, T& q, T& p) {
  bool out = false;
  if (s.lo) {
    const T lb = s.lo[i];
    if (q < lb) {
      q += (T)2 * (lb - q);
      p = -p;
    }
  }
  if (s.hi) {
    const T ub = s.hi[i];
    if (q > ub) {
      q += (T)2 * (ub - q);
      p = -p;
    }
  }
  if (s.lo && q < s.lo[i]) out = true;
  if (s.hi && q > s.hi[i]) out = true;
  return out;
}

template <typename T>
__device__ __forceinline__ T step_factor(const ChainView<T>& s, int64_t c, int64_t n) {
  if (s.seps) return s.seps[(n % s.slen) * s.C + c];
  double ue, ua;
  philox_scalars(s.seed, (uint32_t)c, (uint64_t)n, &ue, &ua);
  return (T)(0.5 + ue);
}

template <typename T>
__device__ __forceinline__ void draw_z4(const ChainView<T>& s, int64_t quad, int64_t c, int64_t n, T z[4]) {
  if (s.sz) {
    const T* base = s.sz + (n % s.slen) * s.d * s.C;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t i = 4 * quad + j;
      z[j] = i < s.d ? base[i * s.C + c] : (T)0;
    }
  } else {
    philox_normal4<T>(s.seed, (uint32_t)quad, (uint32_t)c, (uint64_t)n, PURPOSE_MOMENTUM, z);
  }
}

// FULL mass, step 1: z -> v (the host then forms p = L z and v = M^-1 p).
template <typename T>
__global__ void draw_z_kernel(ChainView<T> s) {
  const int64_t n = s.control[0];
  const int64_t quads = (s.d + 3) / 4;
  const int64_t total = quads * s.C;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t % s.C, qd = t / s.C;
    T z[4];
    draw_z4(s, qd, c, n, z);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t i = 4 * qd + j;
      if (i < s.d) s.v[i * s.C + c] = z[j];
    }
  }
}

// Momentum (UNIT/DIAG; FULL has p and v = M^-1 p already), K0 in FP64, step
// size of this trajectory, first drift and reflection.
template <typename T, int MASS>
__global__ void begin_kernel(ChainView<T> s, double drift) {
  __shared__ double sh[RED_Y][RED_X + 1];
  const int64_t c = blockIdx.x * (int64_t)RED_X + threadIdx.x;
  const bool live = c < s.C;
  const int64_t n = s.control[0];
  T e = (T)0;
  if (live) {
    e = s.eps[c];
    if (s.randomize) e = (T)((double)step_factor(s, c, n) * (double)e);
  }
  const T ce = (T)(drift * (double)e);  // (drift * eps), then times M^-1 p
  double k = 0.0;
  bool oob = false;
  if (live) {
    if (MASS == HMC_MASS_FULL) {
      for (int64_t i = threadIdx.y; i < s.d; i += RED_Y) {
        const int64_t idx = i * s.C + c;
        T p = s.p[idx];
        const T mp = s.v[idx];
        k += (double)p * (double)mp;
        T q = s.q_cur[idx] + ce * mp;
        oob |= reflect(s, i, q, p);
        s.q[idx] = q;
        s.p[idx] = p;
      }
    } else {
      const int64_t quads = (s.d + 3) / 4;
      for (int64_t qd = threadIdx.y; qd < quads; qd += RED_Y) {
        T z[4];
        draw_z4(s, qd, c, n, z);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int64_t i = 4 * qd + j;
          if (i < s.d) {
            const int64_t idx = i * s.C + c;
            T p = MASS == HMC_MASS_DIAG ? (T)sqrt((double)s.mdiag[i]) * z[j] : z[j];
            const T mp = minv_p<T, MASS>(s, i, idx, p);
            k += (double)p * (double)mp;
            T q = s.q_cur[idx] + ce * mp;
            oob |= reflect(s, i, q, p);
            s.q[idx] = q;
            s.p[idx] = p;
          }
        }
      }
    }
  }
  const double ksum = block_chain_sum(k, sh);
  __shared__ int oob_any[RED_X];
  if (threadIdx.y == 0) oob_any[threadIdx.x] = 0;
  __syncthreads();
  if (oob) atomicOr(&oob_any[threadIdx.x], 1);
  __syncthreads();
  if (live && threadIdx.y == 0) {
    s.k_cur[c] = 0.5 * ksum;
    s.eps_local[c] = e;
    s.flags[c] = oob_any[threadIdx.x] ? HMC_FLAG_OUT_OF_BOUNDS : 0;
  }
}

// p -= kick * eps * g; q += drift * eps * M^-1 p; reflect.  For FULL the kick
// and the drift are split around the host-issued v = M^-1 p product.
template <typename T, int MASS, int DO_KICK, int DO_DRIFT>
__global__ void kick_drift_kernel(ChainView<T> s, double kick, double drift) {
  const int64_t total = s.d * s.C;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = idx % s.C, i = idx / s.C;
    const T e = s.eps_local[c];
    T p = s.p[idx];
    if (DO_KICK) {
      const T ck = (T)(kick * (double)e * (s.beta ? s.beta[c] : 1.0));
      p -= ck * s.g[idx];
    }
    if (DO_DRIFT) {
      const T cd = (T)(drift * (double)e);
      T q = s.q[idx] + cd * minv_p<T, MASS>(s, i, idx, p);
      if (s.lo || s.hi) {
        if (reflect(s, i, q, p)) atomicOr(&s.flags[c], HMC_FLAG_OUT_OF_BOUNDS);
      }
      s.q[idx] = q;
    }
    s.p[idx] = p;
  }
}

// FP64 kinetic energy of p (MASS != FULL) or of (p, v = M^-1 p) (FULL).
template <typename T, int MASS>
__device__ __forceinline__ double kinetic_partial(const ChainView<T>& s, const T* p, const T* mp_full, int64_t c) {
  double k = 0.0;
  for (int64_t i = threadIdx.y; i < s.d; i += RED_Y) {
    const int64_t idx = i * s.C + c;
    const T pi = p[idx];
    const T mp = MASS == HMC_MASS_UNIT ? pi : (MASS == HMC_MASS_DIAG ? s.minv[i] * pi : mp_full[idx]);
    k += (double)pi * (double)mp;
  }
  return k;
}

template <typename T, int MASS>
__global__ void kinetic_kernel(ChainView<T> s, const T* p, const T* mp_full, double* out) {
  __shared__ double sh[RED_Y][RED_X + 1];
  const int64_t c = blockIdx.x * (int64_t)RED_X + threadIdx.x;
  const double k = c < s.C ? kinetic_partial<T, MASS>(s, p, mp_full, c) : 0.0;
  const double ks = block_chain_sum(k, sh);
  if (c < s.C && threadIdx.y == 0) out[c] = 0.5 * ks;
}

template <typename T, int MASS>
__global__ void end_kernel(ChainView<T> s) {
  __shared__ double sh[RED_Y][RED_X + 1];
  __shared__ int acc_flag[RED_X];
  const int64_t c = blockIdx.x * (int64_t)RED_X + threadIdx.x;
  const bool live = c < s.C;
  const int64_t n = s.control[0];
  const double k = live ? kinetic_partial<T, MASS>(s, s.p, s.v, c) : 0.0;
  const double ks = block_chain_sum(k, sh);
  if (threadIdx.y == 0) {
    int accept = 0;
    if (live) {
      const double k1 = 0.5 * ks;
      s.k_prop[c] = k1;
      double x1 = s.x_prop[c];
      if (s.flags[c] & HMC_FLAG_OUT_OF_BOUNDS) {
        x1 = INFINITY;
        s.x_prop[c] = x1;
      }
      const double b = s.beta ? s.beta[c] : 1.0;
      const double h0 = (s.beta ? b * s.x_cur[c] : s.x_cur[c]) + s.k_cur[c];
      const double h1 = (s.beta ? b * x1 : x1) + k1;
      const double alpha = exp(h0 - h1);
      if (s.autotune) {
        const T eps_now = s.eps[c];
        if (s.rec_eps && n < s.rec_len) {
          s.rec_eps[n * s.C + c] = (double)eps_now;
          s.rec_acc[n * s.C + c] = alpha;
        }
        const double w = pow((double)(n + 1), -s.kappa);
        const double a = isnan(alpha) ? 0.0 : alpha;
        double e = (double)eps_now - w * (s.target - fmin(a, 1.0));
        if (e <= 0.0) e = fmax(e, s.min_eps);
        s.eps[c] = (T)e;
      }
      double u;
      if (s.su) {
        u = s.su[(n % s.slen) * s.C + c];
      } else {
        double ue;
        philox_scalars(s.seed, (uint32_t)c, (uint64_t)n, &ue, &u);
      }
      accept = alpha > u ? 1 : 0;  // strict; NaN compares false
      if (accept) {
        s.x_cur[c] = x1;
        s.accepted[c] += 1;
      }
    }
    acc_flag[threadIdx.x] = accept;
  }
  __syncthreads();
  const bool record = s.ring_q != nullptr && (n % s.thin) == 0;
  const int64_t slot = record ? (n / s.thin) % s.ring_slots : 0;
  if (live) {
    const bool acc = acc_flag[threadIdx.x] != 0;
    for (int64_t i = threadIdx.y; i < s.d; i += RED_Y) {
      const int64_t idx = i * s.C + c;
      T qv;
      if (acc) {
        qv = s.q[idx];
        s.q_cur[idx] = qv;
      } else if (record) {
        qv = s.q_cur[idx];
      }
      if (record) s.ring_q[slot * s.d * s.C + idx] = qv;
    }
    if (record && threadIdx.y == 0) s.ring_x[slot * s.C + c] = s.beta ? s.beta[c] * s.x_cur[c] : s.x_cur[c];
  }
  // The last block to finish advances the proposal counter.
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    const unsigned long long prev = atomicAdd((unsigned long long*)&s.control[1], 1ull);
    last = prev == (unsigned long long)(gridDim.x - 1);
  }
  __syncthreads();
  if (last && threadIdx.x == 0 && threadIdx.y == 0) {
    s.control[0] = n + 1;
    s.control[1] = 0;
    __threadfence();
  }
}

template <typename T>
int check_state(const hmc_chains* s, const char* who) {
  HMC_REQUIRE(s != nullptr, "%s: null state", who);
  HMC_REQUIRE(s->dims > 0 && s->chains > 0, "%s: dims and chains must be positive", who);
  HMC_REQUIRE(s->chains <= 0xFFFFFFFFll, "%s: too many chains", who);
  HMC_REQUIRE(s->q_cur && s->q && s->p && s->eps && s->eps_local && s->x_cur && s->x_prop && s->k_cur &&
                  s->k_prop && s->accepted && s->flags && s->proposal,
              "%s: missing state buffer", who);
  HMC_REQUIRE(s->mass_kind >= HMC_MASS_UNIT && s->mass_kind <= HMC_MASS_FULL, "%s: bad mass kind", who);
  if (s->mass_kind == HMC_MASS_DIAG)
    HMC_REQUIRE(s->mass_diag && s->mass_inv_diag, "%s: diagonal mass needs diag and inverse", who);
  if (s->mass_kind == HMC_MASS_FULL)
    HMC_REQUIRE(s->mass_chol && s->mass_inv && s->v, "%s: full mass needs cholesky, inverse and v", who);
  if (s->stream_z || s->stream_eps || s->stream_u)
    HMC_REQUIRE(s->stream_z && s->stream_u && s->stream_len > 0 && (s->stream_eps || !s->randomize_stepsize),
                "%s: incomplete injected streams", who);
  if (s->ring_q) HMC_REQUIRE(s->ring_x && s->ring_slots > 0 && s->thinning > 0, "%s: bad sample ring", who);
  return HMC_OK;
}

inline unsigned ew_grid(int64_t n) {
  const unsigned b = blocks_for(n, 256);
  return b > 152u * 32u ? 152u * 32u : b;
}

template <typename T>
int begin_impl(const hmc_chains* s, double drift, cudaStream_t st) {
  HMC_TRY(check_state<T>(s, "hmc_begin_trajectory"));
  ChainView<T> v = view<T>(s);
  const dim3 grid = red_grid(s->chains), block = red_block();
  switch (s->mass_kind) {
    case HMC_MASS_UNIT:
      begin_kernel<T, HMC_MASS_UNIT><<<grid, block, 0, st>>>(v, drift);
      break;
    case HMC_MASS_DIAG:
      begin_kernel<T, HMC_MASS_DIAG><<<grid, block, 0, st>>>(v, drift);
      break;
    default: {
      const int64_t quads = (s->dims + 3) / 4;
      draw_z_kernel<T><<<ew_grid(quads * s->chains), 256, 0, st>>>(v);
      HMC_TRY(check_launch("draw_z_kernel"));
      const int dt = std::is_same<T, double>::value ? HMC_F64 : HMC_F32;
      // p = L z, then v = M^-1 p.
      HMC_TRY(gemm_dispatch(dt, s->dims, s->chains, s->dims, 1.0, s->mass_chol, s->v, nullptr, s->p, 0, st));
      HMC_TRY(gemm_dispatch(dt, s->dims, s->chains, s->dims, 1.0, s->mass_inv, s->p, nullptr, s->v, 0, st));
      begin_kernel<T, HMC_MASS_FULL><<<grid, block, 0, st>>>(v, drift);
    }
  }
  return check_launch("begin_kernel");
}

template <typename T>
int kick_drift_impl(const hmc_chains* s, double kick, double drift, cudaStream_t st) {
  HMC_TRY(check_state<T>(s, "hmc_kick_drift"));
  HMC_REQUIRE(s->g != nullptr, "hmc_kick_drift: missing gradient buffer");
  ChainView<T> v = view<T>(s);
  const unsigned grid = ew_grid(s->dims * s->chains);
  const bool do_drift = drift != 0.0;
  const bool do_kick = kick != 0.0;
  HMC_REQUIRE(do_kick || do_drift, "hmc_kick_drift: kick and drift are both zero");
  switch (s->mass_kind) {
    case HMC_MASS_UNIT:
      if (do_kick && do_drift)
        kick_drift_kernel<T, HMC_MASS_UNIT, 1, 1><<<grid, 256, 0, st>>>(v, kick, drift);
      else if (do_kick)
        kick_drift_kernel<T, HMC_MASS_UNIT, 1, 0><<<grid, 256, 0, st>>>(v, kick, drift);
      else
        kick_drift_kernel<T, HMC_MASS_UNIT, 0, 1><<<grid, 256, 0, st>>>(v, kick, drift);
      break;
    case HMC_MASS_DIAG:
      if (do_kick && do_drift)
        kick_drift_kernel<T, HMC_MASS_DIAG, 1, 1><<<grid, 256, 0, st>>>(v, kick, drift);
      else if (do_kick)
        kick_drift_kernel<T, HMC_MASS_DIAG, 1, 0><<<grid, 256, 0, st>>>(v, kick, drift);
      else
        kick_drift_kernel<T, HMC_MASS_DIAG, 0, 1><<<grid, 256, 0, st>>>(v, kick, drift);
      break;
    default: {
      if (do_kick) {
        kick_drift_kernel<T, HMC_MASS_FULL, 1, 0><<<grid, 256, 0, st>>>(v, kick, drift);
        if (!do_drift) break;
        HMC_TRY(check_launch("kick_kernel"));
      }
      const int dt = std::is_same<T, double>::value ? HMC_F64 : HMC_F32;
      HMC_TRY(gemm_dispatch(dt, s->dims, s->chains, s->dims, 1.0, s->mass_inv, s->p, nullptr, s->v, 0, st));
      kick_drift_kernel<T, HMC_MASS_FULL, 0, 1><<<grid, 256, 0, st>>>(v, kick, drift);
    }
  }
  return check_launch("kick_drift_kernel");
}

template <typename T>
int end_impl(const hmc_chains* s, cudaStream_t st) {
  HMC_TRY(check_state<T>(s, "hmc_end_trajectory"));
  ChainView<T> v = view<T>(s);
  const dim3 grid = red_grid(s->chains), block = red_block();
  switch (s->mass_kind) {
    case HMC_MASS_UNIT:
      end_kernel<T, HMC_MASS_UNIT><<<grid, block, 0, st>>>(v);
      break;
    case HMC_MASS_DIAG:
      end_kernel<T, HMC_MASS_DIAG><<<grid, block, 0, st>>>(v);
      break;
    default: {
      const int dt = std::is_same<T, double>::value ? HMC_F64 : HMC_F32;
      HMC_TRY(gemm_dispatch(dt, s->dims, s->chains, s->dims, 1.0, s->mass_inv, s->p, nullptr, s->v, 0, st));
      end_kernel<T, HMC_MASS_FULL><<<grid, block, 0, st>>>(v);
    }
  }
  return check_launch("end_kernel");
}

template <typename T>
int kinetic_impl(const hmc_chains* s, const void* p, double* out, cudaStream_t st) {
  HMC_REQUIRE(s && p && out, "hmc_kinetic_energy: null argument");
  HMC_REQUIRE(s->dims > 0 && s->chains > 0, "hmc_kinetic_energy: bad sizes");
  ChainView<T> v = view<T>(s);
  const dim3 grid = red_grid(s->chains), block = red_block();
  switch (s->mass_kind) {
    case HMC_MASS_UNIT:
      kinetic_kernel<T, HMC_MASS_UNIT><<<grid, block, 0, st>>>(v, (const T*)p, nullptr, out);
      break;
    case HMC_MASS_DIAG:
      HMC_REQUIRE(s->mass_inv_diag, "hmc_kinetic_energy: missing inverse diagonal");
      kinetic_kernel<T, HMC_MASS_DIAG><<<grid, block, 0, st>>>(v, (const T*)p, nullptr, out);
      break;
    default: {
      HMC_REQUIRE(s->mass_inv && s->v, "hmc_kinetic_energy: full mass needs inverse and v");
      const int dt = std::is_same<T, double>::value ? HMC_F64 : HMC_F32;
      HMC_TRY(gemm_dispatch(dt, s->dims, s->chains, s->dims, 1.0, s->mass_inv, p, nullptr, s->v, 0, st));
      kinetic_kernel<T, HMC_MASS_FULL><<<grid, block, 0, st>>>(v, (const T*)p, (const T*)s->v, out);
    }
  }
  return check_launch("kinetic_kernel");
}

template <typename T>
__global__ void scale_rows_kernel(const T* scale, const T* x, T* out, int64_t d, int64_t C) {
  const int64_t total = d * C;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x)
    out[idx] = scale ? scale[idx / C] * x[idx] : x[idx];
}

template <typename T>
int kinetic_grad_impl(const hmc_chains* s, const void* p, void* out, cudaStream_t st) {
  HMC_REQUIRE(s && p && out, "hmc_kinetic_energy_gradient: null argument");
  HMC_REQUIRE(s->dims > 0 && s->chains > 0, "hmc_kinetic_energy_gradient: bad sizes");
  const int dt = std::is_same<T, double>::value ? HMC_F64 : HMC_F32;
  if (s->mass_kind == HMC_MASS_FULL) {
    HMC_REQUIRE(s->mass_inv, "hmc_kinetic_energy_gradient: missing inverse");
    return gemm_dispatch(dt, s->dims, s->chains, s->dims, 1.0, s->mass_inv, p, nullptr, out, 0, st);
  }
  const T* scale = s->mass_kind == HMC_MASS_DIAG ? (const T*)s->mass_inv_diag : nullptr;
  HMC_REQUIRE(s->mass_kind != HMC_MASS_DIAG || scale, "hmc_kinetic_energy_gradient: missing inverse diagonal");
  scale_rows_kernel<T><<<ew_grid(s->dims * s->chains), 256, 0, st>>>(scale, (const T*)p, (T*)out, s->dims,
                                                                      s->chains);
  return check_launch("scale_rows_kernel");
}

}  // namespace
// ---- replica exchange ----------------------------------------------------
// Decision per pair from the current misfits and inverse temperatures; pairs
// with an index outside [0, C) or a == b never swap.
__global__ void exchange_decide_kernel(int64_t npairs, int64_t C, const int32_t* __restrict__ pairs,
                                       const double* __restrict__ u, const double* __restrict__ beta,
                                       const double* __restrict__ x, int32_t* swapped, int64_t* total) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= npairs) return;
  const int32_t a = pairs[2 * k], b = pairs[2 * k + 1];
  int ok = 0;
  if (a >= 0 && a < C && b >= 0 && b < C && a != b) {
    const double ba = beta ? beta[a] : 1.0, bb = beta ? beta[b] : 1.0;
    ok = exp((ba - bb) * (x[a] - x[b])) > u[k] ? 1 : 0;  // NaN compares false
  }
  swapped[k] = ok;
  if (ok && total) atomicAdd((unsigned long long*)total, 1ull);
}

// Swap the columns of accepted pairs: thread (pair k, dimension i).  The
// exchange follows the last proposal's accept step; when that proposal was
// recorded in the thinned ring, its entry is swapped too, so the recorded
// sample is the post-exchange state, as in the reference (the sample is
// appended after the exchange, Samplers.py:589-678).  Its misfit entry is
// the tempered misfit of the swapped-in model.
template <typename T>
__global__ void exchange_swap_kernel(int64_t npairs, int64_t d, int64_t C, const int32_t* __restrict__ pairs,
                                     const int32_t* __restrict__ swapped, T* q_cur, double* x_cur,
                                     const int64_t* __restrict__ control, T* ring_q, double* ring_x,
                                     int64_t ring_slots, int64_t thin, const double* __restrict__ beta) {
  const int64_t n_last = control ? control[0] - 1 : -1;
  const bool rec = ring_q != nullptr && n_last >= 0 && n_last % thin == 0;
  const int64_t slot = rec ? (n_last / thin) % ring_slots : 0;
  const int64_t total = npairs * d;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = e / d, i = e - k * d;
    if (!swapped[k]) continue;
    const int64_t a = pairs[2 * k], b = pairs[2 * k + 1];
    const T t = q_cur[i * C + a];
    q_cur[i * C + a] = q_cur[i * C + b];
    q_cur[i * C + b] = t;
    if (rec) {
      T* r = ring_q + (slot * d + i) * C;
      r[a] = q_cur[i * C + a];
      r[b] = q_cur[i * C + b];
    }
    if (i == 0) {
      const double tx = x_cur[a];
      x_cur[a] = x_cur[b];
      x_cur[b] = tx;
      if (rec && ring_x) {
        ring_x[slot * C + a] = (beta ? beta[a] : 1.0) * x_cur[a];
        ring_x[slot * C + b] = (beta ? beta[b] : 1.0) * x_cur[b];
      }
    }
  }
}

template <typename T>
int exchange_impl(const hmc_chains* s, int64_t npairs, const int32_t* pairs, const double* u, int32_t* swapped,
                  int64_t* total, cudaStream_t st) {
  HMC_REQUIRE(s->dims > 0 && s->chains > 0 && s->q_cur && s->x_cur, "hmc_exchange: missing state");
  HMC_REQUIRE(npairs >= 0 && 2 * npairs <= s->chains, "hmc_exchange: %lld pairs for %lld chains",
              (long long)npairs, (long long)s->chains);
  if (npairs == 0) return HMC_OK;
  HMC_REQUIRE(pairs && u && swapped, "hmc_exchange: null pairs, uniforms or decisions");
  exchange_decide_kernel<<<blocks_for(npairs, 256), 256, 0, st>>>(npairs, s->chains, pairs, u, s->beta, s->x_cur,
                                                                   swapped, total);
  HMC_TRY(check_launch("exchange_decide_kernel"));
  if (s->ring_q) HMC_REQUIRE(s->ring_slots > 0 && s->thinning > 0, "hmc_exchange: bad sample ring");
  exchange_swap_kernel<T><<<ew_grid(npairs * s->dims), 256, 0, st>>>(
      npairs, s->dims, s->chains, pairs, swapped, (T*)s->q_cur, s->x_cur, s->proposal, (T*)s->ring_q, s->ring_x,
      s->ring_slots, s->thinning, s->beta);
  return check_launch("exchange_swap_kernel");
}

}  // namespace hmc

using namespace hmc;

extern "C" {

int hmc_exchange(const hmc_chains* s, int64_t npairs, const int32_t* pairs, const double* u, int32_t* swapped,
                 int64_t* accepted_total, void* stream) {
  if (!s) return fail(HMC_ERR_INVALID_ARG, "hmc_exchange: null state");
  return HMC_DISPATCH(s->dtype, T, [&] {
    return exchange_impl<T>(s, npairs, pairs, u, swapped, accepted_total, as_stream(stream));
  });
}

int hmc_begin_trajectory(const hmc_chains* s, double drift, void* stream) {
  if (!s) return fail(HMC_ERR_INVALID_ARG, "hmc_begin_trajectory: null state");
  return HMC_DISPATCH(s->dtype, T, [&] { return begin_impl<T>(s, drift, as_stream(stream)); });
}

int hmc_kick_drift(const hmc_chains* s, double kick, double drift, void* stream) {
  if (!s) return fail(HMC_ERR_INVALID_ARG, "hmc_kick_drift: null state");
  return HMC_DISPATCH(s->dtype, T, [&] { return kick_drift_impl<T>(s, kick, drift, as_stream(stream)); });
}

int hmc_end_trajectory(const hmc_chains* s, void* stream) {
  if (!s) return fail(HMC_ERR_INVALID_ARG, "hmc_end_trajectory: null state");
  return HMC_DISPATCH(s->dtype, T, [&] { return end_impl<T>(s, as_stream(stream)); });
}

int hmc_kinetic_energy(const hmc_chains* s, const void* p, double* out, void* stream) {
  if (!s) return fail(HMC_ERR_INVALID_ARG, "hmc_kinetic_energy: null state");
  return HMC_DISPATCH(s->dtype, T, [&] { return kinetic_impl<T>(s, p, out, as_stream(stream)); });
}

int hmc_kinetic_energy_gradient(const hmc_chains* s, const void* p, void* out, void* stream) {
  if (!s) return fail(HMC_ERR_INVALID_ARG, "hmc_kinetic_energy_gradient: null state");
  return HMC_DISPATCH(s->dtype, T, [&] { return kinetic_grad_impl<T>(s, p, out, as_stream(stream)); });
}

}  // extern "C"
