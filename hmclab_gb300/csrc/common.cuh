// Shared helpers of the hmclab_gb300 CUDA library: status handling, dtype
// dispatch, Philox4x32-10 and per-chain FP64 reductions over the [d][C]
// (dimension-major, chain-fastest) layout.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "hmclab_gb300.h"

namespace hmc {

// Records `msg` as the calling thread's last error and returns `code`.
int fail(int code, const char* fmt, ...);
// Maps a CUDA error to HMC_ERR_CUDA with the call site in the message.
int cuda_fail(cudaError_t e, const char* where);
// Counts launches issued by this library (reported to callers for audits).
void count_launch(int n = 1);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Limits of the bounded device waits, read by the launchers of the kernels
// that wait on tensor-copy barriers.  Production: 2 s, nothing withheld.
// hmc_set_wait_limits shortens the limit and makes block 0 of those kernels
// withhold its first barrier arrival, so a test can make a wait run out and
// check the status path without faulting or hanging the GPU.
struct WaitLimits {
  uint64_t ns;
  int withhold;
};
WaitLimits wait_limits();

// Check the launch that was just issued.
inline int check_launch(const char* where) {
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, where);
  return HMC_OK;
}

#define HMC_REQUIRE(cond, ...)                                   \
  do {                                                           \
    if (!(cond)) return ::hmc::fail(HMC_ERR_INVALID_ARG, __VA_ARGS__); \
  } while (0)

#define HMC_TRY(expr)            \
  do {                           \
    int _rc = (expr);            \
    if (_rc != HMC_OK) return _rc; \
  } while (0)

// Dispatch a templated launcher on the dtype code.
#define HMC_DISPATCH(dtype, T, ...)                                   \
  [&]() -> int {                                                      \
    if ((dtype) == HMC_F32) { using T = float; return __VA_ARGS__(); }  \
    if ((dtype) == HMC_F64) { using T = double; return __VA_ARGS__(); } \
    return ::hmc::fail(HMC_ERR_INVALID_ARG, "unknown dtype code %d", (int)(dtype)); \
  }()

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC 2011): 10 rounds of the 4x32 multiply-xorshift round with
// the Weyl key schedule.
// ---------------------------------------------------------------------------
__host__ __device__ inline uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __umulhi(a, b);
#else
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

__host__ __device__ inline uint4 philox4x32_10(uint4 ctr, uint2 key) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      key.x += W0;
      key.y += W1;
    }
    const uint32_t hi0 = mulhi32(M0, ctr.x), lo0 = M0 * ctr.x;
    const uint32_t hi1 = mulhi32(M1, ctr.z), lo1 = M1 * ctr.z;
    ctr = make_uint4(hi1 ^ ctr.y ^ key.x, lo1, hi0 ^ ctr.w ^ key.y, lo0);
  }
  return ctr;
}

// Counter purposes: keep the momentum and scalar streams disjoint.
enum : uint32_t { PURPOSE_MOMENTUM = 0u, PURPOSE_SCALARS = 1u };

// Uniform in (0, 1) from 32 bits (never 0, never 1).
__device__ inline float u01f(uint32_t x) { return ((float)(x >> 8) + 0.5f) * (1.0f / 16777216.0f); }
// Uniform in (0, 1) with 53 bits from two words.
__device__ inline double u01d(uint32_t a, uint32_t b) {
  const uint64_t v = ((uint64_t)a << 21) ^ (uint64_t)(b >> 11);  // 53 bits
  return ((double)v + 0.5) * (1.0 / 9007199254740992.0);
}

// Four standard normals for (row quad, chain, proposal) by Box-Muller.
template <typename T>
__device__ inline void philox_normal4(uint64_t seed, uint32_t quad, uint32_t chain, uint64_t proposal,
                                      uint32_t purpose, T out[4]);

template <>
__device__ inline void philox_normal4<float>(uint64_t seed, uint32_t quad, uint32_t chain,
                                             uint64_t proposal, uint32_t purpose, float out[4]) {
  const uint4 r = philox4x32_10(
      make_uint4(quad, chain, (uint32_t)proposal, ((uint32_t)(proposal >> 32) & 0x0FFFFFFFu) | (purpose << 28)),
      make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
  const float u1 = u01f(r.x), u2 = u01f(r.y), u3 = u01f(r.z), u4 = u01f(r.w);
  const float a = sqrtf(-2.0f * logf(u1)), b = sqrtf(-2.0f * logf(u3));
  const float t1 = 6.283185307179586f * u2, t2 = 6.283185307179586f * u4;
  out[0] = a * cosf(t1);
  out[1] = a * sinf(t1);
  out[2] = b * cosf(t2);
  out[3] = b * sinf(t2);
}

template <>
__device__ inline void philox_normal4<double>(uint64_t seed, uint32_t quad, uint32_t chain,
                                              uint64_t proposal, uint32_t purpose, double out[4]) {
  // Two Philox blocks give 53-bit uniforms for the FP64 verification mode.
  const uint2 key = make_uint2((uint32_t)seed, (uint32_t)(seed >> 32));
  const uint32_t w = ((uint32_t)(proposal >> 32) & 0x07FFFFFFu) | (purpose << 28);
  const uint4 r0 = philox4x32_10(make_uint4(quad, chain, (uint32_t)proposal, w), key);
  const uint4 r1 = philox4x32_10(make_uint4(quad, chain, (uint32_t)proposal, w | 0x08000000u), key);
  const double u1 = u01d(r0.x, r0.y), u2 = u01d(r0.z, r0.w);
  const double u3 = u01d(r1.x, r1.y), u4 = u01d(r1.z, r1.w);
  const double a = sqrt(-2.0 * log(u1)), b = sqrt(-2.0 * log(u3));
  const double t1 = 6.283185307179586 * u2, t2 = 6.283185307179586 * u4;
  out[0] = a * cos(t1);
  out[1] = a * sin(t1);
  out[2] = b * cos(t2);
  out[3] = b * sin(t2);
}

// Per-chain scalar uniforms for proposal n: step factor and accept uniform.
__device__ inline void philox_scalars(uint64_t seed, uint32_t chain, uint64_t proposal, double* u_eps,
                                      double* u_acc) {
  const uint4 r = philox4x32_10(
      make_uint4(0u, chain, (uint32_t)proposal,
                 ((uint32_t)(proposal >> 32) & 0x0FFFFFFFu) | (PURPOSE_SCALARS << 28)),
      make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
  *u_eps = u01d(r.x, r.y);
  *u_acc = u01d(r.z, r.w);
}

// ---------------------------------------------------------------------------
// Per-chain reductions over the [d][C] layout: a block owns 32 consecutive
// chains (threadIdx.x) and RY row lanes (threadIdx.y); rows are strided by RY
// and partial sums are combined in a fixed order, so results are
// bit-reproducible run to run.
// ---------------------------------------------------------------------------
constexpr int RED_X = 32;
constexpr int RED_Y = 8;

__device__ inline double block_chain_sum(double v, double (*sh)[RED_X + 1]) {
  sh[threadIdx.y][threadIdx.x] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.y == 0) {
#pragma unroll
    for (int y = 0; y < RED_Y; ++y) s += sh[y][threadIdx.x];
  }
  __syncthreads();
  return s;  // valid in row lane 0
}

inline dim3 red_grid(int64_t C) { return dim3((unsigned)((C + RED_X - 1) / RED_X)); }
inline dim3 red_block() { return dim3(RED_X, RED_Y); }

inline unsigned blocks_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 0x7FFFFFFF) b = 0x7FFFFFFF;
  return (unsigned)b;
}

}  // namespace hmc
