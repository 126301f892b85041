// Element-wise and data-movement kernels of the MLP gradient surrogate; the
// contractions themselves run in dense_tc.cu (hmc_tc_mlp).
//
// The surrogate maps a normalised position x = (q - mu) / sigma to a
// normalised gradient y = (grad U - g_mu) / g_sigma with two GELU hidden
// layers, BF16 weights and activations and FP32 accumulation; it is trained
// with Adam on FP32 master weights.
#include <cuda_bf16.h>

#include "common.cuh"

namespace hmc {
namespace mlp {

inline unsigned grid_for(int64_t n) {
  const unsigned b = blocks_for(n, 256);
  return b > 152u * 32u ? 152u * 32u : b;
}

// q [d][C] -> x [C][ldx] (normalised, BF16), 32x32 tiles through shared memory.
// Only the d leading columns of each row are written: the contractions read
// exactly K = d columns, and the rest of a row may hold other data.
__global__ void input_kernel(int64_t d, int64_t C, const float* __restrict__ q, const float* __restrict__ mu,
                             const float* __restrict__ inv_s, __nv_bfloat16* x, int64_t ldx) {
  __shared__ float tile[32][33];
  const int64_t i0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t i = i0 + y, c = c0 + threadIdx.x;
    tile[y][threadIdx.x] = (i < d && c < C) ? (q[i * C + c] - mu[i]) * inv_s[i] : 0.f;
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t c = c0 + y, i = i0 + threadIdx.x;
    if (c < C && i < d) x[c * ldx + i] = __float2bfloat16_rn(tile[threadIdx.x][y]);
  }
}

__global__ void gather_kernel(int64_t B, int64_t d, const int32_t* __restrict__ idx, const float* __restrict__ qs,
                              const float* __restrict__ gs, const float* __restrict__ mu,
                              const float* __restrict__ inv_s, const float* __restrict__ gmu,
                              const float* __restrict__ ginv, __nv_bfloat16* x, int64_t ldx, __nv_bfloat16* xt,
                              int64_t ldxt, float* t, int64_t ldt) {
  const int64_t total = B * d;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / d, i = e % d;
    const int64_t row = idx[b];
    const __nv_bfloat16 xv = __float2bfloat16_rn((qs[row * d + i] - mu[i]) * inv_s[i]);
    x[b * ldx + i] = xv;
    xt[i * ldxt + b] = xv;
    t[b * ldt + i] = (gs[row * d + i] - gmu[i]) * ginv[i];
  }
}

// dY = (y - t) / B (BF16, both layouts) and the loss 0.5/B sum (y - t)^2.
__global__ void loss_kernel(int64_t B, int64_t n, const float* __restrict__ y, int64_t ldy,
                            const float* __restrict__ t, int64_t ldt, __nv_bfloat16* dy, int64_t lddy,
                            __nv_bfloat16* dyt, int64_t lddyt, double* loss_partial) {
  __shared__ double sh[256];
  double acc = 0.0;
  const int64_t total = B * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / n, r = e % n;
    const float diff = y[b * ldy + r] - t[b * ldt + r];
    acc += 0.5 * (double)diff * (double)diff;
    const __nv_bfloat16 v = __float2bfloat16_rn(diff / (float)B);
    dy[b * lddy + r] = v;
    dyt[r * lddyt + b] = v;
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss_partial[blockIdx.x] = sh[0];
}

// One warp: lane l adds partials l, l + 32, ...; the lanes' sums are combined
// by a fixed shuffle tree (deterministic).
__global__ void sum_partials_kernel(int n, const double* __restrict__ p, double scale, double* out) {
  double s = 0.0;
  for (int k = threadIdx.x; k < n; k += 32) s += p[k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (threadIdx.x == 0) *out = s * scale;
}

// One warp per row: db[r] = sum_c delta_t[r][c].
__global__ void bias_grad_kernel(int64_t n, int64_t B, const __nv_bfloat16* __restrict__ dt, int64_t ld, float* db) {
  const int64_t r = blockIdx.x * (int64_t)(blockDim.x / 32) + threadIdx.x / 32;
  const int lane = threadIdx.x % 32;
  if (r >= n) return;
  float s = 0.f;
  for (int64_t c = lane; c < B; c += 32) s += __bfloat162float(dt[r * ld + c]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) db[r] = s;
}

__global__ void adam_kernel(int64_t n, float* w, const float* __restrict__ g, float* m, float* v, float lr, float b1,
                            float b2, float eps, float c1, float c2) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const float gk = g[k];
    const float mk = b1 * m[k] + (1.f - b1) * gk;
    const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
    m[k] = mk;
    v[k] = vk;
    w[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
  }
}

__global__ void cast_kernel(int64_t rows, int64_t cols, const float* __restrict__ w, __nv_bfloat16* w16, int64_t ld,
                            __nv_bfloat16* w16t, int64_t ldt) {
  const int64_t total = rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / cols, c = e % cols;
    const __nv_bfloat16 v = __float2bfloat16_rn(w[e]);
    w16[r * ld + c] = v;
    w16t[c * ldt + r] = v;
  }
}

// src [d][C] -> dst rows base + c (each row holds d values).
__global__ void record_kernel(int64_t d, int64_t C, const float* __restrict__ src, float* dst, int64_t base) {
  __shared__ float tile[32][33];
  const int64_t i0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t i = i0 + y, c = c0 + threadIdx.x;
    tile[y][threadIdx.x] = (i < d && c < C) ? src[i * C + c] : 0.f;
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t c = c0 + y, i = i0 + threadIdx.x;
    if (c < C && i < d) dst[(base + c) * d + i] = tile[threadIdx.x][y];
  }
}

}  // namespace mlp
}  // namespace hmc

using namespace hmc;
using namespace hmc::mlp;

extern "C" {

HMC_API int hmc_mlp_input(int64_t d, int64_t C, const float* q, const float* mu, const float* inv_sigma, void* x,
                          int64_t ldx, void* stream) {
  HMC_REQUIRE(d > 0 && C > 0 && ldx >= d, "hmc_mlp_input: bad sizes");
  HMC_REQUIRE(q && mu && inv_sigma && x, "hmc_mlp_input: null argument");
  HMC_REQUIRE((d + 31) / 32 <= 65535, "hmc_mlp_input: too many features");
  const dim3 grid((unsigned)((C + 31) / 32), (unsigned)((d + 31) / 32));
  input_kernel<<<grid, dim3(32, 8), 0, as_stream(stream)>>>(d, C, q, mu, inv_sigma, (__nv_bfloat16*)x, ldx);
  return check_launch("mlp input_kernel");
}

HMC_API int hmc_mlp_gather(int64_t B, int64_t d, const int32_t* idx, const float* q_store, const float* g_store,
                           const float* mu, const float* inv_sigma, const float* g_mu, const float* g_inv_sigma,
                           void* x, int64_t ldx, void* x_t, int64_t ldxt, float* t, int64_t ldt, void* stream) {
  HMC_REQUIRE(B > 0 && d > 0 && ldx >= d && ldxt >= B && ldt >= d, "hmc_mlp_gather: bad sizes");
  HMC_REQUIRE(idx && q_store && g_store && mu && inv_sigma && g_mu && g_inv_sigma && x && x_t && t,
              "hmc_mlp_gather: null argument");
  gather_kernel<<<grid_for(B * d), 256, 0, as_stream(stream)>>>(B, d, idx, q_store, g_store, mu, inv_sigma, g_mu,
                                                               g_inv_sigma, (__nv_bfloat16*)x, ldx,
                                                               (__nv_bfloat16*)x_t, ldxt, t, ldt);
  return check_launch("mlp gather_kernel");
}

HMC_API int hmc_mlp_loss(int64_t B, int64_t n, const float* y, int64_t ldy, const float* t, int64_t ldt, void* dy,
                         int64_t lddy, void* dy_t, int64_t lddyt, double* loss, void* stream) {
  HMC_REQUIRE(B > 0 && n > 0 && ldy >= n && ldt >= n && lddy >= n && lddyt >= B, "hmc_mlp_loss: bad sizes");
  HMC_REQUIRE(y && t && dy && dy_t && loss, "hmc_mlp_loss: null argument");
  // loss partials live in the last 1024 doubles after *loss (caller buffer of 1025 doubles)
  const unsigned grid = grid_for(B * n) > 1024 ? 1024 : grid_for(B * n);
  loss_kernel<<<grid, 256, 0, as_stream(stream)>>>(B, n, y, ldy, t, ldt, (__nv_bfloat16*)dy, lddy,
                                                   (__nv_bfloat16*)dy_t, lddyt, loss + 1);
  HMC_TRY(check_launch("mlp loss_kernel"));
  sum_partials_kernel<<<1, 32, 0, as_stream(stream)>>>((int)grid, loss + 1, 1.0 / (double)B, loss);
  return check_launch("mlp sum_partials_kernel");
}

HMC_API int hmc_mlp_bias_grad(int64_t n, int64_t B, const void* delta_t, int64_t ld, float* db, void* stream) {
  HMC_REQUIRE(n > 0 && B > 0 && ld >= B && delta_t && db, "hmc_mlp_bias_grad: bad arguments");
  bias_grad_kernel<<<blocks_for(n, 8), 256, 0, as_stream(stream)>>>(n, B, (const __nv_bfloat16*)delta_t, ld, db);
  return check_launch("mlp bias_grad_kernel");
}

HMC_API int hmc_mlp_adam(int64_t n, float* w, const float* g, float* m, float* v, float lr, float beta1, float beta2,
                         float eps, int64_t step, void* stream) {
  HMC_REQUIRE(n > 0 && step > 0 && w && g && m && v, "hmc_mlp_adam: bad arguments");
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  adam_kernel<<<grid_for(n), 256, 0, as_stream(stream)>>>(n, w, g, m, v, lr, beta1, beta2, eps, c1, c2);
  return check_launch("mlp adam_kernel");
}

HMC_API int hmc_mlp_cast(int64_t rows, int64_t cols, const float* w, void* w16, int64_t ld, void* w16_t, int64_t ldt,
                         void* stream) {
  HMC_REQUIRE(rows > 0 && cols > 0 && ld >= cols && ldt >= rows && w && w16 && w16_t, "hmc_mlp_cast: bad arguments");
  cast_kernel<<<grid_for(rows * cols), 256, 0, as_stream(stream)>>>(rows, cols, w, (__nv_bfloat16*)w16, ld,
                                                                    (__nv_bfloat16*)w16_t, ldt);
  return check_launch("mlp cast_kernel");
}

HMC_API int hmc_mlp_record(int64_t d, int64_t C, const float* src, float* dst, int64_t base, void* stream) {
  HMC_REQUIRE(d > 0 && C > 0 && base >= 0 && src && dst, "hmc_mlp_record: bad arguments");
  HMC_REQUIRE((d + 31) / 32 <= 65535, "hmc_mlp_record: too many parameters");
  const dim3 grid((unsigned)((C + 31) / 32), (unsigned)((d + 31) / 32));
  record_kernel<<<grid, dim3(32, 8), 0, as_stream(stream)>>>(d, C, src, dst, base);
  return check_launch("mlp record_kernel");
}

}  // extern "C"
