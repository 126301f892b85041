// Element-wise kernels of the scalar-potential surrogate; its contractions run
// in dense_tc.cu (hmc_tc_mlp, OUT and WGRAD modes).
//
// The surrogate is a potential f(x) = w3 . GELU(W2 GELU(W1 x + b1) + b2)
// + x^T A x / 2 + beta . x of the normalised position x = (q - mu) / s; the
// leapfrog uses its exact gradient grad_q f = grad_x f / s, so the surrogate
// field is conservative (the Jacobian of the proposal map it drives is
// symplectic and the surrogate Hamiltonian is conserved up to the
// integrator's error), unlike a network that outputs a gradient directly.
//   gradient pass:  delta2 = w3 * GELU'(z2),  u1 = W2^T delta2,
//                   delta1 = u1 * GELU'(z1),  grad_x f = W1^T delta1 + A x + beta
// It is trained by matching grad_x f to the exact gradients (Sobolev-type
// regression), which needs the derivative of the gradient pass with respect
// to the weights ("double backpropagation", Drucker & Le Cun 1992): with
// e = dLoss / d(grad_x f),
//   dbar1 = W1 e;  ubar1 = dbar1 * GELU'(z1);  zbar1 = dbar1 * u1 * GELU''(z1)
//   dbar2 = W2 ubar1;  zbar2 = dbar2 * w3 * GELU''(z2);  dw3 = sum_b dbar2 * GELU'(z2)
//   abar1 = W2^T zbar2;  zbar1 += abar1 * GELU'(z1)
//   dW1 = delta1^T e + zbar1^T x,  dW2 = delta2^T ubar1 + zbar2^T a1,
//   db1 = sum_b zbar1,  db2 = sum_b zbar2.
// A and beta are the symmetrised ridge fit of the gradients and stay fixed.
#include <cuda_bf16.h>

#include "common.cuh"

namespace hmc {
namespace pot {

// GELU(z) = z Phi(z): first and second derivatives Phi(z) + z phi(z) and
// phi(z) (2 - z^2), with Phi(z) = erfc(-z / sqrt 2) / 2 as in the forward
// epilogue of the contraction kernel.
__device__ __forceinline__ float normal_pdf(float z) { return 0.39894228040143268f * __expf(-0.5f * z * z); }
__device__ __forceinline__ float gelu_d1(float z) {
  return 0.5f * erfcf(-z * 0.70710678118654752f) + z * normal_pdf(z);
}
__device__ __forceinline__ float gelu_d2(float z) { return normal_pdf(z) * (2.f - z * z); }

// One 32 x 32 tile of a [B][n] result per block (block 32 x 8): the value of
// element (b, j) for the selected mode goes to out_bf [B][ld_bf] (BF16), to
// out_t [n][ld_t] (BF16, transposed through shared memory, nullable) and, in
// DBAR1 mode, out_f [B][ldf] receives in * aux * GELU''(z).
__global__ void elementwise_kernel(int mode, int64_t B, int64_t n, const float* __restrict__ in, int64_t ldi,
                                   const float* __restrict__ z, int64_t ldz, const float* __restrict__ aux,
                                   int64_t ldaux, const float* __restrict__ vec, __nv_bfloat16* out_bf,
                                   int64_t ld_bf, __nv_bfloat16* out_t, int64_t ld_t, float* out_f, int64_t ldf) {
  __shared__ float tile[32][33];
  const int64_t j0 = (int64_t)blockIdx.x * 32, b0 = (int64_t)blockIdx.y * 32;
  const int64_t j = j0 + threadIdx.x;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t b = b0 + y;
    float v = 0.f;
    if (b < B && j < n) {
      const float zz = z[b * ldz + j];
      switch (mode) {
        case HMC_POT_DELTA2:
          v = vec[j] * gelu_d1(zz);
          break;
        case HMC_POT_DELTA1:
          v = in[b * ldi + j] * gelu_d1(zz);
          break;
        case HMC_POT_DBAR1: {
          const float x = in[b * ldi + j];
          v = x * gelu_d1(zz);
          out_f[b * ldf + j] = x * aux[b * ldaux + j] * gelu_d2(zz);
          break;
        }
        case HMC_POT_DBAR2:
          v = in[b * ldi + j] * vec[j] * gelu_d2(zz);
          break;
        default:  // HMC_POT_ZBAR1
          v = aux[b * ldaux + j] + in[b * ldi + j] * gelu_d1(zz);
          break;
      }
      out_bf[b * ld_bf + j] = __float2bfloat16_rn(v);
    }
    tile[y][threadIdx.x] = v;
  }
  if (out_t == nullptr) return;
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t jj = j0 + y, b = b0 + threadIdx.x;
    if (jj < n && b < B) out_t[jj * ld_t + b] = __float2bfloat16_rn(tile[threadIdx.x][y]);
  }
}

// dw3[j] = sum_b dbar2[b][j] GELU'(z2[b][j]): a block takes 32 columns, its
// 16 thread rows take every 16th batch row, and the 16 partial sums of a
// column are added in a fixed order (deterministic).
__global__ void w3_grad_kernel(int64_t B, int64_t n, const float* __restrict__ in, int64_t ldi,
                               const float* __restrict__ z, int64_t ldz, float* g) {
  __shared__ float part[16][33];
  const int64_t j = (int64_t)blockIdx.x * 32 + threadIdx.x;
  float s = 0.f;
  if (j < n)
    for (int64_t b = threadIdx.y; b < B; b += 16) s += in[b * ldi + j] * gelu_d1(z[b * ldz + j]);
  part[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && j < n) {
    float t = 0.f;
    for (int y = 0; y < 16; ++y) t += part[y][threadIdx.x];
    g[j] = t;
  }
}

// Loss 0.5 sum_b |y_b - t_b|^2 (partials per block) and e = scale * (y - t) / B
// as BF16 e [B][lde] and e_t [n][ldet].
__global__ void loss_kernel(int64_t B, int64_t n, const float* __restrict__ y, int64_t ldy,
                            const float* __restrict__ t, int64_t ldt, const float* __restrict__ scale,
                            __nv_bfloat16* e, int64_t lde, __nv_bfloat16* et, int64_t ldet, double* partial) {
  __shared__ double sh[256];
  double acc = 0.0;
  const int64_t total = B * n;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = k / n, r = k % n;
    const float diff = y[b * ldy + r] - t[b * ldt + r];
    acc += 0.5 * (double)diff * (double)diff;
    const __nv_bfloat16 v = __float2bfloat16_rn(scale[r] * diff / (float)B);
    e[b * lde + r] = v;
    et[r * ldet + b] = v;
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// One warp: lane l adds partials l, l + 32, ...; the lanes' sums are combined
// by a fixed shuffle tree (deterministic).
__global__ void sum_kernel(int n, const double* __restrict__ p, double scale, double* out) {
  double s = 0.0;
  for (int k = threadIdx.x; k < n; k += 32) s += p[k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (threadIdx.x == 0) *out = s * scale;
}

// Value matching.  The exact misfit U is known wherever an exact gradient
// was taken (the forward simulation that precedes an adjoint gives it), and
// the acceptance of a surrogate trajectory depends on how well f tracks U
// between its end points, so the loss can also match values:
//   L_v = 0.5 w mean_b (r_b - rbar)^2,  r_b = v_b - t_b,  v_b = w3 . a2_b,
// with t_b = U_b minus the (fixed) quadratic part at x_b; centring on the
// batch mean removes the potential's free constant.  dL_v / dv_b =
// w (r_b - rbar) / B = dv_b, and the weight gradients are those of v scaled
// per row: dw3 += sum_b dv_b a2_b, dz2_b = dv_b delta2_b, dz1_b = dv_b delta1_b
// (delta2 = w3 GELU'(z2) and delta1 = (W2^T delta2) GELU'(z1) are the
// gradient pass's own intermediates).
// One block of B <= 1024 threads; a2 is the forward pass's BF16 activation.
__global__ void value_residual_kernel(int B, int h, const __nv_bfloat16* __restrict__ a2, int64_t lda,
                                      const float* __restrict__ w3, const double* __restrict__ targets,
                                      const int32_t* __restrict__ idx, float weight, float* dv, double* loss) {
  __shared__ double sh[1024];
  const int b = threadIdx.x;
  double r = 0.0;
  if (b < B) {
    float v = 0.f;
    for (int j = 0; j < h; ++j) v = fmaf(w3[j], __bfloat162float(a2[(int64_t)b * lda + j]), v);
    r = (double)v - targets[idx[b]];
  }
  sh[b] = r;
  __syncthreads();
  for (int w = 512; w > 0; w >>= 1) {  // fixed-order tree: deterministic
    if (b < w && b + w < (int)blockDim.x) sh[b] += sh[b + w];
    __syncthreads();
  }
  const double rbar = sh[0] / B;
  __syncthreads();
  const double c = b < B ? r - rbar : 0.0;
  if (b < B) dv[b] = (float)(weight * c / B);
  sh[b] = c * c;
  __syncthreads();
  for (int w = 512; w > 0; w >>= 1) {
    if (b < w && b + w < (int)blockDim.x) sh[b] += sh[b + w];
    __syncthreads();
  }
  if (b == 0) *loss = 0.5 * weight * sh[0] / B;
}

// out[j] += sum_b dv[b] in[b][j] (in BF16 [B][ld]); block: 32 columns x 16
// batch rows, partial sums added in a fixed order.
__global__ void weighted_colsum_kernel(int64_t B, int64_t n, const __nv_bfloat16* __restrict__ in, int64_t ld,
                                       const float* __restrict__ dv, float* out) {
  __shared__ float part[16][33];
  const int64_t j = (int64_t)blockIdx.x * 32 + threadIdx.x;
  float s = 0.f;
  if (j < n)
    for (int64_t b = threadIdx.y; b < B; b += 16) s = fmaf(dv[b], __bfloat162float(in[b * ld + j]), s);
  part[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && j < n) {
    float t = 0.f;
    for (int y = 0; y < 16; ++y) t += part[y][threadIdx.x];
    out[j] += t;
  }
}

// out_t[r][b] = in_t[r][b] dv[b] (BF16, rows x B of [rows][ld] arrays).
__global__ void scale_columns_kernel(int64_t rows, int64_t B, const __nv_bfloat16* __restrict__ in_t, int64_t ldi,
                                     const float* __restrict__ dv, __nv_bfloat16* out_t, int64_t ldo) {
  const int64_t total = rows * B;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = k / B, b = k - r * B;
    out_t[r * ldo + b] = __float2bfloat16_rn(__bfloat162float(in_t[r * ldi + b]) * dv[b]);
  }
}

// dst[r][k0 + k] = bf16(scale[r] * src(r, k)) for r < rows, k < cols, with
// src(r, k) = src[k][r] (transposed) or src[r][k].
__global__ void scaled_cast_kernel(int64_t rows, int64_t cols, const float* __restrict__ src, int64_t lds,
                                   int transposed, const float* __restrict__ scale, __nv_bfloat16* dst, int64_t ldd,
                                   int64_t k0) {
  __shared__ float tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  if (transposed) {
    // read src[k][r] along r (coalesced), write dst along k
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
      const int64_t k = c0 + y, r = r0 + threadIdx.x;
      tile[y][threadIdx.x] = (k < cols && r < rows) ? src[k * lds + r] : 0.f;
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
      const int64_t r = r0 + y, k = c0 + threadIdx.x;
      if (r < rows && k < cols) dst[r * ldd + k0 + k] = __float2bfloat16_rn(scale[r] * tile[threadIdx.x][y]);
    }
  } else {
    for (int y = threadIdx.y; y < 32; y += blockDim.y) {
      const int64_t r = r0 + y, k = c0 + threadIdx.x;
      if (r < rows && k < cols) dst[r * ldd + k0 + k] = __float2bfloat16_rn(scale[r] * src[r * lds + k]);
    }
  }
}

}  // namespace pot
}  // namespace hmc

using namespace hmc;
using namespace hmc::pot;

extern "C" {

HMC_API int hmc_pot_elementwise(int mode, int64_t B, int64_t n, const float* in, int64_t ldi, const float* z,
                                int64_t ldz, const float* aux, int64_t ldaux, const float* vec, void* out_bf,
                                int64_t ld_bf, void* out_t, int64_t ld_t, float* out_f, int64_t ldf, void* stream) {
  HMC_REQUIRE(B > 0 && n > 0 && z && out_bf && ldz >= n && ld_bf >= n, "hmc_pot_elementwise: bad arguments");
  HMC_REQUIRE(out_t == nullptr || ld_t >= B, "hmc_pot_elementwise: transposed pitch");
  switch (mode) {
    case HMC_POT_DELTA2:
      HMC_REQUIRE(vec != nullptr, "hmc_pot_elementwise: DELTA2 needs vec");
      break;
    case HMC_POT_DELTA1:
      HMC_REQUIRE(in && ldi >= n, "hmc_pot_elementwise: DELTA1 needs in");
      break;
    case HMC_POT_DBAR1:
      HMC_REQUIRE(in && ldi >= n && aux && ldaux >= n && out_f && ldf >= n, "hmc_pot_elementwise: DBAR1 buffers");
      break;
    case HMC_POT_DBAR2:
      HMC_REQUIRE(in && ldi >= n && vec, "hmc_pot_elementwise: DBAR2 buffers");
      break;
    case HMC_POT_ZBAR1:
      HMC_REQUIRE(in && ldi >= n && aux && ldaux >= n, "hmc_pot_elementwise: ZBAR1 buffers");
      break;
    default:
      return fail(HMC_ERR_INVALID_ARG, "hmc_pot_elementwise: unknown mode %d", mode);
  }
  HMC_REQUIRE((B + 31) / 32 <= 65535, "hmc_pot_elementwise: batch too large");
  const dim3 grid((unsigned)((n + 31) / 32), (unsigned)((B + 31) / 32));
  elementwise_kernel<<<grid, dim3(32, 8), 0, as_stream(stream)>>>(mode, B, n, in, ldi, z, ldz, aux, ldaux, vec,
                                                                  (__nv_bfloat16*)out_bf, ld_bf,
                                                                  (__nv_bfloat16*)out_t, ld_t, out_f, ldf);
  return check_launch("pot elementwise_kernel");
}

HMC_API int hmc_pot_w3_grad(int64_t B, int64_t n, const float* in, int64_t ldi, const float* z, int64_t ldz,
                            float* g, void* stream) {
  HMC_REQUIRE(B > 0 && n > 0 && in && z && g && ldi >= n && ldz >= n, "hmc_pot_w3_grad: bad arguments");
  w3_grad_kernel<<<(unsigned)((n + 31) / 32), dim3(32, 16), 0, as_stream(stream)>>>(B, n, in, ldi, z, ldz, g);
  return check_launch("pot w3_grad_kernel");
}

HMC_API int hmc_pot_loss(int64_t B, int64_t n, const float* y, int64_t ldy, const float* t, int64_t ldt,
                         const float* scale, void* e, int64_t lde, void* e_t, int64_t ldet, double* loss,
                         void* stream) {
  HMC_REQUIRE(B > 0 && n > 0 && ldy >= n && ldt >= n && lde >= n && ldet >= B, "hmc_pot_loss: bad sizes");
  HMC_REQUIRE(y && t && scale && e && e_t && loss, "hmc_pot_loss: null argument");
  const unsigned b = blocks_for(B * n, 256);
  const unsigned grid = b > 1024u ? 1024u : b;
  loss_kernel<<<grid, 256, 0, as_stream(stream)>>>(B, n, y, ldy, t, ldt, scale, (__nv_bfloat16*)e, lde,
                                                   (__nv_bfloat16*)e_t, ldet, loss + 1);
  HMC_TRY(check_launch("pot loss_kernel"));
  sum_kernel<<<1, 32, 0, as_stream(stream)>>>((int)grid, loss + 1, 1.0 / (double)B, loss);
  return check_launch("pot sum_kernel");
}

HMC_API int hmc_pot_value_residual(int64_t B, int64_t h, const void* a2, int64_t lda, const float* w3,
                                   const double* targets, const int32_t* idx, float weight, float* dv, double* loss,
                                   void* stream) {
  HMC_REQUIRE(B > 0 && B <= 1024 && h > 0 && lda >= h, "hmc_pot_value_residual: bad sizes");
  HMC_REQUIRE(a2 && w3 && targets && idx && dv && loss, "hmc_pot_value_residual: null argument");
  value_residual_kernel<<<1, 1024, 0, as_stream(stream)>>>((int)B, (int)h, (const __nv_bfloat16*)a2, lda, w3,
                                                           targets, idx, weight, dv, loss);
  return check_launch("pot value_residual_kernel");
}

HMC_API int hmc_pot_weighted_colsum(int64_t B, int64_t n, const void* in, int64_t ld, const float* dv, float* out,
                                    void* stream) {
  HMC_REQUIRE(B > 0 && n > 0 && ld >= n && in && dv && out, "hmc_pot_weighted_colsum: bad arguments");
  weighted_colsum_kernel<<<(unsigned)((n + 31) / 32), dim3(32, 16), 0, as_stream(stream)>>>(
      B, n, (const __nv_bfloat16*)in, ld, dv, out);
  return check_launch("pot weighted_colsum_kernel");
}

HMC_API int hmc_pot_scale_columns(int64_t rows, int64_t B, const void* in_t, int64_t ldi, const float* dv,
                                  void* out_t, int64_t ldo, void* stream) {
  HMC_REQUIRE(rows > 0 && B > 0 && ldi >= B && ldo >= B && in_t && dv && out_t, "hmc_pot_scale_columns: bad arguments");
  const unsigned g = blocks_for(rows * B, 256);
  scale_columns_kernel<<<g > 4096u ? 4096u : g, 256, 0, as_stream(stream)>>>(
      rows, B, (const __nv_bfloat16*)in_t, ldi, dv, (__nv_bfloat16*)out_t, ldo);
  return check_launch("pot scale_columns_kernel");
}

HMC_API int hmc_pot_scaled_cast(int64_t rows, int64_t cols, const float* src, int64_t lds, int transposed,
                                const float* scale, void* dst, int64_t ldd, int64_t k0, void* stream) {
  HMC_REQUIRE(rows > 0 && cols > 0 && src && scale && dst && k0 >= 0 && ldd >= k0 + cols,
              "hmc_pot_scaled_cast: bad arguments");
  HMC_REQUIRE(lds >= (transposed ? rows : cols), "hmc_pot_scaled_cast: source pitch");
  HMC_REQUIRE((rows + 31) / 32 <= 65535, "hmc_pot_scaled_cast: too many rows");
  const dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
  scaled_cast_kernel<<<grid, dim3(32, 8), 0, as_stream(stream)>>>(rows, cols, src, lds, transposed, scale,
                                                                  (__nv_bfloat16*)dst, ldd, k0);
  return check_launch("pot scaled_cast_kernel");
}

}  // extern "C"
