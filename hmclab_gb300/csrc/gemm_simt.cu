// General row-major matrix product on the CUDA cores:
//   out[m][n] = alpha * A[m][k] B[k][n] + bias[m] + (accumulate ? out : 0).
// Used for the FP64 verification path (dense LinearMatrix at d = 50, full mass
// matrices, full-covariance Normal priors) and for small FP32 products.  The
// FP32 production contraction of the dense LinearMatrix runs on the tensor
// cores (dense_tc.cu).
#include "common.cuh"

namespace hmc {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, TM = 4, TN = 4;

template <typename T>
__global__ void __launch_bounds__(256) gemm_kernel(int64_t M, int64_t N, int64_t K, T alpha, const T* __restrict__ A,
                                                   const T* __restrict__ B, const T* __restrict__ bias, T bias_scale,
                                                   const T* __restrict__ row_scale, T* out, int accumulate) {
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int64_t row0 = (int64_t)blockIdx.y * BM, col0 = (int64_t)blockIdx.x * BN;
  T acc[TM][TN];
#pragma unroll
  for (int a = 0; a < TM; ++a)
#pragma unroll
    for (int b = 0; b < TN; ++b) acc[a][b] = (T)0;

  for (int64_t k0 = 0; k0 < K; k0 += BK) {
    // A tile: BM x BK, 1024 elements, 4 per thread.
    for (int e = threadIdx.x; e < BM * BK; e += 256) {
      const int r = e / BK, kk = e % BK;
      const int64_t gr = row0 + r, gk = k0 + kk;
      As[kk][r] = (gr < M && gk < K) ? A[gr * K + gk] : (T)0;
    }
    for (int e = threadIdx.x; e < BK * BN; e += 256) {
      const int kk = e / BN, cc = e % BN;
      const int64_t gk = k0 + kk, gc = col0 + cc;
      Bs[kk][cc] = (gk < K && gc < N) ? B[gk * N + gc] : (T)0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] += a[i] * b[j];
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int64_t r = row0 + ty + 16 * i;
    if (r >= M) continue;
    const T bv = bias ? bias_scale * bias[r] : (T)0;
    const T rs = row_scale ? row_scale[r] : (T)1;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int64_t c = col0 + tx + 16 * j;
      if (c >= N) continue;
      T v = alpha * acc[i][j] + bv;
      if (row_scale) v *= rs;
      if (accumulate) v += out[r * N + c];
      out[r * N + c] = v;
    }
  }
}

}  // namespace

// out = (alpha * A B + bias_scale * bias[m]) * row_scale[m] + (accumulate ? out : 0)
int gemm_ex(int dtype, int64_t m, int64_t n, int64_t k, double alpha, const void* A, const void* B, const void* bias,
            double bias_scale, const void* row_scale, void* out, int accumulate, cudaStream_t stream) {
  HMC_REQUIRE(m >= 0 && n >= 0 && k >= 0, "hmc_gemm: negative size");
  if (m == 0 || n == 0) return HMC_OK;
  HMC_REQUIRE(A && B && out, "hmc_gemm: null operand");
  HMC_REQUIRE((n + BN - 1) / BN <= 0x7FFFFFFF && (m + BM - 1) / BM <= 65535, "hmc_gemm: matrix too large");
  const dim3 grid((unsigned)((n + BN - 1) / BN), (unsigned)((m + BM - 1) / BM));
  if (dtype == HMC_F32)
    gemm_kernel<float><<<grid, 256, 0, stream>>>(m, n, k, (float)alpha, (const float*)A, (const float*)B,
                                                  (const float*)bias, (float)bias_scale, (const float*)row_scale,
                                                  (float*)out, accumulate);
  else if (dtype == HMC_F64)
    gemm_kernel<double><<<grid, 256, 0, stream>>>(m, n, k, alpha, (const double*)A, (const double*)B,
                                                   (const double*)bias, bias_scale, (const double*)row_scale,
                                                   (double*)out, accumulate);
  else
    return fail(HMC_ERR_INVALID_ARG, "hmc_gemm: unknown dtype %d", dtype);
  return check_launch("gemm_kernel");
}

int gemm_dispatch(int dtype, int64_t m, int64_t n, int64_t k, double alpha, const void* A, const void* B,
                  const void* bias, void* out, int accumulate, cudaStream_t stream) {
  return gemm_ex(dtype, m, n, k, alpha, A, B, bias, 1.0, nullptr, out, accumulate, stream);
}

}  // namespace hmc

extern "C" int hmc_gemm(int dtype, int64_t m, int64_t n, int64_t k, double alpha, const void* A, const void* B,
                        const void* bias, void* out, int accumulate, void* stream) {
  return hmc::gemm_dispatch(dtype, m, n, k, alpha, A, B, bias, out, accumulate, hmc::as_stream(stream));
}
