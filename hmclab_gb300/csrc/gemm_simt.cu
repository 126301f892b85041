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

// blockIdx.z selects the k range [z * k_chunk, (z + 1) * k_chunk); with
// `partial` set, the raw sums of that range go to partial[z][m][n] and the
// epilogue is left to splitk_reduce_kernel.
template <typename T>
__global__ void __launch_bounds__(256) gemm_kernel(int64_t M, int64_t N, int64_t K, T alpha, const T* __restrict__ A,
                                                   const T* __restrict__ B, const T* __restrict__ bias, T bias_scale,
                                                   const T* __restrict__ row_scale, T* out, int accumulate,
                                                   int64_t k_chunk, T* partial) {
  __shared__ T As[BK][BM + 1];
  __shared__ T Bs[BK][BN + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int64_t row0 = (int64_t)blockIdx.y * BM, col0 = (int64_t)blockIdx.x * BN;
  T acc[TM][TN];
#pragma unroll
  for (int a = 0; a < TM; ++a)
#pragma unroll
    for (int b = 0; b < TN; ++b) acc[a][b] = (T)0;

  const int64_t kb = (int64_t)blockIdx.z * k_chunk;
  const int64_t ke = kb + k_chunk < K ? kb + k_chunk : K;
  for (int64_t k0 = kb; k0 < ke; k0 += BK) {
    // A tile: BM x BK, 1024 elements, 4 per thread.
    for (int e = threadIdx.x; e < BM * BK; e += 256) {
      const int r = e / BK, kk = e % BK;
      const int64_t gr = row0 + r, gk = k0 + kk;
      As[kk][r] = (gr < M && gk < ke) ? A[gr * K + gk] : (T)0;
    }
    for (int e = threadIdx.x; e < BK * BN; e += 256) {
      const int kk = e / BN, cc = e % BN;
      const int64_t gk = k0 + kk, gc = col0 + cc;
      Bs[kk][cc] = (gk < ke && gc < N) ? B[gk * N + gc] : (T)0;
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
  if (partial) {
    T* p = partial + (int64_t)blockIdx.z * M * N;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int64_t r = row0 + ty + 16 * i;
      if (r >= M) continue;
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const int64_t c = col0 + tx + 16 * j;
        if (c < N) p[r * N + c] = acc[i][j];
      }
    }
    return;
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

// out = alpha * sum_z partial[z] (+ out), summed in z order.
template <typename T>
__global__ void splitk_reduce_kernel(int64_t mn, int splits, T alpha, const T* __restrict__ partial, T* out,
                                     int accumulate) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < mn; e += (int64_t)gridDim.x * blockDim.x) {
    T s = (T)0;
    for (int z = 0; z < splits; ++z) s += partial[(int64_t)z * mn + e];
    s *= alpha;
    out[e] = accumulate ? out[e] + s : s;
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
  const int64_t kc = k > 0 ? k : 1;
  if (dtype == HMC_F32)
    gemm_kernel<float><<<grid, 256, 0, stream>>>(m, n, k, (float)alpha, (const float*)A, (const float*)B,
                                                  (const float*)bias, (float)bias_scale, (const float*)row_scale,
                                                  (float*)out, accumulate, kc, nullptr);
  else if (dtype == HMC_F64)
    gemm_kernel<double><<<grid, 256, 0, stream>>>(m, n, k, alpha, (const double*)A, (const double*)B,
                                                   (const double*)bias, bias_scale, (const double*)row_scale,
                                                   (double*)out, accumulate, kc, nullptr);
  else
    return fail(HMC_ERR_INVALID_ARG, "hmc_gemm: unknown dtype %d", dtype);
  return check_launch("gemm_kernel");
}

int gemm_splitk(int dtype, int64_t m, int64_t n, int64_t k, double alpha, const void* A, const void* B, void* out,
                int accumulate, void* work, int64_t work_elems, cudaStream_t stream) {
  HMC_REQUIRE(m >= 0 && n >= 0 && k >= 0, "hmc_gemm_splitk: negative size");
  if (m == 0 || n == 0) return HMC_OK;
  HMC_REQUIRE(A && B && out && work, "hmc_gemm_splitk: null operand");
  HMC_REQUIRE(work_elems >= m * n, "hmc_gemm_splitk: work holds fewer than m * n elements");
  HMC_REQUIRE(dtype == HMC_F32 || dtype == HMC_F64, "hmc_gemm_splitk: unknown dtype %d", dtype);
  HMC_REQUIRE((m + BM - 1) / BM <= 65535, "hmc_gemm_splitk: matrix too large");
  const int64_t tiles = ((n + BN - 1) / BN) * ((m + BM - 1) / BM);
  // about four CTAs per SM in total, at least 256 k per split
  int64_t splits = (4 * 152 + tiles - 1) / tiles;
  const int64_t by_k = (k + 255) / 256;
  const int64_t by_work = work_elems / (m * n);
  splits = splits < by_k ? splits : by_k;
  splits = splits < by_work ? splits : by_work;
  splits = splits < 65535 ? splits : 65535;
  splits = splits > 1 ? splits : 1;
  int64_t chunk = k > 0 ? (k + splits - 1) / splits : 1;
  chunk = (chunk + BK - 1) / BK * BK;
  splits = k > 0 ? (k + chunk - 1) / chunk : 1;
  const dim3 grid((unsigned)((n + BN - 1) / BN), (unsigned)((m + BM - 1) / BM), (unsigned)splits);
  const unsigned rblocks = blocks_for(m * n, 256) < 152u * 8u ? blocks_for(m * n, 256) : 152u * 8u;
  if (dtype == HMC_F32) {
    gemm_kernel<float><<<grid, 256, 0, stream>>>(m, n, k, 1.f, (const float*)A, (const float*)B, nullptr, 0.f,
                                                  nullptr, nullptr, 0, chunk, (float*)work);
    HMC_TRY(check_launch("gemm_kernel (split k)"));
    splitk_reduce_kernel<float><<<rblocks, 256, 0, stream>>>(m * n, (int)splits, (float)alpha, (const float*)work,
                                                            (float*)out, accumulate);
  } else {
    gemm_kernel<double><<<grid, 256, 0, stream>>>(m, n, k, 1.0, (const double*)A, (const double*)B, nullptr, 0.0,
                                                   nullptr, nullptr, 0, chunk, (double*)work);
    HMC_TRY(check_launch("gemm_kernel (split k)"));
    splitk_reduce_kernel<double><<<rblocks, 256, 0, stream>>>(m * n, (int)splits, alpha, (const double*)work,
                                                             (double*)out, accumulate);
  }
  return check_launch("splitk_reduce_kernel");
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

extern "C" int hmc_gemm_splitk(int dtype, int64_t m, int64_t n, int64_t k, double alpha, const void* A,
                               const void* B, void* out, int accumulate, void* work, int64_t work_elems,
                               void* stream) {
  return hmc::gemm_splitk(dtype, m, n, k, alpha, A, B, out, accumulate, work, work_elems, hmc::as_stream(stream));
}
