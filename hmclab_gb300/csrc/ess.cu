// Multi-chain effective sample size of every parameter, on the device.
//
// The reference has no ESS estimator (its only mixing diagnostic is
// Helpers/Processing.py:6-13, a numpy autocorrelation).  This follows the
// split-chain multi-chain estimator of Gelman et al., Bayesian Data Analysis
// (3rd ed., section 11.5) as used by Stan: every chain is split into two
// halves (M = 2C half-chains of n = N/2 draws), the lag-t autocorrelation is
//   rho_t = 1 - (W - mean_m gamma_{m,t}) / var+,
// with W the mean within-half-chain variance, var+ = (n-1)/n W + B/n, and the
// sum of rho is truncated by Geyer's initial monotone sequence (pairs
// rho_{2k} + rho_{2k+1} summed while positive, made non-increasing):
//   ESS = M n / (-1 + 2 sum_k P_k).
// Samples are laid out [N][d][C] (the sampler's ring), chain fastest.
#include "common.cuh"

namespace hmc {
namespace {

constexpr int ESS_CH = 32;  // half-chains per block

// Per (parameter, block of half-chains): means, variances and the partial
// autocovariance sums for lags 0..T-1, written to part[(i*nblk + b)*(T+2) + ...]
//   [0] sum of half-chain means, [1] sum of squared means, [2..] sum over
//   half-chains of gamma_{m,t} (with 1/n normalisation).
// STAGE: the half-chains' draws are copied to shared memory (n <= 1024);
// otherwise they are read from the sample array in place (long single runs).
template <typename T, bool STAGE>
__global__ void ess_partial_kernel(const T* __restrict__ x, int64_t N, int64_t d, int64_t C, int n, int lags,
                                   double* __restrict__ part, double* __restrict__ wsum) {
  extern __shared__ float sx_raw[];  // [n][ESS_CH] when staged
  const int64_t i = blockIdx.y;
  const int nblk = gridDim.x;
  const int64_t m = (int64_t)blockIdx.x * ESS_CH + threadIdx.x;  // half-chain index
  const int64_t M = 2 * C;
  const bool live = m < M;
  const int64_t c = m % C, half = m / C;
  // draw k of this half-chain (as FP32, staged or read in place)
  auto draw = [&](int k) -> float {
    return STAGE ? sx_raw[k * ESS_CH + threadIdx.x] : (float)x[((half * n + k) * d + i) * C + c];
  };
  double mean = 0.0;
  if (live) {
    for (int k = 0; k < n; ++k) {
      const float v = (float)x[((half * n + k) * d + i) * C + c];
      if (STAGE) sx_raw[k * ESS_CH + threadIdx.x] = v;
      mean += v;
    }
    mean /= n;
  }
  __syncwarp();
  double var = 0.0;
  __shared__ double red[ESS_CH];
  double* out = part + ((int64_t)i * nblk + blockIdx.x) * (lags + 2);
  // half-chain mean statistics
  red[threadIdx.x] = live ? mean : 0.0;
  __syncwarp();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int j = 0; j < ESS_CH; ++j) s += red[j];
    out[0] = s;
  }
  __syncwarp();
  red[threadIdx.x] = live ? mean * mean : 0.0;
  __syncwarp();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int j = 0; j < ESS_CH; ++j) s += red[j];
    out[1] = s;
  }
  __syncwarp();
  for (int t = 0; t < lags; ++t) {
    double g = 0.0;
    if (live && t < n) {
      for (int k = 0; k + t < n; ++k) g += ((double)draw(k) - mean) * ((double)draw(k + t) - mean);
      g /= n;
      if (t == 0) var = g * n / (n - 1);  // unbiased within-half-chain variance
    }
    red[threadIdx.x] = g;
    __syncwarp();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int j = 0; j < ESS_CH; ++j) s += red[j];
      out[2 + t] = s;
    }
    __syncwarp();
  }
  red[threadIdx.x] = live ? var : 0.0;
  __syncwarp();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int j = 0; j < ESS_CH; ++j) s += red[j];
    wsum[(int64_t)i * nblk + blockIdx.x] = s;
  }
}

// One thread per parameter: combine block partials, Geyer truncation.
__global__ void ess_final_kernel(const double* __restrict__ part, const double* __restrict__ wsum, int64_t d,
                                 int nblk, int64_t M, int n, int lags, double* __restrict__ ess,
                                 double* __restrict__ rhat) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= d) return;
  double smean = 0.0, smean2 = 0.0, W = 0.0;
  for (int b = 0; b < nblk; ++b) {
    const double* p = part + (i * nblk + b) * (lags + 2);
    smean += p[0];
    smean2 += p[1];
    W += wsum[i * nblk + b];
  }
  W /= M;
  const double mu = smean / M;
  const double B = (double)n / (M - 1) * (smean2 - M * mu * mu);  // n * var of half-chain means
  const double varp = (n - 1.0) / n * W + B / n;
  if (rhat) rhat[i] = sqrt(varp / W);
  auto rho = [&](int t) {
    double g = 0.0;
    for (int b = 0; b < nblk; ++b) g += part[(i * nblk + b) * (lags + 2) + 2 + t];
    return 1.0 - (W - g / M) / varp;
  };
  double tau_sum = 0.0, prev = INFINITY;
  int t = 0;
  bool truncated = false;
  for (; t + 1 < lags; t += 2) {
    double P = rho(t) + rho(t + 1);
    if (P < 0.0) {
      truncated = true;
      break;
    }
    if (P > prev) P = prev;  // initial monotone sequence
    prev = P;
    tau_sum += P;
  }
  const double tau = -1.0 + 2.0 * tau_sum;
  double e = M * (double)n / tau;
  if (!truncated) e = -e;  // flag: lag window too short for this parameter
  ess[i] = e;
}

}  // namespace
}  // namespace hmc

using namespace hmc;

extern "C" HMC_API int hmc_ess(int dtype, int64_t N, int64_t d, int64_t C, const void* samples, int lags,
                               double* work, double* ess, double* rhat, void* stream) {
  HMC_REQUIRE(N >= 4 && d > 0 && C > 0, "hmc_ess: need at least 4 draws, 1 parameter, 1 chain");
  HMC_REQUIRE(samples && work && ess, "hmc_ess: null argument");
  HMC_REQUIRE(N / 2 <= (1ll << 30), "hmc_ess: too many draws");
  const int n = (int)(N / 2);
  HMC_REQUIRE(lags >= 2 && lags <= n, "hmc_ess: lags must be in [2, N/2]");
  const bool stage = n <= 1024;
  HMC_REQUIRE(d <= 65535, "hmc_ess: too many parameters for one call");
  const int64_t M = 2 * C;
  const int nblk = (int)((M + ESS_CH - 1) / ESS_CH);
  double* part = work;
  double* wsum = work + d * nblk * (lags + 2);
  const size_t smem = stage ? (size_t)n * ESS_CH * sizeof(float) : 0;
  cudaStream_t st = as_stream(stream);
  const dim3 grid(nblk, (unsigned)d);
  if (dtype == HMC_F32) {
    auto kern = stage ? ess_partial_kernel<float, true> : ess_partial_kernel<float, false>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<grid, ESS_CH, smem, st>>>((const float*)samples, N, d, C, n, lags, part, wsum);
  } else if (dtype == HMC_F64) {
    auto kern = stage ? ess_partial_kernel<double, true> : ess_partial_kernel<double, false>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<grid, ESS_CH, smem, st>>>((const double*)samples, N, d, C, n, lags, part, wsum);
  } else {
    return fail(HMC_ERR_INVALID_ARG, "hmc_ess: unknown dtype %d", dtype);
  }
  HMC_TRY(check_launch("ess_partial_kernel"));
  ess_final_kernel<<<blocks_for(d, 128), 128, 0, st>>>(part, wsum, d, nblk, M, n, lags, ess, rhat);
  return check_launch("ess_final_kernel");
}

namespace hmc {
namespace {
// Mean and variance over all draws and chains of every parameter: one block
// per parameter, fixed-order FP64 reduction.
template <typename T>
__global__ void moments_kernel(const T* __restrict__ x, int64_t N, int64_t d, int64_t C, double* mean, double* var) {
  __shared__ double s1[256], s2[256];
  const int64_t i = blockIdx.x;
  double a = 0.0, b = 0.0;
  const int64_t total = N * C;
  for (int64_t t = threadIdx.x; t < total; t += blockDim.x) {
    const int64_t n = t / C, c = t % C;
    const double v = (double)x[(n * d + i) * C + c];
    a += v;
    b += v * v;
  }
  s1[threadIdx.x] = a;
  s2[threadIdx.x] = b;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      s1[threadIdx.x] += s1[threadIdx.x + w];
      s2[threadIdx.x] += s2[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double m = s1[0] / total;
    mean[i] = m;
    var[i] = s2[0] / total - m * m;
  }
}
}  // namespace
}  // namespace hmc

extern "C" HMC_API int hmc_moments(int dtype, int64_t N, int64_t d, int64_t C, const void* samples, double* mean,
                                   double* var, void* stream) {
  HMC_REQUIRE(N > 0 && d > 0 && C > 0 && d <= 0x7FFFFFFF, "hmc_moments: bad sizes");
  HMC_REQUIRE(samples && mean && var, "hmc_moments: null argument");
  return HMC_DISPATCH(dtype, T, [&] {
    moments_kernel<T><<<(unsigned)d, 256, 0, as_stream(stream)>>>((const T*)samples, N, d, C, mean, var);
    return check_launch("moments_kernel");
  });
}

extern "C" HMC_API int64_t hmc_ess_work_size(int64_t d, int64_t C, int lags) {
  const int64_t nblk = (2 * C + ESS_CH - 1) / ESS_CH;
  return d * nblk * (lags + 2) + d * nblk;
}

// ---- rank normalisation (Vehtari, Gelman, Simpson, Carpenter & Buerkner
// 2021, "Rank-normalization, folding, and localization: an improved R-hat",
// section 4.1): every draw of a parameter is replaced by the normal score of
// its rank among all N x C draws of that parameter,
//   z = Phi^-1((r - 3/8) / (S + 1/4)),  S = N C,
// with tied draws given their average rank.  The split-R-hat and ESS of z are
// the bulk diagnostics of that paper.
namespace hmc {
namespace {
constexpr int RANK_TILE = 2048;

// One thread per draw, blockIdx.y = parameter: the draw is compared with all
// S draws of its parameter, staged through shared memory in tiles.
template <typename T>
__global__ void __launch_bounds__(256) rank_normal_kernel(const T* __restrict__ x, int64_t N, int64_t d, int64_t C,
                                                          int64_t i0, double* __restrict__ z) {
  __shared__ double tile[RANK_TILE];
  const int64_t S = N * C;
  const int64_t i = i0 + blockIdx.y;
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool own = s < S;
  const double v = own ? (double)x[((s / C) * d + i) * C + s % C] : 0.0;
  int less = 0, equal = 0;
  for (int64_t t0 = 0; t0 < S; t0 += RANK_TILE) {
    const int m = (int)(S - t0 < RANK_TILE ? S - t0 : RANK_TILE);
    __syncthreads();
    for (int q = threadIdx.x; q < m; q += blockDim.x) {
      const int64_t u = t0 + q;
      tile[q] = (double)x[((u / C) * d + i) * C + u % C];
    }
    __syncthreads();
    if (own) {
#pragma unroll 8
      for (int q = 0; q < m; ++q) {
        less += tile[q] < v;
        equal += tile[q] == v;
      }
    }
  }
  if (own) {
    const double r = (double)less + 0.5 * (double)(equal + 1);
    z[((s / C) * d + i) * C + s % C] = normcdfinv((r - 0.375) / ((double)S + 0.25));
  }
}
}  // namespace
}  // namespace hmc

extern "C" HMC_API int hmc_rank_normalize(int dtype, int64_t N, int64_t d, int64_t C, const void* samples, double* z,
                                          void* stream) {
  HMC_REQUIRE(N > 0 && d > 0 && C > 0, "hmc_rank_normalize: bad sizes");
  HMC_REQUIRE(samples && z, "hmc_rank_normalize: null argument");
  const int64_t S = N * C;
  HMC_REQUIRE(S < (1ll << 31) / 2, "hmc_rank_normalize: too many draws per parameter");
  // the comparison count is S^2 per parameter: refuse calls that would keep
  // the device busy for more than tens of seconds
  HMC_REQUIRE((double)S * (double)S * (double)d <= 1.1e12,
              "hmc_rank_normalize: S^2 d = %.3g comparisons is beyond this estimator's budget (1.1e12)",
              (double)S * (double)S * (double)d);
  cudaStream_t st = as_stream(stream);
  const unsigned bx = (unsigned)((S + 255) / 256);
  for (int64_t i0 = 0; i0 < d; i0 += 65535) {
    const unsigned dy = (unsigned)(d - i0 < 65535 ? d - i0 : 65535);
    const int rc = HMC_DISPATCH(dtype, T, [&] {
      rank_normal_kernel<T><<<dim3(bx, dy), 256, 0, st>>>((const T*)samples, N, d, C, i0, z);
      return check_launch("rank_normal_kernel");
    });
    if (rc != HMC_OK) return rc;
  }
  return HMC_OK;
}
