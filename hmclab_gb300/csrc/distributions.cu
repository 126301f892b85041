// Batched misfit / gradient kernels of the target distributions on the HMC
// path.  Every misfit is an FP64 per-chain sum; every gradient is written (or
// accumulated, for BayesRule sums) into a [d][C] array of the state dtype.
//
//   Normal (diag / full)   Distributions/base.py:539-574
//   Laplace                Distributions/base.py:689-710
//   LinearMatrix dense     Distributions/LinearMatrix.py:139-222
//   LinearMatrix sparse    Distributions/LinearMatrix.py:309-440
//   SourceLocation3D       Distributions/SourceLocation.py:482-540,697-713
#include <math.h>

#include <type_traits>

#include "common.cuh"

namespace hmc {
int gemm_ex(int dtype, int64_t m, int64_t n, int64_t k, double alpha, const void* A, const void* B, const void* bias,
            double bias_scale, const void* row_scale, void* out, int accumulate, cudaStream_t stream);
}

namespace hmc {
namespace {

inline unsigned ew_grid(int64_t n) {
  const unsigned b = blocks_for(n, 256);
  return b > 152u * 32u ? 152u * 32u : b;
}

// out[i][c] = M[i][c] - mean[i]
template <typename T>
__global__ void centre_kernel(int64_t d, int64_t C, const T* __restrict__ M, const T* __restrict__ mean, T* out) {
  const int64_t total = d * C;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x)
    out[idx] = M[idx] - mean[idx / C];
}

// ---- elementwise priors -----------------------------------------------------
enum PriorKind { PRIOR_NORMAL_DIAG = 0, PRIOR_LAPLACE = 1 };

template <typename T, int KIND>
__global__ void prior_misfit_kernel(int64_t d, int64_t C, const T* __restrict__ M, const T* __restrict__ mean,
                                    const T* __restrict__ w, double* out, int accumulate) {
  __shared__ double sh[RED_Y][RED_X + 1];
  const int64_t c = blockIdx.x * (int64_t)RED_X + threadIdx.x;
  double acc = 0.0;
  if (c < C) {
    for (int64_t i = threadIdx.y; i < d; i += RED_Y) {
      const T m = M[i * C + c];
      if (KIND == PRIOR_NORMAL_DIAG) {
        const T r = mean[i] - m;  // (means - coordinates)
        acc += (double)r * (double)(w[i] * r);
      } else {
        const T r = m - mean[i];
        acc += (double)(fabs(r) * w[i]);
      }
    }
  }
  const double s = block_chain_sum(acc, sh);
  if (c < C && threadIdx.y == 0) {
    const double v = KIND == PRIOR_NORMAL_DIAG ? 0.5 * s : s;
    out[c] = accumulate ? out[c] + v : v;
  }
}

template <typename T>
__device__ __forceinline__ T sgn(T x) {
  return x > (T)0 ? (T)1 : (x < (T)0 ? (T)-1 : (T)0);
}

template <typename T, int KIND>
__global__ void prior_gradient_kernel(int64_t d, int64_t C, const T* __restrict__ M, const T* __restrict__ mean,
                                      const T* __restrict__ w, T* out, int accumulate) {
  const int64_t total = d * C;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = idx / C;
    const T m = M[idx];
    T g;
    if (KIND == PRIOR_NORMAL_DIAG)
      g = -(w[i] * (mean[i] - m));
    else
      g = sgn(m - mean[i]) * w[i];
    out[idx] = accumulate ? out[idx] + g : g;
  }
}

template <typename T, int KIND>
int prior_misfit(int64_t d, int64_t C, const void* M, const void* mean, const void* w, double* out, int accumulate,
                 cudaStream_t st, const char* who) {
  HMC_REQUIRE(d > 0 && C >= 0, "%s: bad sizes", who);
  if (C == 0) return HMC_OK;
  HMC_REQUIRE(M && mean && w && out, "%s: null argument", who);
  prior_misfit_kernel<T, KIND><<<red_grid(C), red_block(), 0, st>>>(d, C, (const T*)M, (const T*)mean,
                                                                    (const T*)w, out, accumulate);
  return check_launch(who);
}

template <typename T, int KIND>
int prior_gradient(int64_t d, int64_t C, const void* M, const void* mean, const void* w, void* out, int accumulate,
                   cudaStream_t st, const char* who) {
  HMC_REQUIRE(d > 0 && C >= 0, "%s: bad sizes", who);
  if (C == 0) return HMC_OK;
  HMC_REQUIRE(M && mean && w && out, "%s: null argument", who);
  prior_gradient_kernel<T, KIND><<<ew_grid(d * C), 256, 0, st>>>(d, C, (const T*)M, (const T*)mean, (const T*)w,
                                                                 (T*)out, accumulate);
  return check_launch(who);
}

// ---- per-chain quadratic forms ---------------------------------------------
// out[c] (+)= scale * (sum_i a[i][c] * (b[i][c] + sb * bvec[i]) + add)
template <typename T>
__global__ void dot_columns_kernel(int64_t d, int64_t C, const T* __restrict__ a, const T* __restrict__ b,
                                   const T* __restrict__ bvec, double sb, double add, double scale, double* out,
                                   int accumulate) {
  __shared__ double sh[RED_Y][RED_X + 1];
  const int64_t c = blockIdx.x * (int64_t)RED_X + threadIdx.x;
  double acc = 0.0;
  if (c < C) {
    for (int64_t i = threadIdx.y; i < d; i += RED_Y) {
      double bv = (double)b[i * C + c];
      if (bvec) bv += sb * (double)bvec[i];
      acc += (double)a[i * C + c] * bv;
    }
  }
  const double s = block_chain_sum(acc, sh);
  if (c < C && threadIdx.y == 0) {
    const double v = scale * (s + add);
    out[c] = accumulate ? out[c] + v : v;
  }
}

// out[c] (+)= 0.5 * sum_j r[j][c]^2 * w[j]
template <typename T>
__global__ void weighted_sq_kernel(int64_t n, int64_t C, const T* __restrict__ r, const T* __restrict__ w,
                                   double* out, int accumulate) {
  __shared__ double sh[RED_Y][RED_X + 1];
  const int64_t c = blockIdx.x * (int64_t)RED_X + threadIdx.x;
  double acc = 0.0;
  if (c < C) {
    for (int64_t j = threadIdx.y; j < n; j += RED_Y) {
      const double rv = (double)r[j * C + c];
      acc += rv * rv * (double)w[j];
    }
  }
  const double s = block_chain_sum(acc, sh);
  if (c < C && threadIdx.y == 0) {
    const double v = 0.5 * s;
    out[c] = accumulate ? out[c] + v : v;
  }
}

// ---- CSR sparse-times-dense (chains fastest) -------------------------------
// out[j][c] = (sum_k val[k] X[col[k]][c] - (bias ? bias[j] : 0)) * (rs ? rs[j] : 1) (+ out)
template <typename T>
__global__ void csr_spmm_kernel(int64_t rows, int64_t C, const int32_t* __restrict__ rp,
                                const int32_t* __restrict__ col, const T* __restrict__ val, const T* __restrict__ X,
                                const T* __restrict__ bias, const T* __restrict__ rs, T* out, int accumulate) {
  const int64_t j = blockIdx.y;
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (j >= rows || c >= C) return;
  T acc = (T)0;
  const int32_t b = rp[j], e = rp[j + 1];
  int32_t k = b;
  // four nonzeros at a time: their rows of X are loaded together (four
  // coalesced 128-byte requests in flight per warp), then accumulated in CSR
  // order, so the sum equals the one-at-a-time loop's
  for (; k + 4 <= e; k += 4) {
    const T x0 = X[(int64_t)col[k] * C + c], x1 = X[(int64_t)col[k + 1] * C + c];
    const T x2 = X[(int64_t)col[k + 2] * C + c], x3 = X[(int64_t)col[k + 3] * C + c];
    acc += val[k] * x0;
    acc += val[k + 1] * x1;
    acc += val[k + 2] * x2;
    acc += val[k + 3] * x3;
  }
  for (; k < e; ++k) acc += val[k] * X[(int64_t)col[k] * C + c];
  if (bias) acc -= bias[j];
  if (rs) acc *= rs[j];
  const int64_t o = j * C + c;
  out[o] = accumulate ? out[o] + acc : acc;
}

template <typename T>
int csr_spmm(int64_t rows, int64_t C, const int32_t* rp, const int32_t* col, const void* val, const void* X,
             const void* bias, const void* rs, void* out, int accumulate, cudaStream_t st) {
  HMC_REQUIRE(rows <= 65535 * 1024ll, "csr: too many rows");
  const int threads = C >= 256 ? 256 : (C >= 128 ? 128 : (C >= 64 ? 64 : 32));
  dim3 grid((unsigned)((C + threads - 1) / threads), 1);
  // grid.y is limited to 65535: split tall matrices into row batches.
  for (int64_t r0 = 0; r0 < rows; r0 += 65535) {
    const int64_t nr = rows - r0 < 65535 ? rows - r0 : 65535;
    grid.y = (unsigned)nr;
    csr_spmm_kernel<T><<<grid, threads, 0, st>>>(nr, C, rp + r0, col, (const T*)val, (const T*)X,
                                                 bias ? (const T*)bias + r0 : nullptr,
                                                 rs ? (const T*)rs + r0 : nullptr, (T*)out + r0 * C, accumulate);
    HMC_TRY(check_launch("csr_spmm_kernel"));
  }
  return HMC_OK;
}

// ---- CSR times a chain block through shared-memory column slabs (FP32) ------
// out[r][c] = (sum_k val[k] X[col[k]][c] - bias[r]) * rs[r] (+ out), as
// csr_spmm_kernel, for a CSR whose columns are sorted within each row.
//
// Each nonzero of the tomography operator multiplies a whole row of the chain
// block, and every column is shared by tens of rows, so gathering X rows from
// L2 once per nonzero moves nnz * C * 4 bytes.  Here a block owns 32 chains
// (one per lane) and a group of CSR_WARPS * RPW rows (warp w: rows
// r0 + w + CSR_WARPS * i).  The columns are walked in slabs of `slab`: X[slab
// columns][the block's 32 chains] is copied into shared memory by
// asynchronous copies (cp.async), double-buffered so that the next slab is in
// flight while the warps add the current slab's nonzeros of their rows
// (slab_ptr[r][s] .. slab_ptr[r][s + 1]) into register accumulators.  Each X
// element is read from L2 once per row group instead of once per nonzero,
// and a shared-memory read is one 128-byte row per nonzero and warp, free of
// bank conflicts.  Nonzeros are added in CSR order with fused multiply-adds,
// so the sums equal csr_spmm_kernel's bit for bit.
constexpr int CSR_WARPS = 16;
constexpr int CSR_THREADS = 32 * CSR_WARPS;

__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool valid) {
  // a chain past C copies nothing and zero-fills (src-size 0)
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src), "r"(valid ? 4 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async16(float* dst, const float* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Issue the copies of slab s (columns s*slab ..) into buffer `buf`.  VEC4:
// C is a multiple of 4 and X 16-byte aligned, so every chain quad of a row is
// one 16-byte copy (the block's 32 chains are 8 quads; quads past C are
// skipped, their lanes never store results).
template <bool VEC4>
__device__ __forceinline__ void csr_slab_fill(float* buf, const float* __restrict__ X, int C, int c0, int cols,
                                              int slab, int s) {
  const int k0 = s * slab;
  const int kn = cols - k0 < slab ? cols - k0 : slab;
  if (VEC4) {
    for (int t = threadIdx.x; t < kn * 8; t += CSR_THREADS) {
      const int row = t >> 3, q = t & 7, cc = c0 + 4 * q;
      if (cc < C) cp_async16(buf + row * 32 + 4 * q, X + (int64_t)(k0 + row) * C + cc);
    }
  } else {
    for (int t = threadIdx.x; t < kn * 32; t += CSR_THREADS) {
      const int row = t >> 5, cc = c0 + (t & 31);
      const bool ok = cc < C;
      cp_async4(buf + t, ok ? X + (int64_t)(k0 + row) * C + cc : X, ok);
    }
  }
  cp_async_commit();
}

// Subtract center[column] from the elements of slab s this thread copied (its
// own copies are complete once it has waited for them).
template <bool VEC4>
__device__ __forceinline__ void csr_slab_centre(float* buf, const float* __restrict__ center, int C, int c0,
                                                int cols, int slab, int s) {
  const int k0 = s * slab;
  const int kn = cols - k0 < slab ? cols - k0 : slab;
  if (VEC4) {
    for (int t = threadIdx.x; t < kn * 8; t += CSR_THREADS) {
      const int row = t >> 3, q = t & 7;
      if (c0 + 4 * q < C) {
        float4* v = (float4*)(buf + row * 32 + 4 * q);
        const float cv = center[k0 + row];
        float4 x = *v;
        x.x -= cv;
        x.y -= cv;
        x.z -= cv;
        x.w -= cv;
        *v = x;
      }
    }
  } else {
    for (int t = threadIdx.x; t < kn * 32; t += CSR_THREADS) buf[t] -= center[k0 + (t >> 5)];
  }
}

template <int RPW, bool VEC4>
__global__ void __launch_bounds__(CSR_THREADS, 2)
    csr_slab_kernel(int rows, int cols, int C, const int32_t* __restrict__ col, const float* __restrict__ val,
                    const int32_t* __restrict__ slab_ptr, int n_slabs, int slab, const float* __restrict__ X,
                    const float* __restrict__ center, const float* __restrict__ bias, const float* __restrict__ rs,
                    float* out, int accumulate) {
  extern __shared__ __align__(16) float sx[];  // two buffers of [slab][32]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int c0 = blockIdx.x * 32, c = c0 + lane;
  const int r0 = blockIdx.y * (CSR_WARPS * RPW);
  float acc[RPW];
#pragma unroll
  for (int i = 0; i < RPW; ++i) acc[i] = 0.f;
  csr_slab_fill<VEC4>(sx, X, C, c0, cols, slab, 0);
  for (int s = 0; s < n_slabs; ++s) {
    float* cur = sx + (s & 1) * slab * 32;
    if (s + 1 < n_slabs) {
      // the other buffer was released by the barrier at the end of slab s - 1
      csr_slab_fill<VEC4>(sx + ((s + 1) & 1) * slab * 32, X, C, c0, cols, slab, s + 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    if (center) csr_slab_centre<VEC4>(cur, center, C, c0, cols, slab, s);
    __syncthreads();  // slab s has landed (and is centred) for every thread's copies
    const int k0 = s * slab;
#pragma unroll
    for (int i = 0; i < RPW; ++i) {
      const int r = r0 + warp + CSR_WARPS * i;
      if (r >= rows) break;  // warp-uniform
      const int64_t sp = (int64_t)r * (n_slabs + 1) + s;
      const int b = slab_ptr[sp], e = slab_ptr[sp + 1];
      float a = acc[i];
      int k = b;
      for (; k + 4 <= e; k += 4) {
        const int j0 = col[k] - k0, j1 = col[k + 1] - k0, j2 = col[k + 2] - k0, j3 = col[k + 3] - k0;
        const float v0 = val[k], v1 = val[k + 1], v2 = val[k + 2], v3 = val[k + 3];
        const float x0 = cur[j0 * 32 + lane], x1 = cur[j1 * 32 + lane], x2 = cur[j2 * 32 + lane],
                    x3 = cur[j3 * 32 + lane];
        a = fmaf(v0, x0, a);
        a = fmaf(v1, x1, a);
        a = fmaf(v2, x2, a);
        a = fmaf(v3, x3, a);
      }
      for (; k < e; ++k) a = fmaf(val[k], cur[(col[k] - k0) * 32 + lane], a);
      acc[i] = a;
    }
    __syncthreads();  // every warp is done with this buffer before it is refilled
  }
  if (c >= C) return;
#pragma unroll
  for (int i = 0; i < RPW; ++i) {
    const int r = r0 + warp + CSR_WARPS * i;
    if (r >= rows) break;
    float v = acc[i];
    if (bias) v -= bias[r];
    if (rs) v *= rs[r];
    const int64_t o = (int64_t)r * C + c;
    out[o] = accumulate ? out[o] + v : v;
  }
}

// ---- gather variants of the FP32 CSR product ---------------------------------
// One block row per CSR row; VEC chains per thread (1, or 4 with 16-byte
// loads of X and stores of out).  The nonzeros of the row are added in CSR
// order with fused multiply-adds (four rows of X in flight), optionally on
// the centred operand X - center[col].
#ifndef HMC_CSR_GATHER_DEPTH
#define HMC_CSR_GATHER_DEPTH 32
#endif
constexpr int GATHER_DEPTH = HMC_CSR_GATHER_DEPTH;

template <int VEC>
__global__ void csr_gather_kernel(int rows, int C, const int32_t* __restrict__ rp, const int32_t* __restrict__ col,
                                  const float* __restrict__ val, const float* __restrict__ X,
                                  const float* __restrict__ center, const float* __restrict__ bias,
                                  const float* __restrict__ rs, float* out, int accumulate) {
  using V = typename std::conditional<VEC == 4, float4, float>::type;
  const int r = blockIdx.y;
  const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * VEC;
  if (r >= rows || c >= C) return;
  float a[VEC];
#pragma unroll
  for (int v = 0; v < VEC; ++v) a[v] = 0.f;
  const int b = rp[r], e = rp[r + 1];
  auto load = [&](int k, float* x) {
    const int j = col[k];
    const float cj = center ? center[j] : 0.f;
    const V xv = *(const V*)(X + (int64_t)j * C + c);
    const float* xs = (const float*)&xv;
#pragma unroll
    for (int v = 0; v < VEC; ++v) x[v] = xs[v] - cj;
  };
  // GATHER_DEPTH rows of X in flight per thread (the product waits on L2
  // gathers), summed in CSR order
  int k = b;
  for (; k + GATHER_DEPTH <= e; k += GATHER_DEPTH) {
    float x[GATHER_DEPTH][VEC], w[GATHER_DEPTH];
#pragma unroll
    for (int u = 0; u < GATHER_DEPTH; ++u) {
      load(k + u, x[u]);
      w[u] = val[k + u];
    }
#pragma unroll
    for (int v = 0; v < VEC; ++v)
#pragma unroll
      for (int u = 0; u < GATHER_DEPTH; ++u) a[v] = fmaf(w[u], x[u][v], a[v]);
  }
  for (; k < e; ++k) {
    float x0[VEC];
    load(k, x0);
    const float v0 = val[k];
#pragma unroll
    for (int v = 0; v < VEC; ++v) a[v] = fmaf(v0, x0[v], a[v]);
  }
  const float bb = bias ? bias[r] : 0.f, ss = rs ? rs[r] : 1.f;
  float* o = out + (int64_t)r * C + c;
  V ov;
  float* os = (float*)&ov;
  if (accumulate) ov = *(const V*)o;
#pragma unroll
  for (int v = 0; v < VEC; ++v) {
    float y = a[v];
    if (bias) y -= bb;
    if (rs) y *= ss;
    os[v] = accumulate ? os[v] + y : y;
  }
  *(V*)o = ov;
}

int csr_gather(const hmc_csr_slabs* A, int64_t C, const float* X, const float* center, const float* bias,
               const float* rs, float* out, int accumulate, cudaStream_t st) {
  HMC_REQUIRE(A->rows <= 65535, "csr gather product: at most 65535 rows per launch");
  if (A->kernel == HMC_CSR_GATHER4) {
    HMC_REQUIRE(C % 4 == 0 && ((uintptr_t)X & 15) == 0 && ((uintptr_t)out & 15) == 0,
                "csr gather product: four chains per thread need C % 4 == 0 and 16-byte aligned operands");
    const int64_t q = C / 4;
    const int threads = q >= 256 ? 256 : (q >= 128 ? 128 : (q >= 64 ? 64 : 32));
    const dim3 grid((unsigned)((q + threads - 1) / threads), (unsigned)A->rows);
    csr_gather_kernel<4><<<grid, threads, 0, st>>>((int)A->rows, (int)C, A->row_ptr, A->col, A->val, X, center, bias,
                                                   rs, out, accumulate);
  } else {
    const int threads = C >= 256 ? 256 : (C >= 128 ? 128 : (C >= 64 ? 64 : 32));
    const dim3 grid((unsigned)((C + threads - 1) / threads), (unsigned)A->rows);
    csr_gather_kernel<1><<<grid, threads, 0, st>>>((int)A->rows, (int)C, A->row_ptr, A->col, A->val, X, center, bias,
                                                   rs, out, accumulate);
  }
  return check_launch("csr_gather_kernel");
}

int csr_slab_check(const hmc_csr_slabs* A, const char* who) {
  HMC_REQUIRE(A != nullptr, "%s: null CSR descriptor", who);
  HMC_REQUIRE(A->kernel >= HMC_CSR_GATHER && A->kernel <= HMC_CSR_SLAB, "%s: unknown CSR kernel %d", who,
              (int)A->kernel);
  HMC_REQUIRE(A->col && A->val, "%s: CSR descriptor has a null array", who);
  HMC_REQUIRE(A->rows > 0 && A->cols > 0 && A->rows < (1ll << 31) && A->cols < (1ll << 31), "%s: bad CSR shape",
              who);
  if (A->kernel != HMC_CSR_SLAB) {
    HMC_REQUIRE(A->row_ptr != nullptr, "%s: the gather kernels need row_ptr", who);
    return HMC_OK;
  }
  HMC_REQUIRE(A->slab_ptr != nullptr, "%s: the slab kernel needs slab_ptr", who);
  HMC_REQUIRE(A->slab >= 32 && A->slab <= 448,
              "%s: slab of %d columns outside 32 .. 448 (two double-buffered blocks per SM)", who, (int)A->slab);
  HMC_REQUIRE(A->rows_per_warp == 4 || A->rows_per_warp == 8 || A->rows_per_warp == 16,
              "%s: rows_per_warp must be 4, 8 or 16", who);
  return HMC_OK;
}

template <int RPW, bool VEC4>
int csr_slab_launch(const hmc_csr_slabs* A, int64_t C, const float* X, const float* center, const float* bias,
                    const float* rs, float* out, int accumulate, cudaStream_t st) {
  const int smem = 2 * A->slab * 32 * (int)sizeof(float);  // double buffer
  static int attr_bytes = 0;  // per instantiation: the largest size enabled so far
  if (smem > 48 * 1024 && smem > attr_bytes) {
    cudaError_t e =
        cudaFuncSetAttribute(csr_slab_kernel<RPW, VEC4>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(csr_slab_kernel)");
    attr_bytes = smem;
  }
  const int n_slabs = (int)((A->cols + A->slab - 1) / A->slab);
  const int64_t groups = (A->rows + CSR_WARPS * RPW - 1) / (CSR_WARPS * RPW);
  HMC_REQUIRE(groups <= 65535, "csr slab product: too many rows");
  const dim3 grid((unsigned)((C + 31) / 32), (unsigned)groups);
  csr_slab_kernel<RPW, VEC4><<<grid, CSR_THREADS, smem, st>>>((int)A->rows, (int)A->cols, (int)C, A->col, A->val,
                                                              A->slab_ptr, n_slabs, A->slab, X, center, bias, rs,
                                                              out, accumulate);
  return check_launch("csr_slab_kernel");
}

template <int RPW>
int csr_slab_launch(const hmc_csr_slabs* A, int64_t C, const float* X, const float* center, const float* bias,
                    const float* rs, float* out, int accumulate, cudaStream_t st) {
  const bool vec4 = C % 4 == 0 && ((uintptr_t)X & 15) == 0;
  return vec4 ? csr_slab_launch<RPW, true>(A, C, X, center, bias, rs, out, accumulate, st)
              : csr_slab_launch<RPW, false>(A, C, X, center, bias, rs, out, accumulate, st);
}

int csr_slab(const hmc_csr_slabs* A, int64_t C, const float* X, const float* center, const float* bias,
             const float* rs, float* out, int accumulate, cudaStream_t st) {
  HMC_REQUIRE(C < (1ll << 31) && (C + 31) / 32 <= 0x7fffffff, "csr slab product: too many chains");
  if (A->kernel != HMC_CSR_SLAB) return csr_gather(A, C, X, center, bias, rs, out, accumulate, st);
  switch (A->rows_per_warp) {
    case 4:
      return csr_slab_launch<4>(A, C, X, center, bias, rs, out, accumulate, st);
    case 8:
      return csr_slab_launch<8>(A, C, X, center, bias, rs, out, accumulate, st);
    default:
      return csr_slab_launch<16>(A, C, X, center, bias, rs, out, accumulate, st);
  }
}

// ---- 3-D source location ----------------------------------------------------
// One thread per (chain, event); stations are staged in shared memory.  The
// per-pair terms mirror SourceLocation.py:495-540, including nansum's skipping
// of NaN terms (missing observations, zero distances).
constexpr int SL_EY = 16;  // event lanes per block (threadIdx.y)

template <typename T, bool GRAD>
__global__ void srcloc_kernel(int64_t E, int64_t S, int64_t C, const T* __restrict__ M, const T* __restrict__ rx,
                              const T* __restrict__ ry, const T* __restrict__ rz, const T* __restrict__ obs,
                              const T* __restrict__ iv, int infer_v, T v_fixed, double* out_x, T* out_g,
                              int accumulate) {
  extern __shared__ unsigned char smem_raw[];
  T* srx = (T*)smem_raw;
  T* sry = srx + S;
  T* srz = sry + S;
  __shared__ double red[SL_EY][RED_X + 1];
  for (int64_t s = threadIdx.y * blockDim.x + threadIdx.x; s < S; s += blockDim.x * blockDim.y) {
    srx[s] = rx[s];
    sry[s] = ry[s];
    srz[s] = rz[s];
  }
  __syncthreads();
  const int64_t c = blockIdx.x * (int64_t)RED_X + threadIdx.x;
  const bool live = c < C;
  const T v = live ? (infer_v ? M[(4 * E) * C + c] : v_fixed) : (T)1;
  const T inv_v = (T)1 / v;
  double mis = 0.0;
  T gv = (T)0;
  if (live) {
    for (int64_t e = threadIdx.y; e < E; e += SL_EY) {
      const T x = M[(4 * e + 0) * C + c], y = M[(4 * e + 1) * C + c], z = M[(4 * e + 2) * C + c],
              t0 = M[(4 * e + 3) * C + c];
      T gx = 0, gy = 0, gz = 0, gT = 0;
      double me = 0.0;
      for (int64_t s = 0; s < S; ++s) {
        const T dx = x - srx[s], dy = y - sry[s], dz = z - srz[s];
        const T r2 = dx * dx + dy * dy + dz * dz;
        // FP32: one reciprocal square root per pair gives both the distance
        // and 1 / distance (within 2 ulp); FP64 keeps the correctly rounded
        // square root of the reference's arithmetic
        T dist, inv_dist;
        if (sizeof(T) == 4) {
          inv_dist = (T)rsqrtf((float)r2);
          dist = r2 > (T)0 ? r2 * inv_dist : (T)0;
        } else {
          dist = sqrt(r2);
          inv_dist = (T)1 / dist;
        }
        const T tc = t0 + dist * inv_v;
        const T o = obs[e * S + s], w = iv[e * S + s];
        if (!GRAD) {
          const T r = o - tc;
          const T term = r * r * w;
          if (!isnan(term)) me += (double)term;
        } else {
          const T mg = (tc - o) * w;  // (t_calc - obs) / std^2
          // one reciprocal per pair; at dist = 0 the partials are 0 * inf =
          // NaN and skipped, like nansum's 0 / 0
          const T inv_vd = inv_v * inv_dist;
          T t;
          t = mg * (dx * inv_vd);
          if (!isnan(t)) gx += t;
          t = mg * (dy * inv_vd);
          if (!isnan(t)) gy += t;
          t = mg * (dz * inv_vd);
          if (!isnan(t)) gz += t;
          if (!isnan(mg)) gT += mg;
          t = mg * (-dist * inv_v * inv_v);
          if (!isnan(t)) gv += t;
        }
      }
      if (GRAD) {
        const int64_t o0 = (4 * e) * C + c;
        if (accumulate) {
          out_g[o0] += gx;
          out_g[o0 + C] += gy;
          out_g[o0 + 2 * C] += gz;
          out_g[o0 + 3 * C] += gT;
        } else {
          out_g[o0] = gx;
          out_g[o0 + C] = gy;
          out_g[o0 + 2 * C] = gz;
          out_g[o0 + 3 * C] = gT;
        }
      } else {
        mis += me;
      }
    }
  }
  // Reduce the velocity gradient (or the misfit) over the event lanes.
  red[threadIdx.y][threadIdx.x] = GRAD ? (double)gv : mis;
  __syncthreads();
  if (threadIdx.y == 0 && live) {
    double s = 0.0;
    for (int y = 0; y < SL_EY; ++y) s += red[y][threadIdx.x];
    if (GRAD) {
      if (infer_v) {
        const int64_t o = (4 * E) * C + c;
        out_g[o] = accumulate ? out_g[o] + (T)s : (T)s;
      }
    } else {
      const double val = 0.5 * s;
      out_x[c] = accumulate ? out_x[c] + val : val;
    }
  }
}

// FP32 source location with the per-pair work cut to the arithmetic that
// matters (the kernel above is issue-bound, so instructions are the lever),
// two stations per instruction on Blackwell's packed FP32 pipe:
//   - stations staged in pairs, (x_a, x_b, y_a, y_b) and (z_a, z_b), and the
//     pair data of 16 events x a chunk of stations as (w_a, w_b, o_a, o_b),
//     (w, o) = (1 / std^2, observed time), in shared memory; a NaN
//     observation or weight, and the padding of an odd chunk, is staged as
//     (0, 0), which makes every term of that pair zero — the nansum of the
//     reference (SourceLocation.py:495-540) without a NaN test per pair;
//   - every arithmetic step runs on both stations at once with the f32x2
//     add / sub / mul / fma instructions (sm_100 and later), one reciprocal
//     square root per station; the squared distance starts from 1e-30, so
//     an event on a station contributes zero partials (nansum's 0 / 0);
//   - 1 / v is factored out of the x, y, z partials and 1 / v^2 out of the
//     velocity partial: per pair k = (t_calc - o) w / dist, and the thread
//     accumulates k dx, k dy, k dz, (t_calc - o) w and (t_calc - o) w dist in
//     two lanes (even and odd stations), added at the end;
//   - misfit terms are summed in FP32 over at most SL_CHUNK stations, then in
//     FP64.
constexpr int SL_CHUNK = 512;
constexpr int SL_PAIRS = SL_CHUNK / 2;

// two FP32 values in one 64-bit register: element a in the low half
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 x2_pack(float a, float b) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void x2_unpack(f32x2 v, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ f32x2 x2_add(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 x2_sub(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 x2_mul(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 x2_fma(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ float x2_sum(f32x2 v) {
  float a, b;
  x2_unpack(v, a, b);
  return a + b;
}

template <bool GRAD>
__global__ void srcloc_f32_kernel(int64_t E, int64_t S, int64_t C, const float* __restrict__ M,
                                  const float* __restrict__ rx, const float* __restrict__ ry,
                                  const float* __restrict__ rz, const float* __restrict__ obs,
                                  const float* __restrict__ iv, int infer_v, float v_fixed, double* out_x,
                                  float* out_g, int accumulate) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ulonglong2* sxy = (ulonglong2*)smem_raw;             // [SL_PAIRS] (x_a, x_b), (y_a, y_b)
  f32x2* sz = (f32x2*)(sxy + SL_PAIRS);                // [SL_PAIRS] (z_a, z_b)
  ulonglong2* swo = (ulonglong2*)(sz + SL_PAIRS);      // [SL_EY][SL_PAIRS] (w_a, w_b), (o_a, o_b)
  __shared__ double red[SL_EY][RED_X + 1];
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
  const int64_t c = blockIdx.x * (int64_t)RED_X + threadIdx.x;
  const bool live = c < C;
  const float v = live ? (infer_v ? M[(4 * E) * C + c] : v_fixed) : 1.f;
  const float inv_v = 1.f / v;
  const f32x2 IV = x2_pack(inv_v, inv_v), EPS = x2_pack(1e-30f, 1e-30f);
  double mis = 0.0, gvd_total = 0.0;
  for (int64_t e0 = 0; e0 < E; e0 += SL_EY) {
    const int64_t e = e0 + threadIdx.y;
    const bool ev = live && e < E;
    float x = 0.f, y = 0.f, z = 0.f, t0 = 0.f;
    if (ev) {
      x = M[(4 * e + 0) * C + c];
      y = M[(4 * e + 1) * C + c];
      z = M[(4 * e + 2) * C + c];
      t0 = M[(4 * e + 3) * C + c];
    }
    const f32x2 X = x2_pack(x, x), Y = x2_pack(y, y), Z = x2_pack(z, z), T0 = x2_pack(t0, t0);
    const f32x2 zero = x2_pack(0.f, 0.f);
    f32x2 gx = zero, gy = zero, gz = zero, gT = zero, gvd = zero;
    for (int64_t s0 = 0; s0 < S; s0 += SL_CHUNK) {
      const int sn = (int)(S - s0 < SL_CHUNK ? S - s0 : SL_CHUNK);
      const int np = (sn + 1) / 2;
      __syncthreads();  // the previous chunk is consumed
      for (int k = tid; k < np; k += nthr) {
        const int a = 2 * k, b = 2 * k + 1;
        const bool hb = b < sn;
        sxy[k] = make_ulonglong2(x2_pack(rx[s0 + a], hb ? rx[s0 + b] : 0.f),
                                 x2_pack(ry[s0 + a], hb ? ry[s0 + b] : 0.f));
        sz[k] = x2_pack(rz[s0 + a], hb ? rz[s0 + b] : 0.f);
      }
      for (int k = tid; k < SL_EY * np; k += nthr) {
        const int ye = k / np, kp = k - ye * np;
        const int64_t ee = e0 + ye;
        float w[2] = {0.f, 0.f}, o[2] = {0.f, 0.f};
        for (int h = 0; h < 2; ++h) {
          const int ks = 2 * kp + h;
          if (ee < E && ks < sn) {
            w[h] = iv[ee * S + s0 + ks];
            o[h] = obs[ee * S + s0 + ks];
            if (isnan(w[h]) || isnan(o[h])) w[h] = o[h] = 0.f;
          }
        }
        swo[ye * SL_PAIRS + kp] = make_ulonglong2(x2_pack(w[0], w[1]), x2_pack(o[0], o[1]));
      }
      __syncthreads();
      if (!ev) continue;
      const ulonglong2* my = swo + threadIdx.y * SL_PAIRS;
      f32x2 ms = zero;
#pragma unroll 4
      for (int k = 0; k < np; ++k) {
        const ulonglong2 q = sxy[k];
        const ulonglong2 p = my[k];
        const f32x2 dx = x2_sub(X, q.x), dy = x2_sub(Y, q.y), dz = x2_sub(Z, sz[k]);
        const f32x2 r2 = x2_fma(dz, dz, x2_fma(dy, dy, x2_fma(dx, dx, EPS)));
        float ra, rb;
        x2_unpack(r2, ra, rb);
        const f32x2 inv = x2_pack(rsqrtf(ra), rsqrtf(rb));
        const f32x2 dist = x2_mul(r2, inv);
        const f32x2 res = x2_sub(x2_fma(dist, IV, T0), p.y);  // t_calc - obs
        if (GRAD) {
          const f32x2 mg = x2_mul(res, p.x);
          const f32x2 k2 = x2_mul(mg, inv);
          gx = x2_fma(k2, dx, gx);
          gy = x2_fma(k2, dy, gy);
          gz = x2_fma(k2, dz, gz);
          gT = x2_add(gT, mg);
          gvd = x2_fma(mg, dist, gvd);
        } else {
          ms = x2_fma(x2_mul(res, res), p.x, ms);
        }
      }
      if (!GRAD) mis += (double)x2_sum(ms);
    }
    if (GRAD && ev) {
      const int64_t o0 = (4 * e) * C + c;
      const float ax = x2_sum(gx) * inv_v, ay = x2_sum(gy) * inv_v, az = x2_sum(gz) * inv_v, aT = x2_sum(gT);
      if (accumulate) {
        out_g[o0] += ax;
        out_g[o0 + C] += ay;
        out_g[o0 + 2 * C] += az;
        out_g[o0 + 3 * C] += aT;
      } else {
        out_g[o0] = ax;
        out_g[o0 + C] = ay;
        out_g[o0 + 2 * C] = az;
        out_g[o0 + 3 * C] = aT;
      }
      gvd_total += (double)x2_sum(gvd);
    }
  }
  // Reduce the velocity partial (or the misfit) over the event lanes.
  red[threadIdx.y][threadIdx.x] = GRAD ? gvd_total : mis;
  __syncthreads();
  if (threadIdx.y == 0 && live) {
    double sum = 0.0;
    for (int yy = 0; yy < SL_EY; ++yy) sum += red[yy][threadIdx.x];
    if (GRAD) {
      if (infer_v) {
        const int64_t o = (4 * E) * C + c;
        const float gv = (float)(-sum) * inv_v * inv_v;
        out_g[o] = accumulate ? out_g[o] + gv : gv;
      }
    } else {
      const double val = 0.5 * sum;
      out_x[c] = accumulate ? out_x[c] + val : val;
    }
  }
}

template <typename T>
int srcloc(bool grad, int64_t E, int64_t S, int64_t C, const void* M, const void* rx, const void* ry, const void* rz,
           const void* obs, const void* iv, int infer_v, double v_fixed, double* out_x, void* out_g, int accumulate,
           cudaStream_t st) {
  const char* who = grad ? "hmc_srcloc3d_gradient" : "hmc_srcloc3d_misfit";
  HMC_REQUIRE(E > 0 && S > 0 && C >= 0, "%s: bad sizes", who);
  if (C == 0) return HMC_OK;
  HMC_REQUIRE(M && rx && ry && rz && obs && iv, "%s: null argument", who);
  HMC_REQUIRE(grad ? out_g != nullptr : out_x != nullptr, "%s: null output", who);
  if (sizeof(T) == 4) {
    const size_t smem = SL_PAIRS * (sizeof(ulonglong2) + sizeof(f32x2)) + (size_t)SL_EY * SL_PAIRS * sizeof(ulonglong2);
    auto k32 = grad ? srcloc_f32_kernel<true> : srcloc_f32_kernel<false>;
    static bool attr_set = false;
    if (!attr_set) {
      cudaError_t e1 = cudaFuncSetAttribute(srcloc_f32_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem);
      cudaError_t e2 = cudaFuncSetAttribute(srcloc_f32_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem);
      if (e1 != cudaSuccess || e2 != cudaSuccess)
        return cuda_fail(e1 != cudaSuccess ? e1 : e2, "cudaFuncSetAttribute(srcloc_f32)");
      attr_set = true;
    }
    k32<<<red_grid(C), dim3(RED_X, SL_EY), smem, st>>>(E, S, C, (const float*)M, (const float*)rx, (const float*)ry,
                                                        (const float*)rz, (const float*)obs, (const float*)iv, infer_v,
                                                        (float)v_fixed, out_x, (float*)out_g, accumulate);
    return check_launch(who);
  }
  const size_t smem = 3 * (size_t)S * sizeof(T);
  HMC_REQUIRE(smem <= 160 * 1024, "%s: too many stations (%lld)", who, (long long)S);
  auto kern = grad ? srcloc_kernel<T, true> : srcloc_kernel<T, false>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(srcloc)");
  }
  kern<<<red_grid(C), dim3(RED_X, SL_EY), smem, st>>>(E, S, C, (const T*)M, (const T*)rx, (const T*)ry,
                                                       (const T*)rz, (const T*)obs, (const T*)iv, infer_v,
                                                       (T)v_fixed, out_x, (T*)out_g, accumulate);
  return check_launch(who);
}

}  // namespace
}  // namespace hmc

using namespace hmc;

extern "C" {

int hmc_normal_diag_misfit(int dtype, int64_t d, int64_t C, const void* M, const void* mean, const void* inv_var,
                           double* out_x, int accumulate, void* stream) {
  return HMC_DISPATCH(dtype, T, [&] {
    return prior_misfit<T, PRIOR_NORMAL_DIAG>(d, C, M, mean, inv_var, out_x, accumulate, as_stream(stream),
                                              "hmc_normal_diag_misfit");
  });
}

int hmc_normal_diag_gradient(int dtype, int64_t d, int64_t C, const void* M, const void* mean, const void* inv_var,
                             void* out_g, int accumulate, void* stream) {
  return HMC_DISPATCH(dtype, T, [&] {
    return prior_gradient<T, PRIOR_NORMAL_DIAG>(d, C, M, mean, inv_var, out_g, accumulate, as_stream(stream),
                                                "hmc_normal_diag_gradient");
  });
}

int hmc_laplace_misfit(int dtype, int64_t d, int64_t C, const void* M, const void* mean, const void* inv_disp,
                       double* out_x, int accumulate, void* stream) {
  return HMC_DISPATCH(dtype, T, [&] {
    return prior_misfit<T, PRIOR_LAPLACE>(d, C, M, mean, inv_disp, out_x, accumulate, as_stream(stream),
                                          "hmc_laplace_misfit");
  });
}

int hmc_laplace_gradient(int dtype, int64_t d, int64_t C, const void* M, const void* mean, const void* inv_disp,
                         void* out_g, int accumulate, void* stream) {
  return HMC_DISPATCH(dtype, T, [&] {
    return prior_gradient<T, PRIOR_LAPLACE>(d, C, M, mean, inv_disp, out_g, accumulate, as_stream(stream),
                                            "hmc_laplace_gradient");
  });
}

// Normal with full covariance (base.py:553-574): with D = m - mu,
// misfit 0.5 D^T S^-1 D and gradient -S^-1 (mu - m) = S^-1 D.
// work holds 2*d*C elements of the state dtype (gradient uses the first d*C).
int hmc_normal_full_misfit(int dtype, int64_t d, int64_t C, const void* M, const void* mean, const void* inv_cov,
                           void* work, double* out_x, int accumulate, void* stream) {
  HMC_REQUIRE(d > 0 && C >= 0, "hmc_normal_full_misfit: bad sizes");
  if (C == 0) return HMC_OK;
  HMC_REQUIRE(M && mean && inv_cov && work && out_x, "hmc_normal_full_misfit: null argument");
  cudaStream_t st = as_stream(stream);
  return HMC_DISPATCH(dtype, T, [&] {
    T* D = (T*)work;
    T* SD = D + d * C;
    centre_kernel<T><<<ew_grid(d * C), 256, 0, st>>>(d, C, (const T*)M, (const T*)mean, D);
    HMC_TRY(check_launch("centre_kernel"));
    HMC_TRY(gemm_ex(dtype, d, C, d, 1.0, inv_cov, D, nullptr, 0.0, nullptr, SD, 0, st));
    dot_columns_kernel<T><<<red_grid(C), red_block(), 0, st>>>(d, C, D, SD, nullptr, 0.0, 0.0, 0.5, out_x,
                                                               accumulate);
    return check_launch("dot_columns_kernel");
  });
}

int hmc_normal_full_gradient(int dtype, int64_t d, int64_t C, const void* M, const void* mean, const void* inv_cov,
                             void* work, void* out_g, int accumulate, void* stream) {
  HMC_REQUIRE(d > 0 && C >= 0, "hmc_normal_full_gradient: bad sizes");
  if (C == 0) return HMC_OK;
  HMC_REQUIRE(M && mean && inv_cov && work && out_g, "hmc_normal_full_gradient: null argument");
  cudaStream_t st = as_stream(stream);
  return HMC_DISPATCH(dtype, T, [&] {
    centre_kernel<T><<<ew_grid(d * C), 256, 0, st>>>(d, C, (const T*)M, (const T*)mean, (T*)work);
    HMC_TRY(check_launch("centre_kernel"));
    return gemm_ex(dtype, d, C, d, 1.0, inv_cov, work, nullptr, 0.0, nullptr, out_g, accumulate, st);
  });
}

int hmc_dense_premul_gradient(int dtype, int64_t d, int64_t C, const void* M, const void* GtG, const void* Gtd0,
                              void* out_g, int accumulate, void* stream) {
  HMC_REQUIRE(d > 0 && C >= 0, "hmc_dense_premul_gradient: bad sizes");
  if (C == 0) return HMC_OK;
  HMC_REQUIRE(M && GtG && Gtd0 && out_g, "hmc_dense_premul_gradient: null argument");
  return gemm_ex(dtype, d, C, d, 1.0, GtG, M, Gtd0, -1.0, nullptr, out_g, accumulate, as_stream(stream));
}

int hmc_dense_premul_misfit(int dtype, int64_t d, int64_t C, const void* M, const void* GtG, const void* Gtd0,
                            double dtd, void* work, double* out_x, int accumulate, void* stream) {
  HMC_REQUIRE(d > 0 && C >= 0, "hmc_dense_premul_misfit: bad sizes");
  if (C == 0) return HMC_OK;
  HMC_REQUIRE(M && GtG && Gtd0 && work && out_x, "hmc_dense_premul_misfit: null argument");
  cudaStream_t st = as_stream(stream);
  // work = GtG m - 2 Gtd0; x = 0.5 * (m^T work + dtd)   (LinearMatrix.py:184-191)
  HMC_TRY(gemm_ex(dtype, d, C, d, 1.0, GtG, M, Gtd0, -2.0, nullptr, work, 0, st));
  return HMC_DISPATCH(dtype, T, [&] {
    dot_columns_kernel<T><<<red_grid(C), red_block(), 0, st>>>(d, C, (const T*)M, (const T*)work, nullptr, 0.0, dtd,
                                                               0.5, out_x, accumulate);
    return check_launch("dot_columns_kernel");
  });
}

int hmc_dense_resid_misfit(int dtype, int64_t n, int64_t d, int64_t C, const void* M, const void* G,
                           const void* data, const void* inv_var, void* resid, double* out_x, int accumulate,
                           void* stream) {
  HMC_REQUIRE(n > 0 && d > 0 && C >= 0, "hmc_dense_resid_misfit: bad sizes");
  if (C == 0) return HMC_OK;
  HMC_REQUIRE(M && G && data && inv_var && resid && out_x, "hmc_dense_resid_misfit: null argument");
  cudaStream_t st = as_stream(stream);
  HMC_TRY(gemm_ex(dtype, n, C, d, 1.0, G, M, data, -1.0, nullptr, resid, 0, st));
  return HMC_DISPATCH(dtype, T, [&] {
    weighted_sq_kernel<T><<<red_grid(C), red_block(), 0, st>>>(n, C, (const T*)resid, (const T*)inv_var, out_x,
                                                               accumulate);
    return check_launch("weighted_sq_kernel");
  });
}

int hmc_dense_resid_gradient(int dtype, int64_t n, int64_t d, int64_t C, const void* M, const void* G,
                             const void* Gt, const void* data, const void* inv_var, void* resid, void* out_g,
                             int accumulate, void* stream) {
  HMC_REQUIRE(n > 0 && d > 0 && C >= 0, "hmc_dense_resid_gradient: bad sizes");
  if (C == 0) return HMC_OK;
  HMC_REQUIRE(M && G && Gt && data && inv_var && resid && out_g, "hmc_dense_resid_gradient: null argument");
  cudaStream_t st = as_stream(stream);
  HMC_TRY(gemm_ex(dtype, n, C, d, 1.0, G, M, data, -1.0, inv_var, resid, 0, st));
  return gemm_ex(dtype, d, C, n, 1.0, Gt, resid, nullptr, 0.0, nullptr, out_g, accumulate, st);
}

int hmc_csr_misfit(int dtype, int64_t n, int64_t d, int64_t C, const void* M, const int32_t* row_ptr,
                   const int32_t* col, const void* val, const void* data, const void* inv_var, void* resid,
                   double* out_x, int accumulate, void* stream) {
  HMC_REQUIRE(n > 0 && d > 0 && C >= 0, "hmc_csr_misfit: bad sizes");
  if (C == 0) return HMC_OK;
  HMC_REQUIRE(M && row_ptr && col && val && data && inv_var && resid && out_x, "hmc_csr_misfit: null argument");
  cudaStream_t st = as_stream(stream);
  return HMC_DISPATCH(dtype, T, [&] {
    HMC_TRY(csr_spmm<T>(n, C, row_ptr, col, val, M, data, nullptr, resid, 0, st));
    weighted_sq_kernel<T><<<red_grid(C), red_block(), 0, st>>>(n, C, (const T*)resid, (const T*)inv_var, out_x,
                                                               accumulate);
    return check_launch("weighted_sq_kernel");
  });
}

int hmc_csr_gradient(int dtype, int64_t n, int64_t d, int64_t C, const void* M, const int32_t* row_ptr,
                     const int32_t* col, const void* val, const int32_t* t_row_ptr, const int32_t* t_col,
                     const void* t_val, const void* data, const void* inv_var, void* resid, void* out_g,
                     int accumulate, void* stream) {
  HMC_REQUIRE(n > 0 && d > 0 && C >= 0, "hmc_csr_gradient: bad sizes");
  if (C == 0) return HMC_OK;
  HMC_REQUIRE(M && row_ptr && col && val && t_row_ptr && t_col && t_val && data && inv_var && resid && out_g,
              "hmc_csr_gradient: null argument");
  cudaStream_t st = as_stream(stream);
  return HMC_DISPATCH(dtype, T, [&] {
    HMC_TRY(csr_spmm<T>(n, C, row_ptr, col, val, M, data, inv_var, resid, 0, st));
    return csr_spmm<T>(d, C, t_row_ptr, t_col, t_val, resid, nullptr, nullptr, out_g, accumulate, st);
  });
}

int hmc_csr_slab_misfit(const hmc_csr_slabs* G, int64_t C, const float* M, const float* center, const float* data,
                        const float* inv_var, float* resid, double* out_x, int accumulate, void* stream) {
  HMC_TRY(csr_slab_check(G, "hmc_csr_slab_misfit"));
  HMC_REQUIRE(C >= 0, "hmc_csr_slab_misfit: bad sizes");
  if (C == 0) return HMC_OK;
  HMC_REQUIRE(M && data && inv_var && resid && out_x, "hmc_csr_slab_misfit: null argument");
  cudaStream_t st = as_stream(stream);
  HMC_TRY(csr_slab(G, C, M, center, data, nullptr, resid, 0, st));
  weighted_sq_kernel<float><<<red_grid(C), red_block(), 0, st>>>(G->rows, C, resid, inv_var, out_x, accumulate);
  return check_launch("weighted_sq_kernel");
}

int hmc_csr_slab_gradient(const hmc_csr_slabs* G, const hmc_csr_slabs* Gt, int64_t C, const float* M,
                          const float* center, const float* data, const float* inv_var, float* resid, float* out_g,
                          int accumulate, void* stream) {
  HMC_TRY(csr_slab_check(G, "hmc_csr_slab_gradient"));
  HMC_TRY(csr_slab_check(Gt, "hmc_csr_slab_gradient"));
  HMC_REQUIRE(Gt->rows == G->cols && Gt->cols == G->rows, "hmc_csr_slab_gradient: G^T shape does not match G");
  HMC_REQUIRE(C >= 0, "hmc_csr_slab_gradient: bad sizes");
  if (C == 0) return HMC_OK;
  HMC_REQUIRE(M && data && inv_var && resid && out_g, "hmc_csr_slab_gradient: null argument");
  cudaStream_t st = as_stream(stream);
  HMC_TRY(csr_slab(G, C, M, center, data, inv_var, resid, 0, st));
  return csr_slab(Gt, C, resid, nullptr, nullptr, nullptr, out_g, accumulate, st);
}

int hmc_srcloc3d_misfit(int dtype, int64_t E, int64_t S, int64_t C, const void* M, const void* rx, const void* ry,
                        const void* rz, const void* obs, const void* inv_var, int infer_velocity,
                        double medium_velocity, double* out_x, int accumulate, void* stream) {
  return HMC_DISPATCH(dtype, T, [&] {
    return srcloc<T>(false, E, S, C, M, rx, ry, rz, obs, inv_var, infer_velocity, medium_velocity, out_x, nullptr,
                     accumulate, as_stream(stream));
  });
}

int hmc_srcloc3d_gradient(int dtype, int64_t E, int64_t S, int64_t C, const void* M, const void* rx, const void* ry,
                          const void* rz, const void* obs, const void* inv_var, int infer_velocity,
                          double medium_velocity, void* out_g, int accumulate, void* stream) {
  return HMC_DISPATCH(dtype, T, [&] {
    return srcloc<T>(true, E, S, C, M, rx, ry, rz, obs, inv_var, infer_velocity, medium_velocity, nullptr, out_g,
                     accumulate, as_stream(stream));
  });
}

}  // extern "C"
