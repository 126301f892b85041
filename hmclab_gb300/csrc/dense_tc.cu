// Tensor-core (tcgen05) contraction of a dense matrix with all chains at once,
// with the HMC step fused into the epilogue.
//
//   D[c][r] = sum_k Q[c][k] A[r][k]          (c: chain, r: matrix row, k: model index)
//
// computed as BF16 hi/lo split products with FP32 accumulation in TMEM:
//   Q A ~ Qhi Ahi + Qhi Alo + Qlo Ahi,  x_hi = bf16(x), x_lo = bf16(x - x_hi).
// A is GtG (gradient of the premultiplied dense LinearMatrix,
// LinearMatrix.py:204-208) or G (residual misfit, LinearMatrix.py:193-202);
// Q holds the chains' positions transposed to chain-major [C][ld] (K-major
// operand), re-split by the epilogue of every fused step.
//
// Kernel structure (one 128-chain x 256-row output tile per CTA, 320 threads):
//   warp 0  TMEM allocation; one lane issues TMA tile loads (128B swizzle)
//   warp 1  one lane issues tcgen05.mma (M=128, N=256, K=16) and commits
//   warps 2-9  epilogue: tcgen05.ld of the accumulator (lane = chain),
//           then one of:
//             EPI_GRAD       g[r][c] (+)= D - bias[r]
//             EPI_STEP       g = D - bias + prior'(q); p -= kick*eps*g;
//                            q += drift*eps*M^-1 p; reflect; write p, q and
//                            the next step's Q hi/lo operand
//             EPI_MISFIT     partial[tile][c] = sum_r (D - data[r])^2 inv_var[r]
// Every mbarrier wait is bounded (2 s of %globaltimer by default, see
// hmc_set_wait_limits); on expiry the CTA sets
// *status = HMC_ERR_TIMEOUT, stops issuing work, waits (bounded) for its own
// copies and MMAs, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "common.cuh"

namespace hmc {
namespace tc {

constexpr int BM = 128;                   // chains per tile (UMMA M)
constexpr int BN = 256;                   // matrix rows per tile (UMMA N)
constexpr int SWZ = 64;                   // swizzle span in bytes (64 or 128)
constexpr int BK = SWZ / 2;               // k per stage = one swizzle row of bf16
constexpr int UK = 16;                    // k per tcgen05.mma (kind::f16)
constexpr int STAGES = SWZ == 64 ? 4 : 2;
constexpr int A_BYTES = BM * BK * 2;      // per operand half (chains)
constexpr int B_BYTES = BN * BK * 2;      // per operand half (rows)
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;  // hi/lo split (3 products)
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
// Stage layout for NPROD products: q_hi | q_lo | a_hi | a_lo (NPROD = 3) or
// q | a (NPROD = 1, plain BF16 operands).
template <int NPROD>
struct Stage {
  static constexpr int bytes = NPROD == 3 ? STAGE_BYTES : A_BYTES + B_BYTES;
  static constexpr int q_lo = A_BYTES;
  static constexpr int a_hi = NPROD == 3 ? 2 * A_BYTES : A_BYTES;
  static constexpr int a_lo = a_hi + B_BYTES;
};
constexpr int THREADS = 320;  // warp 0 TMA, warp 1 MMA, warps 2-9 epilogue
constexpr uint32_t TMEM_COLS = 256;

enum Epi { EPI_GRAD = 0, EPI_STEP = 1, EPI_MISFIT = 2, EPI_MLP_HIDDEN = 3, EPI_MLP_OUT = 4, EPI_MLP_BACK = 5 };
enum Prior { PRIOR_NONE = 0, PRIOR_NORMAL = 1, PRIOR_LAPLACE = 2 };

struct EpiParams {
  int64_t C;        // chains
  int64_t rows;     // rows of A (d for GtG, n for G)
  const float* bias;   // Gtd0 (gradient) or data (misfit), [rows]
  // EPI_GRAD
  float* g;            // [rows][C]
  int accumulate;
  // EPI_STEP
  int prior;
  const float* prior_mean;
  const float* prior_w;  // inverse variance (normal) or inverse dispersion (laplace)
  float* p;              // [d][C]
  float* q;              // [d][C]
  const float* eps_local;  // [C]
  float kick, drift;
  const float* minv;       // [d] inverse mass diagonal or null (unit)
  const float* lo;
  const float* hi;
  const float* center;     // [d] or null: the next operand holds q - center
  int32_t* flags;          // [C]
  __nv_bfloat16* qn_hi;    // next operand [C][ldq]
  __nv_bfloat16* qn_lo;
  int64_t ldq;
  // EPI_MISFIT
  const float* inv_var;    // [rows]
  double* partial;         // [n_tiles][C]
  // EPI_MLP_*: M = batch rows (C), N = features (rows)
  float* z;                // [C][ldz] pre-activations (written by HIDDEN, read by BACK)
  int64_t ldz;
  __nv_bfloat16* act;      // [C][ld_act] activations / deltas (BF16)
  int64_t ld_act;
  __nv_bfloat16* act_t;    // [rows][ld_act_t] the same, transposed
  int64_t ld_act_t;
  float* y;                // [C][ldy] network output (OUT)
  int64_t ldy;
  float* g_state;          // [rows][C] scale * y + shift (OUT, may be null)
  const float* out_scale;
  const float* out_shift;
  int* status;
  uint64_t wait_ns;  // bounded-wait limit (filled by the launcher)
  int withhold;      // test hook: block (0, 0) skips its first stage's copies
};

// GELU(z) = z Phi(z) and its derivative Phi(z) + z phi(z), with
// Phi(z) = erfc(-z / sqrt 2) / 2, which stays accurate in the negative tail
// (1 + erf cancels there in FP32).
__device__ __forceinline__ float std_normal_cdf(float z) { return 0.5f * erfcf(-z * 0.70710678118654752f); }
__device__ __forceinline__ float gelu(float z) { return z * std_normal_cdf(z); }
__device__ __forceinline__ float gelu_grad(float z) {
  return std_normal_cdf(z) + z * 0.39894228040143268f * __expf(-0.5f * z * z);
}

// ---- PTX helpers ------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred P;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, P;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait; false when the limit (2 s in production) expired or another
// role aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                          uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*abort_flag) return false;
    if (globaltimer() - t0 > limit_ns) return false;
  }
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major tile, SWZ-byte swizzle, rows of
// SWZ bytes, 8-row groups 8*SWZ bytes apart (tcgen05 descriptor, version 1).
__device__ __forceinline__ uint64_t sdesc_k_sw(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;              // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)((8 * SWZ) >> 4) << 32;  // stride byte offset
  d |= (uint64_t)1 << 46;              // descriptor version
  d |= (uint64_t)(SWZ == 128 ? 2 : 4) << 61;  // SWIZZLE_128B / SWIZZLE_64B
  return d;
}

// Instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major.
constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred P;\n\t"
      "setp.ne.b32 P, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, P;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// ---- the kernel -------------------------------------------------------------
template <int EPI, int NPROD>
__global__ void __launch_bounds__(THREADS, 1)
    chain_gemm_kernel(const __grid_constant__ CUtensorMap tq_hi, const __grid_constant__ CUtensorMap tq_lo,
                      const __grid_constant__ CUtensorMap ta_hi, const __grid_constant__ CUtensorMap ta_lo,
                      int num_kb, EpiParams ep) {
  using S = Stage<NPROD>;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES * S::bytes);
  uint64_t* empty = full + STAGES;
  uint64_t* accum = empty + STAGES;
  uint32_t* tmem_slot = (uint32_t*)(accum + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int m0 = blockIdx.x * BM;  // first chain of the tile
  const int n0 = blockIdx.y * BN;  // first matrix row of the tile

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(accum, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  int tma_issued_stage_uses = 0;  // producer bookkeeping for the abort drain
  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer ----------------
    const int kb_rot = (int)((blockIdx.x + 7u * blockIdx.y) % (unsigned)num_kb);
    for (int kb = 0; kb < num_kb; ++kb) {
      const int s = kb % STAGES;
      if (kb >= STAGES) {
        if (!mbar_wait(&empty[s], ((kb / STAGES) & 1) ^ 1, abort_flag, ep.wait_ns)) {
          *abort_flag = 1;
          break;
        }
      }
      if (ep.withhold && kb == 0 && blockIdx.x == 0 && blockIdx.y == 0) {
        // test hook: this stage is never armed, so the MMA issuer's wait on
        // it runs out; nothing is in flight for it
        ++tma_issued_stage_uses;
        continue;
      }
      unsigned char* st = smem + s * S::bytes;
      mbar_expect_tx(&full[s], S::bytes);
      // CTAs that share an operand tile start at different k-blocks, so
      // they do not all fetch the same lines from the same L2 slices at once.
      const int kx = ((kb + kb_rot) % num_kb) * BK;
      tma_load_2d(st, &tq_hi, &full[s], kx, m0);
      tma_load_2d(st + S::a_hi, &ta_hi, &full[s], kx, n0);
      if (NPROD == 3) {
        tma_load_2d(st + S::q_lo, &tq_lo, &full[s], kx, m0);
        tma_load_2d(st + S::a_lo, &ta_lo, &full[s], kx, n0);
      }
      ++tma_issued_stage_uses;
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer ----------------
    constexpr uint32_t idesc = idesc_bf16(BM, BN);
    bool ok = true;
    for (int kb = 0; kb < num_kb; ++kb) {
      const int s = kb % STAGES;
      if (!mbar_wait(&full[s], (kb / STAGES) & 1, abort_flag, ep.wait_ns)) {
        *abort_flag = 1;
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t sa_hi = smem_u32(smem + s * S::bytes);
      const uint32_t sa_lo = sa_hi + S::q_lo;
      const uint32_t sb_hi = sa_hi + S::a_hi;
      const uint32_t sb_lo = sa_hi + S::a_lo;
#pragma unroll
      for (int kk = 0; kk < BK / UK; ++kk) {
        const uint32_t off = kk * UK * 2;  // bytes along the swizzled row
        const uint64_t qh = sdesc_k_sw(sa_hi + off);
        const uint64_t ah = sdesc_k_sw(sb_hi + off);
        umma_bf16(tmem, qh, ah, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
        if (NPROD == 3) {
          const uint64_t ql = sdesc_k_sw(sa_lo + off), al = sdesc_k_sw(sb_lo + off);
          umma_bf16(tmem, qh, al, idesc, 1u);
          umma_bf16(tmem, ql, ah, idesc, 1u);
        }
      }
      umma_commit(&empty[s]);  // frees the stage once these MMAs complete
    }
    umma_commit(accum);  // arrives when every MMA issued above completed
    (void)ok;
  } else if (warp >= 2) {
    // ---------------- epilogue ----------------
    // Eight warps: warp w reads TMEM lanes 32*(w%4)..+31 (its chains) and
    // handles every other 16-column chunk of the tile (half = 0 or 1).
    const int quarter = warp % 4;
    const int half = (warp - 2) / 4;
    const int lane_base = 32 * quarter;
    const int64_t c = (int64_t)m0 + lane_base + lane;  // this thread's chain
    float* __restrict__ pp = ep.p;
    float* __restrict__ qq = ep.q;
    const int64_t C = ep.C;
    // While the MMAs run, pull this tile's rows of p and q into L2.
    if (EPI == EPI_STEP) {
      const int et = threadIdx.x - 64;  // 0..255
      const int64_t row = (int64_t)n0 + et;
      if (row < ep.rows && m0 < C) {
        const int64_t cnt = (C - m0) < BM ? (C - m0) : BM;
        for (int64_t off = 0; off < cnt; off += 32) {
          asm volatile("prefetch.global.L2 [%0];" ::"l"(pp + row * C + m0 + off));
          asm volatile("prefetch.global.L2 [%0];" ::"l"(qq + row * C + m0 + off));
        }
      }
    }
    // warp-uniform: the TMEM loads below are warp-collective
    const bool ready = __all_sync(0xffffffffu, mbar_wait(accum, 0, abort_flag, ep.wait_ns) ? 1 : 0) != 0;
    tc_fence_after();
    const bool live_c = ready && c < C;
    const uint32_t tbase = tmem + ((uint32_t)lane_base << 16);
    float eps_k = 0.f, eps_d = 0.f;
    if (EPI == EPI_STEP && live_c) {
      const float e = ep.eps_local[c];
      eps_k = ep.kick * e;
      eps_d = ep.drift * e;
    }
    double misfit_part = 0.0;
    bool oob = false;
    for (int cb = half; cb < BN / 16; cb += 2) {
      float acc[16];
      if (ready) tmem_ld16(tbase + cb * 16, acc);  // warp-collective: every lane takes part
      if (!live_c) continue;
      const int64_t r0 = (int64_t)n0 + cb * 16;
      const int nr = (int)((ep.rows - r0) < 16 ? (ep.rows - r0) : 16);  // valid rows in this chunk
      if (EPI == EPI_MISFIT) {
        float s = 0.f;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          if (j < nr) {
            const float res = acc[j] - ep.bias[r0 + j];
            s = fmaf(res * res, ep.inv_var[r0 + j], s);
          }
        }
        misfit_part += (double)s;
      } else if (EPI == EPI_GRAD) {
        float gold[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) gold[j] = (ep.accumulate && j < nr) ? ep.g[(r0 + j) * C + c] : 0.f;
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (j < nr) ep.g[(r0 + j) * C + c] = acc[j] - (ep.bias ? ep.bias[r0 + j] : 0.f) + gold[j];
      } else if (EPI == EPI_MLP_HIDDEN || EPI == EPI_MLP_BACK) {
        // HIDDEN: z = acc + b, a = GELU(z); BACK: delta = acc * GELU'(z).
        // Both write BF16 [c][r] (next contraction, K = features) and
        // [r][c] (weight gradients, K = batch).
        __align__(16) __nv_bfloat16 a16[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          float v = 0.f;
          if (j < nr) {
            const int64_t r = r0 + j;
            if (EPI == EPI_MLP_HIDDEN) {
              const float zv = acc[j] + ep.bias[r];
              ep.z[c * ep.ldz + r] = zv;
              v = gelu(zv);
            } else {
              v = acc[j] * gelu_grad(ep.z[c * ep.ldz + r]);
            }
          }
          a16[j] = __float2bfloat16_rn(v);
          if (j < nr) ep.act_t[(r0 + j) * ep.ld_act_t + c] = a16[j];
        }
        // only chunks holding valid rows: the columns past `rows` may belong
        // to another array stored in the same row (the output layer's skip input)
        if (nr > 0 && r0 + 16 <= ep.ld_act) {
          uint4* dst = (uint4*)(ep.act + c * ep.ld_act + r0);
          dst[0] = ((const uint4*)a16)[0];
          dst[1] = ((const uint4*)a16)[1];
        }
      } else if (EPI == EPI_MLP_OUT) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          if (j < nr) {
            const int64_t r = r0 + j;
            const float yv = acc[j] + ep.bias[r];
            if (ep.y) ep.y[c * ep.ldy + r] = yv;
            if (ep.g_state) ep.g_state[r * C + c] = ep.out_scale[r] * yv + ep.out_shift[r];
          }
        }
      } else {  // EPI_STEP
        // all loads of the chunk first (independent, in flight together)
        float qv[16], pv[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          qv[j] = j < nr ? qq[(r0 + j) * C + c] : 0.f;
          pv[j] = j < nr ? pp[(r0 + j) * C + c] : 0.f;
        }
        __align__(16) __nv_bfloat16 hi16[16];
        __align__(16) __nv_bfloat16 lo16[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int64_t r = r0 + j;
          float qs = 0.f;
          if (j < nr) {
            float gv = acc[j] - ep.bias[r];
            if (ep.prior == PRIOR_NORMAL) {
              gv += ep.prior_w[r] * (qv[j] - ep.prior_mean[r]);
            } else if (ep.prior == PRIOR_LAPLACE) {
              const float dq = qv[j] - ep.prior_mean[r];
              gv += (dq > 0.f ? 1.f : (dq < 0.f ? -1.f : 0.f)) * ep.prior_w[r];
            }
            pv[j] = pv[j] - eps_k * gv;
            if (eps_d != 0.f) {
              const float mp = ep.minv ? ep.minv[r] * pv[j] : pv[j];
              float qn = qv[j] + eps_d * mp;
              if (ep.lo && qn < ep.lo[r]) {
                qn += 2.f * (ep.lo[r] - qn);
                pv[j] = -pv[j];
              }
              if (ep.hi && qn > ep.hi[r]) {
                qn += 2.f * (ep.hi[r] - qn);
                pv[j] = -pv[j];
              }
              if ((ep.lo && qn < ep.lo[r]) || (ep.hi && qn > ep.hi[r])) oob = true;
              qv[j] = qn;
            }
            qs = ep.center != nullptr ? qv[j] - ep.center[r] : qv[j];
          }
          const __nv_bfloat16 h = __float2bfloat16_rn(qs);
          hi16[j] = h;
          lo16[j] = __float2bfloat16_rn(qs - __bfloat162float(h));
        }
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          if (j < nr) {
            pp[(r0 + j) * C + c] = pv[j];
            if (eps_d != 0.f) qq[(r0 + j) * C + c] = qv[j];
          }
        }
        if (ep.qn_hi != nullptr && r0 < ep.ldq) {
          uint4* dh = (uint4*)(ep.qn_hi + c * ep.ldq + r0);
          uint4* dl = (uint4*)(ep.qn_lo + c * ep.ldq + r0);
          dh[0] = ((const uint4*)hi16)[0];
          dh[1] = ((const uint4*)hi16)[1];
          dl[0] = ((const uint4*)lo16)[0];
          dl[1] = ((const uint4*)lo16)[1];
        }
      }
    }
    if (EPI == EPI_MISFIT && live_c) {
      // two warps share each chain: combine their halves through shared memory
      double* red = (double*)(smem);  // operand stages are idle once the accumulator is ready
      if (half == 1) red[lane_base + lane] = misfit_part;
    }
    if (EPI == EPI_STEP && oob) atomicOr(&ep.flags[c], HMC_FLAG_OUT_OF_BOUNDS);
    if (!ready && threadIdx.x == 64) {
      atomicExch(ep.status, HMC_ERR_TIMEOUT);
      *abort_flag = 1;
    }
    if (EPI == EPI_MISFIT) {
      asm volatile("bar.sync 1, 256;" ::: "memory");  // the eight epilogue warps only
      if (half == 0 && live_c) {
        const double* red = (const double*)(smem);
        ep.partial[(int64_t)blockIdx.y * C + c] = misfit_part + red[lane_base + lane];
      }
    }
  }
  // ---------------- teardown ----------------
  tc_fence_before();
  __syncthreads();
  if (*abort_flag) {
    // Drain what this CTA put in flight before releasing TMEM and smem.
    if (warp == 1 && lane == 0) {
      const uint64_t t0 = globaltimer();
      while (!mbar_try_wait(accum, 0) && globaltimer() - t0 < ep.wait_ns) {
      }
    }
    if (warp == 0 && lane == 0) {
      for (int u = 0; u < tma_issued_stage_uses && u < num_kb; ++u) {
        const int s = u % STAGES;
        const uint64_t t0 = globaltimer();
        while (!mbar_try_wait(&full[s], (u / STAGES) & 1) && globaltimer() - t0 < ep.wait_ns) {
        }
      }
      atomicExch(ep.status, HMC_ERR_TIMEOUT);
    }
    __syncthreads();
  }
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// ---- the leapfrog update as its own pass ------------------------------------
// The update hmc_tc_step_split runs after an EPI_GRAD contraction wrote
// g = GtG q - bias: the prior's gradient, kick, drift and bound reflection
// (the same expressions, in the same order, as the EPI_STEP epilogue, so
// the results are bitwise equal), then the next operand q - center split
// into BF16 hi/lo and transposed to chain-major [C][ldq] through a
// shared-memory tile (rows d..ldq-1 written as zeros).  A thread first loads
// everything its rows need (the state and the per-row prior, mass, bound
// and centre values, bounds absent = -/+inf, which no position crosses)
// into registers, so no load waits behind a store that might alias it.
constexpr int UPDATE_ROWS = 16;  // threadIdx.y extent of the update kernels (swept: 4, 8, 16, 32)
constexpr int UPDATE_RPT = 32 / UPDATE_ROWS;  // rows per thread

struct RowParams {
  float pw, pm, mi, lo, hi, ce;
};
__device__ __forceinline__ RowParams row_params(const EpiParams& ep, int64_t r, int64_t d) {
  RowParams rp{0.f, 0.f, 1.f, -INFINITY, INFINITY, 0.f};
  if (r < d) {
    if (ep.prior != PRIOR_NONE) {
      rp.pw = ep.prior_w[r];
      rp.pm = ep.prior_mean[r];
    }
    if (ep.minv) rp.mi = ep.minv[r];
    if (ep.lo) rp.lo = ep.lo[r];
    if (ep.hi) rp.hi = ep.hi[r];
    if (ep.center) rp.ce = ep.center[r];
  }
  return rp;
}

// One element: returns the next operand's value q - center; updates p, q.
__device__ __forceinline__ float update_one(const EpiParams& ep, const RowParams& rp, float gv, float& qv, float& pv,
                                            float eps_k, float eps_d, bool& oob) {
  if (ep.prior == PRIOR_NORMAL) {
    gv += rp.pw * (qv - rp.pm);
  } else if (ep.prior == PRIOR_LAPLACE) {
    const float dq = qv - rp.pm;
    gv += (dq > 0.f ? 1.f : (dq < 0.f ? -1.f : 0.f)) * rp.pw;
  }
  pv = pv - eps_k * gv;
  if (eps_d != 0.f) {
    const float mp = ep.minv ? rp.mi * pv : pv;
    float qn = qv + eps_d * mp;
    if (qn < rp.lo) {
      qn += 2.f * (rp.lo - qn);
      pv = -pv;
    }
    if (qn > rp.hi) {
      qn += 2.f * (rp.hi - qn);
      pv = -pv;
    }
    if (qn < rp.lo || qn > rp.hi) oob = true;
    qv = qn;
  }
  return ep.center != nullptr ? qv - rp.ce : qv;
}

__global__ void __launch_bounds__(32 * UPDATE_ROWS) step_update_kernel(int64_t d, EpiParams ep,
                                                                        const float* __restrict__ g) {
  __shared__ float tile[32][33];
  const int64_t C = ep.C;
  const int64_t i0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  const int64_t c = c0 + threadIdx.x;
  float eps_k = 0.f, eps_d = 0.f;
  if (c < C) {
    const float e = ep.eps_local[c];
    eps_k = ep.kick * e;
    eps_d = ep.drift * e;
  }
  float qa[UPDATE_RPT], pa[UPDATE_RPT], ga[UPDATE_RPT];
  RowParams rp[UPDATE_RPT];
#pragma unroll
  for (int u = 0; u < UPDATE_RPT; ++u) {
    const int64_t r = i0 + threadIdx.y + u * UPDATE_ROWS;
    const bool in = r < d && c < C;
    const int64_t k = r * C + c;
    qa[u] = in ? ep.q[k] : 0.f;
    pa[u] = in ? ep.p[k] : 0.f;
    ga[u] = in ? g[k] : 0.f;
    rp[u] = row_params(ep, r, d);
  }
  bool oob = false;
#pragma unroll
  for (int u = 0; u < UPDATE_RPT; ++u) {
    const int y = threadIdx.y + u * UPDATE_ROWS;
    const int64_t r = i0 + y;
    float qs = 0.f;
    if (r < d && c < C) {
      qs = update_one(ep, rp[u], ga[u], qa[u], pa[u], eps_k, eps_d, oob);
      const int64_t k = r * C + c;
      ep.p[k] = pa[u];
      if (eps_d != 0.f) ep.q[k] = qa[u];
    }
    tile[y][threadIdx.x] = qs;
  }
  if (oob) atomicOr(&ep.flags[c], HMC_FLAG_OUT_OF_BOUNDS);
  __syncthreads();
#pragma unroll
  for (int u = 0; u < UPDATE_RPT; ++u) {
    const int y = threadIdx.y + u * UPDATE_ROWS;
    const int64_t cc = c0 + y, i = i0 + threadIdx.x;
    if (cc < C && i < ep.ldq) {
      const float v = tile[threadIdx.x][y];
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      ep.qn_hi[cc * ep.ldq + i] = h;
      ep.qn_lo[cc * ep.ldq + i] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
  }
}

// The same update with 16-byte accesses when C is a multiple of 4: a block
// owns 32 rows x 128 chains, a thread four consecutive chains of four rows
// (float4 loads and stores of q, p and g), and the next operand is written
// from a 32 x 129 shared-memory tile, a warp per chain and a lane per row.
__global__ void __launch_bounds__(32 * UPDATE_ROWS) step_update4_kernel(int64_t d, EpiParams ep,
                                                                         const float* __restrict__ g) {
  __shared__ float tile[32][129];
  const int64_t C = ep.C;
  const int64_t i0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 128;
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int64_t c = c0 + 4 * tx;  // first of this thread's four chains
  const bool live = c < C;        // C % 4 == 0: all four or none
  float eps_k[4] = {0.f, 0.f, 0.f, 0.f}, eps_d[4] = {0.f, 0.f, 0.f, 0.f};
  if (live) {
    const float4 e = *(const float4*)(ep.eps_local + c);
    const float ev[4] = {e.x, e.y, e.z, e.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      eps_k[j] = ep.kick * ev[j];
      eps_d[j] = ep.drift * ev[j];
    }
  }
  float4 qa[UPDATE_RPT], pa[UPDATE_RPT], ga[UPDATE_RPT];
  RowParams rp[UPDATE_RPT];
#pragma unroll
  for (int u = 0; u < UPDATE_RPT; ++u) {
    const int64_t r = i0 + ty + u * UPDATE_ROWS;
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    const bool in = live && r < d;
    const int64_t k = r * C + c;
    qa[u] = in ? *(const float4*)(ep.q + k) : z;
    pa[u] = in ? *(const float4*)(ep.p + k) : z;
    ga[u] = in ? *(const float4*)(g + k) : z;
    rp[u] = row_params(ep, r, d);
  }
  bool oob[4] = {false, false, false, false};
#pragma unroll
  for (int u = 0; u < UPDATE_RPT; ++u) {
    const int y = ty + u * UPDATE_ROWS;
    const int64_t r = i0 + y;
    float qv[4] = {qa[u].x, qa[u].y, qa[u].z, qa[u].w};
    float pv[4] = {pa[u].x, pa[u].y, pa[u].z, pa[u].w};
    const float gin[4] = {ga[u].x, ga[u].y, ga[u].z, ga[u].w};
    float qs[4] = {0.f, 0.f, 0.f, 0.f};
    if (live && r < d) {
#pragma unroll
      for (int j = 0; j < 4; ++j) qs[j] = update_one(ep, rp[u], gin[j], qv[j], pv[j], eps_k[j], eps_d[j], oob[j]);
      const int64_t k = r * C + c;
      *(float4*)(ep.p + k) = make_float4(pv[0], pv[1], pv[2], pv[3]);
      // a chain with zero drift keeps its position (the scalar kernels skip its store)
      if (eps_d[0] != 0.f && eps_d[1] != 0.f && eps_d[2] != 0.f && eps_d[3] != 0.f) {
        *(float4*)(ep.q + k) = make_float4(qv[0], qv[1], qv[2], qv[3]);
      } else {
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (eps_d[j] != 0.f) ep.q[k + j] = qv[j];
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) tile[y][4 * tx + j] = qs[j];
  }
#pragma unroll
  for (int j = 0; j < 4; ++j)
    if (oob[j]) atomicOr(&ep.flags[c + j], HMC_FLAG_OUT_OF_BOUNDS);
  __syncthreads();
  for (int cl = ty; cl < 128; cl += UPDATE_ROWS) {
    const int64_t cc = c0 + cl, i = i0 + tx;
    if (cc < C && i < ep.ldq) {
      const float v = tile[tx][cl];
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      ep.qn_hi[cc * ep.ldq + i] = h;
      ep.qn_lo[cc * ep.ldq + i] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
  }
}

// ---- helpers for the operands ------------------------------------------------
// hi/lo split of a row-major FP32 matrix into padded [rows][ld] BF16 arrays
// (columns cols..ld-1 are zero).
__global__ void split_rows_kernel(int64_t rows, int64_t cols, const float* __restrict__ src, int64_t ld,
                                  __nv_bfloat16* hi, __nv_bfloat16* lo) {
  const int64_t total = rows * ld;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / ld, k = t % ld;
    const float v = k < cols ? src[r * cols + k] : 0.f;
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    hi[t] = h;
    lo[t] = __float2bfloat16_rn(v - __bfloat162float(h));
  }
}

// Chain state q [d][C] -> chain-major hi/lo [C][ld] (zero pad), 32x32 tiles.
__global__ void split_transpose_kernel(int64_t d, int64_t C, const float* __restrict__ q,
                                       const float* __restrict__ center, int64_t ld, __nv_bfloat16* hi,
                                       __nv_bfloat16* lo) {
  __shared__ float tile[32][33];
  const int64_t i0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t i = i0 + y, c = c0 + threadIdx.x;
    tile[y][threadIdx.x] = (i < d && c < C) ? (center ? q[i * C + c] - center[i] : q[i * C + c]) : 0.f;
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t c = c0 + y, i = i0 + threadIdx.x;
    if (c < C && i < ld) {
      const float v = tile[threadIdx.x][y];
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      hi[c * ld + i] = h;
      lo[c * ld + i] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
  }
}

// x[c] (+)= 0.5 * sum_t partial[t][c]
__global__ void reduce_partials_kernel(int64_t C, int tiles, const double* __restrict__ partial, double* x,
                                       int accumulate) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= C) return;
  double s = 0.0;
  for (int t = 0; t < tiles; ++t) s += partial[(int64_t)t * C + c];
  x[c] = accumulate ? x[c] + 0.5 * s : 0.5 * s;
}

// ---- host side -----------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
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

// 2-D BF16 tensor map over a [rows][ld] array whose first `cols` columns are
// valid (columns >= cols read as zero), box = box_rows x 64.
int make_map(CUtensorMap* map, const void* base, int64_t rows, int64_t cols, int64_t ld, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return fail(HMC_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
  HMC_REQUIRE(((uintptr_t)base & 15) == 0, "tensor-core operand must be 16-byte aligned");
  HMC_REQUIRE((ld * 2) % 16 == 0 && ld >= cols, "tensor-core operand pitch must be a multiple of 8 elements");
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, SWZ == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(HMC_ERR_INVALID_ARG, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return HMC_OK;
}

template <int EPI, int NPROD = 3>
int launch(int64_t C, int64_t rows, int64_t K, const void* q_hi, const void* q_lo, int64_t ldq, const void* a_hi,
           const void* a_lo, int64_t lda, const EpiParams& ep, cudaStream_t st) {
  HMC_REQUIRE(C > 0 && rows > 0 && K > 0, "tensor-core contraction: bad sizes");
  HMC_REQUIRE(C < (1ll << 31) && rows < (1ll << 31) && K < (1ll << 31), "tensor-core contraction: too large");
  HMC_REQUIRE(ep.status != nullptr, "tensor-core contraction: null status word");
  CUtensorMap mq_hi, mq_lo, ma_hi, ma_lo;
  HMC_TRY(make_map(&mq_hi, q_hi, C, K, ldq, BM));
  HMC_TRY(make_map(&ma_hi, a_hi, rows, K, lda, BN));
  if (NPROD == 3) {
    HMC_TRY(make_map(&mq_lo, q_lo, C, K, ldq, BM));
    HMC_TRY(make_map(&ma_lo, a_lo, rows, K, lda, BN));
  } else {
    mq_lo = mq_hi;
    ma_lo = ma_hi;
  }
  constexpr int smem = STAGES * Stage<NPROD>::bytes + 1024 + 256;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(chain_gemm_kernel<EPI, NPROD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(chain_gemm_kernel)");
    attr_set = true;
  }
  const int num_kb = (int)((K + BK - 1) / BK);
  const dim3 grid((unsigned)((C + BM - 1) / BM), (unsigned)((rows + BN - 1) / BN));
  HMC_REQUIRE(grid.y <= 65535, "tensor-core contraction: too many rows");
  EpiParams e = ep;
  const WaitLimits wl = wait_limits();
  e.wait_ns = wl.ns;
  e.withhold = wl.withhold;
  chain_gemm_kernel<EPI, NPROD><<<grid, THREADS, smem, st>>>(mq_hi, mq_lo, ma_hi, ma_lo, num_kb, e);
  return check_launch("chain_gemm_kernel");
}

}  // namespace tc
}  // namespace hmc

using namespace hmc;
using namespace hmc::tc;

extern "C" {

HMC_API int hmc_split_bf16(int64_t rows, int64_t cols, const float* src, int64_t ld, void* hi, void* lo,
                           void* stream) {
  HMC_REQUIRE(rows >= 0 && cols >= 0 && ld >= cols && ld % 8 == 0, "hmc_split_bf16: bad sizes");
  if (rows == 0) return HMC_OK;
  HMC_REQUIRE(src && hi && lo, "hmc_split_bf16: null argument");
  const unsigned g = blocks_for(rows * ld, 256) > 152u * 16 ? 152u * 16 : blocks_for(rows * ld, 256);
  split_rows_kernel<<<g, 256, 0, as_stream(stream)>>>(rows, cols, src, ld, (__nv_bfloat16*)hi, (__nv_bfloat16*)lo);
  return check_launch("split_rows_kernel");
}

HMC_API int hmc_split_bf16_transpose(int64_t d, int64_t C, const float* q, const float* center, int64_t ld,
                                     void* hi, void* lo, void* stream) {
  HMC_REQUIRE(d > 0 && C >= 0 && ld >= d && ld % 8 == 0, "hmc_split_bf16_transpose: bad sizes");
  if (C == 0) return HMC_OK;
  HMC_REQUIRE(q && hi && lo, "hmc_split_bf16_transpose: null argument");
  HMC_REQUIRE((ld + 31) / 32 <= 65535, "hmc_split_bf16_transpose: too many rows");
  const dim3 grid((unsigned)((C + 31) / 32), (unsigned)((ld + 31) / 32));
  split_transpose_kernel<<<grid, dim3(32, 8), 0, as_stream(stream)>>>(d, C, q, center, ld, (__nv_bfloat16*)hi,
                                                                     (__nv_bfloat16*)lo);
  return check_launch("split_transpose_kernel");
}

HMC_API int hmc_tc_gradient(int64_t rows, int64_t K, int64_t C, const void* a_hi, const void* a_lo, int64_t lda,
                            const void* q_hi, const void* q_lo, int64_t ldq, const float* bias, float* g,
                            int accumulate, int* status, void* stream) {
  HMC_REQUIRE(bias && g, "hmc_tc_gradient: null argument");
  EpiParams ep = {};
  ep.C = C;
  ep.rows = rows;
  ep.bias = bias;
  ep.g = g;
  ep.accumulate = accumulate;
  ep.status = status;
  return launch<EPI_GRAD>(C, rows, K, q_hi, q_lo, ldq, a_hi, a_lo, lda, ep, as_stream(stream));
}

HMC_API int hmc_tc_step(const hmc_chains* s, const void* a_hi, const void* a_lo, int64_t lda, const void* q_hi,
                        const void* q_lo, void* qn_hi, void* qn_lo, int64_t ldq, const float* center,
                        const float* bias, int prior, const float* prior_mean, const float* prior_w, double kick,
                        double drift, int* status, void* stream) {
  HMC_REQUIRE(s != nullptr && s->dtype == HMC_F32, "hmc_tc_step: needs an FP32 chain state");
  HMC_REQUIRE(s->mass_kind == HMC_MASS_UNIT || s->mass_kind == HMC_MASS_DIAG,
              "hmc_tc_step: unit or diagonal mass only");
  HMC_REQUIRE(bias && s->p && s->q && s->eps_local && s->flags, "hmc_tc_step: missing buffer");
  HMC_REQUIRE(prior == PRIOR_NONE || (prior_mean && prior_w), "hmc_tc_step: prior needs mean and weights");
  HMC_REQUIRE(prior >= PRIOR_NONE && prior <= PRIOR_LAPLACE, "hmc_tc_step: unknown prior kind");
  HMC_REQUIRE(ldq % 16 == 0, "hmc_tc_step: operand pitch must be a multiple of 16");
  EpiParams ep = {};
  ep.C = s->chains;
  ep.rows = s->dims;
  ep.bias = bias;
  ep.prior = prior;
  ep.prior_mean = prior_mean;
  ep.prior_w = prior_w;
  ep.p = (float*)s->p;
  ep.q = (float*)s->q;
  ep.eps_local = (const float*)s->eps_local;
  ep.kick = (float)kick;
  ep.drift = (float)drift;
  ep.minv = s->mass_kind == HMC_MASS_DIAG ? (const float*)s->mass_inv_diag : nullptr;
  ep.lo = (const float*)s->lower;
  ep.hi = (const float*)s->upper;
  ep.flags = s->flags;
  ep.center = center;
  HMC_REQUIRE(qn_hi != q_hi && qn_lo != q_lo, "hmc_tc_step: the next operand must not alias the current one");
  ep.qn_hi = (__nv_bfloat16*)qn_hi;
  ep.qn_lo = (__nv_bfloat16*)qn_lo;
  ep.ldq = ldq;
  ep.status = status;
  return launch<EPI_STEP>(s->chains, s->dims, s->dims, q_hi, q_lo, ldq, a_hi, a_lo, lda, ep, as_stream(stream));
}

HMC_API int hmc_tc_step_split(const hmc_chains* s, const void* a_hi, const void* a_lo, int64_t lda,
                              const void* q_hi, const void* q_lo, void* qn_hi, void* qn_lo, int64_t ldq,
                              const float* center, const float* bias, int prior, const float* prior_mean,
                              const float* prior_w, double kick, double drift, int* status, void* stream) {
  HMC_REQUIRE(s != nullptr && s->dtype == HMC_F32, "hmc_tc_step_split: needs an FP32 chain state");
  HMC_REQUIRE(s->mass_kind == HMC_MASS_UNIT || s->mass_kind == HMC_MASS_DIAG,
              "hmc_tc_step_split: unit or diagonal mass only");
  HMC_REQUIRE(bias && s->p && s->q && s->g && s->eps_local && s->flags, "hmc_tc_step_split: missing buffer");
  HMC_REQUIRE(prior == PRIOR_NONE || (prior_mean && prior_w), "hmc_tc_step_split: prior needs mean and weights");
  HMC_REQUIRE(prior >= PRIOR_NONE && prior <= PRIOR_LAPLACE, "hmc_tc_step_split: unknown prior kind");
  HMC_REQUIRE(ldq % 16 == 0 && ldq >= s->dims, "hmc_tc_step_split: operand pitch must be a multiple of 16 >= d");
  HMC_REQUIRE(qn_hi && qn_lo && qn_hi != q_hi && qn_lo != q_lo,
              "hmc_tc_step_split: the next operand must exist and not alias the current one");
  EpiParams eg = {};
  eg.C = s->chains;
  eg.rows = s->dims;
  eg.bias = bias;
  eg.g = (float*)s->g;
  eg.accumulate = 0;
  eg.status = status;
  cudaStream_t st = as_stream(stream);
  HMC_TRY(launch<EPI_GRAD>(s->chains, s->dims, s->dims, q_hi, q_lo, ldq, a_hi, a_lo, lda, eg, st));
  EpiParams ep = {};
  ep.C = s->chains;
  ep.rows = s->dims;
  ep.prior = prior;
  ep.prior_mean = prior_mean;
  ep.prior_w = prior_w;
  ep.p = (float*)s->p;
  ep.q = (float*)s->q;
  ep.eps_local = (const float*)s->eps_local;
  ep.kick = (float)kick;
  ep.drift = (float)drift;
  ep.minv = s->mass_kind == HMC_MASS_DIAG ? (const float*)s->mass_inv_diag : nullptr;
  ep.lo = (const float*)s->lower;
  ep.hi = (const float*)s->upper;
  ep.flags = s->flags;
  ep.center = center;
  ep.qn_hi = (__nv_bfloat16*)qn_hi;
  ep.qn_lo = (__nv_bfloat16*)qn_lo;
  ep.ldq = ldq;
  // 16-byte accesses need every row of the [d][C] state 16-byte aligned
  const bool vec4 = s->chains % 4 == 0 && ((uintptr_t)s->p | (uintptr_t)s->q | (uintptr_t)s->g |
                                           (uintptr_t)s->eps_local) % 16 == 0;
  if (vec4) {
    const dim3 grid((unsigned)((s->chains + 127) / 128), (unsigned)((ldq + 31) / 32));
    step_update4_kernel<<<grid, dim3(32, UPDATE_ROWS), 0, st>>>(s->dims, ep, (const float*)s->g);
    return check_launch("step_update4_kernel");
  }
  const dim3 grid((unsigned)((s->chains + 31) / 32), (unsigned)((ldq + 31) / 32));
  step_update_kernel<<<grid, dim3(32, UPDATE_ROWS), 0, st>>>(s->dims, ep, (const float*)s->g);
  return check_launch("step_update_kernel");
}

HMC_API int hmc_tc_resid_misfit(int64_t n, int64_t d, int64_t C, const void* g_hi, const void* g_lo, int64_t ldg,
                                const void* q_hi, const void* q_lo, int64_t ldq, const float* data,
                                const float* inv_var, double* partial, double* out_x, int accumulate, int* status,
                                void* stream) {
  HMC_REQUIRE(data && inv_var && partial && out_x, "hmc_tc_resid_misfit: null argument");
  EpiParams ep = {};
  ep.C = C;
  ep.rows = n;
  ep.bias = data;
  ep.inv_var = inv_var;
  ep.partial = partial;
  ep.status = status;
  HMC_TRY(launch<EPI_MISFIT>(C, n, d, q_hi, q_lo, ldq, g_hi, g_lo, ldg, ep, as_stream(stream)));
  const int tiles = (int)((n + BN - 1) / BN);
  reduce_partials_kernel<<<blocks_for(C, 256), 256, 0, as_stream(stream)>>>(C, tiles, partial, out_x, accumulate);
  return check_launch("reduce_partials_kernel");
}

HMC_API int64_t hmc_tc_partials_size(int64_t n, int64_t C) { return (n + BN - 1) / BN * C; }

HMC_API int hmc_tc_mlp(int mode, int64_t M, int64_t N, int64_t K, const void* x, int64_t ldx, const void* w,
                       int64_t ldw, const float* bias, const hmc_mlp_out* out, int* status, void* stream) {
  HMC_REQUIRE(out != nullptr && x != nullptr && w != nullptr, "hmc_tc_mlp: null argument");
  HMC_REQUIRE(ldx % 8 == 0 && ldw % 8 == 0, "hmc_tc_mlp: pitches must be multiples of 8 elements");
  EpiParams ep = {};
  ep.C = M;
  ep.rows = N;
  ep.bias = bias;
  ep.status = status;
  ep.z = out->z;
  ep.ldz = out->ldz;
  ep.act = (__nv_bfloat16*)out->act;
  ep.ld_act = out->ld_act;
  ep.act_t = (__nv_bfloat16*)out->act_t;
  ep.ld_act_t = out->ld_act_t;
  ep.y = out->y;
  ep.ldy = out->ldy;
  ep.g_state = out->g_state;
  ep.out_scale = out->out_scale;
  ep.out_shift = out->out_shift;
  ep.g = out->g;
  ep.accumulate = out->accumulate;
  cudaStream_t st = as_stream(stream);
  switch (mode) {
    case HMC_MLP_HIDDEN:
      HMC_REQUIRE(bias && ep.z && ep.act && ep.act_t && ep.ld_act % 16 == 0, "hmc_tc_mlp: hidden outputs");
      return launch<EPI_MLP_HIDDEN, 1>(M, N, K, x, nullptr, ldx, w, nullptr, ldw, ep, st);
    case HMC_MLP_OUT:
      HMC_REQUIRE(bias && (ep.y || (ep.g_state && ep.out_scale && ep.out_shift)), "hmc_tc_mlp: output buffers");
      return launch<EPI_MLP_OUT, 1>(M, N, K, x, nullptr, ldx, w, nullptr, ldw, ep, st);
    case HMC_MLP_BACK:
      HMC_REQUIRE(ep.z && ep.act && ep.act_t && ep.ld_act % 16 == 0, "hmc_tc_mlp: backward buffers");
      return launch<EPI_MLP_BACK, 1>(M, N, K, x, nullptr, ldx, w, nullptr, ldw, ep, st);
    case HMC_MLP_WGRAD:
      HMC_REQUIRE(ep.g != nullptr, "hmc_tc_mlp: weight-gradient output");
      return launch<EPI_GRAD, 1>(M, N, K, x, nullptr, ldx, w, nullptr, ldw, ep, st);
    default:
      return fail(HMC_ERR_INVALID_ARG, "hmc_tc_mlp: unknown mode %d", mode);
  }
}

}  // extern "C"
