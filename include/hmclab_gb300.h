/*
 * hmclab_gb300 — C ABI of the GB300 Hamiltonian Monte Carlo hot path.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (passed as `void*`, NULL = legacy default stream) and returns an int status
 * (HMC_OK = 0).  No C++ exceptions and no framework types cross this boundary;
 * the library never frees or retains caller memory.  `hmc_last_error()` returns
 * a human-readable message for the last failing call on the calling thread.
 *
 * Layout convention: a batch of C chains of a d-dimensional model is stored
 * dimension-major, chain-fastest: element (i, c) of a [d][C] array lives at
 * offset i*C + c.  A single reference-style column vector (d,1) is the C = 1
 * case.  Per-chain scalars (misfits, energies, step sizes) are [C] arrays.
 *
 * dtype codes select the arithmetic type of positions, momenta and gradients:
 * HMC_F32 (production) or HMC_F64 (verification).  Hamiltonian sums, misfits
 * and the accept test are always FP64.
 *
 * Reference interfaces each group replaces are cited per declaration as
 * file:line in the reference project (larsgeb/hmclab).
 */
#ifndef HMCLAB_GB300_H
#define HMCLAB_GB300_H

#include <stdint.h>

#if defined(HMC_BUILDING_LIBRARY) && defined(__GNUC__)
#define HMC_API __attribute__((visibility("default")))
#else
#define HMC_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define HMC_OK 0
#define HMC_ERR_INVALID_ARG 1 /* maps to AssertionError/ValueError host-side */
#define HMC_ERR_CUDA 2        /* CUDA runtime error (launch or execution)    */
#define HMC_ERR_TIMEOUT 3     /* a bounded device wait ran out               */
#define HMC_ERR_NONFINITE 4   /* non-finite state where it is not allowed    */
#define HMC_ERR_UNSUPPORTED 5 /* valid request the library does not provide */

#define HMC_F32 0
#define HMC_F64 1

#define HMC_MASS_UNIT 0
#define HMC_MASS_DIAG 1
#define HMC_MASS_FULL 2

/* per-chain flag bits in hmc_chains.flags */
#define HMC_FLAG_OUT_OF_BOUNDS 1 /* trajectory left the bounds: misfit = +inf */

/* ---- library ------------------------------------------------------------- */
HMC_API int hmc_version(void);
HMC_API const char* hmc_last_error(void);
/* Number of kernels this library has launched since load (host-side counter). */
HMC_API int64_t hmc_launch_count(void);
/* Limits of the bounded waits of the kernels that stage operands through
 * tensor-copy barriers (tensor-core contractions, elastic stencils).  The
 * default is 2 s with nothing withheld.  A test hook: with withhold = 1,
 * block 0 of every such launch skips its first barrier arrival, so its wait
 * runs out after wait_ns (1 us .. 2 s); the kernel then sets its status word
 * (HMC_ERR_TIMEOUT, or 1 for the stencils), frees what it holds and returns.
 * Launches captured in a CUDA graph keep the limits of their capture.
 * Reference counterpart: none (the reference has no device code); it stands
 * for the fault-injection tests of the sampler loop (tests/test_break.py). */
HMC_API int hmc_set_wait_limits(uint64_t wait_ns, int withhold);
/* *capturing = 1 while `stream` is being captured into a CUDA graph (the
 * launch-shape autotuner times nothing then).  No reference counterpart. */
HMC_API int hmc_stream_capturing(void* stream, int* capturing);
/* Zero `bytes` of device memory on `stream` (capturable): the misfit and
 * gradient of a Uniform distribution inside its bounds (reference
 * hmclab/Distributions/base.py:780-786).                                   */
HMC_API int hmc_fill_zero(void* ptr, int64_t bytes, void* stream);

/* ---- counter-based RNG (Philox4x32-10, Salmon et al. 2011) ---------------
 * Replaces the numpy Generator draws of MassMatrices.py:142,227,314 and
 * Samplers.py:1534,1486 in production mode.  out[i][c] = standard normal for
 * counter (i/4, c, proposal, purpose) under key = seed.                      */
HMC_API int hmc_philox_normal(int dtype, int64_t rows, int64_t chains, uint64_t seed,
                      uint64_t proposal, uint32_t purpose, void* out,
                      void* stream);
/* Raw Philox4x32-10 blocks for known-answer tests: n blocks, block k uses
 * counter (ctr0 + k, ctr1, ctr2, ctr3) and key (key0, key1); out is uint32[4n]
 * in device memory. */
HMC_API int hmc_philox_raw(int64_t n, uint32_t ctr0, uint32_t ctr1, uint32_t ctr2,
                   uint32_t ctr3, uint32_t key0, uint32_t key1, uint32_t* out,
                   void* stream);

/* ---- batched chain state of the sampler ----------------------------------
 * Mirrors the per-chain state HMC keeps in Samplers.py:1105-1180
 * (current_model, current_x, current_momentum, stepsize, accepted_proposals)
 * for C chains at once.  All pointers are device memory unless noted.       */
typedef struct hmc_chains {
  int32_t dtype;     /* HMC_F32 / HMC_F64: type of q_cur, q, p, g, v, eps, ring_q */
  int32_t mass_kind; /* HMC_MASS_* */
  int64_t dims;      /* d */
  int64_t chains;    /* C */
  void* q_cur;       /* [d][C] current model of every chain            */
  void* q;           /* [d][C] position along the trajectory           */
  void* p;           /* [d][C] momentum                                */
  void* g;           /* [d][C] gradient of the misfit at q (scratch)   */
  void* v;           /* [d][C] scratch for full-mass products (FULL)   */
  const void* mass_diag;     /* [d] diagonal of M (DIAG)               */
  const void* mass_inv_diag; /* [d] 1/diagonal (DIAG)                  */
  const void* mass_chol;     /* [d][d] lower Cholesky factor of M (FULL) */
  const void* mass_inv;      /* [d][d] M^-1 (FULL)                     */
  const void* lower;         /* [d] lower bounds or NULL               */
  const void* upper;         /* [d] upper bounds or NULL               */
  void* eps;                 /* [C] base step size per chain           */
  void* eps_local;           /* [C] step size of this trajectory       */
  double* x_cur;             /* [C] misfit of q_cur                    */
  double* x_prop;            /* [C] misfit at the trajectory end       */
  double* k_cur;             /* [C] kinetic energy at the start        */
  double* k_prop;            /* [C] kinetic energy at the end          */
  int64_t* accepted;         /* [C] accepted proposals                 */
  int32_t* flags;            /* [C] HMC_FLAG_* of the current trajectory */
  int64_t* proposal;         /* [1] proposals completed (device counter) */
  uint64_t seed;             /* Philox key                             */
  int32_t randomize_stepsize;/* eps_local = U(0.5,1.5) * eps if nonzero */
  int32_t autotune;          /* per-chain Robbins-Monro step adaptation */
  double target_acceptance;  /* autotune target (Samplers.py:1494-1522) */
  double learning_rate;      /* autotune exponent kappa                */
  double minimal_stepsize;   /* autotune floor                         */
  /* Injected random streams (parity mode); NULL selects Philox.
   * stream_z [S][d][C] standard normals, stream_eps [S][C] step factors
   * (already in [0.5,1.5)), stream_u [S][C] accept uniforms; proposal n uses
   * slice n % S.                                                            */
  const void* stream_z;
  const void* stream_eps;
  const double* stream_u;
  int64_t stream_len;
  /* Thinned sample ring: proposal n with n % thinning == 0 is written to slot
   * (n / thinning) % ring_slots as ring_q[slot][d][C], ring_x[slot][C].
   * ring_q may be NULL to disable recording.                               */
  void* ring_q;
  double* ring_x;
  int64_t ring_slots;
  int64_t thinning;
  /* Optional per-proposal records for autotuning: [S][C] step sizes and
   * acceptance rates min(1, exp(H0-H1)); NULL to skip.                     */
  double* rec_stepsize;
  double* rec_acceptance;
  int64_t rec_len;
  /* Optional per-chain inverse temperatures [C] (NULL: all 1): chain c
   * targets exp(-beta[c] * misfit), so kicks scale the gradient by beta[c]
   * and the accept test uses beta[c] * misfit; x_cur / x_prop stay the
   * untempered misfit, ring_x records beta[c] * x_cur (the misfit of the
   * chain's own tempered target, as a tempered distribution would report).  */
  const double* beta;
} hmc_chains;

/* Samplers.py:1463-1469 + 1524-1545 (and MassMatrices.py:100-314):
 * draw momenta p ~ N(0, M), step factors, kinetic energy K(p) in FP64,
 * copy q_cur -> q and make the first drift q += drift * eps_local * M^-1 p,
 * then apply the bound reflection of base.py:239-270.  drift is 0.5 for the
 * leapfrog integrator and a1 for the 3-/4-stage integrators (Samplers.py:
 * 1586-1726).                                                               */
HMC_API int hmc_begin_trajectory(const hmc_chains* s, double drift, void* stream);

/* Samplers.py:1561-1569: p -= kick * eps_local * g, then
 * q += drift * eps_local * M^-1 p, then reflect at the bounds.  drift = 0
 * skips the position update.                                               */
HMC_API int hmc_kick_drift(const hmc_chains* s, double kick, double drift,
                   void* stream);

/* Samplers.py:1471-1492 (+ autotune 1494-1522 and the thinned append of
 * 529-704 lines 675-678): K(p) at the end, H = x + K for both states, accept
 * iff exp(H0 - H1) > u with FP64 arithmetic (NaN rejects), copy q -> q_cur
 * on accept, count, optionally adapt eps, record the thinned sample and
 * advance the proposal counter.  x_prop must hold misfit(q).               */
HMC_API int hmc_end_trajectory(const hmc_chains* s, void* stream);

/* Replica exchange between tempered chains (the exchange step of
 * Samplers.py:589-669, done in place on the device instead of over pipes):
 * for each of the npairs pairs (a, b) = pairs[2k], pairs[2k+1] (distinct
 * chains, each in at most one pair), swap the current models of a and b
 * iff exp((beta[a] - beta[b]) * (x_cur[a] - x_cur[b])) > u[k] (the sum of
 * both chains' misfit improvements; FP64, NaN rejects).  Positions and
 * misfits move; step sizes stay with their chain.  swapped[k] receives the
 * decision; accepted_total (nullable) counts the swaps.  When the last
 * completed proposal (proposal counter - 1) was recorded in the thinned
 * ring, its ring entry is swapped too (the reference appends the sample
 * after the exchange, Samplers.py:675-678), with the tempered misfit of the
 * swapped-in model.                                                        */
HMC_API int hmc_exchange(const hmc_chains* s, int64_t npairs,
                         const int32_t* pairs, const double* u,
                         int32_t* swapped, int64_t* accepted_total,
                         void* stream);

/* MassMatrices.py:100-113,185-198,270-285: out[c] = 0.5 p_c^T M^-1 p_c (FP64).
 * For FULL, s->v is used as scratch.                                       */
HMC_API int hmc_kinetic_energy(const hmc_chains* s, const void* p, double* out,
                       void* stream);
/* MassMatrices.py:115-133,200-218,287-305: out = M^-1 p.                   */
HMC_API int hmc_kinetic_energy_gradient(const hmc_chains* s, const void* p, void* out,
                                void* stream);

/* ---- target distributions: batched misfit / gradient ---------------------
 * misfit: out_x[c] (+)= chi(M[:,c]) in FP64 (accumulate != 0 adds).
 * gradient: out_g[i][c] (+)= d chi / d m_i at M[:,c].                       */

/* base.py:539-574 (Normal, diagonal covariance):
 * chi = 0.5 sum (m - mean)^2 * inv_var, grad = (m - mean) * inv_var.        */
HMC_API int hmc_normal_diag_misfit(int dtype, int64_t d, int64_t C, const void* M,
                           const void* mean, const void* inv_var,
                           double* out_x, int accumulate, void* stream);
HMC_API int hmc_normal_diag_gradient(int dtype, int64_t d, int64_t C, const void* M,
                             const void* mean, const void* inv_var,
                             void* out_g, int accumulate, void* stream);

/* base.py:553-574 (Normal, full covariance): inv_cov is [d][d].  With
 * D = m - mean: chi = 0.5 D^T inv_cov D, grad = inv_cov D.  work is a scratch
 * buffer of 2*d*C elements (misfit) or d*C elements (gradient).             */
HMC_API int hmc_normal_full_misfit(int dtype, int64_t d, int64_t C, const void* M,
                           const void* mean, const void* inv_cov, void* work,
                           double* out_x, int accumulate, void* stream);
HMC_API int hmc_normal_full_gradient(int dtype, int64_t d, int64_t C, const void* M,
                             const void* mean, const void* inv_cov,
                             void* work, void* out_g, int accumulate,
                             void* stream);

/* base.py:689-710 (Laplace): chi = sum |m - mean| * inv_disp,
 * grad = sign(m - mean) * inv_disp, sign(0) = 0.                            */
HMC_API int hmc_laplace_misfit(int dtype, int64_t d, int64_t C, const void* M,
                       const void* mean, const void* inv_disp, double* out_x,
                       int accumulate, void* stream);
HMC_API int hmc_laplace_gradient(int dtype, int64_t d, int64_t C, const void* M,
                         const void* mean, const void* inv_disp, void* out_g,
                         int accumulate, void* stream);

/* LinearMatrix.py:184-208, premultiplied dense form (n > d):
 * grad = GtG m - Gtd0; chi = 0.5 (m^T (GtG m - 2 Gtd0) + dtd).
 * GtG is [d][d] row-major, Gtd0 is [d]; work is a [d][C] scratch.  This is
 * the FP64 verification form; FP32 chains use the residual form below (the
 * premultiplied misfit cancels catastrophically in FP32).                   */
HMC_API int hmc_dense_premul_gradient(int dtype, int64_t d, int64_t C, const void* M,
                              const void* GtG, const void* Gtd0, void* out_g,
                              int accumulate, void* stream);
HMC_API int hmc_dense_premul_misfit(int dtype, int64_t d, int64_t C, const void* M,
                            const void* GtG, const void* Gtd0, double dtd,
                            void* work, double* out_x, int accumulate,
                            void* stream);

/* LinearMatrix.py:193-208, residual dense form:
 * r = (G m - data) * inv_var (n x C), chi = 0.5 sum (G m - data)^2 inv_var,
 * grad = G^T r.  G is [n][d], Gt is [d][n] (both row-major); resid is an
 * [n][C] scratch of the state dtype.                                        */
HMC_API int hmc_dense_resid_misfit(int dtype, int64_t n, int64_t d, int64_t C,
                           const void* M, const void* G, const void* data,
                           const void* inv_var, void* resid, double* out_x,
                           int accumulate, void* stream);
HMC_API int hmc_dense_resid_gradient(int dtype, int64_t n, int64_t d, int64_t C,
                             const void* M, const void* G, const void* Gt,
                             const void* data, const void* inv_var,
                             void* resid, void* out_g, int accumulate,
                             void* stream);

/* No counterpart in the reference.  hmc_dense_resid_misfit for callers that
 * cannot allocate device memory (their host framework owns every device
 * allocation, or cudaMalloc would stall a latency-critical path): the [n][C]
 * residual lives in a library-owned device array of
 * HMC_NOALLOC_SCRATCH_BYTES, held on every GPU that loads the library until
 * exit.  Larger n*C is rejected with HMC_ERR_INVALID_ARG.  No allocation is
 * made; the array's address is looked up on the first call in each device
 * context (make that call before any stream capture), and again on the first
 * call after the context was destroyed and re-created (cudaDeviceReset).
 * Calls share the array: calls that overlap on the GPU race and must be
 * serialised.                                                                */
#define HMC_NOALLOC_SCRATCH_BYTES (16u << 20)
HMC_API int hmc_dense_resid_misfit_noalloc(int dtype, int64_t n, int64_t d,
                                           int64_t C, const void* M,
                                           const void* G, const void* data,
                                           const void* inv_var, double* out_x,
                                           int accumulate, void* stream);

/* LinearMatrix.py:389-426 (sparse G, CSR, simple covariance):
 * G rows (n) in CSR (row_ptr[n+1], col[nnz], val[nnz] of the state dtype);
 * Gt is G^T in CSR (d rows).  resid is an [n][C] scratch.                   */
HMC_API int hmc_csr_misfit(int dtype, int64_t n, int64_t d, int64_t C, const void* M,
                   const int32_t* row_ptr, const int32_t* col, const void* val,
                   const void* data, const void* inv_var, void* resid,
                   double* out_x, int accumulate, void* stream);
HMC_API int hmc_csr_gradient(int dtype, int64_t n, int64_t d, int64_t C,
                     const void* M, const int32_t* row_ptr,
                     const int32_t* col, const void* val,
                     const int32_t* t_row_ptr, const int32_t* t_col,
                     const void* t_val, const void* data,
                     const void* inv_var, void* resid, void* out_g,
                     int accumulate, void* stream);

/* LinearMatrix.py:389-426 (sparse G, simple covariance) in FP32 for a CSR
 * whose column indices are sorted within each row (canonical CSR, scipy's
 * sort_indices).  The chain block is staged through shared memory in
 * double-buffered slabs of `slab` columns (32 .. 448); slab_ptr[r * (n_slabs
 * + 1) + s] is the first
 * nonzero of row r whose column is >= s * slab, with n_slabs =
 * ceil(cols / slab), so slab_ptr[r * (n_slabs + 1)] = row_ptr[r] and the last
 * entry of a row is row_ptr[r + 1].  rows_per_warp (4, 8 or 16) sets the rows
 * a block accumulates per slab pass (16 warps per block).  With center NULL
 * the results equal hmc_csr_misfit / hmc_csr_gradient bit for bit; slab and
 * rows_per_warp only change the speed (picked by the host autotuner, which
 * also times the gather kernels: `kernel` selects the variant, and every
 * variant adds the nonzeros of a row in CSR order with fused multiply-adds,
 * so all give the same sums).
 * center ([cols], may be NULL) makes the first product G (M - center) -
 * data: the caller passes data - G center (formed in FP64) so that the
 * residual is unchanged but the FP32 sums no longer cancel terms of the size
 * of G M (travel times ~1e3 x their residuals in the tomography workload).  */
#define HMC_CSR_GATHER 0  /* one thread per chain, X rows gathered per nonzero   */
#define HMC_CSR_GATHER4 1 /* four chains per thread (16-byte loads; C % 4 == 0)  */
#define HMC_CSR_SLAB 2    /* column slabs of X staged in shared memory          */
typedef struct hmc_csr_slabs {
  const int32_t* col;      /* [nnz] column indices, sorted within rows */
  const float* val;        /* [nnz] values                              */
  const int32_t* slab_ptr; /* [rows][n_slabs + 1] slab starts per row (SLAB) */
  int64_t rows, cols;
  int32_t slab;            /* columns per shared-memory slab (SLAB)     */
  int32_t rows_per_warp;   /* 4, 8 or 16 (SLAB)                         */
  const int32_t* row_ptr;  /* [rows + 1] (GATHER, GATHER4)              */
  int32_t kernel;          /* HMC_CSR_GATHER / GATHER4 / SLAB           */
  int32_t reserved;
} hmc_csr_slabs;
HMC_API int hmc_csr_slab_misfit(const hmc_csr_slabs* G, int64_t C, const float* M,
                                const float* center, const float* data,
                                const float* inv_var, float* resid,
                                double* out_x, int accumulate, void* stream);
HMC_API int hmc_csr_slab_gradient(const hmc_csr_slabs* G, const hmc_csr_slabs* Gt,
                                  int64_t C, const float* M, const float* center,
                                  const float* data, const float* inv_var,
                                  float* resid, float* out_g, int accumulate,
                                  void* stream);

/* SourceLocation.py:482-540 (SourceLocation3D, homogeneous velocity).
 * Parameters are interleaved [x,y,z,T] per event followed by v when
 * infer_velocity != 0, else v = medium_velocity (SourceLocation.py:697-713).
 * rx/ry/rz are [S] station coordinates; obs and inv_var are [E][S];
 * NaN observations are skipped (nansum).                                   */
HMC_API int hmc_srcloc3d_misfit(int dtype, int64_t E, int64_t S, int64_t C,
                        const void* M, const void* rx, const void* ry,
                        const void* rz, const void* obs, const void* inv_var,
                        int infer_velocity, double medium_velocity,
                        double* out_x, int accumulate, void* stream);
HMC_API int hmc_srcloc3d_gradient(int dtype, int64_t E, int64_t S, int64_t C,
                          const void* M, const void* rx, const void* ry,
                          const void* rz, const void* obs,
                          const void* inv_var, int infer_velocity,
                          double medium_velocity, void* out_g, int accumulate,
                          void* stream);

/* ---- tensor-core (tcgen05) contraction of a dense matrix with all chains --
 * FP32 path of LinearMatrix.py:184-208: BF16 hi/lo split operands
 * (x = hi + lo, 3 products hi*hi + hi*lo + lo*hi, FP32 accumulation in
 * TMEM).  A dense matrix A [rows][K] is stored split as a_hi/a_lo with row
 * pitch lda (multiple of 64); the chain positions are stored transposed,
 * chain-major, as q_hi/q_lo [C][ldq].  status is a device int that receives
 * HMC_ERR_TIMEOUT if a bounded wait inside the kernel expired.             */
HMC_API int hmc_split_bf16(int64_t rows, int64_t cols, const float* src,
                           int64_t ld, void* hi, void* lo, void* stream);
/* hi/lo split of (q - center) (center [d] nullable) transposed to [C][ld]. */
HMC_API int hmc_split_bf16_transpose(int64_t d, int64_t C, const float* q,
                                     const float* center, int64_t ld,
                                     void* hi, void* lo, void* stream);
/* g[r][c] (+)= sum_k A[r][k] Q[c][k] - bias[r]   (GtG m - Gtd0)            */
HMC_API int hmc_tc_gradient(int64_t rows, int64_t K, int64_t C,
                            const void* a_hi, const void* a_lo, int64_t lda,
                            const void* q_hi, const void* q_lo, int64_t ldq,
                            const float* bias, float* g, int accumulate,
                            int* status, void* stream);
/* One fused leapfrog kick(+drift) for FP32 chains (Samplers.py:1561-1581)
 * with the posterior gradient GtG q - Gtd0 + prior'(q) (prior: 0 none,
 * 1 Normal diagonal with prior_w = 1/variance, 2 Laplace with prior_w =
 * 1/dispersion; base.py:564-574, 702-710) formed in the epilogue; writes p,
 * q (reflected at the bounds) and the next operand qn_hi/qn_lo = split of
 * (q - center) (must not alias q_hi/q_lo).  With a center c the operands
 * hold q - c and bias must be Gtd0 - GtG c, which keeps the split products
 * accurate near the data-consistent region.  Unit or diagonal mass.         */
HMC_API int hmc_tc_step(const hmc_chains* s, const void* a_hi,
                        const void* a_lo, int64_t lda, const void* q_hi,
                        const void* q_lo, void* qn_hi, void* qn_lo,
                        int64_t ldq, const float* center,
                        const float* bias, int prior,
                        const float* prior_mean, const float* prior_w,
                        double kick, double drift, int* status, void* stream);
/* The same step in two passes with bitwise-equal results: the contraction
 * writes g = GtG q - bias into s->g, then one streaming pass applies the
 * prior, kick, drift and reflection and writes the next operand; the
 * sampler's launch-shape autotuner picks whichever is faster for the shape. */
HMC_API int hmc_tc_step_split(const hmc_chains* s, const void* a_hi,
                              const void* a_lo, int64_t lda, const void* q_hi,
                              const void* q_lo, void* qn_hi, void* qn_lo,
                              int64_t ldq, const float* center,
                              const float* bias, int prior,
                              const float* prior_mean, const float* prior_w,
                              double kick, double drift, int* status,
                              void* stream);
/* Residual misfit 0.5 sum_r (G m - data)_r^2 inv_var_r per chain
 * (LinearMatrix.py:193-202) with FP64 per-chain sums; partial holds
 * hmc_tc_partials_size(n, C) doubles.                                       */
HMC_API int hmc_tc_resid_misfit(int64_t n, int64_t d, int64_t C,
                                const void* g_hi, const void* g_lo,
                                int64_t ldg, const void* q_hi,
                                const void* q_lo, int64_t ldq,
                                const float* data, const float* inv_var,
                                double* partial, double* out_x, int accumulate,
                                int* status, void* stream);
HMC_API int64_t hmc_tc_partials_size(int64_t n, int64_t C);

/* ---- MLP gradient surrogate (no counterpart in the reference: it stands in
 * for the distribution.gradient calls of the leapfrog at Samplers.py:1562,
 * 1573 once trained; the exact misfit still decides acceptance) -----------
 * hmc_tc_mlp: out[m][n] = sum_k x[m][k] w[n][k] on the tensor cores (BF16
 * operands, FP32 accumulation; x is [M][ldx], w is [N][ldw], both BF16), with
 * the epilogue selected by mode:
 *   HMC_MLP_HIDDEN  z = out + bias, a = GELU(z): z -> z [M][ldz] (FP32),
 *                   a -> act [M][ld_act] and act_t [N][ld_act_t] (BF16)
 *   HMC_MLP_OUT     y = out + bias -> y [M][ldy] (FP32, nullable) and/or
 *                   g_state [N][M] = out_scale * y + out_shift
 *   HMC_MLP_BACK    delta = out * GELU'(z) with z [M][ldz]: -> act, act_t
 *   HMC_MLP_WGRAD   g [N][M] (+)= out (FP32, accumulate from `accumulate`)  */
#define HMC_MLP_HIDDEN 0
#define HMC_MLP_OUT 1
#define HMC_MLP_BACK 2
#define HMC_MLP_WGRAD 3
typedef struct hmc_mlp_out {
  float* z;
  int64_t ldz;
  void* act; /* BF16 */
  int64_t ld_act;
  void* act_t; /* BF16 */
  int64_t ld_act_t;
  float* y;
  int64_t ldy;
  float* g_state;
  const float* out_scale;
  const float* out_shift;
  float* g;
  int32_t accumulate;
} hmc_mlp_out;
HMC_API int hmc_tc_mlp(int mode, int64_t M, int64_t N, int64_t K,
                       const void* x, int64_t ldx, const void* w,
                       int64_t ldw, const float* bias, const hmc_mlp_out* out,
                       int* status, void* stream);
/* Network input from the sampler state: x[c][i] = bf16((q[i][c] - mu[i]) *
 * inv_sigma[i]) for q [d][C]; x is [C][ldx], and only its d leading
 * columns are written.                                                     */
HMC_API int hmc_mlp_input(int64_t d, int64_t C, const float* q, const float* mu,
                          const float* inv_sigma, void* x, int64_t ldx,
                          void* stream);
/* Training minibatch: rows idx[0..B) of the sample stores q_store / g_store
 * ([N][d], FP32) -> x [B][ldx], x_t [d][ldxt] (BF16, normalised inputs) and
 * t [B][ldt] (FP32, normalised targets (g - g_mu) * g_inv_sigma).           */
HMC_API int hmc_mlp_gather(int64_t B, int64_t d, const int32_t* idx,
                           const float* q_store, const float* g_store,
                           const float* mu, const float* inv_sigma,
                           const float* g_mu, const float* g_inv_sigma,
                           void* x, int64_t ldx, void* x_t, int64_t ldxt,
                           float* t, int64_t ldt, void* stream);
/* Loss 0.5/B sum (y - t)^2 and dY = (y - t)/B as BF16 dy [B][lddy] and
 * dy_t [n][lddyt].  loss points to 1025 device doubles: loss[0] receives the
 * loss, loss[1..1024] hold block partials.                                  */
HMC_API int hmc_mlp_loss(int64_t B, int64_t n, const float* y, int64_t ldy,
                         const float* t, int64_t ldt, void* dy, int64_t lddy,
                         void* dy_t, int64_t lddyt, double* loss,
                         void* stream);
/* db[r] = sum_{c < B} delta_t[r][c] for BF16 delta_t [n][ld].               */
HMC_API int hmc_mlp_bias_grad(int64_t n, int64_t B, const void* delta_t,
                              int64_t ld, float* db, void* stream);
/* One Adam step (Kingma & Ba 2015) on n FP32 parameters with bias-corrected
 * moments; step is the 1-based step count.                                  */
HMC_API int hmc_mlp_adam(int64_t n, float* w, const float* g, float* m,
                         float* v, float lr, float beta1, float beta2,
                         float eps, int64_t step, void* stream);
/* FP32 weights w [rows][cols] -> BF16 w16 [rows][ld] and w16_t [cols][ldt]. */
HMC_API int hmc_mlp_cast(int64_t rows, int64_t cols, const float* w,
                         void* w16, int64_t ld, void* w16_t, int64_t ldt,
                         void* stream);
/* Append the sampler state src [d][C] as rows base..base+C-1 of dst [N][d]. */
HMC_API int hmc_mlp_record(int64_t d, int64_t C, const float* src, float* dst,
                           int64_t base, void* stream);

/* ---- scalar-potential surrogate (no counterpart in the reference; like the
 * MLP surrogate it stands in for distribution.gradient in the leapfrog,
 * Samplers.py:1562,1573).  f(x) = w3 . GELU(W2 GELU(W1 x + b1) + b2)
 * + x^T A x / 2 + beta . x; the leapfrog uses grad_q f, a conservative field.
 * Its contractions run through hmc_tc_mlp; these are the element-wise steps
 * of the gradient pass and of the double backpropagation that trains it.
 * hmc_pot_elementwise: for every (b < B, j < n), with z [B][ldz]:
 *   HMC_POT_DELTA2  v = vec[j] GELU'(z)
 *   HMC_POT_DELTA1  v = in GELU'(z)
 *   HMC_POT_DBAR1   v = in GELU'(z), and out_f = in aux GELU''(z)
 *   HMC_POT_DBAR2   v = in vec[j] GELU''(z)
 *   HMC_POT_ZBAR1   v = aux + in GELU'(z)
 * v -> out_bf [B][ld_bf] and (nullable) out_t [n][ld_t], both BF16.          */
#define HMC_POT_DELTA2 0
#define HMC_POT_DELTA1 1
#define HMC_POT_DBAR1 2
#define HMC_POT_DBAR2 3
#define HMC_POT_ZBAR1 4
HMC_API int hmc_pot_elementwise(int mode, int64_t B, int64_t n, const float* in,
                                int64_t ldi, const float* z, int64_t ldz,
                                const float* aux, int64_t ldaux,
                                const float* vec, void* out_bf, int64_t ld_bf,
                                void* out_t, int64_t ld_t, float* out_f,
                                int64_t ldf, void* stream);
/* g[j] = sum_b in[b][j] GELU'(z[b][j]) (the gradient of w3).                 */
HMC_API int hmc_pot_w3_grad(int64_t B, int64_t n, const float* in, int64_t ldi,
                            const float* z, int64_t ldz, float* g,
                            void* stream);
/* Loss 0.5/B sum (y - t)^2 -> loss[0] (loss points to 1025 device doubles,
 * loss[1..] hold block partials) and e = scale[j] (y - t) / B as BF16
 * e [B][lde] and e_t [n][ldet].                                             */
HMC_API int hmc_pot_loss(int64_t B, int64_t n, const float* y, int64_t ldy,
                         const float* t, int64_t ldt, const float* scale,
                         void* e, int64_t lde, void* e_t, int64_t ldet,
                         double* loss, void* stream);
/* dst[r][k0 + k] = bf16(scale[r] src(r, k)) for r < rows, k < cols, where
 * src(r, k) = src[k][r] if transposed else src[r][k] (pitch lds).           */
HMC_API int hmc_pot_scaled_cast(int64_t rows, int64_t cols, const float* src,
                                int64_t lds, int transposed, const float* scale,
                                void* dst, int64_t ldd, int64_t k0, void* stream);
/* Value matching of the potential surrogate (no reference counterpart):
 * dv[b] = weight (r_b - rbar) / B and *loss = 0.5 weight mean (r_b - rbar)^2
 * with r_b = w3 . a2[b] - targets[idx[b]] (a2 BF16 [B][lda], B <= 1024);
 * out[j] += sum_b dv[b] in[b][j] (in BF16 [B][ld]); out_t[r][b] =
 * in_t[r][b] dv[b] (BF16 [rows][ld]).                                        */
HMC_API int hmc_pot_value_residual(int64_t B, int64_t h, const void* a2, int64_t lda,
                                   const float* w3, const double* targets,
                                   const int32_t* idx, float weight, float* dv,
                                   double* loss, void* stream);
HMC_API int hmc_pot_weighted_colsum(int64_t B, int64_t n, const void* in, int64_t ld,
                                    const float* dv, float* out, void* stream);
HMC_API int hmc_pot_scale_columns(int64_t rows, int64_t B, const void* in_t,
                                  int64_t ldi, const float* dv, void* out_t,
                                  int64_t ldo, void* stream);

/* ---- 2-D elastic P-SV full-waveform misfit and gradient ------------------
 * Replaces psvWave's forward_simulate / calculate_l2_misfit / adjoint_simulate
 * / map_kernels_to_velocity as called by ElasticFullWaveform2D.misfit and
 * .gradient (ElasticFullWaveform2D.py:138-184): FP32 fourth-order staggered
 * velocity-stress finite differences with a sponge, explosive sources, an L2
 * waveform misfit and the exact discrete adjoint, for C chains at once.
 * Every field is [nz][nx][C] (chain fastest); one shot is run per call.     */
typedef struct hmc_fwi {
  int32_t nx, nz, nt, nrec; /* simulation grid, time steps, receivers       */
  int64_t chains;           /* C                                            */
  float h, dt;              /* grid spacing, time step                      */
  float w;                  /* misfit weight 1 / (sigma^2 * temperature)    */
  const float* taper;       /* [nz][nx] sponge factors                      */
  const float* stf_host;    /* [nt] source time function, HOST memory       */
  const int32_t* rec_map;   /* [nz][nx] receiver index of a cell or -1      */
  const float* rho;         /* [nz][nx][C] model of every chain             */
  const float* vp;
  const float* vs;
  float* bx;                /* [nz][nx][C] derived parameters (work)        */
  float* bz;
  float* l2m;
  float* lam;
  float* muxz;
  float* vx;                /* [nz][nx][C] wavefields (work)                */
  float* vz;
  float* sxx;
  float* szz;
  float* sxz;
  float* store;             /* forward velocities for the adjoint: every
                               step [nt][2][nz][nx][C] (vx, vz after step n)
                               when snapshot_interval <= 1, else per
                               snapshot s = n / k of the steps n = 0, k, 2k,
                               ... [ceil(nt / k)][4][nz][nx][C] (vx, vz after
                               step n, then after step n - 1)               */
  float* rec;               /* [shots][nt][nrec][2][C] synthetic records    */
  const float* obs;         /* [shots][nt][nrec][2] observed records        */
  float* resid;             /* [nt][nrec][2][C] weighted residuals (work)   */
  float* avx;               /* [nz][nx][C] adjoint wavefields (work)        */
  float* avz;
  float* asxx;
  float* aszz;
  float* asxz;
  float* g_bx;              /* [nz][nx][C] gradient accumulators            */
  float* g_bz;
  float* g_l2m;
  float* g_lam;
  float* g_muxz;
  float* t1;                /* [nz][nx][C] adjoint temporaries (work)       */
  float* t2;
  float* t3;
  float* t4;
  float* t5;
  double* partial;          /* [64][C] misfit partial sums (work)           */
  int* status;              /* set to 1 when a tile load timed out (nullable:
                               then the stencils read without staged tiles) */
  int32_t snapshot_interval; /* k: the adjoint correlates the forward and
                               adjoint fields at steps n = 0, k, 2k, ...
                               only, weighted by k (psvWave's
                               snapshot_interval); 0 or 1: every step (the
                               exact discrete gradient)                     */
} hmc_fwi;

/* rho, vp, vs -> buoyancies and moduli on the staggered grid.               */
HMC_API int hmc_fwi_prepare(const hmc_fwi* s, void* stream);
/* One shot with an explosive source at (src_x, src_z) and the wavelet
 * stf_host; records into rec[shot]; stores the velocities of every step when
 * store != 0.  (psvWave fdModel.forward_simulate, called at
 * hmclab/Distributions/ElasticFullWaveform2D.py:175-178.)                   */
HMC_API int hmc_fwi_forward_shot(const hmc_fwi* s, int shot, int src_x,
                                 int src_z, int store, void* stream);
/* A point source of a shot: moment tensor (Mxx, Mzz, Mxz) at simulation cell
 * (x, z) of sxx/szz, fed by its own wavelet.  Per step, sxx and szz of the
 * cell gain M.. * stf[n] * dt / h^2 and each of the four sxz nodes around it
 * gains Mxz * stf[n] * dt / (4 h^2).  An explosion is (1, 1, 0).           */
typedef struct hmc_fwi_source {
  int32_t x, z;             /* 1 <= x < nx, 1 <= z < nz                     */
  float mxx, mzz, mxz;
  const float* stf_host;    /* [nt] wavelet, HOST memory                    */
} hmc_fwi_source;
/* One shot fired by n_src sources at once (the sources of psvWave's
 * which_source_to_fire_in_which_shot; moment tensors from moment_angles,
 * tests/configurations/default_testing_configuration.ini:20-28 of the
 * reference); at most 32 stress terms: 1 per source, 4 with Mxz != 0.       */
HMC_API int hmc_fwi_forward_shot_sources(const hmc_fwi* s, int shot,
                                         const hmc_fwi_source* src, int n_src,
                                         int store, void* stream);
/* out_x[c] (+)= 0.5 * w * sum over shots < nshots of (rec - obs)^2, FP64.   */
HMC_API int hmc_fwi_misfit(const hmc_fwi* s, int nshots, double* out_x,
                           int accumulate, void* stream);
HMC_API int hmc_fwi_zero_gradients(const hmc_fwi* s, void* stream);
/* Cell parametrisation (psvWave's own model vector of absolute vp, vs, rho
 * per cell or block of cells, reference ElasticFullWaveform2D.py:57,194-210):
 * out[cell][c] = base[cell] + (map[cell] >= 0 ? M[map[cell]][c] : 0), and the
 * gradient's segmented sum out[p][c] (+)= sum_{ptr[p] <= k < ptr[p+1]}
 * g[cells[k]][c].  All device memory, [rows][C] chain-fastest.             */
HMC_API int hmc_fwi_cell_model(int64_t cells, int64_t C, const int32_t* map,
                               const float* M, const float* base, float* out,
                               void* stream);
HMC_API int hmc_fwi_cell_gradient(int64_t P, int64_t C, const int32_t* ptr,
                                  const int32_t* cells, const float* g,
                                  float* out, int accumulate, void* stream);
/* Adjoint of the shot just simulated with store != 0; accumulates into the
 * gradient accumulators.                                                   */
HMC_API int hmc_fwi_adjoint_shot(const hmc_fwi* s, int shot, void* stream);
/* Accumulators -> gradients with respect to rho, vp, vs ([nz][nx][C]).     */
HMC_API int hmc_fwi_param_gradient(const hmc_fwi* s, float* g_rho,
                                   float* g_vp, float* g_vs, int accumulate,
                                   void* stream);

/* ---- dense matrix product used by the ops above -------------------------
 * out[m][n] = alpha * A[m][k] B[k][n] + (bias ? bias[m] : 0)
 *             + (accumulate ? out[m][n] : 0), all row-major.                */
HMC_API int hmc_gemm(int dtype, int64_t m, int64_t n, int64_t k, double alpha,
             const void* A, const void* B, const void* bias, void* out,
             int accumulate, void* stream);
/* The same product without bias for a long k and a small m x n (the
 * grid-to-blob projection of the FWI gradient, k = simulation cells): the
 * k range is split over CTAs, each writes its partial product into work
 * (work_elems elements of the dtype, at least m * n; more allows more
 * splits), and a second kernel sums the partials in a fixed order, so the
 * result is deterministic.                                                 */
HMC_API int hmc_gemm_splitk(int dtype, int64_t m, int64_t n, int64_t k,
                            double alpha, const void* A, const void* B,
                            void* out, int accumulate, void* work,
                            int64_t work_elems, void* stream);

/* ---- effective sample size (no counterpart in the reference, whose only
 * mixing diagnostic is Helpers/Processing.py:6-13) --------------------------
 * Split-chain multi-chain ESS per parameter with Geyer's initial monotone
 * sequence (Gelman et al., BDA3 section 11.5): samples are [N][d][C] (the
 * sampler's thinned ring), lags bounds the autocorrelation window; ess[d]
 * is negated where the window was too short to truncate; rhat[d] (nullable)
 * receives split-R-hat.  work holds hmc_ess_work_size(d, C, lags) doubles.  */
HMC_API int hmc_ess(int dtype, int64_t N, int64_t d, int64_t C,
                    const void* samples, int lags, double* work, double* ess,
                    double* rhat, void* stream);
HMC_API int64_t hmc_ess_work_size(int64_t d, int64_t C, int lags);
/* Rank normalisation (Vehtari et al. 2021, section 4.1): z[N][d][C] (FP64)
 * receives, for every draw, Phi^-1((r - 3/8) / (S + 1/4)) with r its rank
 * (ties averaged) among the S = N C draws of its parameter.  The split-R-hat
 * and ESS of z (hmc_ess) are the rank-normalised bulk diagnostics.  Cost
 * S^2 comparisons per parameter; calls with S^2 d > 1.1e12 are refused.    */
HMC_API int hmc_rank_normalize(int dtype, int64_t N, int64_t d, int64_t C,
                               const void* samples, double* z, void* stream);
/* Mean and (population) variance over all draws and chains of every
 * parameter of an [N][d][C] sample array, in FP64.                          */
HMC_API int hmc_moments(int dtype, int64_t N, int64_t d, int64_t C,
                        const void* samples, double* mean, double* var,
                        void* stream);

/* ---- persistent fused proposals for small dense targets -----------------
 * One launch runs `proposals` whole HMC proposals (Samplers.py:1463-1584:
 * momentum draw, first drift, every kick and drift of the integrator, the
 * misfit at the end point, the FP64 accept test of :1471-1492 and the
 * thinned sample record) for every chain, one warp per chain, for the
 * posterior  [prior +] premultiplied dense LinearMatrix
 * (LinearMatrix.py:164-208: gradient GtG m - Gtd0, misfit
 * 0.5 (m^T (GtG m - 2 Gtd0) + dtd)) with d <= 128, GtG held in shared
 * memory.  prior: 0 none, 1 Normal with diagonal inverse variances prior_w
 * (base.py:539-570), 2 Laplace with inverse dispersions prior_w
 * (base.py:689-710).  Unit, diagonal or full mass (a full mass keeps M^-1
 * and its Cholesky factor in shared memory too: 3 d (d|1) elements plus a
 * vector per warp must fit in 227 KB), no bounds, no autotuning, no
 * temperatures.  The proposals are numbered from s->proposal[0] on, as
 * hmc_begin_trajectory / hmc_end_trajectory number them (same random draws,
 * injected streams included), and the counter is advanced by `proposals`.
 * warps_per_block (1, 2, 4, 8 or 16) sets the chains per block; dry != 0
 * runs the arithmetic but writes no state (for timing launch shapes).      */
#define HMC_SCHEDULE_MAX 64
typedef struct hmc_schedule {
  double first_drift;                  /* drift coefficient before the loop */
  int32_t steps;                       /* entries used below                */
  int32_t gradient[HMC_SCHEDULE_MAX];  /* 1: evaluate the gradient, kick    */
  double kick[HMC_SCHEDULE_MAX];       /* kick coefficient (x step size)    */
  double drift[HMC_SCHEDULE_MAX];      /* drift coefficient (x step size)   */
} hmc_schedule;

HMC_API int hmc_persistent_dense(const hmc_chains* s, const void* GtG,
                                 const void* Gtd0, double dtd, int prior,
                                 const void* prior_mean, const void* prior_w,
                                 const hmc_schedule* schedule,
                                 int64_t proposals, int warps_per_block,
                                 int dry, void* stream);

/* Several such targets of different dimensions and chain counts in one
 * launch (one group per target, up to 48 groups; every group has its own
 * chain state, data, step sizes and random draws).  All groups share the
 * dtype, the mass kind, the prior kind and the integrator schedule; each
 * group's proposal counter advances by `proposals`.                        */
typedef struct hmc_dense_group {
  const hmc_chains* chains;
  const void* GtG;
  const void* Gtd0;
  double dtd;
  int prior;
  const void* prior_mean;
  const void* prior_w;
} hmc_dense_group;

HMC_API int hmc_persistent_dense_groups(const hmc_dense_group* groups,
                                        int ngroups,
                                        const hmc_schedule* schedule,
                                        int64_t proposals, int warps_per_block,
                                        int dry, void* stream);

/* ---- CUDA graphs of whole proposals --------------------------------------
 * Capture the work issued on `stream` between begin and end into an
 * executable graph; launch it any number of times.                          */
HMC_API int hmc_graph_begin(void* stream);
HMC_API int hmc_graph_end(void* stream, void** graph_exec);
HMC_API int hmc_graph_launch(void* graph_exec, void* stream);
HMC_API int hmc_graph_destroy(void* graph_exec);

#ifdef __cplusplus
}
#endif

#endif /* HMCLAB_GB300_H */
