// Dense linear misfit for callers that must not allocate device memory.
//
// hmc_dense_resid_misfit needs an [n][C] residual buffer that the caller
// allocates.  Some callers cannot do that: code that runs inside a host
// framework which owns every device allocation (a fixed memory arena or pool
// sized at start-up, where an extra cudaMalloc would fail or fragment it), or
// code on a latency-critical path where cudaMalloc/cudaFree would synchronise
// the device.  This entry point takes the same inputs and outputs but uses a
// fixed-size scratch array that lives in the library's own device image:
//
//   - the array holds HMC_NOALLOC_SCRATCH_BYTES (16 MiB); every GPU that loads
//     this library keeps it until the process exits;
//   - requests whose residual (n * C elements of the dtype) does not fit are
//     rejected with HMC_ERR_INVALID_ARG before any work is issued;
//   - no cudaMalloc, cudaFree or allocating library routine is called;
//   - the device address of the array is looked up once per device, on that
//     device's first call (cudaGetSymbolAddress with the device current), so
//     the first call on each device should be made before any stream capture;
//   - every call shares the one array and the last call's residuals stay in
//     it; they are fully overwritten before being read, so nothing needs
//     clearing, but calls that overlap on the GPU (different streams, or
//     different host threads) race on the array and must be serialised.
#include <mutex>

#include "common.cuh"

namespace {

constexpr size_t kScratchBytes = HMC_NOALLOC_SCRATCH_BYTES;
static_assert(kScratchBytes == (size_t)16 << 20, "scratch size is part of the documented contract");

// Host code must not use this name as an address: on the host it denotes a
// shadow object, not device memory.  The device address comes from
// cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void* g_scratch_address[kMaxDevices] = {};

int scratch_on_current_device(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return hmc::cuda_fail(e, "hmc_dense_resid_misfit_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices)
    return hmc::fail(HMC_ERR_UNSUPPORTED, "hmc_dense_resid_misfit_noalloc: device index %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (g_scratch_address[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return hmc::cuda_fail(e, "hmc_dense_resid_misfit_noalloc: cudaGetSymbolAddress");
    g_scratch_address[dev] = p;
  }
  *out = g_scratch_address[dev];
  return HMC_OK;
}

}  // namespace

extern "C" HMC_API int hmc_dense_resid_misfit_noalloc(int dtype, int64_t n, int64_t d, int64_t C, const void* M,
                                                      const void* G, const void* data, const void* inv_var,
                                                      double* out_x, int accumulate, void* stream) {
  HMC_REQUIRE(dtype == HMC_F32 || dtype == HMC_F64, "hmc_dense_resid_misfit_noalloc: unknown dtype %d", dtype);
  HMC_REQUIRE(n > 0 && d > 0 && C >= 0, "hmc_dense_resid_misfit_noalloc: bad sizes");
  const size_t elem = dtype == HMC_F32 ? 4 : 8;
  const size_t max_elems = kScratchBytes / elem;
  HMC_REQUIRE((size_t)n <= max_elems && (C == 0 || (size_t)C <= max_elems / (size_t)n),
              "hmc_dense_resid_misfit_noalloc: residual of %lld x %lld elements exceeds the %zu-byte scratch "
              "(at most %zu elements of this dtype); use hmc_dense_resid_misfit with a caller buffer",
              (long long)n, (long long)C, kScratchBytes, max_elems);
  if (C == 0) return HMC_OK;
  void* scratch = nullptr;
  HMC_TRY(scratch_on_current_device(&scratch));
  return hmc_dense_resid_misfit(dtype, n, d, C, M, G, data, inv_var, scratch, out_x, accumulate, stream);
}
