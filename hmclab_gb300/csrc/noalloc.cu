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
//   - the device address of the array is looked up once per device context,
//     on the first call made in it (cudaGetSymbolAddress with the device
//     current), so the first call on each device should be made before any
//     stream capture; if the context is destroyed and created again (for
//     example after cudaDeviceReset), the next call sees a new context ID and
//     looks the address up again, so that call too belongs outside a capture;
//   - every call shares the one array and the last call's residuals stay in
//     it; they are fully overwritten before being read, so nothing needs
//     clearing, but calls that overlap on the GPU (different streams, or
//     different host threads) race on the array and must be serialised.
#include <cuda.h>
#include <cudaTypedefs.h>

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
unsigned long long g_scratch_context[kMaxDevices] = {};  // context ID the address belongs to

// Driver entry points, looked up through the runtime so that the library
// needs no link-time dependency on the driver.
struct DriverContextCalls {
  PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
  PFN_cuCtxGetId_v12000 get_id = nullptr;
};

const DriverContextCalls& driver_calls() {
  static DriverContextCalls calls;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      calls.get_current = (PFN_cuCtxGetCurrent_v4000)p;
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      calls.get_id = (PFN_cuCtxGetId_v12000)p;
  });
  return calls;
}

int scratch_on_current_device(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return hmc::cuda_fail(e, "hmc_dense_resid_misfit_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices)
    return hmc::fail(HMC_ERR_UNSUPPORTED, "hmc_dense_resid_misfit_noalloc: device index %d out of range", dev);
  // make the device's primary context current (cudaSetDevice initialises it
  // and allocates nothing), then identify it: a context created again after
  // a reset has a new ID even if its handle value is reused
  e = cudaSetDevice(dev);
  if (e != cudaSuccess) return hmc::cuda_fail(e, "hmc_dense_resid_misfit_noalloc: cudaSetDevice");
  const DriverContextCalls& drv = driver_calls();
  if (!drv.get_current || !drv.get_id)
    return hmc::fail(HMC_ERR_UNSUPPORTED, "hmc_dense_resid_misfit_noalloc: driver context queries unavailable");
  CUcontext ctx = nullptr;
  unsigned long long ctx_id = 0;
  if (drv.get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr || drv.get_id(ctx, &ctx_id) != CUDA_SUCCESS)
    return hmc::fail(HMC_ERR_CUDA, "hmc_dense_resid_misfit_noalloc: no current CUDA context");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (g_scratch_address[dev] == nullptr || g_scratch_context[dev] != ctx_id) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return hmc::cuda_fail(e, "hmc_dense_resid_misfit_noalloc: cudaGetSymbolAddress");
    g_scratch_address[dev] = p;
    g_scratch_context[dev] = ctx_id;
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
