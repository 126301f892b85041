// Library runtime: error reporting, launch accounting, Philox entry points and
// CUDA-graph capture of whole proposals.
#include <stdarg.h>
#include <string.h>

#include <atomic>

#include "common.cuh"

namespace hmc {

static thread_local char g_last_error[512] = "";
static std::atomic<int64_t> g_launches{0};

int fail(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  return fail(HMC_ERR_CUDA, "%s: %s (%s)", where, cudaGetErrorString(e), cudaGetErrorName(e));
}

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

static std::atomic<uint64_t> g_wait_ns{2000000000ull};
static std::atomic<int> g_withhold{0};

WaitLimits wait_limits() { return WaitLimits{g_wait_ns.load(), g_withhold.load()}; }

__global__ void philox_normal_kernel_f32(int64_t rows, int64_t chains, uint64_t seed, uint64_t proposal,
                                         uint32_t purpose, float* out) {
  const int64_t quads = (rows + 3) / 4;
  const int64_t n = quads * chains;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t % chains, q = t / chains;
    float z[4];
    philox_normal4<float>(seed, (uint32_t)q, (uint32_t)c, proposal, purpose, z);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t i = 4 * q + j;
      if (i < rows) out[i * chains + c] = z[j];
    }
  }
}

__global__ void philox_normal_kernel_f64(int64_t rows, int64_t chains, uint64_t seed, uint64_t proposal,
                                         uint32_t purpose, double* out) {
  const int64_t quads = (rows + 3) / 4;
  const int64_t n = quads * chains;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t % chains, q = t / chains;
    double z[4];
    philox_normal4<double>(seed, (uint32_t)q, (uint32_t)c, proposal, purpose, z);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t i = 4 * q + j;
      if (i < rows) out[i * chains + c] = z[j];
    }
  }
}

__global__ void philox_raw_kernel(int64_t n, uint4 ctr, uint2 key, uint32_t* out) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    uint4 c = ctr;
    c.x += (uint32_t)k;
    const uint4 r = philox4x32_10(c, key);
    out[4 * k + 0] = r.x;
    out[4 * k + 1] = r.y;
    out[4 * k + 2] = r.z;
    out[4 * k + 3] = r.w;
  }
}

}  // namespace hmc

using namespace hmc;

extern "C" {

int hmc_version(void) { return 1; }

const char* hmc_last_error(void) { return g_last_error; }

int64_t hmc_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

int hmc_set_wait_limits(uint64_t wait_ns, int withhold) {
  HMC_REQUIRE(wait_ns >= 1000ull && wait_ns <= 2000000000ull, "hmc_set_wait_limits: limit must be 1 us .. 2 s");
  HMC_REQUIRE(withhold == 0 || withhold == 1, "hmc_set_wait_limits: withhold must be 0 or 1");
  g_wait_ns.store(wait_ns);
  g_withhold.store(withhold);
  return HMC_OK;
}

int hmc_philox_normal(int dtype, int64_t rows, int64_t chains, uint64_t seed, uint64_t proposal,
                      uint32_t purpose, void* out, void* stream) {
  HMC_REQUIRE(rows >= 0 && chains >= 0, "hmc_philox_normal: negative size");
  HMC_REQUIRE(purpose < 16u, "hmc_philox_normal: purpose must be < 16");
  if (rows == 0 || chains == 0) return HMC_OK;
  HMC_REQUIRE(out != nullptr, "hmc_philox_normal: null output");
  const int64_t n = (rows + 3) / 4 * chains;
  const unsigned grid = blocks_for(n, 256) > 65535u * 8 ? 65535u * 8 : blocks_for(n, 256);
  if (dtype == HMC_F32)
    philox_normal_kernel_f32<<<grid, 256, 0, as_stream(stream)>>>(rows, chains, seed, proposal, purpose,
                                                                   (float*)out);
  else if (dtype == HMC_F64)
    philox_normal_kernel_f64<<<grid, 256, 0, as_stream(stream)>>>(rows, chains, seed, proposal, purpose,
                                                                   (double*)out);
  else
    return fail(HMC_ERR_INVALID_ARG, "hmc_philox_normal: unknown dtype %d", dtype);
  return check_launch("hmc_philox_normal");
}

int hmc_philox_raw(int64_t n, uint32_t ctr0, uint32_t ctr1, uint32_t ctr2, uint32_t ctr3, uint32_t key0,
                   uint32_t key1, uint32_t* out, void* stream) {
  HMC_REQUIRE(n >= 0, "hmc_philox_raw: negative size");
  if (n == 0) return HMC_OK;
  HMC_REQUIRE(out != nullptr, "hmc_philox_raw: null output");
  philox_raw_kernel<<<blocks_for(n, 128) > 4096 ? 4096 : blocks_for(n, 128), 128, 0, as_stream(stream)>>>(
      n, make_uint4(ctr0, ctr1, ctr2, ctr3), make_uint2(key0, key1), out);
  return check_launch("hmc_philox_raw");
}

int hmc_stream_capturing(void* stream, int* capturing) {
  HMC_REQUIRE(capturing != nullptr, "hmc_stream_capturing: null output");
  cudaStreamCaptureStatus status = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(as_stream(stream), &status);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamIsCapturing");
  *capturing = status != cudaStreamCaptureStatusNone;
  return HMC_OK;
}

int hmc_fill_zero(void* ptr, int64_t bytes, void* stream) {
  HMC_REQUIRE(bytes >= 0 && (ptr != nullptr || bytes == 0), "hmc_fill_zero: bad buffer");
  if (bytes == 0) return HMC_OK;
  cudaError_t e = cudaMemsetAsync(ptr, 0, (size_t)bytes, as_stream(stream));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemsetAsync");
  return HMC_OK;
}

int hmc_graph_begin(void* stream) {
  HMC_REQUIRE(stream != nullptr, "hmc_graph_begin: capture needs a non-default stream");
  cudaError_t e = cudaStreamBeginCapture(as_stream(stream), cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
  return HMC_OK;
}

struct GraphHandle {
  cudaGraphExec_t exec;
  int64_t kernels;  // kernel nodes per replay, for launch accounting
};

int hmc_graph_end(void* stream, void** graph_exec) {
  HMC_REQUIRE(stream != nullptr && graph_exec != nullptr, "hmc_graph_end: null argument");
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(as_stream(stream), &graph);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  size_t n_nodes = 0;
  e = cudaGraphGetNodes(graph, nullptr, &n_nodes);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return cuda_fail(e, "cudaGraphGetNodes");
  }
  int64_t kernels = 0;
  if (n_nodes > 0) {
    cudaGraphNode_t* nodes = new cudaGraphNode_t[n_nodes];
    e = cudaGraphGetNodes(graph, nodes, &n_nodes);
    for (size_t i = 0; e == cudaSuccess && i < n_nodes; ++i) {
      cudaGraphNodeType t;
      if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kernels;
    }
    delete[] nodes;
  }
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  // Launches recorded during capture did not run; only replays count.
  count_launch((int)-kernels);
  *graph_exec = (void*)new GraphHandle{exec, kernels};
  return HMC_OK;
}

int hmc_graph_launch(void* graph_exec, void* stream) {
  HMC_REQUIRE(graph_exec != nullptr, "hmc_graph_launch: null graph");
  GraphHandle* h = (GraphHandle*)graph_exec;
  cudaError_t e = cudaGraphLaunch(h->exec, as_stream(stream));
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
  count_launch((int)h->kernels);
  return HMC_OK;
}

int hmc_graph_destroy(void* graph_exec) {
  if (graph_exec == nullptr) return HMC_OK;
  GraphHandle* h = (GraphHandle*)graph_exec;
  cudaError_t e = cudaGraphExecDestroy(h->exec);
  delete h;
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphExecDestroy");
  return HMC_OK;
}

}  // extern "C"
