// zg_noalloc.cu — zg_run_noalloc: the estimator run for callers that must not allocate device
// memory while they serve queries.
//
// Who cannot allocate: a serving process whose memory manager reserves all device memory at
// start-up (a cudaMalloc from this library would fail or fragment that pool), and callers on a
// latency-critical path, where cudaMalloc / cudaFree can synchronise the whole device and
// stall every other stream.  zg_run / zg_run_async take their per-block scratch from the stream
// allocator on each call; this entry point instead uses one fixed array in the library's own
// device data, so it performs no allocation at all.
//
// The scratch holds the sampling kernel's per-block partial sums: ZG_NOALLOC_MAX_BLOCKS blocks of
// ZG_RESULT_BYTES bytes (16384 x 112 B = 1.75 MiB).  Every GPU that loads the library keeps that
// array until the process exits.  All calls share it and it keeps the last call's contents; each
// block overwrites its own slot before the reduction reads it, so nothing needs clearing.  Calls
// whose executions overlap on the GPU (for example on two streams) race on the array and must be
// serialised by the caller.
#include <mutex>

#include "zg_internal.cuh"

int zg_sample_grid(int kind, int layout);
int zg_check_device();
int zg_launch_sample_with_scratch(const zg_graph* g, const zg_program* p, uint64_t n, uint64_t first, uint64_t seed,
                                  uint32_t stream_id, cudaStream_t s, ZgPartial* scratch, int grid, void* d_result);

static __device__ __align__(256) ZgPartial g_noalloc_scratch[ZG_NOALLOC_MAX_BLOCKS];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
ZgPartial* g_scratch_ptr[kMaxDevices] = {nullptr};

// Once per device, with that device current: the device address of the scratch array.  (Host
// code cannot use &g_noalloc_scratch directly; that is a host-side shadow, not device memory.)
// The array used is the current device's, so the graph must live on the current device; a graph
// on another device is refused.
int scratch_for_current_device(const zg_graph* g, ZgPartial** out) {
  int dev = 0;
  ZG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return zg_set_error(ZG_ERR_INVALID_ARG, "device %d out of range", dev), ZG_ERR_INVALID_ARG;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, g->off) != cudaSuccess) {  // offsets: allocated for every graph
    cudaGetLastError();
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_run_noalloc: the graph's memory is not device memory"), ZG_ERR_INVALID_ARG;
  }
  if (a.type != cudaMemoryTypeDevice || a.device != dev)
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_run_noalloc: the graph lives on device %d, the current device is %d",
                        a.device, dev),
           ZG_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || ptr == nullptr) return zg_check_cuda(e == cudaSuccess ? cudaErrorInvalidSymbol : e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_scratch_ptr[dev] = (ZgPartial*)ptr;
  }
  *out = g_scratch_ptr[dev];
  return ZG_OK;
}

}  // namespace

extern "C" int zg_run_noalloc(const zg_graph* g, const zg_program* p, uint64_t n, uint64_t first_sample,
                              uint64_t seed, uint32_t stream_id, void* cuda_stream, void* d_result) {
  if (!g || !p || !d_result) return zg_set_error(ZG_ERR_INVALID_ARG, "null graph, program or result"), ZG_ERR_INVALID_ARG;
  if (int rc = zg_check_device()) return rc;
  ZgPartial* scratch = nullptr;
  int rc = scratch_for_current_device(g, &scratch);
  if (rc) return rc;
  int grid = zg_sample_grid(p->kind, g->wide ? 1 : g->packed ? 2 : 0);
  uint64_t need = (n + 255) / 256;
  if ((uint64_t)grid > need) grid = (int)(need ? need : 1);
  if (grid > ZG_NOALLOC_MAX_BLOCKS)
    return zg_set_error(ZG_ERR_TOO_LARGE,
                        "zg_run_noalloc: the launch needs %d blocks of scratch but the fixed array holds %d",
                        grid, ZG_NOALLOC_MAX_BLOCKS),
           ZG_ERR_TOO_LARGE;
  return zg_launch_sample_with_scratch(g, p, n, first_sample, seed, stream_id, (cudaStream_t)cuda_stream, scratch,
                                       grid, d_result);
}
