// zg_api.cu — library entry points: device selection, errors, estimator programs.
#include <stdarg.h>
#include <stdio.h>

#include <algorithm>
#include <mutex>
#include <set>
#include <vector>

#include "zg_internal.cuh"

static thread_local char g_err[512] = "";

const char* zg_set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  int n = snprintf(g_err, sizeof(g_err), "[zg %d] ", code);
  vsnprintf(g_err + n, sizeof(g_err) - n, fmt, ap);
  va_end(ap);
  return g_err;
}

int zg_check_cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return ZG_OK;
  zg_set_error(ZG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? ZG_ERR_OOM : ZG_ERR_CUDA;
}

int zg_num_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 1;
  }
  return sms;
}

namespace {
std::mutex g_pool_mu;
cudaMemPool_t g_pool[64];
}  // namespace

cudaError_t zg_malloc_async(void** p, size_t bytes, cudaStream_t s) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaMallocAsync(p, bytes, s);
  cudaMemPool_t pool;
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pool[dev]) {
      cudaMemPoolProps props = {};
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = dev;
      if ((e = cudaMemPoolCreate(&g_pool[dev], &props)) != cudaSuccess) {
        g_pool[dev] = nullptr;
        return e;
      }
      uint64_t keep = 256ull << 20;
      cudaMemPoolSetAttribute(g_pool[dev], cudaMemPoolAttrReleaseThreshold, &keep);
    }
    pool = g_pool[dev];
  }
  return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

extern "C" int zg_version(void) { return 3; }

extern "C" const char* zg_last_error(void) { return g_err; }

extern "C" int zg_init(int device) {
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    zg_set_error(ZG_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
    return ZG_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= count) {
    zg_set_error(ZG_ERR_INVALID_ARG, "device %d of %d", device, count);
    return ZG_ERR_INVALID_ARG;
  }
  ZG_CUDA(cudaSetDevice(device));
  cudaDeviceProp prop;
  ZG_CUDA(cudaGetDeviceProperties(&prop, device));
  if (prop.major * 10 + prop.minor != 103) {
    zg_set_error(ZG_ERR_NO_DEVICE, "device %d is sm_%d%d; the library targets sm_103a", device, prop.major,
                 prop.minor);
    return ZG_ERR_NO_DEVICE;
  }
  ZG_CUDA(cudaFree(nullptr));
  return ZG_OK;
}

extern "C" int zg_set_l2_fetch_granularity(uint32_t bytes, uint32_t* previous) {
  if (bytes != 0 && bytes != 32 && bytes != 64 && bytes != 128)
    return zg_set_error(ZG_ERR_INVALID_ARG, "L2 fetch granularity %u: 0, 32, 64 or 128", bytes), ZG_ERR_INVALID_ARG;
  size_t old = 0;
  ZG_CUDA(cudaDeviceGetLimit(&old, cudaLimitMaxL2FetchGranularity));
  if (previous) *previous = (uint32_t)old;
  if (bytes) ZG_CUDA(cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, bytes));
  return ZG_OK;
}

// ---- programs ---------------------------------------------------------------------------
static uint32_t pair_bit_host(uint32_t i, uint32_t j, uint32_t pv) {
  if (i > j) std::swap(i, j);
  return i * (2 * pv - i - 1) / 2 + (j - i - 1);
}

extern "C" int zg_program_create(int kind, uint32_t param, zg_program** out) {
  if (!out) return zg_set_error(ZG_ERR_INVALID_ARG, "null output"), ZG_ERR_INVALID_ARG;
  if ((kind < ZG_PROG_TRIANGLE || kind > ZG_PROG_CHAIN) && kind != ZG_PROG_FOUR_CLIQUE_UNBIASED)
    return zg_set_error(ZG_ERR_UNSUPPORTED_ESTIMATOR, "unknown program kind %d", kind), ZG_ERR_UNSUPPORTED_ESTIMATOR;
  if (kind == ZG_PROG_CHAIN && (param < 3 || param > ZG_MAX_LIST))
    return zg_set_error(ZG_ERR_INVALID_ARG, "chain order %u outside [3, %d]", param, ZG_MAX_LIST),
           ZG_ERR_INVALID_ARG;
  zg_program* p = new zg_program();
  memset(p, 0, sizeof(*p));
  p->kind = kind;
  p->param = kind == ZG_PROG_CHAIN ? param : 0;
  *out = p;
  return ZG_OK;
}

// SamplerGenerator ctor (src/SamplerGenerator.cpp:344-366, 393-445): every relabelling of the
// pattern in generate_mapping's order, de-duplicated as edge sets; stored as sorted 28-bit masks.
extern "C" int zg_program_create_pattern(uint32_t pv, uint32_t pe, const uint32_t* edges, zg_program** out) {
  if (!out || !edges) return zg_set_error(ZG_ERR_INVALID_ARG, "null argument"), ZG_ERR_INVALID_ARG;
  if (pv < 2 || pv > ZG_MAX_PATTERN_V || pe < 1 || pe > ZG_MAX_LIST - 1)
    return zg_set_error(ZG_ERR_UNSUPPORTED_ESTIMATOR, "pattern with %u vertices / %u edges is outside 2..%d / 1..%d",
                        pv, pe, ZG_MAX_PATTERN_V, ZG_MAX_LIST - 1),
           ZG_ERR_UNSUPPORTED_ESTIMATOR;
  for (uint32_t e = 0; e < pe; ++e)
    if (edges[2 * e] >= pv || edges[2 * e + 1] >= pv || edges[2 * e] == edges[2 * e + 1])
      return zg_set_error(ZG_ERR_INVALID_ARG, "pattern edge %u is invalid", e), ZG_ERR_INVALID_ARG;
  std::vector<uint32_t> perm(pv);
  for (uint32_t i = 0; i < pv; ++i) perm[i] = i;
  std::set<uint32_t> masks;
  do {
    uint32_t mask = 0;
    for (uint32_t e = 0; e < pe; ++e) mask |= 1u << pair_bit_host(perm[edges[2 * e]], perm[edges[2 * e + 1]], pv);
    masks.insert(mask);
  } while (std::next_permutation(perm.begin(), perm.end()));
  std::vector<uint32_t> sorted(masks.begin(), masks.end());
  zg_program* p = new zg_program();
  memset(p, 0, sizeof(*p));
  p->kind = ZG_PROG_PATTERN;
  p->pv = pv;
  p->pe = pe;
  memcpy(p->pedges, edges, sizeof(uint32_t) * 2 * pe);
  p->num_unique = (uint32_t)sorted.size();
  cudaError_t e = cudaMalloc((void**)&p->d_masks, sizeof(uint32_t) * sorted.size());
  if (e == cudaSuccess)
    e = cudaMemcpy(p->d_masks, sorted.data(), sizeof(uint32_t) * sorted.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    if (p->d_masks) cudaFree(p->d_masks);
    delete p;
    return zg_check_cuda(e, "pattern masks");
  }
  *out = p;
  return ZG_OK;
}

extern "C" int zg_program_free(zg_program* p) {
  if (!p) return ZG_OK;
  if (p->d_masks) cudaFree(p->d_masks);
  delete p;
  return ZG_OK;
}

extern "C" int zg_program_info(const zg_program* p, uint32_t* num_unique, uint32_t* cond_calls, uint32_t* vertices) {
  if (!p) return zg_set_error(ZG_ERR_INVALID_ARG, "null program"), ZG_ERR_INVALID_ARG;
  uint32_t cc = 0, vv = 0;
  switch (p->kind) {
    case ZG_PROG_TRIANGLE: cc = 1; vv = 3; break;
    case ZG_PROG_FOUR_CLIQUE:
    case ZG_PROG_FOUR_CLIQUE_UNBIASED: cc = 2; vv = 4; break;
    case ZG_PROG_THREE_CHAIN: cc = 1; vv = 3; break;
    case ZG_PROG_FOUR_CHAIN: cc = 2; vv = 4; break;
    case ZG_PROG_CHAIN: cc = p->param - 2; vv = p->param; break;
    default: cc = p->pe - 1; vv = p->pv; break;
  }
  if (num_unique) *num_unique = p->kind == ZG_PROG_PATTERN ? p->num_unique : 1;
  if (cond_calls) *cond_calls = cc;
  if (vertices) *vertices = vv;
  return ZG_OK;
}

// ---- bandwidth probes: the L2 view of the roofline, random sectors over a graph ------------
int zg_check_device();  // zg_sample.cu
namespace {
__global__ void k_read_probe(const uint4* __restrict__ buf, uint64_t n16, uint32_t reps, uint4* __restrict__ sink) {
  uint4 acc = make_uint4(0, 0, 0, 0);
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint32_t r = 0; r < reps; ++r)
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n16; i += stride) {
      uint4 v = __ldcg(&buf[i]);  // cached in L2 only
      acc.x ^= v.x;
      acc.y ^= v.y;
      acc.z ^= v.z;
      acc.w ^= v.w;
    }
  if ((acc.x ^ acc.y ^ acc.z ^ acc.w) == 0x9E3779B9u) sink[threadIdx.x] = acc;  // keeps the loads live
}

// Random 32-byte sector reads over a graph's sampled arrays (its edge records and its edge-id
// ordered adjacency, each sector of their union equally likely): each thread keeps 8 independent
// 256-bit loads in flight per iteration; one persistent grid at full occupancy.
__global__ void __launch_bounds__(256) k_random_sectors(const char* __restrict__ rec, uint64_t rec_sectors,
                                                        const char* __restrict__ adj, uint64_t adj_sectors,
                                                        uint32_t iters, uint64_t seed,
                                                        unsigned long long* __restrict__ sink) {
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const uint64_t total = rec_sectors + adj_sectors;
  unsigned long long acc = 0;
  for (uint32_t it = 0; it < iters; ++it) {
    unsigned long long v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const uint64_t h = zg_mix64(seed + tid * 0x9E3779B97F4A7C15ull + (((uint64_t)it << 3) | (uint64_t)k));
      const uint64_t sct = __umul64hi(h, total);  // uniform in [0, total)
      const char* p = sct < rec_sectors ? rec + sct * 32 : adj + (sct - rec_sectors) * 32;
      unsigned long long a0, a1, a2, a3;
      asm volatile("ld.global.nc.v4.u64 {%0, %1, %2, %3}, [%4];" : "=l"(a0), "=l"(a1), "=l"(a2), "=l"(a3) : "l"(p));
      v[k] = a0 ^ a1 ^ a2 ^ a3;
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) acc ^= v[k];
  }
  if (acc == 0x9E3779B97F4A7C15ull) sink[threadIdx.x] = acc;  // keeps the loads live
}
}  // namespace

// Random 32-byte sector reads per second over g's records and adjacency (CUDA events, after one
// warm-up launch): the rate at which the memory system serves isolated sectors from the arrays the
// sampling kernels read, the ceiling of kernels whose loads are random sectors.
extern "C" int zg_random_sector_rate(const zg_graph* g, uint32_t iters, void* cuda_stream, double* sectors_per_s) {
  if (!g || !sectors_per_s || iters == 0 || g->d.m == 0)
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_random_sector_rate: bad argument"), ZG_ERR_INVALID_ARG;
  if (int rc = zg_check_device()) return rc;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  const uint64_t m = g->d.m;
  const uint64_t rec_sectors = (g->wide ? 32ull : 16ull) * m / 32;  // whole sectors of the record array
  const uint64_t adj_sectors = 16ull * m / 32;                      // of adj_e (2m entries of 8 bytes)
  unsigned long long* sink = nullptr;
  cudaError_t e = cudaMalloc(&sink, 256 * sizeof(unsigned long long));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return zg_set_error(ZG_ERR_OOM, "zg_random_sector_rate: %s", cudaGetErrorString(e)), ZG_ERR_OOM;
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_random_sectors, 256, 0);
  const int grid = (per_sm < 1 ? 1 : per_sm) * zg_num_sms();
  const char* rec = (const char*)g->rec;
  const char* adj = (const char*)g->adj_e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_random_sectors<<<grid, 256, 0, s>>>(rec, rec_sectors, adj, adj_sectors, 4, 1, sink);  // warm-up
  cudaEventRecord(e0, s);
  k_random_sectors<<<grid, 256, 0, s>>>(rec, rec_sectors, adj, adj_sectors, iters, 2, sink);
  cudaEventRecord(e1, s);
  e = cudaEventSynchronize(e1);
  float ms = 0;
  if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (e != cudaSuccess) return zg_check_cuda(e, "zg_random_sector_rate");
  *sectors_per_s = ms > 0 ? (double)grid * 256 * iters * 8 / (ms / 1000.0) : 0.0;
  return ZG_OK;
}

// Read bandwidth of a device buffer of `bytes` read `reps` times by one persistent grid (CUDA
// events): a buffer well below the 129 MB L2 measures L2 bandwidth, one well above it HBM.
extern "C" int zg_read_bandwidth(uint64_t bytes, uint32_t reps, void* cuda_stream, double* gbs) {
  if (!gbs || bytes < 16 || reps == 0) return zg_set_error(ZG_ERR_INVALID_ARG, "zg_read_bandwidth: bad argument"), ZG_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  uint64_t n16 = bytes / 16;
  uint4 *buf = nullptr, *sink = nullptr;
  cudaError_t e;
  if ((e = cudaMalloc(&buf, n16 * 16)) || (e = cudaMalloc(&sink, 256 * 16))) {
    if (buf) cudaFree(buf);
    cudaGetLastError();
    return zg_set_error(ZG_ERR_OOM, "zg_read_bandwidth: %s", cudaGetErrorString(e)), ZG_ERR_OOM;
  }
  cudaMemsetAsync(buf, 1, n16 * 16, s);
  int grid = 4 * zg_num_sms();
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_read_probe<<<grid, 256, 0, s>>>(buf, n16, 1, sink);  // warm the cache
  cudaEventRecord(e0, s);
  k_read_probe<<<grid, 256, 0, s>>>(buf, n16, reps, sink);
  cudaEventRecord(e1, s);
  e = cudaEventSynchronize(e1);
  float ms = 0;
  if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  cudaFree(sink);
  if (e != cudaSuccess) return zg_check_cuda(e, "zg_read_bandwidth");
  *gbs = ms > 0 ? (double)n16 * 16 * reps / (ms / 1000.0) / 1e9 : 0.0;
  return ZG_OK;
}
