// zg_batch.cu — many estimator queries of uneven program, predicate and budget in one
// persistent launch, replayed through a CUDA graph.
//
// The reference runs one calculate() at a time (src/ZGraphInstance.cpp:257-297; a predicate
// query first rebuilds its filtered graph, src/ZGraphInstance.cpp:492-525).  Here a batch is:
//   * a filtered-graph cache: each distinct predicate (op, t0, t1) is filtered, shuffled and
//     rebuilt once on the device (zg_graph_filter) and kept, least recently used first out, within
//     a byte budget;
//   * a work list of (query, chunk) items, chunk = 2^chunk_log2 consecutive sample indices of one
//     query, taken by the blocks of one persistent kernel from an atomic counter; each item's
//     block-reduced partial lands in its own slot;
//   * a finalize kernel that reduces every query's slots in chunk order (exact integer sums, so
//     the estimate equals zg_run's on the same draws; the double variance term is summed in a
//     fixed order, so a batch is deterministic);
//   * one CUDA graph per batch object (copy in, reset the counter, the two kernels, copy out),
//     instantiated once and replayed by every submit: the kernels read the batch size from
//     device memory, so one graph serves every batch up to the object's capacity.
#include <algorithm>
#include <math.h>
#include <map>
#include <tuple>
#include <vector>

#include "zg_programs.cuh"

int zg_graph_filter_sampling(const zg_graph* g, int pred_op, int64_t t0, int64_t t1, uint64_t shuffle_seed,
                             cudaStream_t s, uint64_t* out_m, zg_graph** out);

namespace {

constexpr int kBB = 256;  // threads per block

struct BatchQuery {
  ZgDevGraph g;
  ZgProgParams pp;  // pp.kind == ZG_QUERY_THREE_MOTIF: chain + triangle on the same wedges
  uint64_t n, seed, first;
  uint64_t slot0;  // first partial slot of this query (two partials per chunk)
  uint32_t stream;
  uint32_t nchunks;
};

struct BatchWork {
  uint32_t query, chunk;
};

// Work items [0, nsimple) run in k_batch, [nsimple, nwork) (pattern programs, whose per-sample
// state is larger) in k_batch_pattern, each kernel taking items from its own counter.
struct BatchHeader {
  uint32_t nwork, nsimple, nq, chunk_log2;
};

// The 3-motif sample: a 3-chain estimator whose wedge the triangle estimator closes
// (applications/ThreeMotif.cpp:48-121 with the cache; the fused form of zg_run_three_motif).
__device__ __forceinline__ void motif_sample(const ZgDevGraph& g, Ctx& c, Res& r, Res& rt) {
  if (g.m == 0) {
    r.fail = true;
    return;
  }
  uint64_t e0 = c.draw(0, g.m - 1);
  uint4 q, qp;
  edge_rec(g, e0, q, qp);
  uint64_t S = (uint64_t)q.z + q.w;
  if (S == 0) {
    r.fail = true;
    return;
  }
  uint64_t r1 = c.draw(0, S - 1);
  const bool on_y = r1 >= q.z;
  if (on_y) r1 -= q.z;
  const uint32_t other = on_y ? q.x : q.y, base = after_edge(g, q, qp, on_y);
  res_mul(r, g.m);
  res_mul(r, S);
  r.hit = true;
  uint2 e1 = ZG_LDG(&g.adj_e[base + (uint32_t)r1]);
  uint32_t a1 = 1 + (e1.x == q.x || e1.x == q.y);
  if (a1 == 2) r.shift = 1;
  rt.hit = a1 == 1 && edge_after(g, other, e1.x, e1.y + 1);
  rt.num = r.num;
  rt.shift = r.shift;
}

// One work item: a chunk of one query's samples, reduced into its partial slot(s).
template <bool PATTERN>
__device__ __forceinline__ void batch_item(const BatchQuery& sq, uint32_t chunk, uint32_t clog,
                                           ZgPartial* __restrict__ parts) {
  const uint64_t lo = (uint64_t)chunk << clog;
  const uint64_t end = lo + (1ull << clog);
  const uint64_t hi = end < sq.n ? end : sq.n;
  const bool motif = !PATTERN && sq.pp.kind == ZG_QUERY_THREE_MOTIF;
  Acc a, at;
  acc_init(a);
  acc_init(at);
  // The sums of a (the 3-motif's triangle sums stay in at) live in shared-memory slots, as in
  // k_sample's long programs: the registers they free let more warps stay resident without
  // spilling (each thread adds its hits in the same order, so the sums are the same).
  __shared__ AccSlots<kBB> sl;
  acc_slots_init(sl);
  for (uint64_t i = lo + threadIdx.x; i < hi; i += kBB) {
    Ctx c{sq.seed, sq.first + i, sq.stream, 0, nullptr, 0};
    Res r;
    res_init(r);
    if (PATTERN) {
      prog_pattern<false>(sq.g, sq.pp, c, r);
      acc_add_slots(a, sl, r, sq.pp.den_log2);
    } else if (motif) {
      Res rt;
      res_init(rt);
      motif_sample(sq.g, c, r, rt);
      acc_add_slots(a, sl, r, 1);
      acc_add(at, rt, 1);
    } else {
      switch (sq.pp.kind) {
        case ZG_PROG_TRIANGLE: prog_triangle<false>(sq.g, c, r); break;
        case ZG_PROG_FOUR_CLIQUE: prog_four_clique<false>(sq.g, c, r); break;
        case ZG_PROG_FOUR_CLIQUE_UNBIASED: prog_four_clique<false, true>(sq.g, c, r); break;
        case ZG_PROG_THREE_CHAIN: prog_three_chain<false>(sq.g, c, r); break;
        case ZG_PROG_FOUR_CHAIN: prog_four_chain<false>(sq.g, c, r); break;
        default: prog_chain<false>(sq.g, (int)sq.pp.param, c, r); break;  // ZG_PROG_CHAIN
      }
      acc_add_slots(a, sl, r, sq.pp.den_log2);
    }
  }
  acc_from_slots(a, sl);
  const uint64_t slot = 2 * (sq.slot0 + chunk);
  block_reduce_store<kBB>(a, &parts[slot]);
  __syncthreads();
  if (motif) block_reduce_store<kBB>(at, &parts[slot + 1]);
}

template <bool PATTERN, int MINB>
__global__ void __launch_bounds__(kBB, MINB)
    k_batch(const BatchHeader* __restrict__ hdr, const BatchQuery* __restrict__ qs, const BatchWork* __restrict__ work,
            ZgPartial* __restrict__ parts, unsigned int* __restrict__ counters) {
  __shared__ BatchQuery sq;
  __shared__ uint32_t sw;
  const uint32_t base = PATTERN ? hdr->nsimple : 0, limit = PATTERN ? hdr->nwork : hdr->nsimple;
  const uint32_t clog = hdr->chunk_log2;
  for (;;) {
    if (threadIdx.x == 0) sw = base + atomicAdd(&counters[PATTERN ? 1 : 0], 1u);
    __syncthreads();
    const uint32_t w = sw;
    if (w >= limit) break;
    const BatchWork wk = work[w];
    {
      // the query descriptor into shared memory, one word per thread
      const uint32_t* src = reinterpret_cast<const uint32_t*>(&qs[wk.query]);
      uint32_t* dst = reinterpret_cast<uint32_t*>(&sq);
      for (uint32_t i = threadIdx.x; i < sizeof(BatchQuery) / 4; i += kBB) dst[i] = src[i];
    }
    __syncthreads();
    batch_item<PATTERN>(sq, wk.chunk, clog, parts);
    __syncthreads();  // sq and sw are rewritten by the next item
  }
}

// One block per query: its chunks' partials (two per chunk) in chunk order.
__global__ void __launch_bounds__(kBB) k_batch_finalize(const BatchHeader* __restrict__ hdr,
                                                        const BatchQuery* __restrict__ qs,
                                                        const ZgPartial* __restrict__ parts,
                                                        ZgPartial* __restrict__ out) {
  const uint32_t q = blockIdx.x;
  if (q >= hdr->nq) return;
  const uint64_t slot0 = qs[q].slot0;
  const uint32_t nch = qs[q].nchunks;
  for (int half = 0; half < 2; ++half) {
    unsigned long long v[12] = {0};
    double d0 = 0, d1 = 0;
    for (uint32_t c = threadIdx.x; c < nch; c += kBB) {
      const ZgPartial& p = parts[2 * (slot0 + c) + half];
      v[0] += p.samples;
      v[1] += p.hits;
      v[2] += p.fails;
      v[3] += p.overflow;
      for (int i = 0; i < 8; ++i) v[4 + i] += p.lane[i];
      d0 += p.sum_w4;
      d1 += p.sum_w2;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
      for (int i = 0; i < 12; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
      d0 += __shfl_xor_sync(0xffffffffu, d0, o);
      d1 += __shfl_xor_sync(0xffffffffu, d1, o);
    }
    __shared__ unsigned long long sv[kBB / 32][12];
    __shared__ double sd[kBB / 32][2];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
      for (int i = 0; i < 12; ++i) sv[warp][i] = v[i];
      sd[warp][0] = d0;
      sd[warp][1] = d1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      ZgPartial p;
      unsigned long long t[12] = {0};
      double s0 = 0, s1 = 0;
      for (int w = 0; w < kBB / 32; ++w) {
        for (int i = 0; i < 12; ++i) t[i] += sv[w][i];
        s0 += sd[w][0];
        s1 += sd[w][1];
      }
      p.samples = t[0];
      p.hits = t[1];
      p.fails = t[2];
      p.overflow = t[3];
      for (int i = 0; i < 8; ++i) p.lane[i] = t[4 + i];
      p.sum_w4 = s0;
      p.sum_w2 = s1;
      out[2 * q + half] = p;
    }
    __syncthreads();
  }
}

typedef void (*BatchKernel)(const BatchHeader*, const BatchQuery*, const BatchWork*, ZgPartial*, unsigned int*);
constexpr int kBatchVariants = 3;  // 2, 3 or 4 resident blocks of 256 threads
BatchKernel batch_kernel(int v, bool pattern) {
  switch (v) {
    case 0: return pattern ? k_batch<true, 2> : k_batch<false, 2>;
    case 1: return pattern ? k_batch<true, 3> : k_batch<false, 3>;
    default: return pattern ? k_batch<true, 4> : k_batch<false, 4>;
  }
}

template <typename T>
int dalloc(T** p, size_t count) {
  cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    zg_set_error(ZG_ERR_OOM, "cudaMalloc(%zu bytes) failed: %s", sizeof(T) * count, cudaGetErrorString(e));
    return ZG_ERR_OOM;
  }
  return ZG_OK;
}

uint32_t den_of(int kind, uint32_t param, const zg_program* prog) {
  switch (kind) {
    case ZG_PROG_TRIANGLE: return 1;
    case ZG_PROG_FOUR_CLIQUE: return 2;
    case ZG_PROG_FOUR_CLIQUE_UNBIASED: return 2;
    case ZG_PROG_THREE_CHAIN: return 1;
    case ZG_PROG_FOUR_CHAIN: return 2;
    case ZG_PROG_CHAIN: return param - 2;
    case ZG_QUERY_THREE_MOTIF: return 1;
    default: return prog ? prog->pe - 1 : 0;
  }
}

}  // namespace

void zg_partial_to_counters(const void* partial, uint32_t den, zg_counters* out);

struct zg_batch {
  const zg_graph* base;
  uint32_t max_queries, max_work;
  uint64_t cache_bytes, filter_seed;
  // filtered-graph cache
  struct Entry {
    zg_graph* g;
    uint64_t bytes, last_use;
  };
  std::map<std::tuple<int, int64_t, int64_t>, Entry> cache;
  uint64_t cached_bytes = 0, use_clock = 0;
  // device buffers
  BatchHeader* d_hdr = nullptr;
  BatchQuery* d_q = nullptr;
  BatchWork* d_work = nullptr;
  ZgPartial* d_parts = nullptr;
  ZgPartial* d_out = nullptr;
  unsigned int* d_counter = nullptr;
  // pinned host staging
  BatchHeader* h_hdr = nullptr;
  BatchQuery* h_q = nullptr;
  BatchWork* h_work = nullptr;
  ZgPartial* h_out = nullptr;
  std::vector<uint32_t> den;
  uint32_t nq = 0;
  // graph
  int variant = 2;
  int grid = 0, grid_pattern = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t last_stream = nullptr;
  bool submitted = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // around the graph launch
  float last_ms = 0;
};

namespace {

void batch_release_graph(zg_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

// copy in, reset the counter, the persistent kernel, the finalize kernel, copy out
int batch_enqueue(zg_batch* b, cudaStream_t s) {
  cudaError_t e;
  if ((e = cudaMemcpyAsync(b->d_hdr, b->h_hdr, sizeof(BatchHeader), cudaMemcpyHostToDevice, s)) ||
      (e = cudaMemcpyAsync(b->d_q, b->h_q, sizeof(BatchQuery) * b->max_queries, cudaMemcpyHostToDevice, s)) ||
      (e = cudaMemcpyAsync(b->d_work, b->h_work, sizeof(BatchWork) * b->max_work, cudaMemcpyHostToDevice, s)) ||
      (e = cudaMemsetAsync(b->d_counter, 0, 2 * sizeof(unsigned int), s)))
    return zg_check_cuda(e, "batch copy-in");
  batch_kernel(b->variant, false)<<<b->grid, kBB, 0, s>>>(b->d_hdr, b->d_q, b->d_work, b->d_parts, b->d_counter);
  batch_kernel(b->variant, true)<<<b->grid_pattern, kBB, 0, s>>>(b->d_hdr, b->d_q, b->d_work, b->d_parts,
                                                                 b->d_counter);
  k_batch_finalize<<<b->max_queries, kBB, 0, s>>>(b->d_hdr, b->d_q, b->d_parts, b->d_out);
  if ((e = cudaMemcpyAsync(b->h_out, b->d_out, sizeof(ZgPartial) * 2 * b->max_queries, cudaMemcpyDeviceToHost, s)))
    return zg_check_cuda(e, "batch copy-out");
  return ZG_OK;
}

int batch_build_graph(zg_batch* b) {
  batch_release_graph(b);
  cudaStream_t cs;
  cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e) return zg_check_cuda(e, "capture stream");
  int rc = ZG_OK;
  if ((e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal))) {
    cudaStreamDestroy(cs);
    return zg_check_cuda(e, "begin capture");
  }
  rc = batch_enqueue(b, cs);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(cs, &g);
  cudaStreamDestroy(cs);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e) return zg_check_cuda(e, "end capture");
  b->graph = g;
  if ((e = cudaGraphInstantiate(&b->exec, g, 0))) {
    cudaGraphDestroy(g);
    b->graph = nullptr;
    return zg_check_cuda(e, "graph instantiate");
  }
  return ZG_OK;
}

int batch_set_variant(zg_batch* b, int v) {
  b->variant = v;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel(v, false), kBB, 0);
  b->grid = (per_sm < 1 ? 1 : per_sm) * zg_num_sms();
  per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel(v, true), kBB, 0);
  b->grid_pattern = (per_sm < 1 ? 1 : per_sm) * zg_num_sms();
  return batch_build_graph(b);
}

uint64_t filter_seed_of(uint64_t base, int op, int64_t t0, int64_t t1) {
  return zg_mix64(base ^ zg_mix64((uint64_t)op * 0x9E3779B97F4A7C15ull ^ zg_mix64((uint64_t)t0) ^
                                  (zg_mix64((uint64_t)t1) << 1)));
}

// Frees the least recently used cached graph that is neither `keep` nor used by the batch being
// prepared (`pinned`); false when there is none.
bool batch_evict_one(zg_batch* b, const std::vector<const zg_graph*>& pinned, const zg_graph* keep) {
  auto victim = b->cache.end();
  for (auto jt = b->cache.begin(); jt != b->cache.end(); ++jt) {
    if (jt->second.g == keep || std::find(pinned.begin(), pinned.end(), jt->second.g) != pinned.end()) continue;
    if (victim == b->cache.end() || jt->second.last_use < victim->second.last_use) victim = jt;
  }
  if (victim == b->cache.end()) return false;
  b->cached_bytes -= victim->second.bytes;
  zg_graph_free(victim->second.g);
  b->cache.erase(victim);
  return true;
}

// The cached filtered graph of (op, t0, t1), built on first use; `pinned` holds the graphs the
// batch being prepared uses (never evicted for it).  A build that runs out of device memory frees
// cached graphs, least recently used first, and tries again.
int batch_filtered(zg_batch* b, int op, int64_t t0, int64_t t1, cudaStream_t s,
                   const std::vector<const zg_graph*>& pinned, const zg_graph** out) {
  auto key = std::make_tuple(op, t0, op == ZG_PRED_RANGE ? t1 : 0);
  auto it = b->cache.find(key);
  if (it != b->cache.end()) {
    it->second.last_use = ++b->use_clock;
    *out = it->second.g;
    return ZG_OK;
  }
  zg_graph* g = nullptr;
  uint64_t m = 0;
  int rc;
  do {
    rc = zg_graph_filter_sampling(b->base, op, t0, t1, filter_seed_of(b->filter_seed, op, t0, t1), s, &m, &g);
  } while (rc == ZG_ERR_OOM && batch_evict_one(b, pinned, nullptr));
  if (rc) return rc;
  zg_graph_meta meta;
  zg_graph_get_meta(g, &meta);
  b->cache[key] = {g, meta.device_bytes, ++b->use_clock};
  b->cached_bytes += meta.device_bytes;
  // evict least recently used graphs not used by this batch while over budget
  while (b->cached_bytes > b->cache_bytes && batch_evict_one(b, pinned, g)) {
  }
  *out = g;
  return ZG_OK;
}

}  // namespace

extern "C" int zg_batch_create(const zg_graph* base, uint32_t max_queries, uint64_t cache_bytes, uint64_t filter_seed,
                               zg_batch** out) {
  if (!base || !out || max_queries == 0)
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_batch_create: null argument or zero capacity"), ZG_ERR_INVALID_ARG;
  if (max_queries > ZG_BATCH_MAX_QUERIES)
    return zg_set_error(ZG_ERR_TOO_LARGE, "zg_batch_create: at most %u queries", ZG_BATCH_MAX_QUERIES), ZG_ERR_TOO_LARGE;
  zg_batch* b = new zg_batch();
  b->base = base;
  b->max_queries = max_queries;
  b->max_work = ZG_BATCH_MAX_CHUNKS + max_queries;
  b->cache_bytes = cache_bytes;
  b->filter_seed = filter_seed;
  int rc;
  cudaError_t e;
  if ((rc = dalloc(&b->d_hdr, 1)) || (rc = dalloc(&b->d_q, max_queries)) || (rc = dalloc(&b->d_work, b->max_work)) ||
      (rc = dalloc(&b->d_parts, 2 * (size_t)b->max_work)) || (rc = dalloc(&b->d_out, 2 * (size_t)max_queries)) ||
      (rc = dalloc(&b->d_counter, 2))) {
    zg_batch_free(b);
    return rc;
  }
  if ((e = cudaMallocHost((void**)&b->h_hdr, sizeof(BatchHeader))) ||
      (e = cudaMallocHost((void**)&b->h_q, sizeof(BatchQuery) * max_queries)) ||
      (e = cudaMallocHost((void**)&b->h_work, sizeof(BatchWork) * b->max_work)) ||
      (e = cudaMallocHost((void**)&b->h_out, sizeof(ZgPartial) * 2 * max_queries))) {
    cudaGetLastError();
    zg_batch_free(b);
    return zg_set_error(ZG_ERR_OOM, "pinned host buffers: %s", cudaGetErrorString(e)), ZG_ERR_OOM;
  }
  if ((e = cudaEventCreate(&b->ev0)) || (e = cudaEventCreate(&b->ev1))) {
    zg_batch_free(b);
    return zg_check_cuda(e, "batch events");
  }
  memset(b->h_hdr, 0, sizeof(BatchHeader));
  memset(b->h_q, 0, sizeof(BatchQuery) * max_queries);
  memset(b->h_work, 0, sizeof(BatchWork) * b->max_work);
  if ((rc = batch_set_variant(b, 2))) {
    zg_batch_free(b);
    return rc;
  }
  *out = b;
  return ZG_OK;
}

extern "C" int zg_batch_free(zg_batch* b) {
  if (!b) return ZG_OK;
  if (b->submitted && b->last_stream) cudaStreamSynchronize(b->last_stream);
  batch_release_graph(b);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  for (auto& kv : b->cache) zg_graph_free(kv.second.g);
  cudaFree(b->d_hdr);
  cudaFree(b->d_q);
  cudaFree(b->d_work);
  cudaFree(b->d_parts);
  cudaFree(b->d_out);
  cudaFree(b->d_counter);
  if (b->h_hdr) cudaFreeHost(b->h_hdr);
  if (b->h_q) cudaFreeHost(b->h_q);
  if (b->h_work) cudaFreeHost(b->h_work);
  if (b->h_out) cudaFreeHost(b->h_out);
  delete b;
  return ZG_OK;
}

extern "C" int zg_batch_filtered_graph(zg_batch* b, int pred_op, int64_t t0, int64_t t1, void* cuda_stream,
                                       const zg_graph** out) {
  if (!b || !out || pred_op < ZG_PRED_GE || pred_op > ZG_PRED_RANGE)
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_batch_filtered_graph: bad argument"), ZG_ERR_INVALID_ARG;
  if (b->submitted && b->last_stream) {
    cudaError_t e = cudaStreamSynchronize(b->last_stream);  // a running batch may use a cached graph
    if (e) return zg_check_cuda(e, "previous batch");
  }
  return batch_filtered(b, pred_op, t0, t1, (cudaStream_t)cuda_stream, {}, out);
}

extern "C" int zg_batch_submit(zg_batch* b, const zg_batch_query* q, uint32_t nq, void* cuda_stream) {
  if (!b || (nq && !q)) return zg_set_error(ZG_ERR_INVALID_ARG, "zg_batch_submit: null argument"), ZG_ERR_INVALID_ARG;
  if (nq > b->max_queries)
    return zg_set_error(ZG_ERR_TOO_LARGE, "zg_batch_submit: %u queries > capacity %u", nq, b->max_queries),
           ZG_ERR_TOO_LARGE;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  if (b->submitted && b->last_stream) {
    cudaError_t e = cudaStreamSynchronize(b->last_stream);  // the staging buffers are reused
    if (e) return zg_check_cuda(e, "previous batch");
  }
  // validate, then programs (built-in kinds are created here; patterns come with the query)
  for (uint32_t i = 0; i < nq; ++i) {
    const zg_batch_query& x = q[i];
    if (x.n == 0) return zg_set_error(ZG_ERR_INVALID_ARG, "query %u: zero estimators", i), ZG_ERR_INVALID_ARG;
    bool builtin = (x.kind >= ZG_PROG_TRIANGLE && x.kind <= ZG_PROG_CHAIN) || x.kind == ZG_PROG_FOUR_CLIQUE_UNBIASED;
    bool pattern = x.kind == ZG_PROG_PATTERN && x.program && x.program->kind == ZG_PROG_PATTERN;
    if (!builtin && !pattern && x.kind != ZG_QUERY_THREE_MOTIF)
      return zg_set_error(ZG_ERR_UNSUPPORTED_ESTIMATOR, "query %u: kind %d%s", i, x.kind,
                          x.kind == ZG_PROG_PATTERN ? " needs its pattern program" : ""),
             ZG_ERR_UNSUPPORTED_ESTIMATOR;
  }
  std::vector<const zg_graph*> graphs(nq);
  std::vector<zg_program*> own(nq, nullptr);
  int rc = ZG_OK;
  for (uint32_t i = 0; i < nq && rc == ZG_OK; ++i) {
    const zg_batch_query& x = q[i];
    if ((x.kind >= ZG_PROG_TRIANGLE && x.kind <= ZG_PROG_CHAIN) || x.kind == ZG_PROG_FOUR_CLIQUE_UNBIASED)
      rc = zg_program_create(x.kind, x.param, &own[i]);
    if (rc == ZG_OK) {
      if (x.pred_op) rc = batch_filtered(b, x.pred_op, x.t0, x.t1, s, graphs, &graphs[i]);
      else graphs[i] = b->base;
    }
  }
  if (rc) {
    for (auto* p : own)
      if (p) zg_program_free(p);
    return rc;
  }
  // chunk size: the smallest power of two >= 2^12 that keeps the work list within capacity
  uint32_t clog = 12;
  for (;;) {
    uint64_t items = 0;
    for (uint32_t i = 0; i < nq; ++i) items += (q[i].n + (1ull << clog) - 1) >> clog;
    if (items <= b->max_work) break;
    ++clog;
  }
  b->den.assign(nq, 0);
  std::vector<uint32_t> nch(nq);
  std::vector<char> is_pattern(nq, 0);
  uint64_t slot = 0;
  for (uint32_t i = 0; i < nq; ++i) {
    const zg_batch_query& x = q[i];
    const zg_program* p = own[i] ? own[i] : x.program;  // null for the 3-motif
    BatchQuery& d = b->h_q[i];
    memset(&d, 0, sizeof(d));
    d.g = graphs[i]->d;
    if (p) {
      d.pp.kind = p->kind;
      d.pp.param = p->param;
      d.pp.pv = p->pv;
      d.pp.pe = p->pe;
      d.pp.num_unique = p->num_unique;
      d.pp.masks = p->d_masks;
    } else {
      d.pp.kind = ZG_QUERY_THREE_MOTIF;
    }
    is_pattern[i] = p && p->kind == ZG_PROG_PATTERN;
    d.pp.den_log2 = den_of(x.kind, x.param, p);
    b->den[i] = d.pp.den_log2;
    d.n = x.n;
    d.seed = x.seed;
    d.first = x.first_sample;
    d.stream = x.stream_id;
    nch[i] = (uint32_t)((x.n + (1ull << clog) - 1) >> clog);
    d.nchunks = nch[i];
    d.slot0 = slot;
    slot += nch[i];
  }
  // work items, built-in programs first, then patterns; within each, round-robin over queries so
  // long and short queries mix
  uint32_t nwork = 0, nsimple = 0;
  for (int pass = 0; pass < 2; ++pass) {
    for (uint32_t round = 0, left = 1; left; ++round) {
      left = 0;
      for (uint32_t i = 0; i < nq; ++i)
        if (is_pattern[i] == pass && round < nch[i]) {
          b->h_work[nwork++] = {i, round};
          left = 1;
        }
    }
    if (pass == 0) nsimple = nwork;
  }
  b->h_hdr->nwork = nwork;
  b->h_hdr->nsimple = nsimple;
  b->h_hdr->nq = nq;
  b->h_hdr->chunk_log2 = clog;
  b->nq = nq;
  // built-in programs carry no device tables: their descriptors are complete without them
  for (auto* p : own)
    if (p) zg_program_free(p);
  cudaEventRecord(b->ev0, s);
  cudaError_t e = cudaGraphLaunch(b->exec, s);
  if (e) return zg_check_cuda(e, "batch graph launch");
  cudaEventRecord(b->ev1, s);
  b->last_stream = s;
  b->submitted = true;
  return ZG_OK;
}

extern "C" int zg_batch_wait(zg_batch* b, zg_counters* out) {
  if (!b || !out) return zg_set_error(ZG_ERR_INVALID_ARG, "zg_batch_wait: null argument"), ZG_ERR_INVALID_ARG;
  if (!b->submitted) return zg_set_error(ZG_ERR_INVALID_ARG, "zg_batch_wait: nothing submitted"), ZG_ERR_INVALID_ARG;
  cudaError_t e = cudaStreamSynchronize(b->last_stream);
  if (e) return zg_check_cuda(e, "batch");
  cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1);
  for (uint32_t i = 0; i < b->nq; ++i) {
    zg_partial_to_counters(&b->h_out[2 * i], b->den[i], &out[2 * i]);
    zg_partial_to_counters(&b->h_out[2 * i + 1], b->den[i], &out[2 * i + 1]);
  }
  b->submitted = false;
  return ZG_OK;
}

extern "C" int zg_batch_size_learned(zg_batch* b, const zg_mlp* net, zg_batch_query* q, uint32_t nq, double error,
                                     double confidence, uint64_t pilot_samples, void* cuda_stream) {
  if (!b || !net || (nq && !q))
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_batch_size_learned: null argument"), ZG_ERR_INVALID_ARG;
  if (!(error > 0) || !(confidence > 0 && confidence < 1))
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_batch_size_learned: error %g / confidence %g", error, confidence),
           ZG_ERR_INVALID_ARG;
  const bool adaptive = pilot_samples == 0;  // as zg_graph_features: 2^16 .. 2^22 until 8 hits
  if (adaptive) pilot_samples = 1ull << 16;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  // the queries to size, as pilot queries: the pilot zg_graph_features would run for each
  std::vector<uint32_t> idx;
  std::vector<zg_batch_query> pilot;
  for (uint32_t i = 0; i < nq; ++i) {
    if (q[i].n != 0) continue;
    if (q[i].kind == ZG_QUERY_THREE_MOTIF)
      return zg_set_error(ZG_ERR_INVALID_ARG, "query %u: a 3-motif query needs its sample count", i),
             ZG_ERR_INVALID_ARG;
    zg_batch_query x = q[i];
    x.n = pilot_samples;
    x.first_sample = 0;
    x.stream_id = ZG_ELP_STREAM + 1;
    idx.push_back(i);
    pilot.push_back(x);
  }
  if (idx.empty()) return ZG_OK;
  const uint32_t k = (uint32_t)idx.size();
  std::vector<zg_counters> c(2 * (size_t)k);
  int rc = zg_batch_submit(b, pilot.data(), k, cuda_stream);
  if (rc == ZG_OK) rc = zg_batch_wait(b, c.data());
  if (rc) return rc;
  // adaptive pilots: the queries below 8 hits again with 4x the estimators, up to 2^22
  for (uint64_t n = pilot_samples << 2; adaptive && n <= (1ull << 22); n <<= 2) {
    std::vector<uint32_t> again;
    std::vector<zg_batch_query> more;
    for (uint32_t j = 0; j < k; ++j)
      if (c[2 * j].hits < 8) {
        again.push_back(j);
        more.push_back(pilot[j]);
        more.back().n = n;
      }
    if (again.empty()) break;
    std::vector<zg_counters> c2(2 * again.size());
    if ((rc = zg_batch_submit(b, more.data(), (uint32_t)more.size(), cuda_stream)) ||
        (rc = zg_batch_wait(b, c2.data())))
      return rc;
    for (size_t a = 0; a < again.size(); ++a) c[2 * again[a]] = c2[2 * a];
  }
  // features: the query graph's degree statistics, the program class, the pilot
  std::vector<float> X((size_t)k * ZG_MLP_FEATURES), Y((size_t)k * ZG_MLP_OUTPUTS);
  std::vector<const zg_graph*> none;
  for (uint32_t j = 0; j < k && rc == ZG_OK; ++j) {
    const zg_batch_query& x = q[idx[j]];
    const zg_graph* g = b->base;
    if (x.pred_op) rc = batch_filtered(b, x.pred_op, x.t0, x.t1, s, none, &g);
    zg_program* own = nullptr;
    if (rc == ZG_OK && x.kind != ZG_PROG_PATTERN) rc = zg_program_create(x.kind, x.param, &own);
    float* f = &X[(size_t)j * ZG_MLP_FEATURES];
    if (rc == ZG_OK) rc = zg_degree_features(g, s, f);
    if (rc == ZG_OK) zg_query_features(own ? own : x.program, c[2 * j], f);
    if (own) zg_program_free(own);
  }
  if (rc == ZG_OK) rc = zg_mlp_predict(net, X.data(), k, Y.data());
  if (rc) return rc;
  for (uint32_t j = 0; j < k; ++j) q[idx[j]].n = zg_learned_n(Y[(size_t)j * ZG_MLP_OUTPUTS], error, confidence);
  return ZG_OK;
}

double zg_exact_mean_host(const uint64_t s[5], uint32_t den, uint64_t n);

namespace {
double exact_mean_of(const zg_counters& c) { return zg_exact_mean_host(c.sum_num, c.den_log2, c.samples); }
// a += c for two runs of one query over disjoint sample ranges (same den_log2): exact.
void merge_into(zg_counters& a, const zg_counters& c) {
  unsigned __int128 carry = 0;
  for (int i = 0; i < 5; ++i) {
    unsigned __int128 t = (unsigned __int128)a.sum_num[i] + c.sum_num[i] + carry;
    a.sum_num[i] = (uint64_t)t;
    carry = t >> 64;
  }
  a.samples += c.samples;
  a.hits += c.hits;
  a.fails += c.fails;
  a.overflow |= c.overflow;
  a.sum_w2 += c.sum_w2;
  a.sum_w4 += c.sum_w4;
  a.estimate = exact_mean_of(a);
  a.sum_w = zg_exact_mean_host(a.sum_num, a.den_log2, 1);  // the exact sum, rounded once
}
}  // namespace

extern "C" int zg_batch_bounded(zg_batch* b, const zg_mlp* net, const zg_batch_query* q, uint32_t nq, double error,
                                double confidence, uint32_t max_rounds, uint64_t max_samples, void* cuda_stream,
                                zg_counters* out, uint32_t* bound_met, uint32_t* rounds_run) {
  if (!b || !net || (nq && (!q || !out || !bound_met)))
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_batch_bounded: null argument"), ZG_ERR_INVALID_ARG;
  if (max_rounds == 0) max_rounds = 4;
  if (max_samples == 0) max_samples = 1ull << 40;
  std::vector<zg_batch_query> sized(q, q + nq);
  int rc = zg_batch_size_learned(b, net, sized.data(), nq, error, confidence, 0, cuda_stream);
  if (rc) return rc;
  const cudaStream_t s = (cudaStream_t)cuda_stream;
  std::vector<uint64_t> ran(nq, 0), want(nq);
  std::vector<uint32_t> pending;
  for (uint32_t i = 0; i < nq; ++i) {
    want[i] = sized[i].n;
    bound_met[i] = 0;
    pending.push_back(i);
    memset(&out[2 * i], 0, 2 * sizeof(zg_counters));
  }
  uint32_t rounds = 0;
  std::vector<zg_batch_query> sub;
  std::vector<zg_counters> res;
  while (!pending.empty() && rounds < max_rounds) {
    sub.clear();
    for (uint32_t i : pending) {
      zg_batch_query x = sized[i];
      x.n = want[i];
      x.first_sample = sized[i].first_sample + ran[i];  // fresh sample indices
      sub.push_back(x);
    }
    res.assign(2 * sub.size(), zg_counters{});
    if ((rc = zg_batch_submit(b, sub.data(), (uint32_t)sub.size(), cuda_stream)) ||
        (rc = zg_batch_wait(b, res.data())))
      return rc;
    ++rounds;
    std::vector<uint32_t> next;
    for (size_t j = 0; j < pending.size(); ++j) {
      const uint32_t i = pending[j];
      if (sized[i].kind == ZG_QUERY_THREE_MOTIF) {  // its given budgets, once
        out[2 * i] = res[2 * j];
        out[2 * i + 1] = res[2 * j + 1];
        continue;
      }
      if (ran[i] == 0) out[2 * i] = res[2 * j];
      else merge_into(out[2 * i], res[2 * j]);
      ran[i] += want[i];
      const zg_counters& t = out[2 * i];
      const double n = (double)t.samples;
      double var = n > 0 ? t.sum_w2 / n - t.estimate * t.estimate : 0.0;
      if (var < 0) var = 0;
      // a filtered graph's estimators are bounded by the base graph's range (fewer edges, lower degrees)
      double range = 0, half = 0;
      uint32_t method = 0;
      if ((rc = zg_weight_range(b->base, sized[i].kind, sized[i].param,
                                sized[i].program ? sized[i].program->pe : 0, s, &range)))
        return rc;
      const double ew4 = n > 0 ? t.sum_w4 / n : 0.0;
      if (zg_bound_check(t.estimate, var, ew4, t.samples, t.hits, error, confidence, range, &half, &method)) {
        bound_met[i] = 1;
        continue;
      }
      const double need = zg_samples_needed(t.estimate, var, ew4, t.samples, t.hits, error, confidence);
      if (ran[i] >= max_samples) continue;
      const double cap = (double)max_samples;
      const uint64_t target = (uint64_t)(need < cap ? need : cap);
      want[i] = target > ran[i] ? target - ran[i] : 0;
      if (want[i] < ran[i] / 4 + 1) want[i] = ran[i] / 4 + 1;
      if (want[i] > max_samples - ran[i]) want[i] = max_samples - ran[i];
      next.push_back(i);
    }
    pending.swap(next);
  }
  if (rounds_run) *rounds_run = rounds;
  return ZG_OK;
}

extern "C" int zg_batch_tune(zg_batch* b, const zg_batch_query* q, uint32_t nq, void* cuda_stream, int* best_variant,
                             float* ms_per_variant) {
  if (!b || !q) return zg_set_error(ZG_ERR_INVALID_ARG, "zg_batch_tune: null argument"), ZG_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  std::vector<zg_counters> tmp(2 * (size_t)nq);
  float best_ms = 0;
  int best = b->variant;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int rc = ZG_OK;
  for (int v = 0; v < kBatchVariants && rc == ZG_OK; ++v) {
    if ((rc = batch_set_variant(b, v))) break;
    float vbest = 0;
    for (int rep = 0; rep < 3 && rc == ZG_OK; ++rep) {
      cudaEventRecord(e0, s);
      if ((rc = zg_batch_submit(b, q, nq, cuda_stream))) break;
      cudaEventRecord(e1, s);
      if ((rc = zg_batch_wait(b, tmp.data()))) break;
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep == 0 || ms < vbest) vbest = ms;
    }
    if (ms_per_variant) ms_per_variant[v] = vbest;
    if (v == 0 || vbest < best_ms) {
      best_ms = vbest;
      best = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  if (best_variant) *best_variant = best;
  return batch_set_variant(b, best);
}

extern "C" int zg_batch_elapsed_ms(const zg_batch* b, float* ms) {
  if (!b || !ms) return zg_set_error(ZG_ERR_INVALID_ARG, "zg_batch_elapsed_ms: null argument"), ZG_ERR_INVALID_ARG;
  *ms = b->last_ms;
  return ZG_OK;
}

extern "C" int zg_batch_copy_bytes(const zg_batch* b, uint64_t* h2d, uint64_t* d2h) {
  if (!b || !h2d || !d2h) return zg_set_error(ZG_ERR_INVALID_ARG, "zg_batch_copy_bytes: null argument"), ZG_ERR_INVALID_ARG;
  *h2d = sizeof(BatchHeader) + sizeof(BatchQuery) * (uint64_t)b->max_queries + sizeof(BatchWork) * (uint64_t)b->max_work;
  *d2h = sizeof(ZgPartial) * 2 * (uint64_t)b->max_queries;
  return ZG_OK;
}
