// zg_graph.cu — device graph store: the GB300 counterpart of Graph<E> + CSRConstructor
// (include/Graph.hpp:148-210, src/Graph.cpp:215-377), GraphFilter (src/GraphFilters.cpp:17-177)
// and GraphSampler (src/Graph.cpp:629-780).
//
// Build = validate + degree count + one exclusive scan + two stable radix sorts (CUB):
//   1. half-edges (v, nbr, eid) in edge-id order, sorted stably by v -> adj_e: each list is
//      in edge-id order exactly as the reference's outgoing_adj_list;
//   2. adj_e's (v:nbr) keys sorted stably -> adj_n (ties keep edge-id order);
//   3. per edge and endpoint, the suffix count (entries after it in that endpoint's list).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_reduce.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <vector>

#include "zg_internal.cuh"

namespace {

template <typename T>
int dev_alloc(T** p, size_t count) {
  size_t bytes = sizeof(T) * (count ? count : 1);
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    zg_set_error(ZG_ERR_OOM, "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
    return ZG_ERR_OOM;
  }
  return ZG_OK;
}

// RAII holder for temporaries.
struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  int alloc(size_t bytes) {
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 1);
    if (e != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      zg_set_error(ZG_ERR_OOM, "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
      return ZG_ERR_OOM;
    }
    return ZG_OK;
  }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
  }
  template <typename T>
  T* as() {
    return (T*)p;
  }
};

int grid_for(uint64_t n, int block) {
  uint64_t g = (n + block - 1) / block;
  uint64_t cap = (uint64_t)zg_num_sms() * 32;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

int bits_for(uint64_t maxval) {
  int b = 1;
  while (b < 64 && (maxval >> b)) ++b;
  return b;
}

// Validate the COO (src/Graph.cpp:454 asserts src != dst), count degrees, emit half-edges.
__global__ void k_validate_count(const uint2* __restrict__ coo, uint64_t m, uint32_t nv,
                                 unsigned long long* __restrict__ deg, uint32_t* __restrict__ keys,
                                 unsigned long long* __restrict__ vals, void* __restrict__ rec, uint32_t wide,
                                 unsigned int* __restrict__ bad) {
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
       e += (uint64_t)gridDim.x * blockDim.x) {
    uint2 c = coo[e];
    if (c.x >= nv || c.y >= nv || c.x == c.y) {
      atomicOr(bad, 1u);
      continue;
    }
    atomicAdd(&deg[c.x], 1ull);
    atomicAdd(&deg[c.y], 1ull);
    keys[2 * e] = c.x;
    keys[2 * e + 1] = c.y;
    vals[2 * e] = (unsigned long long)c.y | ((unsigned long long)e << 32);
    vals[2 * e + 1] = (unsigned long long)c.x | ((unsigned long long)e << 32);
    if (wide) {
      ((ZgRec*)rec)[e].e = make_uint4(c.x, c.y, 0u, 0u);
      ((ZgRec*)rec)[e].p = make_uint4(0u, 0u, 0u, 0u);
    } else {
      ((uint4*)rec)[e] = make_uint4(c.x, c.y, 0u, 0u);
    }
  }
}

// Per edge and endpoint: entries after it in the endpoint's list (wide records: also its own slot
// and the entries before it); (v:nbr) keys for the neighbour sort.
__global__ void k_suffix(const uint32_t* __restrict__ vkeys, const uint2* __restrict__ adj_e,
                         uint64_t n2, const int64_t* __restrict__ off, void* __restrict__ rec, uint32_t wide,
                         unsigned long long* __restrict__ nkeys, uint32_t* __restrict__ nvals) {
  for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < n2;
       g += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t v = vkeys[g];
    uint2 a = adj_e[g];
    uint32_t suf = (uint32_t)(off[v + 1] - 1 - (int64_t)g);
    if (wide) {
      uint32_t pre = (uint32_t)((int64_t)g - off[v]);
      ZgRec* r = &((ZgRec*)rec)[a.y];
      if (r->e.x == v) {
        r->e.z = suf;
        r->p.x = (uint32_t)g;
        r->p.z = pre;
      } else {
        r->e.w = suf;
        r->p.y = (uint32_t)g;
        r->p.w = pre;
      }
    } else {
      uint4* r = &((uint4*)rec)[a.y];
      if (r->x == v)
        r->z = suf;
      else
        r->w = suf;
    }
    if (nkeys) {
      nkeys[g] = ((unsigned long long)v << 32) | a.x;
      nvals[g] = a.y;
    }
  }
}

__global__ void k_adj_n(const unsigned long long* __restrict__ nkeys, const uint32_t* __restrict__ nvals,
                        uint64_t n2, uint2* __restrict__ adj_n, unsigned int* __restrict__ dup) {
  for (uint64_t g = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; g < n2;
       g += (uint64_t)gridDim.x * blockDim.x) {
    unsigned long long k = nkeys[g];
    adj_n[g] = make_uint2((uint32_t)k, nvals[g]);
    if (g > 0 && nkeys[g - 1] == k) atomicOr(dup, 1u);
  }
}

__global__ void k_off32(const int64_t* __restrict__ off, uint64_t n, uint32_t* __restrict__ off32) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    off32[i] = (uint32_t)off[i];
}

// Wide records (as built) into 16-byte ones: packed bit fields (the slots included) or compact
// (src, dst, suf_src, suf_dst).
__global__ void k_narrow(const ZgRec* __restrict__ wide, uint64_t m, uint4* __restrict__ out, uint32_t packed,
                         uint32_t vb, uint32_t sb, uint32_t pb) {
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
    const ZgRec r = wide[e];
    if (packed) {
      const uint64_t w0 = (uint64_t)r.e.x | ((uint64_t)r.e.y << vb) | ((uint64_t)r.e.z << (2 * vb));
      const uint64_t w1 = (uint64_t)r.e.w | ((uint64_t)r.p.x << sb) | ((uint64_t)r.p.y << (sb + pb));
      out[e] = make_uint4((uint32_t)w0, (uint32_t)(w0 >> 32), (uint32_t)w1, (uint32_t)(w1 >> 32));
    } else {
      out[e] = r.e;
    }
  }
}

// Bucketed two-choice cuckoo insertion of every edge's entry (fingerprint << 32 | edge id).  A
// thread claims an empty slot of either bucket with atomicCAS; when both are full it swaps its
// entry into slot 1..3 of one (atomicExch) and carries the evicted entry to that entry's other
// bucket (its key is rebuilt from rec).  Whenever an entry goes to its second bucket, its first
// bucket (full then, so slot 0 holds an entry) gets the overflow flag in slot 0, which is only
// ever written by that first claim and by these flags.  After kMaxKicks swaps it gives up and
// raises *fail: the host rebuilds with new hash seeds.  Every loop here is bounded.
constexpr int kMaxKicks = 128;

__device__ __forceinline__ bool cuckoo_try(unsigned long long* ent, uint32_t b, unsigned long long x) {
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    unsigned long long* slot = &ent[4 * (uint64_t)b + j];
    if (*(volatile unsigned long long*)slot != ZG_HASH_EMPTY) continue;
    if (atomicCAS(slot, ZG_HASH_EMPTY, x) == ZG_HASH_EMPTY) return true;
  }
  return false;
}

__global__ void k_cuckoo_insert(const ZgDevGraph d, uint64_t m, unsigned long long* ent, uint32_t bits,
                                uint64_t seed, unsigned int* __restrict__ fail) {
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
    uint4 r = zg_rec_e(d, e);
    unsigned long long k = zg_edge_key(r.x, r.y);
    unsigned long long x = ((unsigned long long)zg_fingerprint(k, seed) << 32) | e;
    uint32_t from = 0xFFFFFFFFu;  // the bucket the carried entry was evicted from
    bool placed = false;
    for (int kick = 0; kick < kMaxKicks; ++kick) {
      const uint32_t b1 = zg_bucket1(k, seed, bits), b2 = zg_bucket2(k, seed, bits);
      if (cuckoo_try(ent, b1, x)) {
        placed = true;
        break;
      }
      if (b2 != b1 && cuckoo_try(ent, b2, x)) {
        atomicOr(&ent[4 * (uint64_t)b1], ZG_HASH_OVERFLOW);
        placed = true;
        break;
      }
      const uint32_t vb = from == b1 ? b2 : from == b2 ? b1 : (((e + kick) & 1) ? b2 : b1);
      if (vb != b1) atomicOr(&ent[4 * (uint64_t)b1], ZG_HASH_OVERFLOW);
      const unsigned long long old = atomicExch(&ent[4 * (uint64_t)vb + 1 + (e + (uint64_t)kick) % 3], x);
      if (old == ZG_HASH_EMPTY) {
        placed = true;
        break;
      }
      x = old;
      uint4 ro = zg_rec_e(d, (uint32_t)old);
      k = zg_edge_key(ro.x, ro.y);
      from = vb;
    }
    if (!placed) atomicOr(fail, 1u);
  }
}

// Every edge must be found in one of its two buckets (an insertion that gave up lost one), and
// one found only in its second bucket needs the overflow flag on its first.
__global__ void k_cuckoo_check(const ZgDevGraph d, uint64_t m, const unsigned long long* __restrict__ ent,
                               uint32_t bits, uint64_t seed, unsigned int* __restrict__ fail) {
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
    uint4 r = zg_rec_e(d, e);
    unsigned long long k = zg_edge_key(r.x, r.y);
    unsigned long long x = ((unsigned long long)zg_fingerprint(k, seed) << 32) | e;
    const uint32_t b1 = zg_bucket1(k, seed, bits), b2 = zg_bucket2(k, seed, bits);
    bool in1 = false, in2 = false;
    for (int j = 0; j < 4; ++j) {
      in1 |= (ent[4 * (uint64_t)b1 + j] & ~ZG_HASH_OVERFLOW) == x;
      in2 |= (ent[4 * (uint64_t)b2 + j] & ~ZG_HASH_OVERFLOW) == x;
    }
    const unsigned long long s0 = ent[4 * (uint64_t)b1];
    const bool flagged = s0 != ZG_HASH_EMPTY && (s0 & ZG_HASH_OVERFLOW);
    if (!(in1 || (in2 && flagged))) atomicOr(fail, 1u);
  }
}

// The cuckoo table of the graph's edges: buckets for a load of at most 0.8 (0.5, see below), up to
// 8 seeds, and the table doubled after every 4 failed seeds.
int build_hash(zg_graph* g, cudaStream_t s) {
  const uint64_t m = g->d.m;
  uint32_t bits = 1;
  // Load up to 0.8, or up to 0.5 for a graph far larger than L2 (wide records) whose table then
  // stays within 4 GiB: such a graph is read from HBM either way, and with more first buckets
  // holding an empty slot more absent edges are settled by one sector (edge_candidate).  Larger
  // tables keep the 0.8 load: doubling one of tens of GB cost more in address translation than
  // it saved (R-MAT scale 26: 709 -> 794 ms per batch; the 43 M-edge Chung-Lu batch: 74 -> 70 ms).
  while ((4ull << bits) * 4 < m * 5) ++bits;  // 4 * 2^bits slots >= m / 0.8
  uint32_t roomy = 1;
  while ((4ull << roomy) < m * 2) ++roomy;  // 4 * 2^roomy slots >= m / 0.5
  if (g->wide && (8ull * (4ull << roomy)) <= (4ull << 30)) bits = roomy;
  DevBuf fail;
  int rc;
  if ((rc = fail.alloc(sizeof(unsigned int)))) return rc;
  const int B = 256;
  for (int attempt = 0; attempt < 8; ++attempt) {
    if (attempt && attempt % 4 == 0) ++bits;
    const uint64_t slots = 4ull << bits;
    if (g->hent) cudaFree(g->hent);
    g->hent = nullptr;
    if ((rc = dev_alloc(&g->hent, slots))) return rc;
    uint64_t seed = zg_mix64(0x5A4748415348ull + attempt);
    cudaError_t ce;
    if ((ce = cudaMemsetAsync(g->hent, 0xFF, sizeof(unsigned long long) * slots, s)) ||
        (ce = cudaMemsetAsync(fail.p, 0, sizeof(unsigned int), s)))
      return zg_check_cuda(ce, "hash memset");
    if (m) {
      k_cuckoo_insert<<<grid_for(m, B), B, 0, s>>>(g->d, m, g->hent, bits, seed, fail.as<unsigned int>());
      k_cuckoo_check<<<grid_for(m, B), B, 0, s>>>(g->d, m, g->hent, bits, seed, fail.as<unsigned int>());
    }
    unsigned int hf = 0;
    if ((ce = cudaMemcpyAsync(&hf, fail.p, sizeof(hf), cudaMemcpyDeviceToHost, s)) || (ce = cudaStreamSynchronize(s)))
      return zg_check_cuda(ce, "hash build");
    if (!hf) {
      g->d.hent = g->hent;
      g->d.hbits = bits;
      g->d.hseed = seed;
      g->bytes += slots * sizeof(unsigned long long);
      return ZG_OK;
    }
  }
  zg_set_error(ZG_ERR_CUDA, "cuckoo table of %llu edges did not build", (unsigned long long)m);
  return ZG_ERR_CUDA;
}

// Record layout of the graphs built from now on (zg_set_record_layout).
int g_record_layout = ZG_RECORDS_AUTO;

// Wide records when the compact layout's sampling working set (records 16 B, edge-id adjacency
// 16 B, cuckoo table about 10 B per edge, offsets) is more than twice the L2: such a graph is
// served from HBM either way, and the wide record saves a dependent read and two sectors per step.
// Near the L2 size the compact layout keeps more of the graph resident.
bool wide_records(uint64_t m, uint32_t nv) {
  if (g_record_layout == ZG_RECORDS_WIDE) return true;
  if (g_record_layout == ZG_RECORDS_COMPACT || g_record_layout == ZG_RECORDS_PACKED) return false;
  int dev = 0, l2 = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const uint64_t hot = 42ull * m + 4ull * ((uint64_t)nv + 1);
  return hot > 2ull * (uint64_t)l2;
}

// Builds a graph from a device COO (consumed: freed by the caller afterwards).
// sampling_only: skip the neighbour-ordered adjacency (exports only) and its duplicate check; for
// graphs derived from an already validated graph (filters, subsamples) that only sampling reads.
int build_graph(const uint2* d_coo, const uint32_t* d_w_in, uint64_t m, uint32_t nv,
                cudaStream_t s, zg_graph** out, bool sampling_only = false) {
  // edge ids and adjacency positions (< 2m) are 32-bit
  if (m > 0x7FFFFFFFull)
    return zg_set_error(ZG_ERR_TOO_LARGE, "at most 2^31-1 edges (32-bit positions): m=%llu", (unsigned long long)m),
           ZG_ERR_TOO_LARGE;
  if (nv == 0 && m > 0) return zg_set_error(ZG_ERR_INVALID_GRAPH, "edges on a graph with 0 vertices"), ZG_ERR_INVALID_GRAPH;
  zg_graph* g = new zg_graph();
  memset(g, 0, sizeof(*g));
  int rc;
  auto fail = [&](int code) {
    zg_graph_free(g);
    return code;
  };
  uint64_t n2 = 2 * m;
  // packed records are made from wide ones once the degrees are known (else compact ones)
  const bool try_packed =
      !wide_records(m, nv) && m && (g_record_layout == ZG_RECORDS_AUTO || g_record_layout == ZG_RECORDS_PACKED);
  g->wide = try_packed || wide_records(m, nv);
  const size_t rec_bytes = (g->wide ? sizeof(ZgRec) : sizeof(uint4)) * m;
  // adj_e, 8 entries of slack (lb_eid_win's windows may read up to 7 entries past the last one),
  // and off32 share one allocation
  const size_t adj_bytes = sizeof(uint2) * (n2 + 8);
  g->hot_bytes = adj_bytes + sizeof(uint32_t) * ((size_t)nv + 1);
  if ((rc = dev_alloc((char**)&g->hot, g->hot_bytes)) || (rc = dev_alloc((char**)&g->rec, rec_bytes)) ||
      (rc = dev_alloc(&g->off, (size_t)nv + 1)) || (!sampling_only && (rc = dev_alloc(&g->adj_n, n2))))
    return fail(rc);
  g->adj_e = (uint2*)g->hot;
  g->off32 = (uint32_t*)((char*)g->hot + adj_bytes);
  if (d_w_in) {
    if ((rc = dev_alloc(&g->w, m))) return fail(rc);
    if (m) {
      cudaError_t e = cudaMemcpyAsync(g->w, d_w_in, sizeof(uint32_t) * m, cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return fail(zg_check_cuda(e, "copy weights"));
    }
  }
  g->bytes = rec_bytes + (sizeof(int64_t) + sizeof(uint32_t)) * ((size_t)nv + 1) +
             (sampling_only ? 1 : 2) * sizeof(uint2) * n2 + (d_w_in ? sizeof(uint32_t) * m : 0);
  DevBuf deg, keys, keys2, vals, vals2, flags, tmp, nk, nk2, nv1, nv2;
  if ((rc = deg.alloc(sizeof(unsigned long long) * ((size_t)nv + 1))) ||
      (rc = keys.alloc(sizeof(uint32_t) * n2)) || (rc = keys2.alloc(sizeof(uint32_t) * n2)) ||
      (rc = vals.alloc(sizeof(unsigned long long) * n2)) || (rc = flags.alloc(sizeof(unsigned int) * 2)))
    return fail(rc);
  cudaError_t ce;
  if ((ce = cudaMemsetAsync(deg.p, 0, sizeof(unsigned long long) * ((size_t)nv + 1), s)) ||
      (ce = cudaMemsetAsync(flags.p, 0, sizeof(unsigned int) * 2, s)))
    return fail(zg_check_cuda(ce, "memset"));
  const int B = 256;
  if (m) {
    k_validate_count<<<grid_for(m, B), B, 0, s>>>(d_coo, m, nv, deg.as<unsigned long long>(),
                                                   keys.as<uint32_t>(), vals.as<unsigned long long>(),
                                                   g->rec, g->wide, flags.as<unsigned int>());
  }
  // offsets = exclusive scan of degrees (deg[nv] = 0 gives off[nv] = 2m)
  size_t tb = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tb, deg.as<unsigned long long>(),
                                (unsigned long long*)g->off, (int64_t)nv + 1, s);
  if ((rc = tmp.alloc(tb))) return fail(rc);
  cub::DeviceScan::ExclusiveSum(tmp.p, tb, deg.as<unsigned long long>(), (unsigned long long*)g->off,
                                (int64_t)nv + 1, s);
  unsigned int hflags[2] = {0, 0};
  if ((ce = cudaMemcpyAsync(hflags, flags.p, sizeof(hflags), cudaMemcpyDeviceToHost, s)) ||
      (ce = cudaStreamSynchronize(s)))
    return fail(zg_check_cuda(ce, "graph validation"));
  if (hflags[0]) {
    zg_set_error(ZG_ERR_INVALID_GRAPH, "edge list holds a self-loop or a vertex id >= %u", nv);
    return fail(ZG_ERR_INVALID_GRAPH);
  }
  if (m) {
    // 1. stable sort of half-edges by vertex -> edge-id-ordered adjacency
    int vb = bits_for(nv > 0 ? nv - 1 : 0);
    tmp.reset();
    tb = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tb, keys.as<uint32_t>(), keys2.as<uint32_t>(),
                                    vals.as<unsigned long long>(), (unsigned long long*)g->adj_e,
                                    (int64_t)n2, 0, vb, s);
    if ((rc = tmp.alloc(tb))) return fail(rc);
    cub::DeviceRadixSort::SortPairs(tmp.p, tb, keys.as<uint32_t>(), keys2.as<uint32_t>(),
                                    vals.as<unsigned long long>(), (unsigned long long*)g->adj_e,
                                    (int64_t)n2, 0, vb, s);
    vals.reset();
    keys.reset();
    // 2. suffix counts and (v:nbr) keys
    if (!sampling_only &&
        ((rc = nk.alloc(sizeof(unsigned long long) * n2)) || (rc = nk2.alloc(sizeof(unsigned long long) * n2)) ||
         (rc = nv1.alloc(sizeof(uint32_t) * n2)) || (rc = nv2.alloc(sizeof(uint32_t) * n2))))
      return fail(rc);
    k_suffix<<<grid_for(n2, B), B, 0, s>>>(keys2.as<uint32_t>(), g->adj_e, n2, g->off, g->rec, g->wide,
                                           nk.as<unsigned long long>(), nv1.as<uint32_t>());
    keys2.reset();
    if (!sampling_only) {
      // 3. neighbour order within each vertex (stable: duplicates keep edge-id order)
      tmp.reset();
      tb = 0;
      cub::DeviceRadixSort::SortPairs(nullptr, tb, nk.as<unsigned long long>(), nk2.as<unsigned long long>(),
                                      nv1.as<uint32_t>(), nv2.as<uint32_t>(), (int64_t)n2, 0, 32 + vb, s);
      if ((rc = tmp.alloc(tb))) return fail(rc);
      cub::DeviceRadixSort::SortPairs(tmp.p, tb, nk.as<unsigned long long>(), nk2.as<unsigned long long>(),
                                      nv1.as<uint32_t>(), nv2.as<uint32_t>(), (int64_t)n2, 0, 32 + vb, s);
      k_adj_n<<<grid_for(n2, B), B, 0, s>>>(nk2.as<unsigned long long>(), nv2.as<uint32_t>(), n2, g->adj_n,
                                            flags.as<unsigned int>() + 1);
    }
    // max degree (src/Graph.cpp:467-474)
    tmp.reset();
    DevBuf dmax;
    if ((rc = dmax.alloc(sizeof(unsigned long long)))) return fail(rc);
    tb = 0;
    cub::DeviceReduce::Max(nullptr, tb, deg.as<unsigned long long>(), dmax.as<unsigned long long>(),
                           (int64_t)nv, s);
    if ((rc = tmp.alloc(tb))) return fail(rc);
    cub::DeviceReduce::Max(tmp.p, tb, deg.as<unsigned long long>(), dmax.as<unsigned long long>(),
                           (int64_t)nv, s);
    unsigned long long hmax = 0;
    if ((ce = cudaMemcpyAsync(&hmax, dmax.p, sizeof(hmax), cudaMemcpyDeviceToHost, s)) ||
        (ce = cudaMemcpyAsync(hflags, flags.p, sizeof(hflags), cudaMemcpyDeviceToHost, s)) ||
        (ce = cudaStreamSynchronize(s)))
      return fail(zg_check_cuda(ce, "graph build"));
    if (hflags[1]) {
      zg_set_error(ZG_ERR_INVALID_GRAPH, "edge list holds a duplicate edge");
      return fail(ZG_ERR_INVALID_GRAPH);
    }
    g->max_degree = hmax;
  }
  if (try_packed) {
    const uint32_t vb = (uint32_t)bits_for(nv - 1), sb = (uint32_t)bits_for(g->max_degree);
    const uint32_t pb = (uint32_t)bits_for(n2 - 1);
    const bool fits = 2 * vb + sb <= 64 && sb + 2 * pb <= 64;
    uint4* r16 = nullptr;
    if ((rc = dev_alloc(&r16, m))) return fail(rc);
    k_narrow<<<grid_for(m, B), B, 0, s>>>((const ZgRec*)g->rec, m, r16, fits, vb, sb, pb);
    if ((ce = cudaStreamSynchronize(s)) != cudaSuccess) {
      cudaFree(r16);
      return fail(zg_check_cuda(ce, "record narrowing"));
    }
    cudaFree(g->rec);
    g->rec = r16;
    g->wide = 0;
    g->packed = fits;
    g->bytes -= (sizeof(ZgRec) - sizeof(uint4)) * m;
    g->d.pk_v = vb;
    g->d.pk_s = sb;
    g->d.pk_p = pb;
  }
  k_off32<<<grid_for((uint64_t)nv + 1, B), B, 0, s>>>(g->off, (uint64_t)nv + 1, g->off32);
  g->d.m = m;
  g->d.rec = g->rec;
  g->d.wide = g->wide;
  g->d.packed = g->packed;
  g->d.off32 = g->off32;
  if ((rc = build_hash(g, s))) return fail(rc);
  ce = cudaGetLastError();
  if (ce != cudaSuccess) return fail(zg_check_cuda(ce, "graph build kernels"));
  g->d.nv = nv;
  g->d.off32 = g->off32;
  g->d.rec = g->rec;
  g->d.off = g->off;
  g->d.adj_e = g->adj_e;
  g->d.adj_n = g->adj_n;
  g->d.w = g->w;
  g->num_edges = m;
  *out = g;
  return ZG_OK;
}

__global__ void k_perm_keys(uint64_t m, uint64_t seed, unsigned long long* keys, unsigned long long* idx) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x) {
    keys[i] = zg_draw(seed, ZG_STREAM_SHUFFLE, i, 0, 0, ~0ull);
    idx[i] = i;
  }
}

// out[i] = in[perm[i]]; optional weight gather and parent-index composition.
__global__ void k_gather(uint64_t m, const unsigned long long* __restrict__ perm, const uint2* __restrict__ coo_in,
                         const uint32_t* __restrict__ w_in, const unsigned long long* __restrict__ parent_in,
                         uint2* __restrict__ coo_out, uint32_t* __restrict__ w_out,
                         unsigned long long* __restrict__ parent_out) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m;
       i += (uint64_t)gridDim.x * blockDim.x) {
    unsigned long long j = perm[i];
    coo_out[i] = coo_in[j];
    if (w_in) w_out[i] = w_in[j];
    parent_out[i] = parent_in ? parent_in[j] : j;
  }
}

// Permutes (coo, w, parent) in place through temporaries: sort (Philox key, index) pairs.
int permute(uint2** coo, uint32_t** w, unsigned long long** parent, uint64_t m, uint64_t seed,
            cudaStream_t s) {
  if (m == 0) return ZG_OK;
  DevBuf k1, k2, i1, i2, tmp;
  int rc;
  if ((rc = k1.alloc(8 * m)) || (rc = k2.alloc(8 * m)) || (rc = i1.alloc(8 * m)) || (rc = i2.alloc(8 * m)))
    return rc;
  const int B = 256;
  k_perm_keys<<<grid_for(m, B), B, 0, s>>>(m, seed, k1.as<unsigned long long>(), i1.as<unsigned long long>());
  size_t tb = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tb, k1.as<unsigned long long>(), k2.as<unsigned long long>(),
                                  i1.as<unsigned long long>(), i2.as<unsigned long long>(), (int64_t)m, 0, 64, s);
  if ((rc = tmp.alloc(tb))) return rc;
  cub::DeviceRadixSort::SortPairs(tmp.p, tb, k1.as<unsigned long long>(), k2.as<unsigned long long>(),
                                  i1.as<unsigned long long>(), i2.as<unsigned long long>(), (int64_t)m, 0, 64, s);
  uint2* coo2 = nullptr;
  uint32_t* w2 = nullptr;
  unsigned long long* p2 = nullptr;
  if ((rc = dev_alloc(&coo2, m))) return rc;
  if (*w && (rc = dev_alloc(&w2, m))) {
    cudaFree(coo2);
    return rc;
  }
  if ((rc = dev_alloc(&p2, m))) {
    cudaFree(coo2);
    if (w2) cudaFree(w2);
    return rc;
  }
  k_gather<<<grid_for(m, B), B, 0, s>>>(m, i2.as<unsigned long long>(), *coo, *w, *parent, coo2, w2, p2);
  cudaError_t ce = cudaStreamSynchronize(s);
  cudaFree(*coo);
  if (*w) cudaFree(*w);
  if (*parent) cudaFree(*parent);
  *coo = coo2;
  *w = w2;
  *parent = p2;
  if (ce != cudaSuccess) return zg_check_cuda(ce, "permute");
  return ZG_OK;
}

// Predicate flags for GraphFilter / keep draws for GraphSampler.
__global__ void k_select(uint64_t m, const uint32_t* __restrict__ w, int op, int64_t t0, int64_t t1,
                         double rate, uint64_t keep_seed, int mode, unsigned long long* __restrict__ flag) {
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
       e += (uint64_t)gridDim.x * blockDim.x) {
    bool keep;
    if (mode == 0) {
      int64_t x = (int64_t)w[e];
      switch (op) {
        case ZG_PRED_GE: keep = x >= t0; break;
        case ZG_PRED_LT: keep = x < t0; break;
        case ZG_PRED_GT: keep = x > t0; break;
        case ZG_PRED_LE: keep = x <= t0; break;
        case ZG_PRED_EQ: keep = x == t0; break;
        case ZG_PRED_NE: keep = x != t0; break;
        default: keep = x >= t0 && x < t1; break;
      }
    } else {
      // src/Graph.cpp:652-664: rand_int(1, 2^30) <= (unsigned long long)(rate * 2^30)
      const unsigned long long max_rand_int = 1ull << 30;
      unsigned long long threshold = (unsigned long long)(rate * (double)max_rand_int);
      keep = zg_draw(keep_seed, ZG_STREAM_SUBSAMPLE, e, 0, 1, max_rand_int) <= threshold;
    }
    flag[e] = keep ? 1ull : 0ull;
  }
}

__global__ void k_compact(uint64_t m, const unsigned long long* __restrict__ flag,
                          const unsigned long long* __restrict__ pos, const ZgDevGraph src,
                          const uint32_t* __restrict__ w, uint2* __restrict__ coo_out,
                          uint32_t* __restrict__ w_out, unsigned long long* __restrict__ parent) {
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
       e += (uint64_t)gridDim.x * blockDim.x) {
    if (!flag[e]) continue;
    unsigned long long p = pos[e];
    uint4 r = zg_rec_e(src, e);
    coo_out[p] = make_uint2(r.x, r.y);
    if (w) w_out[p] = w[e];
    parent[p] = e;
  }
}

// GraphFilter::generate_graph / GraphSampler::sample_graph on the device.
int derive(bool sampling_only, const zg_graph* g, int mode, int op, int64_t t0, int64_t t1, double rate,
           uint64_t keep_seed,
           uint64_t shuffle_seed, cudaStream_t s, uint64_t* parent_index, uint64_t* out_m, zg_graph** out) {
  if (!g || !out) return zg_set_error(ZG_ERR_INVALID_ARG, "null argument"), ZG_ERR_INVALID_ARG;
  if (mode == 0 && !g->w) return zg_set_error(ZG_ERR_INVALID_ARG, "graph has no edge weights"), ZG_ERR_INVALID_ARG;
  if (mode == 0 && (op < ZG_PRED_GE || op > ZG_PRED_RANGE))
    return zg_set_error(ZG_ERR_INVALID_ARG, "unknown predicate op %d", op), ZG_ERR_INVALID_ARG;
  uint64_t m = g->d.m;
  DevBuf flag, pos, tmp;
  int rc;
  if ((rc = flag.alloc(8 * (m + 1))) || (rc = pos.alloc(8 * (m + 1)))) return rc;
  const int B = 256;
  cudaError_t ce;
  if ((ce = cudaMemsetAsync(flag.p, 0, 8 * (m + 1), s))) return zg_check_cuda(ce, "memset");
  if (m)
    k_select<<<grid_for(m, B), B, 0, s>>>(m, g->w, op, t0, t1, rate, keep_seed, mode,
                                          flag.as<unsigned long long>());
  size_t tb = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tb, flag.as<unsigned long long>(), pos.as<unsigned long long>(),
                                (int64_t)m + 1, s);
  if ((rc = tmp.alloc(tb))) return rc;
  cub::DeviceScan::ExclusiveSum(tmp.p, tb, flag.as<unsigned long long>(), pos.as<unsigned long long>(),
                                (int64_t)m + 1, s);
  unsigned long long kept = 0;
  if ((ce = cudaMemcpyAsync(&kept, pos.as<unsigned long long>() + m, 8, cudaMemcpyDeviceToHost, s)) ||
      (ce = cudaStreamSynchronize(s)))
    return zg_check_cuda(ce, "filter count");
  uint2* coo = nullptr;
  uint32_t* w = nullptr;
  unsigned long long* parent = nullptr;
  if ((rc = dev_alloc(&coo, kept)) || (g->w && (rc = dev_alloc(&w, kept))) || (rc = dev_alloc(&parent, kept))) {
    if (coo) cudaFree(coo);
    if (w) cudaFree(w);
    return rc;
  }
  if (m)
    k_compact<<<grid_for(m, B), B, 0, s>>>(m, flag.as<unsigned long long>(), pos.as<unsigned long long>(),
                                           g->d, g->w, coo, w, parent);
  if (shuffle_seed != ZG_NO_SHUFFLE) rc = permute(&coo, &w, &parent, kept, shuffle_seed, s);
  if (rc == ZG_OK) rc = build_graph(coo, w, kept, g->d.nv, s, out, sampling_only);
  if (rc == ZG_OK) {
    // src/GraphFilters.cpp:90-135 (identical in src/Graph.cpp:704-749)
    double sample_rate_after_partition =
        g->num_edges ? (double)g->d.m / (double)g->num_edges : 1.0;
    (*out)->num_edges = (uint64_t)(1. * (double)kept / sample_rate_after_partition);
    (*out)->max_degree = (uint64_t)((double)(*out)->max_degree / sample_rate_after_partition);
    if (parent_index && kept)
      ce = cudaMemcpy(parent_index, parent, 8 * kept, cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) rc = zg_check_cuda(ce, "parent index");
  }
  if (out_m) *out_m = kept;
  cudaFree(coo);
  if (w) cudaFree(w);
  cudaFree(parent);
  return rc;
}

int upload_coo(const uint32_t* edges, const uint32_t* weights, uint64_t m, cudaStream_t s, uint2** coo,
               uint32_t** w) {
  int rc;
  *coo = nullptr;
  *w = nullptr;
  if ((rc = dev_alloc(coo, m))) return rc;
  if (weights && (rc = dev_alloc(w, m))) {
    cudaFree(*coo);
    return rc;
  }
  cudaError_t ce = cudaSuccess;
  if (m) ce = cudaMemcpyAsync(*coo, edges, sizeof(uint2) * m, cudaMemcpyHostToDevice, s);
  if (ce == cudaSuccess && weights && m)
    ce = cudaMemcpyAsync(*w, weights, sizeof(uint32_t) * m, cudaMemcpyHostToDevice, s);
  if (ce != cudaSuccess) {
    cudaFree(*coo);
    if (*w) cudaFree(*w);
    return zg_check_cuda(ce, "upload edges");
  }
  return ZG_OK;
}

}  // namespace

// zg_graph_filter / zg_graph_subsample without the neighbour-ordered adjacency: derived graphs that
// only the sampling kernels read (the batch cache, the error profile's subsample).
int zg_graph_filter_sampling(const zg_graph* g, int pred_op, int64_t t0, int64_t t1, uint64_t shuffle_seed,
                             cudaStream_t s, uint64_t* out_m, zg_graph** out) {
  return derive(true, g, 0, pred_op, t0, t1, 0.0, 0, shuffle_seed, s, nullptr, out_m, out);
}
int zg_graph_subsample_sampling(const zg_graph* g, double rate, uint64_t keep_seed, uint64_t shuffle_seed,
                                cudaStream_t s, uint64_t* out_m, zg_graph** out) {
  return derive(true, g, 1, 0, 0, 0, rate, keep_seed, shuffle_seed, s, nullptr, out_m, out);
}

// A graph from a device COO in edge-id order (the device generators' entry into the build).
int zg_build_graph_device(const uint2* d_coo, const uint32_t* d_w, uint64_t m, uint32_t nv, cudaStream_t s,
                          zg_graph** out, bool sampling_only) {
  return build_graph(d_coo, d_w, m, nv, s, out, sampling_only);
}

extern "C" int zg_graph_create(const uint32_t* edges, uint64_t m, uint32_t num_vertices,
                               const uint32_t* weights, void* cuda_stream, zg_graph** out) {
  if (!out || (m && !edges)) return zg_set_error(ZG_ERR_INVALID_ARG, "null argument"), ZG_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  uint2* coo;
  uint32_t* w;
  int rc = upload_coo(edges, weights, m, s, &coo, &w);
  if (rc) return rc;
  rc = build_graph(coo, w, m, num_vertices, s, out);
  cudaStreamSynchronize(s);
  cudaFree(coo);
  if (w) cudaFree(w);
  return rc;
}

extern "C" int zg_graph_permuted(const uint32_t* edges, uint64_t m, uint32_t num_vertices,
                                 const uint32_t* weights, uint64_t shuffle_seed, void* cuda_stream,
                                 uint64_t* parent_index, zg_graph** out) {
  if (!out || (m && !edges)) return zg_set_error(ZG_ERR_INVALID_ARG, "null argument"), ZG_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  uint2* coo;
  uint32_t* w;
  unsigned long long* parent = nullptr;
  int rc = upload_coo(edges, weights, m, s, &coo, &w);
  if (rc) return rc;
  rc = permute(&coo, &w, &parent, m, shuffle_seed, s);
  if (rc == ZG_OK) rc = build_graph(coo, w, m, num_vertices, s, out);
  if (rc == ZG_OK && parent_index && m) {
    cudaError_t ce = cudaMemcpy(parent_index, parent, 8 * m, cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) rc = zg_check_cuda(ce, "parent index");
  }
  cudaStreamSynchronize(s);
  cudaFree(coo);
  if (w) cudaFree(w);
  if (parent) cudaFree(parent);
  return rc;
}

extern "C" int zg_set_record_layout(int layout) {
  if (layout < ZG_RECORDS_AUTO || layout > ZG_RECORDS_PACKED)
    return zg_set_error(ZG_ERR_INVALID_ARG, "unknown record layout %d", layout), ZG_ERR_INVALID_ARG;
  g_record_layout = layout;
  return ZG_OK;
}

extern "C" int zg_graph_free(zg_graph* g) {
  if (!g) return ZG_OK;
  if (g->rec) cudaFree(g->rec);
  if (g->off) cudaFree(g->off);
  if (g->hent) cudaFree(g->hent);
  if (g->hot) cudaFree(g->hot);  // adj_e and off32
  if (g->adj_n) cudaFree(g->adj_n);
  if (g->w) cudaFree(g->w);
  delete g;
  return ZG_OK;
}

extern "C" int zg_graph_get_meta(const zg_graph* g, zg_graph_meta* out) {
  if (!g || !out) return zg_set_error(ZG_ERR_INVALID_ARG, "null argument"), ZG_ERR_INVALID_ARG;
  out->num_vertices = g->d.nv;
  out->weighted = g->w != nullptr;
  out->num_local_edges = g->d.m;
  out->num_edges = g->num_edges;
  out->max_degree = g->max_degree;
  out->device_bytes = g->bytes;
  out->record_bytes = g->wide ? (uint32_t)sizeof(ZgRec) : (uint32_t)sizeof(uint4);
  out->record_layout = g->wide ? ZG_RECORDS_WIDE : g->packed ? ZG_RECORDS_PACKED : ZG_RECORDS_COMPACT;
  return ZG_OK;
}

extern "C" int zg_graph_set_meta(zg_graph* g, uint64_t num_edges, uint64_t max_degree) {
  if (!g) return zg_set_error(ZG_ERR_INVALID_ARG, "null graph"), ZG_ERR_INVALID_ARG;
  g->num_edges = num_edges;
  g->max_degree = max_degree;
  return ZG_OK;
}

namespace {
// Edge e0 + i's (src, dst) and suffix sizes out of its record, in any layout.
__global__ void k_export_rec(ZgDevGraph g, uint64_t e0, uint64_t cnt, uint32_t* __restrict__ edges,
                             uint32_t* __restrict__ suffix) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < cnt; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint4 q = zg_rec_e(g, e0 + i);
    if (edges) reinterpret_cast<uint2*>(edges)[i] = make_uint2(q.x, q.y);
    if (suffix) reinterpret_cast<uint2*>(suffix)[i] = make_uint2(q.z, q.w);
  }
}
}  // namespace

extern "C" int zg_graph_download(const zg_graph* g, uint32_t* edges, uint32_t* weights, int64_t* offsets,
                                 uint32_t* adj_e, uint32_t* adj_n, uint32_t* suffix) {
  if (!g) return zg_set_error(ZG_ERR_INVALID_ARG, "null graph"), ZG_ERR_INVALID_ARG;
  uint64_t m = g->d.m;
  cudaError_t ce = cudaSuccess;
  if ((edges || suffix) && m) {
    // unpacked on the device in chunks of at most 2^27 edges (1 GiB per array), then copied out
    const uint64_t chunk = m < (1ull << 27) ? m : (1ull << 27);
    uint32_t *d_e = nullptr, *d_s = nullptr;
    if (edges) ce = cudaMalloc((void**)&d_e, 8 * chunk);
    if (ce == cudaSuccess && suffix) ce = cudaMalloc((void**)&d_s, 8 * chunk);
    for (uint64_t e0 = 0; ce == cudaSuccess && e0 < m; e0 += chunk) {
      const uint64_t cnt = m - e0 < chunk ? m - e0 : chunk;
      const int grid = (int)std::min<uint64_t>((cnt + 255) / 256, (uint64_t)zg_num_sms() * 16);
      k_export_rec<<<grid, 256>>>(g->d, e0, cnt, d_e, d_s);
      ce = cudaGetLastError();
      if (ce == cudaSuccess && edges) ce = cudaMemcpy(edges + 2 * e0, d_e, 8 * cnt, cudaMemcpyDeviceToHost);
      if (ce == cudaSuccess && suffix) ce = cudaMemcpy(suffix + 2 * e0, d_s, 8 * cnt, cudaMemcpyDeviceToHost);
    }
    if (d_e) cudaFree(d_e);
    if (d_s) cudaFree(d_s);
    if (ce != cudaSuccess) return zg_check_cuda(ce, "download records");
  }
  if (weights && g->w && m) ce = cudaMemcpy(weights, g->w, 4 * m, cudaMemcpyDeviceToHost);
  if (ce == cudaSuccess && offsets)
    ce = cudaMemcpy(offsets, g->off, 8 * ((size_t)g->d.nv + 1), cudaMemcpyDeviceToHost);
  if (ce == cudaSuccess && adj_e && m) ce = cudaMemcpy(adj_e, g->adj_e, 16 * m, cudaMemcpyDeviceToHost);
  if (adj_n && m && !g->adj_n)
    return zg_set_error(ZG_ERR_INVALID_ARG, "this derived graph has no neighbour-ordered adjacency"),
           ZG_ERR_INVALID_ARG;
  if (ce == cudaSuccess && adj_n && m) ce = cudaMemcpy(adj_n, g->adj_n, 16 * m, cudaMemcpyDeviceToHost);
  if (ce != cudaSuccess) return zg_check_cuda(ce, "download");
  return ZG_OK;
}

extern "C" int zg_graph_filter(const zg_graph* g, int pred_op, int64_t t0, int64_t t1, uint64_t shuffle_seed,
                               void* cuda_stream, uint64_t* parent_index, uint64_t* out_m, zg_graph** out) {
  return derive(false, g, 0, pred_op, t0, t1, 0.0, 0, shuffle_seed, (cudaStream_t)cuda_stream, parent_index, out_m,
                out);
}

extern "C" int zg_graph_subsample(const zg_graph* g, double rate, uint64_t keep_seed, uint64_t shuffle_seed,
                                  void* cuda_stream, uint64_t* parent_index, uint64_t* out_m, zg_graph** out) {
  if (!(rate >= 0.0 && rate <= 1.0))
    return zg_set_error(ZG_ERR_INVALID_ARG, "sample rate %g outside [0,1]", rate), ZG_ERR_INVALID_ARG;
  return derive(false, g, 1, 0, 0, 0, rate, keep_seed, shuffle_seed, (cudaStream_t)cuda_stream, parent_index, out_m,
                out);
}
