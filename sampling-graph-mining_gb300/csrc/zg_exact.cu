// zg_exact.cu — exact subgraph counts on the device, bit-exact with naive_implementation/:
//   triangles (TriangleCounting.cpp), wedges (ThreeChain.cpp), 3-edge paths (FourChain.cpp),
//   K1,4 stars (FiveStar.cpp), 4-cliques (FourClique.cpp), houses (FiveHouse.cpp), 4-edge paths
//   (FiveChain.cpp) and the predicate-weighted triangles (WeightedTriangleCounting.cpp,
//   AtLeastOneWeightedTriangleCounting.cpp).
//
// Degree orientation: every edge points from the endpoint with the smaller (degree, id) to the
// larger, which bounds every out-list by sqrt(2m) and counts each clique once from its lowest
// vertex.  The out-lists come from one radix sort of (src:dst) keys.  Work is edge-parallel, one
// thread per oriented edge; an edge whose shorter out-list is long goes to a queue that a second
// kernel runs with one warp per edge, so the few edges between hubs do not hold a thread each for
// the whole launch:
//   triangles  = sum over oriented (u,v) of |out(u) ∩ out(v)|
//   4-cliques  = sum over oriented (u,v), w in out(u) ∩ out(v), of |out(w) ∩ out(u) ∩ out(v)|
//   3-paths    = sum over edges of (d_u - 1)(d_v - 1) - 3 * triangles
//   wedges     = sum C(d,2),  stars = sum C(d,4)  (exact 128-bit; the naive FiveStar wraps in 64)
// A predicate on the edge data keeps only the passing edges in the orientation (weighted
// triangles: data >= T; at least one >= T: all triangles minus those whose edges are all < T).
// Houses and 4-edge paths come from per-edge triangle counts t(e) and 4-cycle counts c4(e), one
// warp per edge over the full sorted neighbour lists (identities checked against the naive walks
// in oracle/zg_oracle.c):
//   houses       = sum_e t(e) c4(e) - 2 sum_e t(e)^2 + 6 T
//   4-edge paths = (sum_v (S1(v)^2 - S2(v)) + 2 sum_e t(e)(3 - d_a - d_b) - 2 sum_e c4(e)) / 2
// with c4(a,b) = sum over x in N(a) \ {b} of (|N(x) ∩ N(b)| - 1), S1(v) = sum over w in N(v) of
// (d_w - 1), S2(v) the sum of the squares.  Sums are reduced per block in 128 bits (two's
// complement for the signed terms) and folded on the host.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <vector>

#include "zg_internal.cuh"

namespace {

constexpr int kB = 256;

struct U128 {
  unsigned long long lo, hi;
};

__device__ __forceinline__ void add128(U128& a, unsigned long long v) {
  unsigned long long o = a.lo;
  a.lo += v;
  a.hi += a.lo < o;
}

__device__ __forceinline__ void add128w(U128& a, unsigned __int128 v) {
  add128(a, (unsigned long long)v);
  a.hi += (unsigned long long)(v >> 64);
}

__device__ void block_store(U128 a, U128* out) {
  __shared__ unsigned long long slo[kB], shi[kB];
  slo[threadIdx.x] = a.lo;
  shi[threadIdx.x] = a.hi;
  __syncthreads();
  if (threadIdx.x == 0) {
    U128 t = {0, 0};
    for (int i = 0; i < kB; ++i) {
      add128(t, slo[i]);
      t.hi += shi[i];
    }
    out[blockIdx.x] = t;
  }
}

__device__ __forceinline__ uint64_t deg(const ZgDevGraph& g, uint32_t v) { return (uint64_t)(g.off[v + 1] - g.off[v]); }

// (degree, id) order
__device__ __forceinline__ bool lower(const ZgDevGraph& g, uint32_t a, uint32_t b) {
  uint64_t da = deg(g, a), db = deg(g, b);
  return da < db || (da == db && a < b);
}

// Edge predicate of the weighted counts: 0 keeps every edge, 1 keeps data >= t, 2 keeps data < t.
__device__ __forceinline__ bool keep_edge(const ZgDevGraph& g, uint64_t e, int pred, uint32_t t) {
  if (pred == 0) return true;
  const uint32_t w = g.w[e];
  return pred == 1 ? w >= t : w < t;
}

__global__ void k_orient(ZgDevGraph g, int pred, uint32_t t, unsigned long long* __restrict__ keys,
                         unsigned long long* __restrict__ outdeg) {
  for (uint64_t e = blockIdx.x * (uint64_t)kB + threadIdx.x; e < g.m; e += (uint64_t)gridDim.x * kB) {
    if (!keep_edge(g, e, pred, t)) {
      keys[e] = ~0ull;  // sorts after every kept edge
      continue;
    }
    uint4 r = zg_rec_e(g, e);
    uint32_t a = r.x, b = r.y;
    if (!lower(g, a, b)) {
      uint32_t t = a;
      a = b;
      b = t;
    }
    keys[e] = ((unsigned long long)a << 32) | b;
    atomicAdd(&outdeg[a], 1ull);
  }
}

__device__ __forceinline__ bool bsearch(const uint32_t* __restrict__ a, int64_t lo, int64_t hi, uint32_t key) {
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    uint32_t x = __ldg(&a[mid]);
    if (x == key) return true;
    if (x < key)
      lo = mid + 1;
    else
      hi = mid;
  }
  return false;
}

constexpr int64_t kHeavy = 48;  // an edge whose shorter out-list is longer goes to the warp kernel

// |out(w) ∩ out(u) ∩ out(v)| summed over w in out(u) ∩ out(v), or |out(u) ∩ out(v)|, for the
// entries [i0, es) of the shorter list with stride di (1: one thread; 32: the lanes of a warp)
__device__ __forceinline__ unsigned long long dag_edge(const uint32_t* __restrict__ nbr, const int64_t* __restrict__ ooff,
                                                       int kind, int64_t bu, int64_t eu, int64_t bv, int64_t ev,
                                                       int64_t i0, int64_t di) {
  bool swap = (eu - bu) > (ev - bv);
  int64_t es = swap ? ev : eu, bl = swap ? bu : bv, el = swap ? eu : ev;
  unsigned long long c = 0;
  for (int64_t i = i0; i < es; i += di) {
    uint32_t w = __ldg(&nbr[i]);
    if (!bsearch(nbr, bl, el, w)) continue;
    if (kind != ZG_EXACT_FOUR_CLIQUE) {
      ++c;
      continue;
    }
    int64_t bw = ooff[w], ew = ooff[w + 1];
    for (int64_t j = bw; j < ew; ++j) {
      uint32_t x = __ldg(&nbr[j]);
      if (bsearch(nbr, bu, eu, x) && bsearch(nbr, bv, ev, x)) ++c;
    }
  }
  return c;
}

// one thread per oriented edge (u,v): keys sorted, so u = key >> 32; heavy edges are queued
__global__ void __launch_bounds__(kB) k_dag_count(uint64_t m, const unsigned long long* __restrict__ keys,
                                                  const uint32_t* __restrict__ nbr, const int64_t* __restrict__ ooff,
                                                  int kind, U128* __restrict__ parts, uint32_t* __restrict__ heavy,
                                                  unsigned long long* __restrict__ nheavy) {
  U128 acc = {0, 0};
  for (uint64_t e = blockIdx.x * (uint64_t)kB + threadIdx.x; e < m; e += (uint64_t)gridDim.x * kB) {
    unsigned long long k = keys[e];
    uint32_t u = (uint32_t)(k >> 32), v = (uint32_t)k;
    int64_t bu = ooff[u], eu = ooff[u + 1], bv = ooff[v], ev = ooff[v + 1];
    int64_t shorter = (eu - bu) < (ev - bv) ? (eu - bu) : (ev - bv);
    if (shorter > kHeavy) {  // the queue holds every edge (m < 2^32)
      heavy[atomicAdd(nheavy, 1ull)] = (uint32_t)e;
      continue;
    }
    bool swap = (eu - bu) > (ev - bv);
    add128(acc, dag_edge(nbr, ooff, kind, bu, eu, bv, ev, swap ? bv : bu, 1));
  }
  block_store(acc, parts);
}

// one warp per queued edge, the lanes splitting its shorter out-list
__global__ void __launch_bounds__(kB) k_dag_heavy(const uint32_t* __restrict__ heavy, uint64_t nheavy,
                                                  const unsigned long long* __restrict__ keys,
                                                  const uint32_t* __restrict__ nbr, const int64_t* __restrict__ ooff,
                                                  int kind, U128* __restrict__ parts) {
  U128 acc = {0, 0};
  const int lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t)gridDim.x * (kB / 32);
  for (uint64_t h = blockIdx.x * (uint64_t)(kB / 32) + (threadIdx.x >> 5); h < nheavy; h += warps) {
    unsigned long long k = keys[heavy[h]];
    uint32_t u = (uint32_t)(k >> 32), v = (uint32_t)k;
    int64_t bu = ooff[u], eu = ooff[u + 1], bv = ooff[v], ev = ooff[v + 1];
    bool swap = (eu - bu) > (ev - bv);
    add128(acc, dag_edge(nbr, ooff, kind, bu, eu, bv, ev, (swap ? bv : bu) + lane, 32));
  }
  block_store(acc, parts);
}

__global__ void k_low32(const unsigned long long* __restrict__ keys, uint64_t m, uint32_t* __restrict__ out) {
  for (uint64_t e = blockIdx.x * (uint64_t)kB + threadIdx.x; e < m; e += (uint64_t)gridDim.x * kB)
    out[e] = (uint32_t)keys[e];
}

// per-vertex degree terms and per-edge (d_u - 1)(d_v - 1)
__global__ void __launch_bounds__(kB) k_degree_terms(ZgDevGraph g, int kind, U128* __restrict__ parts) {
  U128 acc = {0, 0};
  uint64_t tid = blockIdx.x * (uint64_t)kB + threadIdx.x, stride = (uint64_t)gridDim.x * kB;
  if (kind == ZG_EXACT_THREE_PATH) {
    for (uint64_t e = tid; e < g.m; e += stride) {
      uint4 r = zg_rec_e(g, e);
      add128w(acc, (unsigned __int128)(deg(g, r.x) - 1) * (deg(g, r.y) - 1));
    }
  } else {
    for (uint64_t v = tid; v < g.nv; v += stride) {
      uint64_t d = deg(g, (uint32_t)v);
      if (kind == ZG_EXACT_WEDGE) add128(acc, d * (d - 1) / 2);
      else if (d >= 4) add128w(acc, (unsigned __int128)d * (d - 1) * (d - 2) * (d - 3) / 24);
    }
  }
  block_store(acc, parts);
}

struct Dev {
  void* p = nullptr;
  ~Dev() {
    if (p) cudaFree(p);
  }
};

int fold(U128* parts, int grid, cudaStream_t s, unsigned __int128* out) {
  std::vector<U128> h(grid);
  cudaError_t ce = cudaMemcpyAsync(h.data(), parts, sizeof(U128) * grid, cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return zg_check_cuda(ce, "exact count");
  unsigned __int128 t = 0;
  for (int i = 0; i < grid; ++i) t += ((unsigned __int128)h[i].hi << 64) | h[i].lo;
  *out = t;
  return ZG_OK;
}

int alloc(Dev& d, size_t bytes) {
  cudaError_t e = cudaMalloc(&d.p, bytes ? bytes : 1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    d.p = nullptr;
    return zg_check_cuda(e, "exact count scratch");
  }
  return ZG_OK;
}

// triangles (kind TRIANGLE) or 4-cliques over the degree-oriented DAG of the edges that pass the
// predicate (pred 0: every edge)
int dag_count(const zg_graph* g, int kind, int pred, uint32_t t, cudaStream_t s, unsigned __int128* out) {
  uint64_t m = g->d.m;
  uint32_t nv = g->d.nv;
  if (m == 0) {
    *out = 0;
    return ZG_OK;
  }
  Dev k1, k2, od, ooff, tmp, parts, hv, nh;
  int rc;
  int grid = zg_num_sms() * 8;
  if ((rc = alloc(k1, 8 * m)) || (rc = alloc(k2, 8 * m)) || (rc = alloc(od, 8 * ((size_t)nv + 1))) ||
      (rc = alloc(ooff, 8 * ((size_t)nv + 1))) || (rc = alloc(parts, sizeof(U128) * 2 * grid)) ||
      (rc = alloc(hv, 4 * m)) || (rc = alloc(nh, 8)))
    return rc;
  cudaMemsetAsync(od.p, 0, 8 * ((size_t)nv + 1), s);
  cudaMemsetAsync(nh.p, 0, 8, s);
  k_orient<<<grid, kB, 0, s>>>(g->d, pred, t, (unsigned long long*)k1.p, (unsigned long long*)od.p);
  size_t tb = 0;
  int bits = 32;
  while (bits < 64 && ((uint64_t)(nv ? nv - 1 : 0) >> (bits - 32))) ++bits;
  if (pred) bits = 64;  // the dropped edges' key ~0 must sort last
  cub::DeviceRadixSort::SortKeys(nullptr, tb, (unsigned long long*)k1.p, (unsigned long long*)k2.p, (int64_t)m, 0,
                                 bits, s);
  if ((rc = alloc(tmp, tb))) return rc;
  cub::DeviceRadixSort::SortKeys(tmp.p, tb, (unsigned long long*)k1.p, (unsigned long long*)k2.p, (int64_t)m, 0,
                                 bits, s);
  size_t tb2 = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, tb2, (unsigned long long*)od.p, (unsigned long long*)ooff.p,
                                (int64_t)nv + 1, s);
  if (tb2 > tb) {
    cudaFree(tmp.p);
    tmp.p = nullptr;
    if ((rc = alloc(tmp, tb2))) return rc;
  }
  cub::DeviceScan::ExclusiveSum(tmp.p, tb2, (unsigned long long*)od.p, (unsigned long long*)ooff.p,
                                (int64_t)nv + 1, s);
  // the kept edges: the total out-degree
  unsigned long long mk = m;
  cudaError_t ce = cudaMemcpyAsync(&mk, (unsigned long long*)ooff.p + nv, 8, cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return zg_check_cuda(ce, "exact count (kept edges)");
  // neighbour column of the sorted keys, reusing k1 as the uint32 array
  uint32_t* nbr = (uint32_t*)k1.p;
  k_low32<<<grid, kB, 0, s>>>((const unsigned long long*)k2.p, mk, nbr);
  k_dag_count<<<grid, kB, 0, s>>>(mk, (const unsigned long long*)k2.p, nbr, (const int64_t*)ooff.p, kind,
                                  (U128*)parts.p, (uint32_t*)hv.p, (unsigned long long*)nh.p);
  unsigned long long nheavy = 0;
  ce = cudaMemcpyAsync(&nheavy, nh.p, 8, cudaMemcpyDeviceToHost, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) return zg_check_cuda(ce, "exact count kernel");
  k_dag_heavy<<<grid, kB, 0, s>>>((const uint32_t*)hv.p, nheavy, (const unsigned long long*)k2.p, nbr,
                                  (const int64_t*)ooff.p, kind, (U128*)parts.p + grid);
  ce = cudaGetLastError();
  if (ce != cudaSuccess) return zg_check_cuda(ce, "exact count kernel");
  return fold((U128*)parts.p, 2 * grid, s, out);
}

// ---- houses and 4-edge paths -------------------------------------------------------------------
// Sorted full neighbour lists aligned with g->off: from the neighbour-ordered adjacency when the
// graph has one, else by a radix sort of both directions' (src:dst) keys.
__global__ void k_both_keys(ZgDevGraph g, unsigned long long* __restrict__ keys) {
  for (uint64_t e = blockIdx.x * (uint64_t)kB + threadIdx.x; e < g.m; e += (uint64_t)gridDim.x * kB) {
    uint4 r = zg_rec_e(g, e);
    keys[2 * e] = ((unsigned long long)r.x << 32) | r.y;
    keys[2 * e + 1] = ((unsigned long long)r.y << 32) | r.x;
  }
}
__global__ void k_adj_nbr(const uint2* __restrict__ adj, uint64_t n, uint32_t* __restrict__ out) {
  for (uint64_t i = blockIdx.x * (uint64_t)kB + threadIdx.x; i < n; i += (uint64_t)gridDim.x * kB) out[i] = adj[i].x;
}

// |N(x) ∩ N(y)|: iterate the shorter list, binary-search the longer
__device__ __forceinline__ unsigned long long common(const uint32_t* __restrict__ nbr, const int64_t* __restrict__ off,
                                                     uint32_t x, uint32_t y) {
  int64_t bx = off[x], ex = off[x + 1], by = off[y], ey = off[y + 1];
  if (ex - bx > ey - by) {
    int64_t t0 = bx, t1 = ex;
    bx = by;
    ex = ey;
    by = t0;
    ey = t1;
  }
  unsigned long long c = 0;
  for (int64_t i = bx; i < ex; ++i) c += bsearch(nbr, by, ey, __ldg(&nbr[i]));
  return c;
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// one warp per edge (a, b), a the endpoint of smaller degree: t(e) and c4(e), then the edge's term
__global__ void __launch_bounds__(kB) k_house_chain(ZgDevGraph g, const uint32_t* __restrict__ nbr,
                                                    const int64_t* __restrict__ off, int kind, U128* __restrict__ parts) {
  U128 acc = {0, 0};
  const int lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t)gridDim.x * (kB / 32);
  for (uint64_t e = blockIdx.x * (uint64_t)(kB / 32) + (threadIdx.x >> 5); e < g.m; e += warps) {
    uint4 r = zg_rec_e(g, e);
    uint32_t a = r.x, b = r.y;
    int64_t da = off[a + 1] - off[a], db = off[b + 1] - off[b];
    if (da > db) {
      uint32_t t = a;
      a = b;
      b = t;
      int64_t x = da;
      da = db;
      db = x;
    }
    unsigned long long tl = 0;
    for (int64_t i = off[a] + lane; i < off[a + 1]; i += 32) tl += bsearch(nbr, off[b], off[b + 1], __ldg(&nbr[i]));
    const unsigned long long te = warp_sum(tl);
    if (kind == ZG_EXACT_FIVE_HOUSE && te == 0) continue;
    unsigned long long cl = 0;
    for (int64_t i = off[a] + lane; i < off[a + 1]; i += 32) {
      const uint32_t x = __ldg(&nbr[i]);
      if (x != b) cl += common(nbr, off, x, b) - 1;  // a is in both lists
    }
    const unsigned long long c4 = warp_sum(cl);
    if (lane == 0) {
      __int128 v;
      if (kind == ZG_EXACT_FIVE_HOUSE)
        v = (__int128)te * c4 - 2 * (__int128)te * te + 2 * (__int128)te;  // 6 T = 2 sum_e t(e)
      else
        v = 2 * (__int128)te * (3 - (__int128)da - (__int128)db) - 2 * (__int128)c4;
      add128w(acc, (unsigned __int128)v);
    }
  }
  block_store(acc, parts);
}

// one warp per vertex: S1(v)^2 - S2(v)
__global__ void __launch_bounds__(kB) k_chain_vertex(uint32_t nv, const uint32_t* __restrict__ nbr,
                                                     const int64_t* __restrict__ off, U128* __restrict__ parts) {
  U128 acc = {0, 0};
  const int lane = threadIdx.x & 31;
  const uint64_t warps = (uint64_t)gridDim.x * (kB / 32);
  for (uint64_t v = blockIdx.x * (uint64_t)(kB / 32) + (threadIdx.x >> 5); v < nv; v += warps) {
    unsigned long long s1 = 0;
    unsigned __int128 s2 = 0;
    for (int64_t i = off[v] + lane; i < off[v + 1]; i += 32) {
      const uint32_t w = __ldg(&nbr[i]);
      const unsigned long long dw = (unsigned long long)(off[w + 1] - off[w]) - 1;
      s1 += dw;
      s2 += (unsigned __int128)dw * dw;
    }
    s1 = warp_sum(s1);
    // exact 128-bit warp sum of s2: 64-bit halves, each low-half addition's carry into the high half
    unsigned long long slo = (unsigned long long)s2, shi = (unsigned long long)(s2 >> 64);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long olo = __shfl_xor_sync(0xffffffffu, slo, o), ohi = __shfl_xor_sync(0xffffffffu, shi, o);
      const unsigned long long n = slo + olo;
      shi += ohi + (n < slo);
      slo = n;
    }
    if (lane == 0) {
      const unsigned __int128 S2 = ((unsigned __int128)shi << 64) | slo;
      add128w(acc, (unsigned __int128)s1 * s1 - S2);
    }
  }
  block_store(acc, parts);
}

int house_chain(const zg_graph* g, int kind, cudaStream_t s, unsigned __int128* out) {
  const uint64_t m = g->d.m;
  const uint32_t nv = g->d.nv;
  if (m == 0) {
    *out = 0;
    return ZG_OK;
  }
  Dev nb, parts, k1, k2, tmp;
  int rc;
  const int grid = zg_num_sms() * 8;
  if ((rc = alloc(nb, 4 * 2 * m)) || (rc = alloc(parts, sizeof(U128) * 2 * grid))) return rc;
  if (g->adj_n) {
    k_adj_nbr<<<grid, kB, 0, s>>>(g->adj_n, 2 * m, (uint32_t*)nb.p);
  } else {
    if ((rc = alloc(k1, 8 * 2 * m)) || (rc = alloc(k2, 8 * 2 * m))) return rc;
    k_both_keys<<<grid, kB, 0, s>>>(g->d, (unsigned long long*)k1.p);
    size_t tb = 0;
    cub::DeviceRadixSort::SortKeys(nullptr, tb, (unsigned long long*)k1.p, (unsigned long long*)k2.p, (int64_t)(2 * m),
                                   0, 64, s);
    if ((rc = alloc(tmp, tb))) return rc;
    cub::DeviceRadixSort::SortKeys(tmp.p, tb, (unsigned long long*)k1.p, (unsigned long long*)k2.p, (int64_t)(2 * m),
                                   0, 64, s);
    k_low32<<<grid, kB, 0, s>>>((const unsigned long long*)k2.p, 2 * m, (uint32_t*)nb.p);
  }
  cudaMemsetAsync(parts.p, 0, sizeof(U128) * 2 * grid, s);
  k_house_chain<<<grid, kB, 0, s>>>(g->d, (const uint32_t*)nb.p, g->off, kind, (U128*)parts.p);
  if (kind == ZG_EXACT_FIVE_CHAIN)
    k_chain_vertex<<<grid, kB, 0, s>>>(nv, (const uint32_t*)nb.p, g->off, (U128*)parts.p + grid);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return zg_check_cuda(ce, "exact count kernel");
  unsigned __int128 r = 0;
  if ((rc = fold((U128*)parts.p, 2 * grid, s, &r))) return rc;
  *out = kind == ZG_EXACT_FIVE_CHAIN ? (unsigned __int128)((__int128)r / 2) : r;
  return ZG_OK;
}

int degree_terms(const zg_graph* g, int kind, cudaStream_t s, unsigned __int128* out) {
  int grid = zg_num_sms() * 8;
  Dev parts;
  int rc = alloc(parts, sizeof(U128) * grid);
  if (rc) return rc;
  k_degree_terms<<<grid, kB, 0, s>>>(g->d, kind, (U128*)parts.p);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return zg_check_cuda(ce, "exact count kernel");
  return fold((U128*)parts.p, grid, s, out);
}

}  // namespace

extern "C" int zg_exact_count(const zg_graph* g, int kind, void* cuda_stream, uint64_t out[2]) {
  if (!g || !out) return zg_set_error(ZG_ERR_INVALID_ARG, "null argument"), ZG_ERR_INVALID_ARG;
  if (kind < ZG_EXACT_TRIANGLE || kind > ZG_EXACT_FIVE_CHAIN)
    return zg_set_error(ZG_ERR_INVALID_ARG, "unknown exact-count kind %d (the weighted triangles take "
                        "zg_exact_count_weighted)", kind), ZG_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  unsigned __int128 r = 0, t = 0;
  int rc = ZG_OK;
  switch (kind) {
    case ZG_EXACT_TRIANGLE:
    case ZG_EXACT_FOUR_CLIQUE: rc = dag_count(g, kind, 0, 0, s, &r); break;
    case ZG_EXACT_WEDGE:
    case ZG_EXACT_FIVE_STAR: rc = degree_terms(g, kind, s, &r); break;
    case ZG_EXACT_THREE_PATH:
      rc = degree_terms(g, kind, s, &r);
      if (rc == ZG_OK) rc = dag_count(g, ZG_EXACT_TRIANGLE, 0, 0, s, &t);
      r -= 3 * t;
      break;
    case ZG_EXACT_FIVE_HOUSE:
    case ZG_EXACT_FIVE_CHAIN: rc = house_chain(g, kind, s, &r); break;
  }
  if (rc) return rc;
  out[0] = (uint64_t)r;
  out[1] = (uint64_t)(r >> 64);
  return ZG_OK;
}

extern "C" int zg_exact_count_weighted(const zg_graph* g, int kind, uint32_t threshold, void* cuda_stream,
                                       uint64_t out[2]) {
  if (!g || !out) return zg_set_error(ZG_ERR_INVALID_ARG, "null argument"), ZG_ERR_INVALID_ARG;
  if (kind != ZG_EXACT_WEIGHTED_TRIANGLE && kind != ZG_EXACT_AT_LEAST_ONE_TRIANGLE)
    return zg_set_error(ZG_ERR_INVALID_ARG, "unknown weighted exact-count kind %d", kind), ZG_ERR_INVALID_ARG;
  if (!g->w) return zg_set_error(ZG_ERR_INVALID_ARG, "the graph has no edge data"), ZG_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  unsigned __int128 r = 0, below = 0;
  int rc;
  if (kind == ZG_EXACT_WEIGHTED_TRIANGLE) {
    rc = dag_count(g, ZG_EXACT_TRIANGLE, 1, threshold, s, &r);
  } else {
    rc = dag_count(g, ZG_EXACT_TRIANGLE, 0, 0, s, &r);
    if (rc == ZG_OK) rc = dag_count(g, ZG_EXACT_TRIANGLE, 2, threshold, s, &below);
    r -= below;
  }
  if (rc) return rc;
  out[0] = (uint64_t)r;
  out[1] = (uint64_t)(r >> 64);
  return ZG_OK;
}
