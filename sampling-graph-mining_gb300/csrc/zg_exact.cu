// zg_exact.cu — exact subgraph counts on the device, bit-exact with naive_implementation/:
//   triangles (TriangleCounting.cpp), wedges (ThreeChain.cpp), 3-edge paths (FourChain.cpp),
//   K1,4 stars (FiveStar.cpp) and 4-cliques (FourClique.cpp).
//
// Degree orientation: every edge points from the endpoint with the smaller (degree, id) to the
// larger, which bounds every out-list by sqrt(2m) and counts each clique once from its lowest
// vertex.  The out-lists come from one radix sort of (src:dst) keys.  Work is edge-parallel:
//   triangles  = sum over oriented (u,v) of |out(u) ∩ out(v)|
//   4-cliques  = sum over oriented (u,v), w in out(u) ∩ out(v), of |out(w) ∩ out(u) ∩ out(v)|
//   3-paths    = sum over edges of (d_u - 1)(d_v - 1) - 3 * triangles
//   wedges     = sum C(d,2),  stars = sum C(d,4)  (exact 128-bit; the naive FiveStar wraps in 64)
// Sums are reduced per block in 128 bits and folded on the host.
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

__global__ void k_orient(ZgDevGraph g, unsigned long long* __restrict__ keys, unsigned long long* __restrict__ outdeg) {
  for (uint64_t e = blockIdx.x * (uint64_t)kB + threadIdx.x; e < g.m; e += (uint64_t)gridDim.x * kB) {
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

// one thread per oriented edge (u,v): keys sorted, so u = key >> 32
__global__ void __launch_bounds__(kB) k_dag_count(ZgDevGraph g, const unsigned long long* __restrict__ keys,
                                                  const uint32_t* __restrict__ nbr, const int64_t* __restrict__ ooff,
                                                  int kind, U128* __restrict__ parts) {
  U128 acc = {0, 0};
  for (uint64_t e = blockIdx.x * (uint64_t)kB + threadIdx.x; e < g.m; e += (uint64_t)gridDim.x * kB) {
    unsigned long long k = keys[e];
    uint32_t u = (uint32_t)(k >> 32), v = (uint32_t)k;
    int64_t bu = ooff[u], eu = ooff[u + 1], bv = ooff[v], ev = ooff[v + 1];
    // iterate the shorter list, search the longer
    bool swap = (eu - bu) > (ev - bv);
    int64_t bs = swap ? bv : bu, es = swap ? ev : eu, bl = swap ? bu : bv, el = swap ? eu : ev;
    if (kind == ZG_EXACT_FOUR_CLIQUE) {
      for (int64_t i = bs; i < es; ++i) {
        uint32_t w = __ldg(&nbr[i]);
        if (!bsearch(nbr, bl, el, w)) continue;
        int64_t bw = ooff[w], ew = ooff[w + 1];
        for (int64_t j = bw; j < ew; ++j) {
          uint32_t x = __ldg(&nbr[j]);
          if (bsearch(nbr, bu, eu, x) && bsearch(nbr, bv, ev, x)) add128(acc, 1);
        }
      }
    } else {
      uint64_t c = 0;
      for (int64_t i = bs; i < es; ++i)
        if (bsearch(nbr, bl, el, __ldg(&nbr[i]))) ++c;
      add128(acc, c);
    }
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

// triangles (kind TRIANGLE) or 4-cliques over the degree-oriented DAG
int dag_count(const zg_graph* g, int kind, cudaStream_t s, unsigned __int128* out) {
  uint64_t m = g->d.m;
  uint32_t nv = g->d.nv;
  if (m == 0) {
    *out = 0;
    return ZG_OK;
  }
  Dev k1, k2, od, ooff, tmp, parts;
  int rc;
  int grid = zg_num_sms() * 8;
  if ((rc = alloc(k1, 8 * m)) || (rc = alloc(k2, 8 * m)) || (rc = alloc(od, 8 * ((size_t)nv + 1))) ||
      (rc = alloc(ooff, 8 * ((size_t)nv + 1))) || (rc = alloc(parts, sizeof(U128) * grid)))
    return rc;
  cudaMemsetAsync(od.p, 0, 8 * ((size_t)nv + 1), s);
  k_orient<<<grid, kB, 0, s>>>(g->d, (unsigned long long*)k1.p, (unsigned long long*)od.p);
  size_t tb = 0;
  int bits = 32;
  while (bits < 64 && ((uint64_t)(nv ? nv - 1 : 0) >> (bits - 32))) ++bits;
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
  // neighbour column of the sorted keys, reusing k1 as the uint32 array
  uint32_t* nbr = (uint32_t*)k1.p;
  k_low32<<<grid, kB, 0, s>>>((const unsigned long long*)k2.p, m, nbr);
  k_dag_count<<<grid, kB, 0, s>>>(g->d, (const unsigned long long*)k2.p, nbr, (const int64_t*)ooff.p, kind,
                                  (U128*)parts.p);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return zg_check_cuda(ce, "exact count kernel");
  return fold((U128*)parts.p, grid, s, out);
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
  if (kind < ZG_EXACT_TRIANGLE || kind > ZG_EXACT_FOUR_CLIQUE)
    return zg_set_error(ZG_ERR_INVALID_ARG, "unknown exact-count kind %d", kind), ZG_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  unsigned __int128 r = 0, t = 0;
  int rc = ZG_OK;
  switch (kind) {
    case ZG_EXACT_TRIANGLE:
    case ZG_EXACT_FOUR_CLIQUE: rc = dag_count(g, kind, s, &r); break;
    case ZG_EXACT_WEDGE:
    case ZG_EXACT_FIVE_STAR: rc = degree_terms(g, kind, s, &r); break;
    case ZG_EXACT_THREE_PATH:
      rc = degree_terms(g, kind, s, &r);
      if (rc == ZG_OK) rc = dag_count(g, ZG_EXACT_TRIANGLE, s, &t);
      r -= 3 * t;
      break;
  }
  if (rc) return rc;
  out[0] = (uint64_t)r;
  out[1] = (uint64_t)(r >> 64);
  return ZG_OK;
}
