// zg_exact.cu — exact subgraph counts on the device, bit-exact with naive_implementation/:
//   triangles (TriangleCounting.cpp), wedges (ThreeChain.cpp), 3-edge paths (FourChain.cpp),
//   K1,4 stars (FiveStar.cpp) and 4-cliques (FourClique.cpp).
// One warp per vertex u walks u's neighbour-sorted list; for each neighbour v > u a lane
// intersects the two sorted lists by binary search over the longer one.  Counts are summed in
// 128 bits per block and folded on the host.
#include <vector>

#include "zg_internal.cuh"

namespace {

constexpr int kB = 256;

// first index in adj[lo,hi) with nbr >= key
__device__ __forceinline__ int64_t lb_nbr(const uint2* __restrict__ adj, int64_t lo, int64_t hi, uint32_t key) {
  while (lo < hi) {
    int64_t mid = (lo + hi) >> 1;
    if (__ldg(&adj[mid]).x < key)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

__device__ __forceinline__ bool contains(const uint2* __restrict__ adj, int64_t lo, int64_t hi, uint32_t key) {
  int64_t p = lb_nbr(adj, lo, hi, key);
  return p < hi && __ldg(&adj[p]).x == key;
}

// number of w in N(u) ∩ N(v) with w > lim
__device__ uint64_t common_above(const ZgDevGraph& g, uint32_t u, uint32_t v, uint32_t lim) {
  int64_t bu = g.off[u], eu = g.off[u + 1], bv = g.off[v], ev = g.off[v + 1];
  if (eu - bu > ev - bv) {
    int64_t t = bu; bu = bv; bv = t;
    t = eu; eu = ev; ev = t;
  }
  uint64_t c = 0;
  for (int64_t i = lb_nbr(g.adj_n, bu, eu, lim + 1); i < eu; ++i) {
    uint32_t w = __ldg(&g.adj_n[i]).x;
    if (contains(g.adj_n, bv, ev, w)) ++c;
  }
  return c;
}

// |N(u) ∩ N(v)|
__device__ uint64_t common_all(const ZgDevGraph& g, uint32_t u, uint32_t v) {
  int64_t bu = g.off[u], eu = g.off[u + 1], bv = g.off[v], ev = g.off[v + 1];
  if (eu - bu > ev - bv) {
    int64_t t = bu; bu = bv; bv = t;
    t = eu; eu = ev; ev = t;
  }
  uint64_t c = 0;
  for (int64_t i = bu; i < eu; ++i)
    if (contains(g.adj_n, bv, ev, __ldg(&g.adj_n[i]).x)) ++c;
  return c;
}

struct U128 {
  unsigned long long lo, hi;
};

__device__ __forceinline__ void add128(U128& a, unsigned long long v) {
  unsigned long long o = a.lo;
  a.lo += v;
  a.hi += a.lo < o;
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

// kind-specific per-vertex work, warp per vertex
__global__ void __launch_bounds__(kB) k_exact(ZgDevGraph g, int kind, U128* __restrict__ parts) {
  U128 acc = {0, 0};
  int lane = threadIdx.x & 31;
  uint64_t warp = (blockIdx.x * (uint64_t)kB + threadIdx.x) >> 5;
  uint64_t nwarps = ((uint64_t)gridDim.x * kB) >> 5;
  for (uint64_t u64 = warp; u64 < g.nv; u64 += nwarps) {
    uint32_t u = (uint32_t)u64;
    int64_t b = g.off[u], e = g.off[u + 1];
    uint64_t du = (uint64_t)(e - b);
    if (kind == ZG_EXACT_WEDGE) {
      if (lane == 0) add128(acc, du * (du - 1) / 2);
      continue;
    }
    if (kind == ZG_EXACT_FIVE_STAR) {
      if (lane == 0 && du >= 4) {
        // C(d,4) exactly: d(d-1)(d-2)(d-3)/24 in 128 bits
        unsigned __int128 x = (unsigned __int128)du * (du - 1) * (du - 2) * (du - 3) / 24;
        add128(acc, (unsigned long long)x);
        acc.hi += (unsigned long long)(x >> 64);
      }
      continue;
    }
    for (int64_t i = lb_nbr(g.adj_n, b, e, u + 1) + lane; i < e; i += 32) {
      uint32_t v = __ldg(&g.adj_n[i]).x;  // v > u
      if (kind == ZG_EXACT_TRIANGLE) {
        add128(acc, common_above(g, u, v, v));
      } else if (kind == ZG_EXACT_THREE_PATH) {
        // (d_u - 1)(d_v - 1) - |N(u) ∩ N(v)|, summed over edges: 3-paths + 3T - 3T
        uint64_t dv = (uint64_t)(g.off[v + 1] - g.off[v]);
        unsigned __int128 x = (unsigned __int128)(du - 1) * (dv - 1);
        x -= common_all(g, u, v);
        add128(acc, (unsigned long long)x);
        acc.hi += (unsigned long long)(x >> 64);
      } else {  // ZG_EXACT_FOUR_CLIQUE: w in N(u)∩N(v), w > v; x in N(w), x > w, x in N(u)∩N(v)
        int64_t bv = g.off[v], ev = g.off[v + 1];
        for (int64_t k = lb_nbr(g.adj_n, b, e, v + 1); k < e; ++k) {
          uint32_t w = __ldg(&g.adj_n[k]).x;
          if (!contains(g.adj_n, bv, ev, w)) continue;
          int64_t bw = g.off[w], ew = g.off[w + 1];
          for (int64_t j = lb_nbr(g.adj_n, bw, ew, w + 1); j < ew; ++j) {
            uint32_t x = __ldg(&g.adj_n[j]).x;
            if (contains(g.adj_n, b, e, x) && contains(g.adj_n, bv, ev, x)) add128(acc, 1);
          }
        }
      }
    }
  }
  block_store(acc, parts);
}

}  // namespace

extern "C" int zg_exact_count(const zg_graph* g, int kind, void* cuda_stream, uint64_t out[2]) {
  if (!g || !out) return zg_set_error(ZG_ERR_INVALID_ARG, "null argument"), ZG_ERR_INVALID_ARG;
  if (kind < ZG_EXACT_TRIANGLE || kind > ZG_EXACT_FOUR_CLIQUE)
    return zg_set_error(ZG_ERR_INVALID_ARG, "unknown exact-count kind %d", kind), ZG_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  int grid = zg_num_sms() * 8;
  U128* parts = nullptr;
  ZG_CUDA(cudaMallocAsync((void**)&parts, sizeof(U128) * grid, s));
  k_exact<<<grid, kB, 0, s>>>(g->d, kind, parts);
  std::vector<U128> h(grid);
  cudaError_t ce = cudaMemcpyAsync(h.data(), parts, sizeof(U128) * grid, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(parts, s);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
  if (ce == cudaSuccess) ce = cudaGetLastError();
  if (ce != cudaSuccess) return zg_check_cuda(ce, "zg_exact_count");
  unsigned __int128 t = 0;
  for (int i = 0; i < grid; ++i) t += ((unsigned __int128)h[i].hi << 64) | h[i].lo;
  out[0] = (uint64_t)t;
  out[1] = (uint64_t)(t >> 64);
  return ZG_OK;
}
