// zg_gen_device.cu — the seeded generators of zg_gen.cpp run on the device and feed the graph
// build directly: the same Philox draws, the same dedup and the same seeded edge order and
// orientation, so zg_graph_gen_rmat(...) equals zg_graph_create(zg_gen_rmat(...)) edge for edge,
// without the host round trip (R-MAT scale 26 / edge factor 24 has 1.6 G raw edges).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>

#include <vector>

#include "zg_internal.cuh"

int zg_build_graph_device(const uint2* d_coo, const uint32_t* d_w, uint64_t m, uint32_t nv, cudaStream_t s,
                          zg_graph** out, bool sampling_only);

namespace {

// the generators' Philox streams (zg_gen.cpp)
constexpr uint32_t kStreamRmat = 0xFFFFFF00u;
constexpr uint32_t kStreamOrder = 0xFFFFFF01u;
constexpr uint32_t kStreamCL = 0xFFFFFF02u;
constexpr uint32_t kStreamW = 0xFFFFFF03u;
constexpr unsigned long long kSelfLoop = ~0ull;

// Philox4x32-10, all four output words (counter: ctr lo/hi, d, stream; key: seed).
__device__ __forceinline__ uint4 philox4(uint64_t seed, uint32_t stream, uint64_t ctr, uint32_t d) {
  uint32_t c0 = (uint32_t)ctr, c1 = (uint32_t)(ctr >> 32), c2 = d, c3 = stream;
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  return make_uint4(c0, c1, c2, c3);
}

__device__ __forceinline__ unsigned long long canon(uint32_t u, uint32_t v) {
  return u == v ? kSelfLoop : (u < v ? ((unsigned long long)u << 32 | v) : ((unsigned long long)v << 32 | u));
}

__global__ void k_rmat_keys(uint64_t n, uint32_t scale, uint64_t ta, uint64_t tb, uint64_t tc, uint64_t seed,
                            unsigned long long* __restrict__ keys) {
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t u = 0, v = 0;
    uint4 o = make_uint4(0, 0, 0, 0);
    for (uint32_t lvl = 0; lvl < scale; ++lvl) {
      if ((lvl & 3) == 0) o = philox4(seed, kStreamRmat, k, lvl >> 2);
      uint32_t w = (lvl & 3) == 0 ? o.x : (lvl & 3) == 1 ? o.y : (lvl & 3) == 2 ? o.z : o.w;
      uint64_t r = w;
      uint32_t bu = r >= tb, bv = (r >= ta && r < tb) || r >= tc;
      u = (u << 1) | bu;
      v = (v << 1) | bv;
    }
    keys[k] = canon(u, v);
  }
}

__global__ void k_cl_keys(uint64_t draws, const double* __restrict__ cdf, uint32_t n, double total, uint64_t seed,
                          unsigned long long* __restrict__ keys) {
  for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < draws;
       k += (uint64_t)gridDim.x * blockDim.x) {
    uint4 o = philox4(seed, kStreamCL, k, 0);
    double r0 = (double)(((uint64_t)o.y << 21) ^ o.x) * 0x1p-53 * total;
    double r1 = (double)(((uint64_t)o.w << 21) ^ o.z) * 0x1p-53 * total;
    uint32_t uv[2];
    double rr[2] = {r0, r1};
    for (int j = 0; j < 2; ++j) {  // upper_bound: first index with cdf > r
      uint32_t lo = 0, hi = n;
      while (lo < hi) {
        uint32_t mid = lo + ((hi - lo) >> 1);
        if (cdf[mid] > rr[j])
          hi = mid;
        else
          lo = mid + 1;
      }
      uv[j] = lo >= n ? n - 1 : lo;
    }
    keys[k] = canon(uv[0], uv[1]);
  }
}

__global__ void k_order_keys(uint64_t m, uint64_t seed, unsigned long long* __restrict__ okey,
                             unsigned long long* __restrict__ idx) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
    uint4 o = philox4(seed, kStreamOrder, i, 0);
    okey[i] = ((unsigned long long)o.y << 32) | o.x;
    idx[i] = i;
  }
}

__global__ void k_emit(uint64_t m, uint64_t seed, const unsigned long long* __restrict__ keys,
                       const unsigned long long* __restrict__ idx, uint2* __restrict__ coo) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
    unsigned long long j = idx[i];
    unsigned long long k = keys[j];
    uint32_t u = (uint32_t)(k >> 32), v = (uint32_t)k;
    uint4 o = philox4(seed, kStreamOrder, j, 1);
    coo[i] = (o.x & 1) ? make_uint2(v, u) : make_uint2(u, v);
  }
}

__global__ void k_weights(uint64_t m, uint32_t max_value, uint64_t seed, uint32_t* __restrict__ w) {
  for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m; e += (uint64_t)gridDim.x * blockDim.x) {
    uint4 o = philox4(seed, kStreamW, e, 0);
    w[e] = (uint32_t)(((uint64_t)o.x * max_value) >> 32);
  }
}

int grid_n(uint64_t n) {
  uint64_t g = (n + 255) / 256, cap = (uint64_t)zg_num_sms() * 32;
  return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

struct Buf {
  void* p = nullptr;
  ~Buf() { release(); }
  int alloc(size_t bytes) {
    if (cudaMalloc(&p, bytes ? bytes : 1) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      zg_set_error(ZG_ERR_OOM, "cudaMalloc(%zu bytes) failed", bytes);
      return ZG_ERR_OOM;
    }
    return ZG_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
  }
  template <typename T>
  T* as() {
    return (T*)p;
  }
};

// keys (raw, n of them; consumed) -> sorted unique canonical edges -> seeded order and orientation
// -> device graph (with seeded weights when max_weight > 0).
int finish_device(Buf& keys, uint64_t n, uint32_t nv, uint64_t seed, uint32_t max_weight, uint64_t weight_seed,
                  uint32_t flags, cudaStream_t s, zg_graph** out) {
  int rc;
  cudaError_t ce;
  Buf k2, tmp, cnt;
  if ((rc = k2.alloc(8 * n)) || (rc = cnt.alloc(8))) return rc;
  size_t tb = 0;
  cub::DeviceRadixSort::SortKeys(nullptr, tb, keys.as<unsigned long long>(), k2.as<unsigned long long>(), (int64_t)n,
                                 0, 64, s);
  if ((rc = tmp.alloc(tb))) return rc;
  cub::DeviceRadixSort::SortKeys(tmp.p, tb, keys.as<unsigned long long>(), k2.as<unsigned long long>(), (int64_t)n, 0,
                                 64, s);
  tmp.release();
  tb = 0;
  cub::DeviceSelect::Unique(nullptr, tb, k2.as<unsigned long long>(), keys.as<unsigned long long>(),
                            cnt.as<unsigned long long>(), (int64_t)n, s);
  if ((rc = tmp.alloc(tb))) return rc;
  cub::DeviceSelect::Unique(tmp.p, tb, k2.as<unsigned long long>(), keys.as<unsigned long long>(),
                            cnt.as<unsigned long long>(), (int64_t)n, s);
  tmp.release();
  k2.release();
  unsigned long long m = 0, last = 0;
  if ((ce = cudaMemcpyAsync(&m, cnt.p, 8, cudaMemcpyDeviceToHost, s)) || (ce = cudaStreamSynchronize(s)))
    return zg_check_cuda(ce, "generator dedup");
  if (m) {
    if ((ce = cudaMemcpy(&last, keys.as<unsigned long long>() + m - 1, 8, cudaMemcpyDeviceToHost)))
      return zg_check_cuda(ce, "generator dedup");
    if (last == kSelfLoop) --m;  // the self-loop marker sorts last
  }
  Buf okey, okey2, idx, idx2;
  if ((rc = okey.alloc(8 * m)) || (rc = okey2.alloc(8 * m)) || (rc = idx.alloc(8 * m)) || (rc = idx2.alloc(8 * m)))
    return rc;
  if (m) k_order_keys<<<grid_n(m), 256, 0, s>>>(m, seed, okey.as<unsigned long long>(), idx.as<unsigned long long>());
  tb = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tb, okey.as<unsigned long long>(), okey2.as<unsigned long long>(),
                                  idx.as<unsigned long long>(), idx2.as<unsigned long long>(), (int64_t)m, 0, 64, s);
  if ((rc = tmp.alloc(tb))) return rc;
  cub::DeviceRadixSort::SortPairs(tmp.p, tb, okey.as<unsigned long long>(), okey2.as<unsigned long long>(),
                                  idx.as<unsigned long long>(), idx2.as<unsigned long long>(), (int64_t)m, 0, 64, s);
  tmp.release();
  okey.release();
  okey2.release();
  idx.release();
  Buf coo, w;
  if ((rc = coo.alloc(8 * m))) return rc;
  if (m) k_emit<<<grid_n(m), 256, 0, s>>>(m, seed, keys.as<unsigned long long>(), idx2.as<unsigned long long>(),
                                          coo.as<uint2>());
  idx2.release();
  keys.release();
  if (max_weight) {
    if ((rc = w.alloc(4 * m))) return rc;
    if (m) k_weights<<<grid_n(m), 256, 0, s>>>(m, max_weight, weight_seed, w.as<uint32_t>());
  }
  if ((ce = cudaGetLastError())) return zg_check_cuda(ce, "generator kernels");
  return zg_build_graph_device(coo.as<uint2>(), max_weight ? w.as<uint32_t>() : nullptr, m, nv, s, out,
                               (flags & ZG_GRAPH_SAMPLING_ONLY) != 0);
}

}  // namespace

extern "C" int zg_graph_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                                 uint32_t max_weight, uint64_t weight_seed, uint32_t flags, void* cuda_stream,
                                 zg_graph** out) {
  if (!out || scale < 1 || scale > 31 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
    return zg_set_error(ZG_ERR_INVALID_ARG, "invalid R-MAT parameters"), ZG_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  const uint64_t n = (uint64_t)edge_factor << scale;
  const double two32 = 4294967296.0;
  uint64_t ta = (uint64_t)(a * two32), tb = (uint64_t)((a + b) * two32), tc = (uint64_t)((a + b + c) * two32);
  Buf keys;
  int rc = keys.alloc(8 * n);
  if (rc) return rc;
  if (n) k_rmat_keys<<<grid_n(n), 256, 0, s>>>(n, scale, ta, tb, tc, seed, keys.as<unsigned long long>());
  return finish_device(keys, n, 1u << scale, seed, max_weight, weight_seed, flags, s, out);
}

extern "C" int zg_graph_gen_chung_lu(uint32_t nv, double exponent, double avg_degree, uint64_t seed,
                                     uint32_t max_weight, uint64_t weight_seed, uint32_t flags, void* cuda_stream,
                                 zg_graph** out) {
  if (!out || nv < 2 || exponent <= 1.0 || avg_degree <= 0)
    return zg_set_error(ZG_ERR_INVALID_ARG, "invalid Chung-Lu parameters"), ZG_ERR_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)cuda_stream;
  // the cumulative weights on the host, in the generator's order of additions (zg_gen.cpp)
  std::vector<double> cdf(nv);
  double gam = 1.0 / (exponent - 1.0), tot = 0;
  for (uint32_t i = 0; i < nv; ++i) {
    tot += pow((double)i + 1.0, -gam);
    cdf[i] = tot;
  }
  const uint64_t draws = (uint64_t)(avg_degree * nv / 2.0);
  Buf dcdf, keys;
  int rc;
  if ((rc = dcdf.alloc(8ull * nv)) || (rc = keys.alloc(8 * draws))) return rc;
  cudaError_t ce = cudaMemcpyAsync(dcdf.p, cdf.data(), 8ull * nv, cudaMemcpyHostToDevice, s);
  if (ce) return zg_check_cuda(ce, "Chung-Lu weights");
  if (draws)
    k_cl_keys<<<grid_n(draws), 256, 0, s>>>(draws, dcdf.as<double>(), nv, tot, seed, keys.as<unsigned long long>());
  if ((ce = cudaStreamSynchronize(s))) return zg_check_cuda(ce, "Chung-Lu keys");
  dcdf.release();
  return finish_device(keys, draws, nv, seed, max_weight, weight_seed, flags, s, out);
}
