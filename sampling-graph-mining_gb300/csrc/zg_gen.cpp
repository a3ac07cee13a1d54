// zg_gen.cpp — seeded synthetic graphs for benchmarks and tests (the reference ships none; its
// SNAP datasets are download scripts).  Every random number is a Philox draw keyed by the
// seed, so the same call yields the same graph on any host.
//   R-MAT (Chakrabarti, Zhan, Faloutsos, SDM'04) and Chung-Lu (Chung & Lu 2002) power-law
//   graphs; undirected, self-loops and duplicate edges removed, emitted in a seeded random
//   order with a seeded random orientation (the reference's loader shuffles edges the same way
//   before it assigns edge ids, src/Graph.cpp:218-231).
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "zg_internal.cuh"

namespace {

constexpr uint32_t kStreamRmat = 0xFFFFFF00u;
constexpr uint32_t kStreamOrder = 0xFFFFFF01u;
constexpr uint32_t kStreamCL = 0xFFFFFF02u;
constexpr uint32_t kStreamW = 0xFFFFFF03u;

void philox4(uint64_t seed, uint32_t stream, uint64_t ctr, uint32_t d, uint32_t out[4]) {
  uint32_t c0 = (uint32_t)ctr, c1 = (uint32_t)(ctr >> 32), c2 = d, c3 = stream;
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    c0 = n0;
    c1 = (uint32_t)p1;
    c2 = n2;
    c3 = (uint32_t)p0;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

template <typename F>
void parallel_for(uint64_t n, F f) {
  unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  if (n < 65536) nt = 1;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t)
    th.emplace_back([&, t] {
      uint64_t lo = n / nt * t, hi = t == nt - 1 ? n : lo + n / nt;
      for (uint64_t i = lo; i < hi; ++i) f(i);
    });
  for (auto& x : th) x.join();
}

// canonical (min,max) keys -> unique -> seeded order and orientation
int finish(std::vector<uint64_t>& keys, uint64_t seed, uint64_t capacity, uint32_t* edges, uint64_t* m_out) {
  std::sort(keys.begin(), keys.end());
  keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
  if (keys.size() && keys.back() == ~0ull) keys.pop_back();  // self-loop marker
  uint64_t m = keys.size();
  *m_out = m;
  if (!edges) return ZG_OK;
  if (m > capacity) return zg_set_error(ZG_ERR_TOO_LARGE, "capacity %llu < %llu edges", (unsigned long long)capacity, (unsigned long long)m), ZG_ERR_TOO_LARGE;
  std::vector<std::pair<uint64_t, uint64_t>> order(m);
  parallel_for(m, [&](uint64_t i) {
    uint32_t o[4];
    philox4(seed, kStreamOrder, i, 0, o);
    order[i] = {((uint64_t)o[1] << 32) | o[0], i};
  });
  std::sort(order.begin(), order.end());
  parallel_for(m, [&](uint64_t i) {
    uint64_t k = keys[order[i].second];
    uint32_t u = (uint32_t)(k >> 32), v = (uint32_t)k;
    uint32_t o[4];
    philox4(seed, kStreamOrder, order[i].second, 1, o);
    if (o[0] & 1) std::swap(u, v);
    edges[2 * i] = u;
    edges[2 * i + 1] = v;
  });
  return ZG_OK;
}

}  // namespace

extern "C" int zg_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                           uint64_t capacity, uint32_t* edges, uint64_t* m_out) {
  if (!m_out || scale < 1 || scale > 31 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
    return zg_set_error(ZG_ERR_INVALID_ARG, "invalid R-MAT parameters"), ZG_ERR_INVALID_ARG;
  uint64_t n = (uint64_t)edge_factor << scale;
  const double two32 = 4294967296.0;
  uint64_t ta = (uint64_t)(a * two32), tb = (uint64_t)((a + b) * two32), tc = (uint64_t)((a + b + c) * two32);
  std::vector<uint64_t> keys(n);
  parallel_for(n, [&](uint64_t k) {
    uint32_t u = 0, v = 0;
    uint32_t o[4];
    for (uint32_t lvl = 0; lvl < scale; ++lvl) {
      if ((lvl & 3) == 0) philox4(seed, kStreamRmat, k, lvl >> 2, o);
      uint64_t r = o[lvl & 3];
      uint32_t bu = 0, bv = 0;
      if (r < ta) {
      } else if (r < tb) {
        bv = 1;
      } else if (r < tc) {
        bu = 1;
      } else {
        bu = 1;
        bv = 1;
      }
      u = (u << 1) | bu;
      v = (v << 1) | bv;
    }
    if (u == v)
      keys[k] = ~0ull;
    else
      keys[k] = u < v ? ((uint64_t)u << 32 | v) : ((uint64_t)v << 32 | u);
  });
  return finish(keys, seed, capacity, edges, m_out);
}

// Chung-Lu with expected degrees w_i ∝ (i + i0)^(-1/(exponent-1)), scaled to avg_degree; endpoints
// drawn independently proportional to w (inverse-CDF on the prefix sums).
extern "C" int zg_gen_chung_lu(uint32_t n, double exponent, double avg_degree, uint64_t seed, uint64_t capacity,
                               uint32_t* edges, uint64_t* m_out) {
  if (!m_out || n < 2 || exponent <= 1.0 || avg_degree <= 0)
    return zg_set_error(ZG_ERR_INVALID_ARG, "invalid Chung-Lu parameters"), ZG_ERR_INVALID_ARG;
  std::vector<double> cdf(n);
  double gam = 1.0 / (exponent - 1.0), s = 0;
  for (uint32_t i = 0; i < n; ++i) {
    s += pow((double)i + 1.0, -gam);
    cdf[i] = s;
  }
  uint64_t draws = (uint64_t)(avg_degree * n / 2.0);
  std::vector<uint64_t> keys(draws);
  parallel_for(draws, [&](uint64_t k) {
    uint32_t o[4];
    philox4(seed, kStreamCL, k, 0, o);
    double r0 = (((uint64_t)o[1] << 21) ^ o[0]) * 0x1p-53 * s;
    double r1 = (((uint64_t)o[3] << 21) ^ o[2]) * 0x1p-53 * s;
    uint32_t u = (uint32_t)(std::upper_bound(cdf.begin(), cdf.end(), r0) - cdf.begin());
    uint32_t v = (uint32_t)(std::upper_bound(cdf.begin(), cdf.end(), r1) - cdf.begin());
    if (u >= n) u = n - 1;
    if (v >= n) v = n - 1;
    keys[k] = u == v ? ~0ull : (u < v ? ((uint64_t)u << 32 | v) : ((uint64_t)v << 32 | u));
  });
  return finish(keys, seed, capacity, edges, m_out);
}

// Edge data uniform in [0, max_value) (datasets/toolkits/get_weighted_datasets.cpp:28-43 uses
// rand() % 79; the batched workload asks for [0, 100)).
extern "C" int zg_gen_weights(uint64_t m, uint32_t max_value, uint64_t seed, uint32_t* w) {
  if ((m && !w) || max_value == 0) return zg_set_error(ZG_ERR_INVALID_ARG, "invalid weight request"), ZG_ERR_INVALID_ARG;
  parallel_for(m, [&](uint64_t e) {
    uint32_t o[4];
    philox4(seed, kStreamW, e, 0, o);
    w[e] = (uint32_t)(((uint64_t)o[0] * max_value) >> 32);
  });
  return ZG_OK;
}
