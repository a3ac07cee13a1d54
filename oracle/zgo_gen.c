/*
 * zgo_gen.c — CPU ORACLE side (test infrastructure only; see zg_oracle.h): seeded synthetic
 * inputs for the CPU arm of the benchmark, produced on the host without the GPU library.
 *
 * zgo_gen_rmat yields the same edge list, edge for edge and in the same order and orientation,
 * as the library's zg_gen_rmat / zg_graph_gen_rmat (tests/test_oracle_gen.py checks this), so the
 * CPU arm and the GPU arm sample the same graph.  The algorithm is that generator's:
 *   R-MAT (Chakrabarti, Zhan, Faloutsos, SDM'04): edge k descends `scale` levels; level l takes
 *   32-bit word l & 3 of Philox4x32-10 block (k, l >> 2) on the R-MAT stream and picks the
 *   quadrant by comparing it with floor(a, a+b, a+b+c scaled by 2^32);
 *   canonical (min, max) keys, duplicates and self-loops removed, ascending;
 *   output edge i is the unique key of rank order[i], where order sorts (word of block (j, 0) on
 *   the order stream, j) lexicographically; word 0 of block (order[i], 1) flips its orientation
 *   when odd.
 * The reference itself has no generator (its SNAP inputs come from download scripts,
 * datasets/*\/scripts/download.sh); its loader shuffles edges before assigning ids
 * (src/Graph.cpp:218-231), which the seeded order stands in for.
 *
 * Sorting is a parallel least-significant-digit radix sort (stable), so ties in the order words
 * fall back to ascending j exactly as the lexicographic pair order does.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "zg_oracle.h"

#define ZGO_STREAM_RMAT  0xFFFFFF00u
#define ZGO_STREAM_ORDER 0xFFFFFF01u

static void philox_block(uint64_t seed, uint32_t stream, uint64_t ctr, uint32_t d, uint32_t out[4]) {
  uint32_t c[4] = {(uint32_t)ctr, (uint32_t)(ctr >> 32), d, stream};
  uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  zgo_philox4x32_10(c, k, out);
}

static int nthreads(uint64_t n) {
#ifdef _OPENMP
  return n < 65536 ? 1 : omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

static int thread_id(void) {
#ifdef _OPENMP
  return omp_get_thread_num();
#else
  return 0;
#endif
}

#define RADIX_BITS 13
#define RADIX (1u << RADIX_BITS)

/* Stable parallel LSD radix sort of keys[0..n) on bits [0, bits), carrying an optional uint32
 * payload.  Scratch buffers are allocated here; the sorted data ends in keys/payload. */
static int radix_sort(uint64_t* keys, uint32_t* payload, uint64_t n, int bits) {
  if (n < 2) return ZG_OK;
  int nt = nthreads(n);
  uint64_t* k2 = (uint64_t*)malloc(sizeof(uint64_t) * n);
  uint32_t* p2 = payload ? (uint32_t*)malloc(sizeof(uint32_t) * n) : NULL;
  uint64_t* hist = (uint64_t*)malloc(sizeof(uint64_t) * RADIX * (size_t)nt);
  if (!k2 || (payload && !p2) || !hist) {
    free(k2); free(p2); free(hist);
    return ZG_ERR_OOM;
  }
  uint64_t *src = keys, *dst = k2;
  uint32_t *psrc = payload, *pdst = p2;
  for (int shift = 0; shift < bits; shift += RADIX_BITS) {
    memset(hist, 0, sizeof(uint64_t) * RADIX * (size_t)nt);
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
    {
      int t = thread_id();
      uint64_t lo = n / (uint64_t)nt * (uint64_t)t, hi = t == nt - 1 ? n : lo + n / (uint64_t)nt;
      uint64_t* h = hist + (size_t)t * RADIX;
      for (uint64_t i = lo; i < hi; ++i) h[(src[i] >> shift) & (RADIX - 1)]++;
    }
    /* bucket-major, thread-minor exclusive offsets keep the sort stable */
    uint64_t run = 0;
    int single = 0;
    for (uint32_t b = 0; b < RADIX; ++b) {
      uint64_t tot = 0;
      for (int t = 0; t < nt; ++t) tot += hist[(size_t)t * RADIX + b];
      if (tot == n) single = 1;
      for (int t = 0; t < nt; ++t) {
        uint64_t c = hist[(size_t)t * RADIX + b];
        hist[(size_t)t * RADIX + b] = run;
        run += c;
      }
    }
    if (single) continue; /* every key has the same digit: the pass would be the identity */
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
    {
      int t = thread_id();
      uint64_t lo = n / (uint64_t)nt * (uint64_t)t, hi = t == nt - 1 ? n : lo + n / (uint64_t)nt;
      uint64_t* h = hist + (size_t)t * RADIX;
      for (uint64_t i = lo; i < hi; ++i) {
        uint64_t pos = h[(src[i] >> shift) & (RADIX - 1)]++;
        dst[pos] = src[i];
        if (psrc) pdst[pos] = psrc[i];
      }
    }
    uint64_t* tk = src; src = dst; dst = tk;
    uint32_t* tp = psrc; psrc = pdst; pdst = tp;
  }
  if (src != keys) {
    memcpy(keys, src, sizeof(uint64_t) * n);
    if (payload) memcpy(payload, psrc, sizeof(uint32_t) * n);
  }
  free(k2); free(p2); free(hist);
  return ZG_OK;
}

int zgo_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                 uint64_t capacity, uint32_t* edges, uint64_t* m_out) {
  if (!m_out || scale < 1 || scale > 31 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return ZG_ERR_INVALID_ARG;
  const uint64_t n = (uint64_t)edge_factor << scale;
  const double two32 = 4294967296.0;
  const uint64_t ta = (uint64_t)(a * two32), tb = (uint64_t)((a + b) * two32), tc = (uint64_t)((a + b + c) * two32);
  const uint64_t marker = (scale == 31) ? ~0ull >> 2 : (1ull << (2 * scale)) - 1; /* u == v == 2^scale - 1 */
  uint64_t* keys = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
  if (!keys) return ZG_ERR_OOM;
  int nt = nthreads(n);
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
  for (uint64_t k = 0; k < n; ++k) {
    uint32_t u = 0, v = 0, o[4] = {0, 0, 0, 0};
    for (uint32_t lvl = 0; lvl < scale; ++lvl) {
      if ((lvl & 3) == 0) philox_block(seed, ZGO_STREAM_RMAT, k, lvl >> 2, o);
      uint64_t r = o[lvl & 3];
      uint32_t bu = r >= tc ? 1u : (r >= tb ? 1u : 0u);
      uint32_t bv = r >= tc ? 1u : (r >= tb ? 0u : (r >= ta ? 1u : 0u));
      u = (u << 1) | bu;
      v = (v << 1) | bv;
    }
    /* canonical key (min << scale | max); a self-loop becomes the marker, which sorts last */
    keys[k] = u == v ? marker : (u < v ? ((uint64_t)u << scale | v) : ((uint64_t)v << scale | u));
  }
  int rc = radix_sort(keys, NULL, n, 2 * (int)scale);
  if (rc) { free(keys); return rc; }
  uint64_t m = 0;
  for (uint64_t i = 0; i < n; ++i)
    if (keys[i] != marker && (m == 0 || keys[m - 1] != keys[i])) keys[m++] = keys[i];
  *m_out = m;
  if (!edges) { free(keys); return ZG_OK; }
  if (m > capacity) { free(keys); return ZG_ERR_TOO_LARGE; }
  uint64_t* w = (uint64_t*)malloc(sizeof(uint64_t) * (m ? m : 1));
  uint32_t* idx = (uint32_t*)malloc(sizeof(uint32_t) * (m ? m : 1));
  if (!w || !idx || m > 0xFFFFFFFFull) { free(keys); free(w); free(idx); return w && idx ? ZG_ERR_TOO_LARGE : ZG_ERR_OOM; }
  nt = nthreads(m);
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
  for (uint64_t i = 0; i < m; ++i) {
    uint32_t o[4];
    philox_block(seed, ZGO_STREAM_ORDER, i, 0, o);
    w[i] = ((uint64_t)o[1] << 32) | o[0];
    idx[i] = (uint32_t)i;
  }
  rc = radix_sort(w, idx, m, 64);
  free(w);
  if (rc) { free(keys); free(idx); return rc; }
  const uint64_t vmask = (1ull << scale) - 1;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
  for (uint64_t i = 0; i < m; ++i) {
    uint64_t k = keys[idx[i]];
    uint32_t u = (uint32_t)(k >> scale), v = (uint32_t)(k & vmask), o[4];
    philox_block(seed, ZGO_STREAM_ORDER, idx[i], 1, o);
    if (o[0] & 1) { uint32_t t = u; u = v; v = t; }
    edges[2 * i] = u;
    edges[2 * i + 1] = v;
  }
  free(keys);
  free(idx);
  return ZG_OK;
}

int zgo_subsample_edges(const uint32_t* edges, uint64_t m, double rate, uint64_t keep_seed, uint64_t shuffle_seed,
                        uint64_t capacity, uint32_t* out, uint64_t* k_out) {
  if (!k_out || (m && !edges) || m >= ((uint64_t)1 << 32)) return ZG_ERR_INVALID_ARG;
  int nt = nthreads(m);
  uint8_t* keep = (uint8_t*)malloc(m ? m : 1);
  uint64_t* cnt = (uint64_t*)calloc((size_t)nt + 1, sizeof(uint64_t));
  if (!keep || !cnt) {
    free(keep); free(cnt);
    return ZG_ERR_OOM;
  }
  /* the keep draws, counted per contiguous range of edges */
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
  {
    int t = thread_id();
    uint64_t lo = m / (uint64_t)nt * (uint64_t)t, hi = t == nt - 1 ? m : lo + m / (uint64_t)nt, c = 0;
    for (uint64_t e = lo; e < hi; ++e) c += keep[e] = (uint8_t)zgo_subsample_keep(rate, keep_seed, e);
    cnt[t + 1] = c;
  }
  for (int t = 0; t < nt; ++t) cnt[t + 1] += cnt[t];
  const uint64_t k = cnt[nt];
  *k_out = k;
  if (!out) {
    free(keep); free(cnt);
    return ZG_OK;
  }
  if (capacity < k) {
    free(keep); free(cnt);
    return ZG_ERR_INVALID_ARG;
  }
  uint32_t* pos = (uint32_t*)malloc(sizeof(uint32_t) * (k ? k : 1));
  uint64_t* keys = (uint64_t*)malloc(sizeof(uint64_t) * (k ? k : 1));
  uint32_t* order = (uint32_t*)malloc(sizeof(uint32_t) * (k ? k : 1));
  if (!pos || !keys || !order) {
    free(keep); free(cnt); free(pos); free(keys); free(order);
    return ZG_ERR_OOM;
  }
  /* the kept positions in ascending order, and the shuffle key of each kept rank */
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
  {
    int t = thread_id();
    uint64_t lo = m / (uint64_t)nt * (uint64_t)t, hi = t == nt - 1 ? m : lo + m / (uint64_t)nt, j = cnt[t];
    for (uint64_t e = lo; e < hi; ++e)
      if (keep[e]) pos[j++] = (uint32_t)e;
  }
  int nk = nthreads(k);
#ifdef _OPENMP
#pragma omp parallel for num_threads(nk) schedule(static)
#endif
  for (int64_t j = 0; j < (int64_t)k; ++j) {
    keys[j] = zgo_shuffle_key(shuffle_seed, (uint64_t)j);
    order[j] = (uint32_t)j;
  }
  /* stable on the keys: ties keep ascending rank, the (key, rank) order of zgo_shuffle_perm */
  int rc = radix_sort(keys, order, k, 64);
  if (rc == ZG_OK) {
#ifdef _OPENMP
#pragma omp parallel for num_threads(nk) schedule(static)
#endif
    for (int64_t i = 0; i < (int64_t)k; ++i) {
      const uint64_t e = pos[order[i]];
      out[2 * i] = edges[2 * e];
      out[2 * i + 1] = edges[2 * e + 1];
    }
  }
  free(keep); free(cnt); free(pos); free(keys); free(order);
  return rc;
}
