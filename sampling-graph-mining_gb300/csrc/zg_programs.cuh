// zg_programs.cuh — the estimator programs on the device, shared by the sampling kernels
// (zg_sample.cu) and the batched-query kernel (zg_batch.cu).
//
// One estimator (sample) per thread.  Every estimator draws from its own Philox4x32-10 counter
// stream (seed, stream_id, sample index, draw index), so results do not depend on the launch
// shape.  Each program restates one application estimate() (cited) on the device layout of
// zg_internal.cuh:
//   * a conditional step from an edge's endpoints reads its suffix sizes S and the entries'
//     addresses from the edge's record (no search; see zg_internal.cuh for the two layouts);
//   * later steps find lower bounds by interpolation search inside ranges the per-edge suffix
//     counts already narrow;
//   * closure checks (conditional_close, src/ZGraphInstance.cpp:372-407) look the edge up in the
//     cuckoo table.
// Weights are exact: numerator m*prod(S_i) (192-bit) over 2^shift.  The debug variant (DBG)
// additionally records every draw, the access-model sector count and the reference's double 1/p
// computed with the same IEEE operation sequence as the application (x87 extended arithmetic
// restated in integers for ChainMining).
#pragma once

#include "zg_internal.cuh"

// Internal linkage: every translation unit that includes this header gets its own copy.
namespace {

struct Ctx {
  uint64_t seed;
  uint64_t sample;
  uint32_t stream;
  uint32_t nd;
  zg_sample_trace* tr;  // debug only
  uint32_t sectors;     // debug only: access model, 32-byte sectors
  uint32_t closures;    // debug only: access model, closure checks
  const ZgKeys* rk;     // the seed's round keys (a grid-constant parameter), or null
  __device__ __forceinline__ uint64_t draw(uint64_t lo, uint64_t hi) { return take(word(nd), lo, hi); }
  // The Philox word of draw k, computable before the range it maps to is known (so the integer
  // work overlaps the loads that determine the range); take() maps the next draw's word.
  __device__ __forceinline__ uint64_t word(uint32_t k) const {
    return rk ? zg_sample_word_k(*rk, stream, sample, k) : zg_sample_word(seed, stream, sample, k);
  }
  __device__ __forceinline__ uint64_t take(uint64_t w, uint64_t lo, uint64_t hi) {
    uint64_t v = zg_draw_map(w, lo, hi);
    if (tr && nd < ZG_MAX_DRAWS) {
      tr->lo[nd] = lo;
      tr->hi[nd] = hi;
      tr->val[nd] = v;
    }
    ++nd;
    return v;
  }
};

struct Res {
  bool hit;
  bool fail;
  bool ovf;
  uint32_t shift;
  ZgU192 num;
  double w;  // debug: reference double
};

__device__ __forceinline__ void res_init(Res& r) {
  r.hit = false;
  r.fail = false;
  r.ovf = false;
  r.shift = 0;
  zg_u192_set(r.num, 1);
  r.w = 0.0;
}
// Every factor of a weight is below 2^32: the edge count (at most 2^31 - 1, the build's limit),
// a suffix sum S over distinct anchors (at most 2m) or a small constant.  A factor that broke this
// would be reported as an overflow, never truncated silently.
__device__ __forceinline__ void res_mul(Res& r, uint64_t f) {
  if (zg_u192_mul32(r.num, (uint32_t)f) || (f >> 32)) r.ovf = true;
}

// First index in adj_e[lo, hi) whose edge id >= key, where every edge id in the range is known
// to lie in [vlo, vhi].  The build shuffles the edge ids (a uniformly random permutation), so an
// edge-id-ordered list is a sorted uniform sample of [0, m): interpolation finds the bound in
// O(log log d) expected probes instead of log2 d.  After 8 interpolation probes it bisects, which
// bounds the worst case (unshuffled input) by 8 + log2 d probes.
__device__ __forceinline__ uint32_t lb_eid(const uint2* __restrict__ adj, uint32_t lo, uint32_t hi, uint32_t key,
                                           uint32_t vlo, uint32_t vhi) {
  for (int it = 0; hi - lo > 4; ++it) {
    if (key <= vlo) return lo;  // every id in the range is >= key
    if (key > vhi) return hi;   // every id in the range is < key
    uint32_t n = hi - lo, p;
    if (it < 8) {
      float f = __fdividef((float)(key - vlo), (float)(vhi - vlo) + 1.0f);
      uint32_t est = (uint32_t)(f * (float)n);
      p = lo + (est < n ? est : n - 1);
    } else {
      p = lo + (n >> 1);
    }
    uint32_t v = ZG_LDG(&adj[p]).y;
    if (v < key) {
      lo = p + 1;
      vlo = v + 1;
    } else {
      hi = p;
      vhi = v - 1;  // v >= key > vlo >= 0
    }
  }
  // at most 4 entries left (sorted): load them together and count those below the key
  uint32_t n = hi - lo, below = 0;
#pragma unroll
  for (uint32_t i = 0; i < 4; ++i)
    if (i < n) below += ZG_LDG(&adj[lo + i]).y < key;
  return lo + below;
}

// The edge ids of adjacency entries s .. s+7 (s a multiple of 4: two 32-byte-aligned 256-bit
// loads).  The build leaves 8 entries of slack after adj_e, so s < 2m never reads past it.
__device__ __forceinline__ void ld_ids8(const uint2* adj, uint32_t s, uint32_t (&id)[8]) {
  unsigned long long a0, a1, a2, a3, b0, b1, b2, b3;
  ZG_NOTE_LOAD(adj + s, 64);
  asm("ld.global.nc.v4.u64 {%0, %1, %2, %3}, [%4];" : "=l"(a0), "=l"(a1), "=l"(a2), "=l"(a3) : "l"(adj + s));
  asm("ld.global.nc.v4.u64 {%0, %1, %2, %3}, [%4];" : "=l"(b0), "=l"(b1), "=l"(b2), "=l"(b3) : "l"(adj + s + 4));
  id[0] = (uint32_t)(a0 >> 32);
  id[1] = (uint32_t)(a1 >> 32);
  id[2] = (uint32_t)(a2 >> 32);
  id[3] = (uint32_t)(a3 >> 32);
  id[4] = (uint32_t)(b0 >> 32);
  id[5] = (uint32_t)(b1 >> 32);
  id[6] = (uint32_t)(b2 >> 32);
  id[7] = (uint32_t)(b3 >> 32);
}

// lb_eid with a window of 8 entries (two sectors) read around each interpolated estimate: the
// bound is found inside the window, or the window and every entry on its wrong side drop out, so
// short lists take one dependent read.  Costs registers: used where warps run one search each.
__device__ __forceinline__ uint32_t lb_eid_win(const uint2* __restrict__ adj, uint32_t lo, uint32_t hi, uint32_t key,
                                               uint32_t vlo, uint32_t vhi) {
  for (int it = 0; lo < hi; ++it) {
    if (key <= vlo) return lo;
    if (key > vhi) return hi;
    const uint32_t n = hi - lo;
    uint32_t c;
    if (it < 8) {
      float f = __fdividef((float)(key - vlo), (float)(vhi - vlo) + 1.0f);
      uint32_t est = (uint32_t)(f * (float)n);
      c = lo + (est < n ? est : n - 1);
    } else {
      c = lo + (n >> 1);
    }
    const uint32_t s = (c >= 3 ? c - 3 : 0u) & ~3u;  // window [s, s + 8) holds c
    uint32_t id[8];
    ld_ids8(adj, s, id);
    const uint32_t wl = s > lo ? s : lo, wh = s + 8 < hi ? s + 8 : hi;  // its part of [lo, hi), not empty
    uint32_t below = 0, idf = 0, idl = 0;
#pragma unroll
    for (uint32_t i = 0; i < 8; ++i) {
      const uint32_t p = s + i;
      below += p >= wl && p < wh && id[i] < key;
      idf = p == wl ? id[i] : idf;
      idl = p == wh - 1 ? id[i] : idl;
    }
    if (below == 0) {  // the bound is at or before the window
      if (wl == lo) return lo;
      hi = wl;
      vhi = idf - 1;  // idf >= key > vlo >= 0
    } else if (below == wh - wl) {  // the bound is after the window
      if (wh == hi) return hi;
      lo = wh;
      vlo = idl + 1;
    } else {
      return wl + below;
    }
  }
  return lo;
}

// Does edge (x,y) exist with edge id >= min_valid?  conditional_close's question
// (src/ZGraphInstance.cpp:372-407): the pattern edges still to close join two sampled vertices,
// so "found in some sampled vertex's list with id >= min_valid" is "edge (x,y) exists with such
// an id".  Answered by the cuckoo table (one 32-byte sector per bucket): a fingerprint match is
// confirmed against rec, so the answer is exact.  Two phases, so a caller with several look-ups
// can stop before any dependent load: edge_candidate() reads the key's first bucket, and its
// second behind an overflow flag (edge_candidate_both: both at once), and returns the first entry
// whose fingerprint matches (or the empty marker: then the edge does not exist); edge_confirm()
// checks the candidate against rec and, in the rare case of a second fingerprint match, rescans.
// The result is the edge id, or -1 when the edge does not exist.
// One bucket = one 32-byte sector, read with a single 256-bit load (sm_100 family).
__device__ __forceinline__ void ld_bucket(const unsigned long long* p, ulonglong2& lo, ulonglong2& hi) {
  ZG_NOTE_LOAD(p, 32);
  asm("ld.global.nc.v4.u64 {%0, %1, %2, %3}, [%4];" : "=l"(lo.x), "=l"(lo.y), "=l"(hi.x), "=l"(hi.y) : "l"(p));
}

// One wide edge record (32 bytes, one sector) in a single 256-bit load.
__device__ __forceinline__ void ld_rec(const ZgRec* r, uint4& e, uint4& p) {
  unsigned long long a, b, c, d;
  ZG_NOTE_LOAD(r, 32);
  asm("ld.global.nc.v4.u64 {%0, %1, %2, %3}, [%4];" : "=l"(a), "=l"(b), "=l"(c), "=l"(d) : "l"(r));
  e = make_uint4((uint32_t)a, (uint32_t)(a >> 32), (uint32_t)b, (uint32_t)(b >> 32));
  p = make_uint4((uint32_t)c, (uint32_t)(c >> 32), (uint32_t)d, (uint32_t)(d >> 32));
}

// Edge e's record with both endpoints unknown: e = (src, dst, suf_src, suf_dst), p = (pos_src,
// pos_dst, pre_src, pre_dst).  Wide layout: one read.  Compact: the record, then the endpoints'
// offsets (the pre_* loads vanish where a caller does not use them).
__device__ __forceinline__ void edge_rec(const ZgDevGraph& g, uint64_t e, uint4& q, uint4& p) {
  if (g.wide) {
    ld_rec(&((const ZgRec*)g.rec)[e], q, p);
    return;
  }
  if (g.packed) {  // the slots from the record, the predecessor counts from the offsets (if used)
    uint2 pos;
    zg_rec_packed(g, e, q, pos);
    p.x = pos.x;
    p.y = pos.y;
    p.z = p.x - ZG_LDG(&g.off32[q.x]);
    p.w = p.y - ZG_LDG(&g.off32[q.y]);
    return;
  }
  q = ZG_LDG(&((const uint4*)g.rec)[e]);
  p.x = ZG_LDG(&g.off32[q.x + 1]) - q.z - 1;
  p.y = ZG_LDG(&g.off32[q.y + 1]) - q.w - 1;
  p.z = p.x - ZG_LDG(&g.off32[q.x]);
  p.w = p.y - ZG_LDG(&g.off32[q.y]);
}

// The first entry after edge (q, p) in its src's (dst = false) or dst's list.  Compact layout:
// one offset read, of the chosen endpoint only.
__device__ __forceinline__ uint32_t after_edge(const ZgDevGraph& g, const uint4& q, const uint4& p, bool dst) {
  if (g.wide || g.packed) return (dst ? p.y : p.x) + 1;
  return ZG_LDG(&g.off32[(dst ? q.y : q.x) + 1]) - (dst ? q.w : q.z);
}

// Edge e seen from its endpoint v (already known): entries after it in v's list and its own slot
// there.  Compact layout: the record and v's end offset are read together.
struct EdgeAt {
  uint32_t suf, pos, pre;  // pre: wide layout only (see edge_at_start)
};
__device__ __forceinline__ EdgeAt edge_at(const ZgDevGraph& g, uint64_t e, uint32_t v) {
  EdgeAt r;
  if (g.wide) {
    uint4 q, p;
    ld_rec(&((const ZgRec*)g.rec)[e], q, p);
    const bool s = q.x == v;
    r.suf = s ? q.z : q.w;
    r.pos = s ? p.x : p.y;
    r.pre = s ? p.z : p.w;
    return r;
  }
  if (g.packed) {
    uint4 q;
    uint2 pos;
    zg_rec_packed(g, e, q, pos);
    const bool s = q.x == v;
    r.suf = s ? q.z : q.w;
    r.pos = s ? pos.x : pos.y;
    r.pre = 0;
    return r;
  }
  const uint4 q = ZG_LDG(&((const uint4*)g.rec)[e]);
  const uint32_t end = ZG_LDG(&g.off32[v + 1]);
  r.suf = q.x == v ? q.z : q.w;
  r.pos = end - r.suf - 1;
  r.pre = 0;
  return r;
}
// The first slot of v's list, for a step that searches it (compact layout: v's start offset, a
// read independent of the record, issued only where a search needs it).
__device__ __forceinline__ uint32_t edge_at_start(const ZgDevGraph& g, const EdgeAt& a, uint32_t v) {
  return g.wide ? a.pos - a.pre : ZG_LDG(&g.off32[v]);
}

struct EdgeProbe {
  unsigned long long key, cand;
};

// The key's first bucket is read first, and its second only if the first carries the overflow
// flag (slot 0, bit 63): the build sets it on a bucket whenever one of the keys whose first bucket
// it is goes to its second bucket, so an unflagged first bucket without a matching fingerprint
// proves the edge absent after one sector.
__device__ __forceinline__ unsigned long long bucket_match(const ulonglong2& a0, const ulonglong2& a1, uint32_t fp) {
  unsigned long long e = ZG_HASH_EMPTY;  // an empty entry never matches: no fingerprint is 0x7FFFFFFF
  e = zg_entry_fp(a1.y) == fp ? a1.y : e;
  e = zg_entry_fp(a1.x) == fp ? a1.x : e;
  e = zg_entry_fp(a0.y) == fp ? a0.y : e;
  e = zg_entry_fp(a0.x) == fp ? a0.x : e;
  return e;
}
__device__ __forceinline__ bool bucket_overflow(const ulonglong2& a0) {
  return a0.x != ZG_HASH_EMPTY && (a0.x & ZG_HASH_OVERFLOW);
}

__device__ __forceinline__ EdgeProbe edge_candidate(const ZgDevGraph& g, uint32_t x, uint32_t y) {
  EdgeProbe pr;
  pr.key = zg_edge_key(x, y);
  const uint32_t fp = zg_fingerprint(pr.key, g.hseed);
  ulonglong2 a0, a1;
  ld_bucket(g.hent + 4ull * zg_bucket1(pr.key, g.hseed, g.hbits), a0, a1);
  unsigned long long e = bucket_match(a0, a1, fp);
  if (e == ZG_HASH_EMPTY && bucket_overflow(a0)) {
    ulonglong2 c0, c1;
    ld_bucket(g.hent + 4ull * zg_bucket2(pr.key, g.hseed, g.hbits), c0, c1);
    e = bucket_match(c0, c1, fp);
  }
  pr.cand = e;
  return pr;
}

// The same look-up with both buckets read at once (two sectors, one dependent step): for the
// latency-bound 4-clique, whose early rejection waits on this look-up.
__device__ __forceinline__ EdgeProbe edge_candidate_both(const ZgDevGraph& g, uint32_t x, uint32_t y) {
  EdgeProbe pr;
  pr.key = zg_edge_key(x, y);
  const uint32_t fp = zg_fingerprint(pr.key, g.hseed);
  ulonglong2 a0, a1, c0, c1;
  ld_bucket(g.hent + 4ull * zg_bucket1(pr.key, g.hseed, g.hbits), a0, a1);
  ld_bucket(g.hent + 4ull * zg_bucket2(pr.key, g.hseed, g.hbits), c0, c1);
  const unsigned long long e = bucket_match(a0, a1, fp);
  pr.cand = e != ZG_HASH_EMPTY ? e : bucket_match(c0, c1, fp);
  return pr;
}

// another entry of the two buckets with the same fingerprint (probability ~ 8 / 2^31 a look-up)
__device__ __noinline__ int64_t edge_rescan(const ZgDevGraph& g, unsigned long long key, unsigned long long cand) {
  uint64_t b1 = 4ull * zg_bucket1(key, g.hseed, g.hbits), b2 = 4ull * zg_bucket2(key, g.hseed, g.hbits);
  uint32_t fp = zg_fingerprint(key, g.hseed);
  for (int i = 0; i < 8; ++i) {
    unsigned long long x = ZG_LDG(&g.hent[(i < 4 ? b1 : b2) + (i & 3)]);
    if (x == cand || zg_entry_fp(x) != fp) continue;
    uint4 q = zg_rec_e(g, (uint32_t)x);
    if (zg_edge_key(q.x, q.y) == key) return (int64_t)(uint32_t)x;
  }
  return -1;
}

__device__ __forceinline__ int64_t edge_confirm(const ZgDevGraph& g, const EdgeProbe& pr) {
  if (pr.cand == ZG_HASH_EMPTY) return -1;
  uint4 r = zg_rec_e(g, (uint32_t)pr.cand);
  if (zg_edge_key(r.x, r.y) == pr.key) return (int64_t)(uint32_t)pr.cand;
  return edge_rescan(g, pr.key, pr.cand);
}

__device__ __forceinline__ bool edge_after(const ZgDevGraph& g, uint32_t x, uint32_t y, uint32_t min_valid) {
  return edge_confirm(g, edge_candidate(g, x, y)) >= (int64_t)min_valid;
}

// ---- access model (debug): algorithmic bytes of a sample in 32-byte sectors ---------------
// sample_edge 1; a conditional step: per anchor v with d_v > 0, 1 + max(1, ceil(log2 d_v) - 2),
// plus 1 for the chosen entry; a closure edge: 2 + max(1, ceil(log2 min(d_x, d_y)) - 2),
// counted for every edge checked up to the first miss.
__device__ __forceinline__ uint32_t model_search(uint64_t d) {
  uint32_t l = d <= 1 ? 0u : (uint32_t)(64 - __clzll(d - 1));
  return l > 3 ? l - 2 : 1u;
}
__device__ __forceinline__ uint64_t degree(const ZgDevGraph& g, uint32_t v) {
  return (uint64_t)(ZG_LDG(&g.off32[v + 1]) - ZG_LDG(&g.off32[v]));
}
__device__ __forceinline__ uint32_t model_anchor(const ZgDevGraph& g, uint32_t v) {
  uint64_t d = degree(g, v);
  return d ? 1 + model_search(d) : 0;
}
__device__ __forceinline__ uint32_t model_close(const ZgDevGraph& g, uint32_t x, uint32_t y) {
  uint64_t dx = degree(g, x), dy = degree(g, y);
  return 2 + model_search(dx < dy ? dx : dy);
}

// ---- reference doubles (debug) ---------------------------------------------------------
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double u2d(uint64_t v) { return __ull2double_rn(v); }

// x87 extended (64-bit mantissa, round-to-nearest-even), restated in integers.
struct Ext {
  uint64_t m;
  int32_t e;
};
__device__ __forceinline__ Ext ext_from_double(double d) {
  uint64_t b = (uint64_t)__double_as_longlong(d);
  int ex = (int)((b >> 52) & 0x7ff);
  Ext r;
  r.m = ((b & ((1ull << 52) - 1)) | (1ull << 52)) << 11;
  r.e = ex - 1075 - 11;
  return r;
}
__device__ __forceinline__ Ext ext_mul(Ext a, Ext b) {
  uint64_t lo = a.m * b.m, hi = __umul64hi(a.m, b.m);
  uint64_t keep, rem, half = 1ull << 63;
  Ext r;
  if (hi >> 63) {
    keep = hi;
    rem = lo;
    r.e = a.e + b.e + 64;
  } else {
    keep = (hi << 1) | (lo >> 63);
    rem = lo << 1;
    r.e = a.e + b.e + 63;
  }
  if (rem > half || (rem == half && (keep & 1))) {
    keep++;
    if (keep == 0) {
      keep = 1ull << 63;
      r.e++;
    }
  }
  r.m = keep;
  return r;
}
// 2^127 / m for m in (2^63, 2^64): restoring division, 64 quotient bits.
__device__ __forceinline__ Ext ext_inv(Ext a) {
  Ext r;
  if (a.m == (1ull << 63)) {
    r.m = 1ull << 63;
    r.e = -126 - a.e;
    return r;
  }
  // remainder arithmetic on 65-bit values: rem < m < 2^64
  uint64_t q = 0, rem = 1ull << 63;  // 2^127 = 2^63 * 2^64: start with rem = 2^63, shift in 64 zero bits
  for (int i = 0; i < 64; ++i) {
    bool top = rem >> 63;
    rem <<= 1;
    q <<= 1;
    if (top || rem >= a.m) {
      rem -= a.m;
      q |= 1;
    }
  }
  r.e = -127 - a.e;
  // round: compare 2*rem with m
  bool top = rem >> 63;
  uint64_t rem2 = rem << 1;
  bool gt = top || rem2 > a.m;
  bool eq = !top && rem2 == a.m;
  if (gt || (eq && (q & 1))) {
    q++;
    if (q == 0) {
      q = 1ull << 63;
      r.e++;
    }
  }
  r.m = q;
  return r;
}
__device__ __forceinline__ double ext_to_double(Ext a) {
  uint64_t keep = a.m >> 11, rem = a.m & 0x7ff;
  int e = a.e + 11;
  if (rem > 0x400 || (rem == 0x400 && (keep & 1))) {
    keep++;
    if (keep == (1ull << 53)) {
      keep >>= 1;
      e++;
    }
  }
  return scalbn(u2d(keep), e);
}

// ---- Triangle: applications/Triangle.cpp:48-73 -----------------------------------------
template <bool DBG>
__device__ void prog_triangle(const ZgDevGraph& g, Ctx& c, Res& r) {
  if (g.m == 0) {
    r.fail = true;
    return;
  }
  const uint64_t w1 = c.word(1);  // the second draw's Philox work overlaps the first loads
  uint64_t e0 = c.draw(0, g.m - 1);
  uint4 q, qp;
  edge_rec(g, e0, q, qp);
  uint64_t S = (uint64_t)q.z + q.w;
  if (DBG) c.sectors += 1 + model_anchor(g, q.x) + model_anchor(g, q.y);
  if (S == 0) {
    r.fail = true;
    return;
  }
  if (DBG) c.sectors += 1;
  uint64_t r1 = c.take(w1, 0, S - 1);
  const bool on_y = r1 >= q.z;  // the conditional edge hangs off dst
  const uint32_t other = on_y ? q.x : q.y;
  uint32_t idx = after_edge(g, q, qp, on_y) + (uint32_t)(on_y ? r1 - q.z : r1);
  uint2 e1 = ZG_LDG(&g.adj_e[idx]);
  uint32_t a1 = 1 + (e1.x == q.x || e1.x == q.y);
  res_mul(r, g.m);
  res_mul(r, S);
  if (a1 == 2) r.shift = 1;
  bool closed = (a1 == 1) && edge_after(g, other, e1.x, e1.y + 1);
  if (DBG) {
    c.sectors += model_close(g, other, e1.x);
    c.closures++;
  }
  r.hit = closed;
  if (DBG && closed) {
    double p = 1.0;
    p = dmul(p, ddiv(1.0, u2d(g.m)));
    p = dmul(p, ddiv(1.0 * a1, u2d(S)));
    r.w = ddiv(1.0, p);
  }
}

// ---- ThreeChain: applications/ThreeChain.cpp:315-330 -------------------------------------
template <bool DBG>
__device__ void prog_three_chain(const ZgDevGraph& g, Ctx& c, Res& r) {
  if (g.m == 0) {
    r.fail = true;
    return;
  }
  uint64_t e0 = c.draw(0, g.m - 1);
  uint4 q = zg_rec_e(g, e0);
  uint64_t S = (uint64_t)q.z + q.w;
  if (DBG) c.sectors += 1 + model_anchor(g, q.x) + model_anchor(g, q.y);
  if (S == 0) {
    r.fail = true;
    return;
  }
  if (DBG) c.sectors += 1;
  uint64_t r1 = c.draw(0, S - 1);
  // The chosen edge only sets the appearance count a, which is 1 on a simple graph
  // (zg_graph_create rejects duplicate edges); the debug variant reads it and checks.
  uint32_t a1 = 1;
  if (DBG) {
    uint4 q2, qp;
    edge_rec(g, e0, q2, qp);
    uint32_t base = qp.x + 1;
    if (r1 >= q.z) {
      r1 -= q.z;
      base = qp.y + 1;
    }
    uint2 e1 = ZG_LDG(&g.adj_e[base + (uint32_t)r1]);
    a1 = 1 + (e1.x == q.x || e1.x == q.y);
  }
  res_mul(r, g.m);
  res_mul(r, S);
  if (a1 == 2) r.shift = 1;
  r.hit = true;
  if (DBG) {
    double p = 1.0;
    p = dmul(p, ddiv(1.0, u2d(g.m)));
    p = dmul(p, ddiv(1.0 * a1, u2d(S)));
    r.w = ddiv(1.0, p);
  }
}

// ---- the canonical-path test of the unbiased 4-clique program (no counterpart in the reference)
// Vertices by slot: 0 = a, 1 = b (e0's ends), 2 = c (e1's new end, e1 hangs off slot s1), 3 = d
// (e2's new end, e2 hangs off slot s2).  The three unsampled pairs must be edges (any id; looked
// up in the order (the other of a and b, c), then the two pairs at d in slot order, up to the first
// missing one, the debug access model counting each look-up), and the sample must be the clique's
// canonical path: id0 the smallest of the six ids, id1 the
// smallest of the four edges joining {a, b} to {c, d}, id2 the smallest id above id1 at d.
template <bool DBG>
__device__ __forceinline__ bool canonical_four_clique(const ZgDevGraph& g, Ctx& c, uint32_t va, uint32_t vb,
                                                      uint32_t vc, uint32_t vd, int s1, int s2, uint32_t id0,
                                                      uint32_t id1, uint32_t id2, const EdgeProbe& pc) {
  auto vslot = [&](int i) { return i == 0 ? va : i == 1 ? vb : i == 2 ? vc : vd; };
  // the unsampled pairs in slot order: (1 - s1, 2), then the two (x, 3) with x != s2
  const int x0 = 1 - s1, x1 = s2 == 0 ? 1 : 0, x2 = s2 == 2 ? 1 : 2;
  int64_t h0, h1 = -1, h2 = -1;
  if (DBG) {
    h0 = edge_confirm(g, edge_candidate(g, vslot(x0), vc));
    c.sectors += model_close(g, vslot(x0), vc);
    c.closures++;
    if (h0 >= 0) {
      h1 = edge_confirm(g, edge_candidate(g, vslot(x1), vd));
      c.sectors += model_close(g, vslot(x1), vd);
      c.closures++;
    }
    if (h0 >= 0 && h1 >= 0) {
      h2 = edge_confirm(g, edge_candidate(g, vslot(x2), vd));
      c.sectors += model_close(g, vslot(x2), vd);
      c.closures++;
    }
  } else {
    const EdgeProbe& p0 = pc;  // the caller's look-up of (slot x0, c)
    if (p0.cand == ZG_HASH_EMPTY) return false;
    EdgeProbe p1 = edge_candidate(g, vslot(x1), vd), p2 = edge_candidate(g, vslot(x2), vd);
    if (p1.cand == ZG_HASH_EMPTY || p2.cand == ZG_HASH_EMPTY) return false;
    h0 = edge_confirm(g, p0);
    h1 = edge_confirm(g, p1);
    h2 = edge_confirm(g, p2);
  }
  if (h0 < 0 || h1 < 0 || h2 < 0) return false;
  const uint32_t i_c = (uint32_t)h0, i_x1 = (uint32_t)h1, i_x2 = (uint32_t)h2;
  // ids of the pairs at d by slot: the sampled one (s2) and the two looked up
  const uint32_t d0 = s2 == 0 ? id2 : (x1 == 0 ? i_x1 : i_x2);
  const uint32_t d1 = s2 == 1 ? id2 : (x1 == 1 ? i_x1 : i_x2);
  const uint32_t d2 = s2 == 2 ? id2 : (x1 == 2 ? i_x1 : i_x2);
  // (i) e0 is the smallest (e1, e2 are larger by construction)
  if (i_c < id0 || i_x1 < id0 || i_x2 < id0) return false;
  // (ii) e1 is the smallest of {a, b} x {c, d}: the other {a, b}-c edge and both {a, b}-d edges
  if (i_c < id1 || d0 < id1 || d1 < id1) return false;
  // (iii) no edge at d with an id strictly between id1 and id2
  if ((d0 > id1 && d0 < id2) || (d1 > id1 && d1 < id2) || (d2 > id1 && d2 < id2)) return false;
  return true;
}

// ---- FourClique: applications/FourClique.cpp:176-234 -------------------------------------
// Vertices in insertion order a (e0.src), b (e0.dst), c (e1's new end), d (e2's new end); all
// state in scalars (no dynamically indexed arrays, which would live in local memory).
template <bool DBG, bool UNBIASED = false>
__device__ void prog_four_clique(const ZgDevGraph& g, Ctx& c, Res& r) {
  if (g.m == 0) {
    r.fail = true;
    return;
  }
  const uint64_t w1 = c.word(1);  // the second draw's Philox work overlaps the first loads
  // (the third draw's is done where it is needed: most samples end before it)
  uint64_t e0 = c.draw(0, g.m - 1);
  uint4 q, qp;
  edge_rec(g, e0, q, qp);
  uint64_t S1 = (uint64_t)q.z + q.w;
  if (DBG) c.sectors += 1 + model_anchor(g, q.x) + model_anchor(g, q.y);
  if (S1 == 0) {
    r.fail = true;
    return;
  }
  if (DBG) c.sectors += 1;
  uint64_t r1 = c.take(w1, 0, S1 - 1);
  const uint32_t va = q.x, vb = q.y;
  const bool s1b = r1 >= q.z;  // the first conditional edge hangs off b
  const uint32_t r1o = (uint32_t)(s1b ? r1 - q.z : r1);  // its place among the anchor's entries after e0
  const uint32_t suf_own = s1b ? q.w : q.z, suf_oth = s1b ? q.z : q.w;
  const uint32_t base_own = after_edge(g, q, qp, s1b);  // the anchor's first entry after e0
  const uint32_t idx1 = base_own + r1o;
  uint2 e1 = ZG_LDG(&g.adj_e[idx1]);
  const uint32_t vc = e1.x;
  uint32_t a1 = 1 + (vc == va || vc == vb);
  res_mul(r, g.m);
  res_mul(r, S1);
  if (a1 == 2) r.shift++;
  // Every hit of either program is a 4-clique and so contains the pair (x0, c), x0 the end of e0
  // that e1 does not hang off.  Its two buckets are read before the second step: when neither
  // holds its fingerprint the pair is absent and the sample is a miss, unless the second step has
  // no candidate at all (then it fails, as below).  With entries after e1 left in the anchor's own
  // list that cannot happen, and the sample ends here; the counters are those of the full path.
  const uint32_t x0 = s1b ? va : vb;
  const uint32_t own = suf_own - r1o - 1;  // the anchor's entries after e1
  EdgeProbe p0{0ull, ZG_HASH_EMPTY};
  if (!DBG) {
    // near-L2 graphs (compact records): both buckets in one step; graphs read from HBM (wide):
    // the first bucket, the second behind its overflow flag (fewer sectors).  Measured: R-MAT
    // scale 20 1.88 vs 1.92 ms, R-MAT scale 26 631.6 vs 622.4 ms per batch.
    p0 = g.wide ? edge_candidate(g, x0, vc) : edge_candidate_both(g, x0, vc);
    if (p0.cand == ZG_HASH_EMPTY && own != 0) return;
  }
  // second conditional step: anchors [a, b, c], min_valid = id1 + 1
  uint32_t mv = e1.y + 1;
  const EdgeAt ac = edge_at(g, e1.y, vc);
  const uint32_t lbC = ac.pos + 1;  // c's entries after e1
  const uint32_t endC = lbC + ac.suf;
  // the anchor's own list continues right after e1; the other endpoint's list needs a search
  // (that suffix holds edge ids in [id0 + 1, m - 1])
  const uint32_t base_oth = after_edge(g, q, qp, !s1b);
  const uint32_t end_own = base_own + suf_own, end_oth = base_oth + suf_oth;
  if (!DBG && p0.cand == ZG_HASH_EMPTY) {
    // a miss or a failure, nothing else: the step has a candidate unless c has no entries after
    // e1 and the other endpoint's largest id after e0 (its list's last entry) is below id1 + 1
    const bool any = (a1 == 1 && ac.suf != 0) || (suf_oth != 0 && ZG_LDG(&g.adj_e[end_oth - 1]).y >= mv);
    r.fail = !any;
    return;
  }
  uint32_t lo = lb_eid(g.adj_e, base_oth, end_oth, mv, (uint32_t)e0 + 1, (uint32_t)(g.m - 1));
  uint32_t lbA = s1b ? lo : idx1 + 1, lbB = s1b ? idx1 + 1 : lo;
  uint64_t lenA = (s1b ? end_oth : end_own) - lbA, lenB = (s1b ? end_own : end_oth) - lbB;
  // when c coincides with a or b (duplicate edges) the reference lists only two vertices
  uint64_t lenC = a1 == 1 ? (uint64_t)(endC - lbC) : 0;
  uint64_t S2 = lenA + lenB + lenC;
  if (DBG) c.sectors += model_anchor(g, va) + model_anchor(g, vb) + (a1 == 1 ? model_anchor(g, vc) : 0);
  if (S2 == 0) {
    r.fail = true;
    return;
  }
  if (DBG) c.sectors += 1;
  uint64_t r2 = c.take(c.word(2), 0, S2 - 1);
  int s2;
  uint32_t pos2;
  if (r2 < lenA) {
    s2 = 0;
    pos2 = lbA + (uint32_t)r2;
  } else if (r2 - lenA < lenB) {
    s2 = 1;
    pos2 = lbB + (uint32_t)(r2 - lenA);
  } else {
    s2 = 2;
    pos2 = lbC + (uint32_t)(r2 - lenA - lenB);
  }
  uint2 e2 = ZG_LDG(&g.adj_e[pos2]);
  const uint32_t vd = e2.x;
  bool dup = vd == va || vd == vb || (a1 == 1 && vd == vc);
  uint32_t a2 = 1 + (dup ? 1 : 0);
  res_mul(r, S2);
  if (a2 == 2) r.shift++;
  if (a1 != 1 || dup) return;  // three vertices: a triangle was sampled (FourClique.cpp:224-226)
  if (UNBIASED) {
    r.hit = canonical_four_clique<DBG>(g, c, va, vb, vc, vd, s1b ? 1 : 0, s2, (uint32_t)e0, e1.y, e2.y, p0);
  } else {
    // closure: the 3 vertex pairs not sampled, all with edge id >= id2 + 1.  Sampled pairs are
    // (a,b), (anchor of e1, c) and (anchor of e2, d).  The reference checks the pairs in slot order
    // up to the first miss (the debug access model follows that).
    const int s1 = s1b ? 1 : 0;
    uint32_t mv2 = e2.y + 1;
    auto vslot = [&](int i) { return i == 0 ? va : i == 1 ? vb : i == 2 ? vc : vd; };
    bool ok = true;
    if (DBG) {
      for (int i = 0; i < 4; ++i)
        for (int j = i + 1; j < 4; ++j) {
          bool sampled = (i == 0 && j == 1) || (i == s1 && j == 2) || (i == s2 && j == 3);
          if (!sampled && ok) {
            ok = edge_after(g, vslot(i), vslot(j), mv2);
            c.sectors += model_close(g, vslot(i), vslot(j));
            c.closures++;
          }
        }
    } else {
      // (x0, c) has a candidate (p0, read above); the two pairs (?, d) other than e2's own
      uint32_t x1 = vslot(s2 == 0 ? 1 : 0);
      uint32_t x2 = vslot(s2 == 2 ? 1 : 2);
      EdgeProbe p1 = edge_candidate(g, x1, vd), p2 = edge_candidate(g, x2, vd);
      ok = p1.cand != ZG_HASH_EMPTY && p2.cand != ZG_HASH_EMPTY;
      if (ok)
        ok = edge_confirm(g, p0) >= (int64_t)mv2 && edge_confirm(g, p1) >= (int64_t)mv2 &&
             edge_confirm(g, p2) >= (int64_t)mv2;
    }
    r.hit = ok;
  }
  if (DBG && r.hit) {
    double p = 1.0;
    p = dmul(p, ddiv(1.0, u2d(g.m)));
    p = dmul(p, ddiv(1.0 * a1, u2d(S1)));
    p = dmul(p, ddiv(1.0 * a2, u2d(S2)));
    r.w = ddiv(1.0, p);
  }
}

// ---- FourChain: applications/FourChain.cpp:24-124 ----------------------------------------
// sel_known: the program draw (1..3) when the caller has already drawn it, else 0.
template <bool DBG>
__device__ void prog_four_chain(const ZgDevGraph& g, Ctx& c, Res& r, uint32_t sel_known = 0) {
  const uint64_t w2 = c.word(2), w3 = c.word(3);  // Philox work of the later draws, up front
  uint64_t sel;
  if (sel_known) {
    sel = sel_known;
    ++c.nd;
  } else {
    sel = c.draw(1, 3);
  }
  res_mul(r, 3);
  if (g.m == 0) {
    r.fail = true;
    return;
  }
  uint64_t e0 = c.draw(0, g.m - 1);
  res_mul(r, g.m);
  uint4 q, qp;
  edge_rec(g, e0, q, qp);
  const uint32_t a = q.x, b = q.y;
  if (!DBG && sel == 3) {
    // vertices [a] give e1, vertices [b] give e2: both entries' addresses follow from e0's record,
    // so their loads go out together (the same counters as the shared chain below)
    const uint64_t S1 = q.z, S2 = q.w;
    if (S1 == 0 || S2 == 0) {
      r.fail = true;
      return;
    }
    const uint64_t r1 = c.take(w2, 0, S1 - 1), r2 = c.take(w3, 0, S2 - 1);
    const uint2 e1 = ZG_LDG(&g.adj_e[after_edge(g, q, qp, false) + (uint32_t)r1]);
    const uint2 e2 = ZG_LDG(&g.adj_e[after_edge(g, q, qp, true) + (uint32_t)r2]);
    res_mul(r, S1);
    if (e1.x == a) r.shift++;
    res_mul(r, S2);
    if (e2.x == b) r.shift++;
    r.hit = !(b == a || b == e1.x) && !(e2.x == a || e2.x == e1.x);
    return;
  }
  if (DBG) c.sectors += 1;
  // The three programs share one chain of dependent loads (edge record, [anchor offset,] e1,
  // [e1's record and] the second anchor's offset, e2; bracketed reads: compact layout or some
  // programs only) so a warp whose lanes drew different programs walks it once.
  //   sel 1, 2: vertices [a, b] give e1; its far end nw gives e2 (edges [e0, e1] resp. [e0])
  //   sel 3:    vertices [a] give e1; vertices [b] give e2 (edges [e0])
  const bool split = sel == 3;
  const uint64_t S1 = split ? (uint64_t)q.z : (uint64_t)q.z + q.w;
  if (DBG) c.sectors += model_anchor(g, a) + (split ? 0 : model_anchor(g, b));
  if (S1 == 0) {
    r.fail = true;
    return;
  }
  if (DBG) c.sectors += 1;
  uint64_t r1 = c.take(w2, 0, S1 - 1);
  const bool on_b = !split && r1 >= q.z;  // e1 hangs off b
  if (on_b) r1 -= q.z;
  const uint32_t anchor = on_b ? b : a;
  const uint2 e1 = ZG_LDG(&g.adj_e[after_edge(g, q, qp, on_b) + (uint32_t)r1]);
  const uint32_t a1 = 1 + (e1.x == a || (!split && e1.x == b));
  res_mul(r, S1);
  if (a1 == 2) r.shift++;
  // the second step's anchor: b, or the vertex of e1 not shared with e0 (FourChain.cpp:44-54)
  uint32_t v2;
  if (split) v2 = b;
  else if (a == anchor) v2 = e1.x;
  else if (a == e1.x) v2 = anchor;
  else if (b == anchor) v2 = e1.x;
  else v2 = anchor;
  uint32_t lb2, end2;
  if (split) {
    lb2 = after_edge(g, q, qp, true);  // sel 3: b's entries after e0
    end2 = lb2 + q.w;
  } else {
    const EdgeAt a1v = edge_at(g, e1.y, v2);  // e1 in v2's list
    lb2 = a1v.pos + 1;                          // sel 1: min_valid = id1 + 1
    end2 = lb2 + a1v.suf;
    if (sel == 2)  // min_valid = id0 + 1, at or before e1's own slot in v2's list
      lb2 = lb_eid_win(g.adj_e, edge_at_start(g, a1v, v2), lb2, (uint32_t)e0 + 1, 0u, e1.y);
  }
  const uint64_t S2 = (uint64_t)(end2 - lb2);
  if (DBG) c.sectors += model_anchor(g, v2);
  if (S2 == 0) {
    r.fail = true;
    return;
  }
  if (DBG) c.sectors += 1;
  const uint64_t r2 = c.take(w3, 0, S2 - 1);
  const uint2 e2 = ZG_LDG(&g.adj_e[lb2 + (uint32_t)r2]);
  const uint32_t a2 = 1 + (e2.x == v2);
  res_mul(r, S2);
  if (a2 == 2) r.shift++;
  bool ok;
  if (split) {
    ok = !(b == a || b == e1.x) && !(e2.x == a || e2.x == e1.x);
  } else {
    ok = !(v2 == a || v2 == b) && !(e2.x == a || e2.x == b);
    if (sel == 2) ok = ok && !(e2.y >= e1.y);
  }
  r.hit = ok;
  if (DBG && ok) {
    double p = 1. / 3;
    p = dmul(p, ddiv(1.0, u2d(g.m)));
    p = dmul(p, ddiv(1.0 * a1, u2d(S1)));
    p = dmul(p, ddiv(1.0 * a2, u2d(S2)));
    r.w = ddiv(1.0, p);
  }
}

// canonicality_check (applications/ChainMining.cpp:218-235, src/SamplerGenerator.cpp:368-385)
__device__ __forceinline__ bool canonical(const uint32_t* es, const uint32_t* ed, const uint32_t* ei, int ne,
                                          uint32_t s, uint32_t d, uint32_t id) {
  if (ne <= 1) return true;
  bool found = false;
  for (int i = 0; i < ne; ++i) {
    if (!found) {
      if (s == es[i] || s == ed[i] || d == es[i] || d == ed[i]) found = true;
    } else if (ei[i] >= id) {
      return false;
    }
  }
  return true;
}


// Two 4-chain samples of the same program (sel, already drawn by the caller) per thread, their
// dependent-load chains interleaved stage by stage so that each stage's loads of both samples are
// in flight together: the same draws, tests and weights as prog_four_chain<false> on each.
template <int N>
__device__ __forceinline__ void prog_four_chain_n(const ZgDevGraph& g, Ctx (&c)[N], Res (&r)[N], uint32_t sel) {
  uint64_t w2[N], w3[N], e0[N];
  uint4 q[N], qp[N];
  bool live[N];
#pragma unroll
  for (int i = 0; i < N; ++i) {
    w2[i] = c[i].word(2);
    w3[i] = c[i].word(3);
    ++c[i].nd;  // the program draw
    res_mul(r[i], 3);
    live[i] = g.m != 0;
    if (!live[i]) r[i].fail = true;
  }
#pragma unroll
  for (int i = 0; i < N; ++i)
    if (live[i]) {
      e0[i] = c[i].draw(0, g.m - 1);
      res_mul(r[i], g.m);
      edge_rec(g, e0[i], q[i], qp[i]);
    }
  if (sel == 3) {  // vertices [a] give e1, vertices [b] give e2: both loads at once
    uint2 e1[N], e2[N];
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (live[i]) {
        const uint64_t S1 = q[i].z, S2 = q[i].w;
        if (S1 == 0 || S2 == 0) {
          r[i].fail = true;
          live[i] = false;
          continue;
        }
        const uint64_t r1 = c[i].take(w2[i], 0, S1 - 1), r2 = c[i].take(w3[i], 0, S2 - 1);
        e1[i] = ZG_LDG(&g.adj_e[after_edge(g, q[i], qp[i], false) + (uint32_t)r1]);
        e2[i] = ZG_LDG(&g.adj_e[after_edge(g, q[i], qp[i], true) + (uint32_t)r2]);
        res_mul(r[i], S1);
        res_mul(r[i], S2);
      }
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (live[i]) {
        const uint32_t a = q[i].x, b = q[i].y;
        if (e1[i].x == a) r[i].shift++;
        if (e2[i].x == b) r[i].shift++;
        r[i].hit = !(b == a || b == e1[i].x) && !(e2[i].x == a || e2[i].x == e1[i].x);
      }
    return;
  }
  // sel 1, 2: vertices [a, b] give e1; its far end v2 gives e2
  uint2 e1[N];
  uint32_t v2[N];
#pragma unroll
  for (int i = 0; i < N; ++i)
    if (live[i]) {
      const uint64_t S1 = (uint64_t)q[i].z + q[i].w;
      if (S1 == 0) {
        r[i].fail = true;
        live[i] = false;
        continue;
      }
      uint64_t r1 = c[i].take(w2[i], 0, S1 - 1);
      const bool on_b = r1 >= q[i].z;
      if (on_b) r1 -= q[i].z;
      e1[i] = ZG_LDG(&g.adj_e[after_edge(g, q[i], qp[i], on_b) + (uint32_t)r1]);
      res_mul(r[i], S1);
      v2[i] = on_b ? q[i].y : q[i].x;  // the anchor, resolved below
    }
  EdgeAt a1v[N];
#pragma unroll
  for (int i = 0; i < N; ++i)
    if (live[i]) {
      const uint32_t a = q[i].x, b = q[i].y, anchor = v2[i];
      if (e1[i].x == a || e1[i].x == b) r[i].shift++;
      // the second step's anchor: the vertex of e1 not shared with e0 (FourChain.cpp:44-54)
      uint32_t v;
      if (a == anchor) v = e1[i].x;
      else if (a == e1[i].x) v = anchor;
      else if (b == anchor) v = e1[i].x;
      else v = anchor;
      v2[i] = v;
      a1v[i] = edge_at(g, e1[i].y, v);  // e1 in v's list
    }
  uint32_t lb2[N], end2[N];
#pragma unroll
  for (int i = 0; i < N; ++i)
    if (live[i]) {
      lb2[i] = a1v[i].pos + 1;  // sel 1: min_valid = id1 + 1
      end2[i] = lb2[i] + a1v[i].suf;
      if (sel == 2)  // min_valid = id0 + 1, at or before e1's own slot in v2's list
        lb2[i] = lb_eid_win(g.adj_e, edge_at_start(g, a1v[i], v2[i]), lb2[i], (uint32_t)e0[i] + 1, 0u, e1[i].y);
    }
  uint2 e2[N];
#pragma unroll
  for (int i = 0; i < N; ++i)
    if (live[i]) {
      const uint64_t S2 = (uint64_t)(end2[i] - lb2[i]);
      if (S2 == 0) {
        r[i].fail = true;
        live[i] = false;
        continue;
      }
      const uint64_t r2 = c[i].take(w3[i], 0, S2 - 1);
      e2[i] = ZG_LDG(&g.adj_e[lb2[i] + (uint32_t)r2]);
      res_mul(r[i], S2);
    }
#pragma unroll
  for (int i = 0; i < N; ++i)
    if (live[i]) {
      const uint32_t a = q[i].x, b = q[i].y;
      if (e2[i].x == v2[i]) r[i].shift++;
      bool ok = !(v2[i] == a || v2[i] == b) && !(e2[i].x == a || e2[i].x == b);
      if (sel == 2) ok = ok && !(e2[i].y >= e1[i].y);
      r[i].hit = ok;
    }
}
// ---- ChainMining: applications/ChainMining.cpp:240-84 ------------------------------------
template <bool DBG>
__device__ void prog_chain(const ZgDevGraph& g, int order, Ctx& c, Res& r) {
  if (g.m == 0) {
    r.fail = true;
    return;
  }
  uint64_t e0 = c.draw(0, g.m - 1);
  res_mul(r, g.m);
  uint4 q, qp;
  edge_rec(g, e0, q, qp);
  uint32_t es[ZG_MAX_LIST], ed[ZG_MAX_LIST], ei[ZG_MAX_LIST];
  uint32_t vs[ZG_MAX_LIST];
  int ne = 1, nvtx = 2;
  es[0] = q.x;
  ed[0] = q.y;
  ei[0] = (uint32_t)e0;
  vs[0] = q.x;
  vs[1] = q.y;
  uint32_t f[2] = {q.x, q.y};
  uint32_t fe[2], fl[2];
  fl[0] = qp.x + 1;
  fl[1] = qp.y + 1;
  fe[0] = fl[0] + q.z;
  fe[1] = fl[1] + q.w;
  Ext p;
  if (DBG) p = ext_from_double(ddiv(1.0, u2d(g.m)));
  if (DBG) c.sectors += 1;
  uint32_t mv = (uint32_t)e0 + 1;
  for (int i = 0; i < order - 2; ++i) {
    uint64_t l0 = (uint64_t)(fe[0] - fl[0]), l1 = (uint64_t)(fe[1] - fl[1]);
    uint64_t S = l0 + l1;
    if (DBG) c.sectors += model_anchor(g, f[0]) + model_anchor(g, f[1]);
    if (S == 0) {
      r.fail = true;
      return;
    }
    if (DBG) c.sectors += 1;
    uint64_t rr = c.draw(0, S - 1);
    int side = 0;
    if (rr >= l0) {
      rr -= l0;
      side = 1;
    }
    uint2 e = ZG_LDG(&g.adj_e[fl[side] + (uint32_t)rr]);
    uint32_t src = f[side];
    uint32_t av = (f[0] == src) + (f[1] == src) + (f[0] == e.x) + (f[1] == e.x);
    res_mul(r, S);
    if (av == 2) r.shift++;
    if (DBG) p = ext_mul(p, ext_from_double(ddiv(1.0 * av, u2d(S))));
    if (!canonical(es, ed, ei, ne, src, e.x, e.y)) return;
    es[ne] = src;
    ed[ne] = e.x;
    ei[ne] = e.y;
    ++ne;
    bool seen = false;
    for (int k = 0; k < nvtx; ++k) seen |= (vs[k] == e.x);
    if (!seen) vs[nvtx++] = e.x;
    if (nvtx != i + 3) return;
    // frontier update (ChainMining.cpp:265-80); here src is a frontier vertex and e.x is new
    int upd = (f[0] == src) ? 0 : 1;
    f[upd] = e.x;
    if (!DBG && i + 1 >= order - 2) break;  // the last step: the new frontier's range is not used
    const EdgeAt ae = edge_at(g, e.y, e.x);  // e in the new frontier's list
    fe[upd] = ae.pos + 1 + ae.suf;
    fl[upd] = lb_eid(g.adj_e, edge_at_start(g, ae, e.x), ae.pos + 1, mv, 0u, e.y);
  }
  r.hit = true;
  if (DBG) r.w = ext_to_double(ext_inv(p));
}

// ---- SamplerGenerator<Empty>::estimate: src/SamplerGenerator.cpp:461-546 ----------------
__device__ __forceinline__ uint32_t pair_bit(uint32_t i, uint32_t j, uint32_t pv) {
  if (i > j) {
    uint32_t t = i;
    i = j;
    j = t;
  }
  return i * (2 * pv - i - 1) / 2 + (j - i - 1);
}

// prog_pattern for patterns of at most MV vertices and ME edges with every per-sample array in
// registers: loops run to the compile-time bounds under guards, writes at a run-time position go
// to every slot under a predicate, and the sampled edges are kept as the vertex slots of their
// ends (4 bits each, packed) plus their edge ids.  Same draws, same tests in the same order as
// prog_pattern (the canonicality test compares vertex slots: the vertices are distinct).
template <int MV, int ME>
__device__ void prog_pattern_small(const ZgDevGraph& g, const ZgProgParams& pp, Ctx& c, Res& r) {
  uint64_t e0 = c.draw(0, g.m - 1);
  res_mul(r, g.m);
  uint4 q, qp;
  edge_rec(g, e0, q, qp);
  uint32_t vs[MV], vl[MV], ve[MV], ei[ME];
#pragma unroll
  for (int i = 0; i < MV; ++i) vs[i] = vl[i] = ve[i] = 0;
#pragma unroll
  for (int i = 0; i < ME; ++i) ei[i] = 0;
  vs[0] = q.x;
  vs[1] = q.y;
  vl[0] = qp.x + 1;
  vl[1] = qp.y + 1;
  ve[0] = vl[0] + q.z;
  ve[1] = vl[1] + q.w;
  uint32_t es = 0u, ed = 1u;  // edge k's end slots at bits 4k..4k+3
  ei[0] = (uint32_t)e0;
  const uint32_t mv = (uint32_t)e0 + 1;
  int nvtx = 2, ne = 1;
#pragma unroll
  for (int k = 1; k < ME; ++k) {
    if ((uint32_t)k >= pp.pe) break;
    uint64_t S = 0;
#pragma unroll
    for (int i = 0; i < MV; ++i) S += i < nvtx ? (uint64_t)(ve[i] - vl[i]) : 0ull;
    if (S == 0) {
      r.fail = true;
      return;
    }
    uint64_t rr = c.draw(0, S - 1);
    // the anchor slot: the first whose entries hold rr (prog_pattern's scan, unrolled)
    int side = nvtx - 1;
    uint32_t base = 0, src = 0;
    bool done = false;
#pragma unroll
    for (int i = 0; i < MV - 1; ++i) {
      const uint64_t len = (uint64_t)(ve[i] - vl[i]);
      const bool here = !done && i < nvtx - 1 && rr < len;
      if (!done && i < nvtx - 1 && !here) rr -= len;
      if (here) side = i;
      done = done || here || i >= nvtx - 1;
    }
#pragma unroll
    for (int i = 0; i < MV; ++i)
      if (i == side) {
        base = vl[i];
        src = vs[i];
      }
    uint2 e = ZG_LDG(&g.adj_e[base + (uint32_t)rr]);
    int nbr_slot = -1;
#pragma unroll
    for (int i = 0; i < MV; ++i)
      if (i < nvtx && vs[i] == e.x) nbr_slot = i;
    res_mul(r, S);
    if (nbr_slot >= 0) r.shift++;
    // canonicality_check (src/SamplerGenerator.cpp:368-385) on vertex slots
    const int ds = nbr_slot >= 0 ? nbr_slot : nvtx;  // the new edge's far end (a new slot if new)
    if (ne > 1) {
      bool found = false, canon = true;
#pragma unroll
      for (int i = 0; i < ME; ++i) {
        if (i >= ne) break;
        const int a = (int)((es >> (4 * i)) & 15u), b = (int)((ed >> (4 * i)) & 15u);
        if (!found) {
          if (side == a || side == b || ds == a || ds == b) found = true;
        } else if (ei[i] >= e.y) {
          canon = false;
        }
      }
      if (!canon) return;
    }
    es |= (uint32_t)side << (4 * ne);
    ed |= (uint32_t)ds << (4 * ne);
#pragma unroll
    for (int i = 0; i < ME; ++i)
      if (i == ne) ei[i] = e.y;
    ++ne;
    if (nbr_slot < 0) {
      if (nvtx >= MV) return;  // more vertices than the pattern (pv <= MV): not a hit
      // the new vertex's list range past min_valid: needed only if another step draws from it.
      // Its list comes from the vertex offsets, not from the sampled edge's record: the vertex is
      // reached through a random edge, so high-degree vertices come up most often and their
      // offsets tend to be L2 hits, where the record of a random edge is a DRAM read.  The bound
      // is searched over the whole list (the sampled edge, id >= min_valid, lies in it).
      uint32_t nve = 0, nvl = 0;
      if ((uint32_t)k + 1 < pp.pe) {
        const uint32_t ls = ZG_LDG(&g.off32[e.x]);
        nve = ZG_LDG(&g.off32[e.x + 1]);
        nvl = lb_eid(g.adj_e, ls, nve, mv, 0u, (uint32_t)(g.m - 1));
      }
#pragma unroll
      for (int i = 0; i < MV; ++i)
        if (i == nvtx) {
          vs[i] = e.x;
          ve[i] = nve;
          vl[i] = nvl;
        }
      ++nvtx;
      if ((uint32_t)nvtx > pp.pv) return;
    }
  }
  if ((uint32_t)nvtx != pp.pv) return;
  // relabel by ascending vertex id (SamplerGenerator.cpp:493-527) and test the edge set
  uint32_t rank[MV];
#pragma unroll
  for (int i = 0; i < MV; ++i) {
    uint32_t rk = 0;
#pragma unroll
    for (int j = 0; j < MV; ++j) rk += (j < nvtx && vs[j] < vs[i]) ? 1u : 0u;
    rank[i] = rk;
  }
  uint32_t mask = 0;
#pragma unroll
  for (int k = 0; k < ME; ++k) {
    if (k >= ne) break;
    const int a = (int)((es >> (4 * k)) & 15u), b = (int)((ed >> (4 * k)) & 15u);
    uint32_t ri = 0, rj = 0;
#pragma unroll
    for (int i = 0; i < MV; ++i) {
      if (i == a) ri = rank[i];
      if (i == b) rj = rank[i];
    }
    mask |= 1u << pair_bit(ri, rj, pp.pv);
  }
  int lo = 0, hi = (int)pp.num_unique;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (ZG_LDG(&pp.masks[mid]) < mask)
      lo = mid + 1;
    else
      hi = mid;
  }
  r.hit = lo < (int)pp.num_unique && ZG_LDG(&pp.masks[lo]) == mask;
}

template <bool DBG>
__device__ void prog_pattern(const ZgDevGraph& g, const ZgProgParams& pp, Ctx& c, Res& r) {
  if (g.m == 0) {
    r.fail = true;
    return;
  }
  if (!DBG && pp.pv <= 5 && pp.pe <= 6) {  // 5-star, 5-house, triangle, ...: registers only
    prog_pattern_small<5, 6>(g, pp, c, r);
    return;
  }
  uint64_t e0 = c.draw(0, g.m - 1);
  res_mul(r, g.m);
  uint4 q, qp;
  edge_rec(g, e0, q, qp);
  const int MV = ZG_MAX_PATTERN_V + 1;
  uint32_t vs[MV];
  uint32_t vl[MV], ve[MV];
  uint32_t es[ZG_MAX_LIST], ed[ZG_MAX_LIST], ei[ZG_MAX_LIST];
  int nvtx = 2, ne = 1;
  vs[0] = q.x;
  vs[1] = q.y;
  vl[0] = qp.x + 1;
  vl[1] = qp.y + 1;
  ve[0] = vl[0] + q.z;
  ve[1] = vl[1] + q.w;
  es[0] = q.x;
  ed[0] = q.y;
  ei[0] = (uint32_t)e0;
  uint32_t mv = (uint32_t)e0 + 1;
  double p = 1.0;
  if (DBG) p = dmul(p, ddiv(1.0, u2d(g.m)));
  if (DBG) c.sectors += 1;
  for (uint32_t k = 1; k < pp.pe; ++k) {
    uint64_t S = 0;
    for (int i = 0; i < nvtx; ++i) S += (uint64_t)(ve[i] - vl[i]);
    if (DBG)
      for (int i = 0; i < nvtx; ++i) c.sectors += model_anchor(g, vs[i]);
    if (S == 0) {
      r.fail = true;
      return;
    }
    if (DBG) c.sectors += 1;
    uint64_t rr = c.draw(0, S - 1);
    int side = 0;
    for (; side < nvtx - 1; ++side) {
      uint64_t len = (uint64_t)(ve[side] - vl[side]);
      if (rr < len) break;
      rr -= len;
    }
    uint2 e = ZG_LDG(&g.adj_e[vl[side] + (uint32_t)rr]);
    uint32_t src = vs[side];
    int nbr_slot = -1;
    for (int i = 0; i < nvtx; ++i)
      if (vs[i] == e.x) nbr_slot = i;
    uint32_t av = 1 + (nbr_slot >= 0);
    res_mul(r, S);
    if (av == 2) r.shift++;
    if (DBG) p = dmul(p, ddiv(1.0 * av, u2d(S)));
    if (!canonical(es, ed, ei, ne, src, e.x, e.y)) return;
    es[ne] = src;
    ed[ne] = e.x;
    ei[ne] = e.y;
    ++ne;
    if (nbr_slot < 0) {
      vs[nvtx] = e.x;
      const EdgeAt ae = edge_at(g, e.y, e.x);  // e in the new vertex's list
      ve[nvtx] = ae.pos + 1 + ae.suf;
      vl[nvtx] = lb_eid(g.adj_e, edge_at_start(g, ae, e.x), ae.pos + 1, mv, 0u, e.y);
      ++nvtx;
      if ((uint32_t)nvtx > pp.pv) return;
    }
  }
  if ((uint32_t)nvtx != pp.pv) return;
  // relabel by ascending vertex id (SamplerGenerator.cpp:493-527) and test the edge set
  uint32_t rank[MV];
  for (int i = 0; i < nvtx; ++i) {
    uint32_t rk = 0;
    for (int j = 0; j < nvtx; ++j) rk += vs[j] < vs[i];
    rank[i] = rk;
  }
  uint32_t mask = 0;
  for (int k = 0; k < ne; ++k) {
    uint32_t ri = 0, rj = 0;
    for (int i = 0; i < nvtx; ++i) {
      if (vs[i] == es[k]) ri = rank[i];
      if (vs[i] == ed[k]) rj = rank[i];
    }
    mask |= 1u << pair_bit(ri, rj, pp.pv);
  }
  int lo = 0, hi = (int)pp.num_unique;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (ZG_LDG(&pp.masks[mid]) < mask)
      lo = mid + 1;
    else
      hi = mid;
  }
  bool ok = lo < (int)pp.num_unique && ZG_LDG(&pp.masks[lo]) == mask;
  r.hit = ok;
  if (DBG && ok) r.w = ddiv(1.0, p);
}

// ---- per-thread exact accumulation and block reduction ----------------------------------
// Per-thread state kept small: one thread handles < 2^32 estimators, so 32-bit counters.
struct Acc {
  uint32_t samples, hits, fails, ovf;
  uint64_t s[4];
  double sw2;  // the mean's sum is the exact s[]; only the variance terms are doubles
  double sw4;  // sum of w^4: the uncertainty of the variance (heavy-tailed weights)
};

__device__ __forceinline__ void acc_init(Acc& a) {
  a.samples = a.hits = a.fails = a.ovf = 0;
  a.s[0] = a.s[1] = a.s[2] = a.s[3] = 0;
  a.sw2 = 0.0;
  a.sw4 = 0.0;
}

// num / 2^shift as a double truncated to 53 bits, built from integer operations only: GB300's
// FP64 pipe is narrow, and this runs once per hit (the variance terms; the mean is exact).
__device__ __forceinline__ double u192_scaled_to_double(const ZgU192& n, uint32_t shift) {
  uint64_t top = n.l[0], next = 0;
  int base = 0;
  if (n.l[2]) {
    top = n.l[2];
    next = n.l[1];
    base = 128;
  } else if (n.l[1]) {
    top = n.l[1];
    next = n.l[0];
    base = 64;
  }
  if (top == 0) return 0.0;
  int lz = __clzll(top);
  uint64_t mant = (top << lz) | (lz ? next >> (64 - lz) : 0ull);
  int64_t e = (int64_t)base + 63 - lz - (int64_t)shift;  // value = mant * 2^(e - 63)
  uint64_t bits = ((uint64_t)(e + 1023) << 52) | ((mant >> 11) & ((1ull << 52) - 1));
  return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ void acc_add(Acc& a, const Res& r, uint32_t den) {
  a.samples++;
  a.fails += r.fail;
  if (!r.hit) return;
  a.hits++;
  a.ovf += r.ovf;
  uint32_t sh = den - r.shift;  // < 64
  uint64_t v0 = r.num.l[0] << sh;
  uint64_t v1 = sh ? (r.num.l[1] << sh) | (r.num.l[0] >> (64 - sh)) : r.num.l[1];
  uint64_t v2 = sh ? (r.num.l[2] << sh) | (r.num.l[1] >> (64 - sh)) : r.num.l[2];
  uint64_t v3 = sh ? (r.num.l[2] >> (64 - sh)) : 0;
  asm("add.cc.u64 %0, %0, %4;\n\t"
      "addc.cc.u64 %1, %1, %5;\n\t"
      "addc.cc.u64 %2, %2, %6;\n\t"
      "addc.u64 %3, %3, %7;"
      : "+l"(a.s[0]), "+l"(a.s[1]), "+l"(a.s[2]), "+l"(a.s[3])
      : "l"(v0), "l"(v1), "l"(v2), "l"(v3));
  // sum_w is taken from the exact integer sum at the end; only the square needs the FP64 pipe
  double w = u192_scaled_to_double(r.num, r.shift);
  const double w2 = w * w;
  a.sw2 = fma(w, w, a.sw2);
  a.sw4 = fma(w2, w2, a.sw4);
}

// One thread's counters, 320-bit sum and variance term kept in shared memory (slot threadIdx.x of
// arrays of BLOCK entries) instead of registers: a latency-bound sampling loop then fits a smaller
// register budget, i.e. more resident warps and more loads in flight.  Each thread adds its hits
// in the same order as with acc_add, so the results are identical.
template <int BLOCK>
struct AccSlots {
  unsigned long long s[4][BLOCK];
  double sw2[BLOCK], sw4[BLOCK];
  uint32_t samples[BLOCK], hits[BLOCK], fails[BLOCK], ovf[BLOCK];
};

template <int BLOCK>
__device__ __forceinline__ void acc_slots_init(AccSlots<BLOCK>& sl) {
  const int t = threadIdx.x;
  sl.s[0][t] = sl.s[1][t] = sl.s[2][t] = sl.s[3][t] = 0;
  sl.sw2[t] = 0.0;
  sl.sw4[t] = 0.0;
  sl.samples[t] = sl.hits[t] = sl.fails[t] = sl.ovf[t] = 0;
}

template <int BLOCK>
__device__ __forceinline__ void acc_add_slots(Acc& a, AccSlots<BLOCK>& sl, const Res& r, uint32_t den) {
  const int t = threadIdx.x;
  sl.samples[t]++;
  sl.fails[t] += r.fail;
  if (!r.hit) return;
  sl.hits[t]++;
  sl.ovf[t] += r.ovf;
  uint32_t sh = den - r.shift;  // < 64
  uint64_t v0 = r.num.l[0] << sh;
  uint64_t v1 = sh ? (r.num.l[1] << sh) | (r.num.l[0] >> (64 - sh)) : r.num.l[1];
  uint64_t v2 = sh ? (r.num.l[2] << sh) | (r.num.l[1] >> (64 - sh)) : r.num.l[2];
  uint64_t v3 = sh ? (r.num.l[2] >> (64 - sh)) : 0;
  unsigned long long s0 = sl.s[0][t], s1 = sl.s[1][t], s2 = sl.s[2][t], s3 = sl.s[3][t];
  asm("add.cc.u64 %0, %0, %4;\n\t"
      "addc.cc.u64 %1, %1, %5;\n\t"
      "addc.cc.u64 %2, %2, %6;\n\t"
      "addc.u64 %3, %3, %7;"
      : "+l"(s0), "+l"(s1), "+l"(s2), "+l"(s3)
      : "l"(v0), "l"(v1), "l"(v2), "l"(v3));
  sl.s[0][t] = s0;
  sl.s[1][t] = s1;
  sl.s[2][t] = s2;
  sl.s[3][t] = s3;
  double w = u192_scaled_to_double(r.num, r.shift);
  const double w2 = w * w;
  sl.sw2[t] = fma(w, w, sl.sw2[t]);
  sl.sw4[t] = fma(w2, w2, sl.sw4[t]);
}

// The slots back into the thread's accumulator (after its loop).
template <int BLOCK>
__device__ __forceinline__ void acc_from_slots(Acc& a, const AccSlots<BLOCK>& sl) {
  const int t = threadIdx.x;
  a.samples = sl.samples[t];
  a.hits = sl.hits[t];
  a.fails = sl.fails[t];
  a.ovf = sl.ovf[t];
  a.s[0] = sl.s[0][t];
  a.s[1] = sl.s[1][t];
  a.s[2] = sl.s[2][t];
  a.s[3] = sl.s[3][t];
  a.sw2 = sl.sw2[t];
  a.sw4 = sl.sw4[t];
}

template <int BLOCK>
__device__ void block_reduce_store(Acc& a, ZgPartial* out) {
  unsigned long long v[14];
  v[0] = a.samples;
  v[1] = a.hits;
  v[2] = a.fails;
  v[3] = a.ovf;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    v[4 + 2 * i] = (uint32_t)a.s[i];
    v[5 + 2 * i] = a.s[i] >> 32;
  }
  double d1 = a.sw2, d4 = a.sw4;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int i = 0; i < 12; ++i) v[i] += __shfl_xor_sync(0xffffffffu, v[i], o);
    d1 += __shfl_xor_sync(0xffffffffu, d1, o);
    d4 += __shfl_xor_sync(0xffffffffu, d4, o);
  }
  __shared__ unsigned long long sv[BLOCK / 32][12];
  __shared__ double sd[BLOCK / 32][2];
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < 12; ++i) sv[warp][i] = v[i];
    sd[warp][0] = d1;
    sd[warp][1] = d4;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    ZgPartial p;
    unsigned long long t[12] = {0};
    double s1 = 0, s4 = 0;
    for (int w = 0; w < BLOCK / 32; ++w) {
      for (int i = 0; i < 12; ++i) t[i] += sv[w][i];
      s1 += sd[w][0];
      s4 += sd[w][1];
    }
    p.samples = t[0];
    p.hits = t[1];
    p.fails = t[2];
    p.overflow = t[3];
    for (int i = 0; i < 8; ++i) p.lane[i] = t[4 + i];
    p.sum_w4 = s4;
    p.sum_w2 = s1;
    *out = p;
  }
}


}  // namespace
