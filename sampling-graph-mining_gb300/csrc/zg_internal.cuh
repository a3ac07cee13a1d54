// zg_internal.cuh — shared device/host definitions of libzgraph_gpu.
//
// Device graph layout (all arrays in HBM, built by zg_graph.cu):
//   rec[m]    one record per edge in edge-id order (edge id = position, src/Graph.cpp:295-306), in
//             one of three layouts chosen when the graph is built (results are identical):
//             compact, uint4 (src, dst, suf_src, suf_dst): the COO plus, per endpoint, how many
//               entries follow this edge in that endpoint's edge-id-ordered list;
//             wide, ZgRec (32 bytes, one sector): e = the compact record, p = (pos_src, pos_dst,
//               pre_src, pre_dst), the index of the edge's own entry in adj_e within each
//               endpoint's list and how many entries precede it there;
//             packed (16 bytes): src, dst, suf_src, suf_dst, pos_src, pos_dst as bit fields of
//               two words, w0 = src | dst << V | suf_src << 2V and w1 = suf_dst | pos_src << S |
//               pos_dst << (S + P) (V, S, P: the graph's vertex, suffix and slot bits), where
//               they fit.
//             A conditional step from an edge's endpoints needs S = suf_src + suf_dst and the
//             entries' addresses pos + 1 .. pos + suf: the wide and packed records give both in
//             one read, the compact one needs the endpoints' offsets (off32) as a second,
//             dependent read.  The 16-byte layouts keep graphs whose working set is near the L2
//             size resident; the wide one saves a dependent read and two sectors per step on graphs
//             far larger than L2 (where the packed fields would not fit either).
//   off[V+1]  int64 offsets shared by both adjacency arrays (outgoing_adj_index).
//   adj_e[2m] uint2 (nbr, edge_id) sorted by edge id per vertex (outgoing_adj_list order,
//             asserted at src/Graph.cpp:324-334): the sampling order.  Followed by 8 entries of
//             slack that the windowed search may read but never uses.
//   adj_n[2m] uint2 (nbr, edge_id) sorted by (nbr, edge_id) per vertex (exports, exact counts).
//   w[m]      uint32 edge data (Graph<VertexId>) or null.
//   off32[V+1] the offsets as uint32 (2m < 2^32), read by the compact layout's steps.
//   hent[4B]  the edge set as a two-choice bucketed cuckoo table, B = 2^hbits buckets of 4
//             entries (one 32-byte sector); entry = (fingerprint << 32) | edge id for the key
//             (min(u,v) << 32) | max(u,v) (31-bit fingerprint; bit 63 of slot 0 flags a bucket
//             some of whose keys live in their second bucket).  A closure check ("edge (x,y)
//             exists with id >= min_valid") reads the first bucket, and the second only behind an
//             overflow flag; a fingerprint match is confirmed against the record of that edge id,
//             so the answer is exact.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/zgraph_gpu.h"

#define ZG_STREAM_SHUFFLE 0xFFFFFFF0u
#define ZG_STREAM_SUBSAMPLE 0xFFFFFFF1u

struct __align__(32) ZgRec {
  uint4 e;  // src, dst, suf_src, suf_dst
  uint4 p;  // pos_src, pos_dst, pre_src, pre_dst
};

struct ZgDevGraph {
  uint32_t nv;
  uint32_t hbits;  // log2 of the cuckoo table's bucket count
  uint64_t m;
  const void* rec;  // ZgRec[m] when wide, else uint4[m] (compact) or ulonglong2[m] (packed)
  uint32_t wide;
  uint32_t packed;
  uint32_t pk_v, pk_s, pk_p;  // packed: vertex, suffix and slot field bits
  const int64_t* off;
  const uint2* adj_e;
  const uint2* adj_n;
  const uint32_t* w;
  const uint32_t* off32;
  const unsigned long long* hent;
  uint64_t hseed;
};

#define ZG_HASH_EMPTY 0xFFFFFFFFFFFFFFFFull
// Set in slot 0 of a bucket (never empty then) when an entry whose first bucket it is lives in its
// second bucket: only then can a key absent from its first bucket be in its second.
#define ZG_HASH_OVERFLOW 0x8000000000000000ull

// A packed record's fields: q = (src, dst, suf_src, suf_dst), pos = (pos_src, pos_dst).
__host__ __device__ __forceinline__ void zg_unpack(uint32_t vb, uint32_t sb, uint32_t pb, uint64_t w0, uint64_t w1,
                                                   uint32_t& src, uint32_t& dst, uint32_t& suf_src, uint32_t& suf_dst,
                                                   uint32_t& pos_src, uint32_t& pos_dst) {
  const uint32_t vm = (uint32_t)((1ull << vb) - 1), sm = (uint32_t)((1ull << sb) - 1), pm = (uint32_t)((1ull << pb) - 1);
  src = (uint32_t)w0 & vm;
  dst = (uint32_t)(w0 >> vb) & vm;
  suf_src = (uint32_t)(w0 >> (2 * vb)) & sm;
  suf_dst = (uint32_t)w1 & sm;
  pos_src = (uint32_t)(w1 >> sb) & pm;
  pos_dst = (uint32_t)(w1 >> (sb + pb)) & pm;
}

#ifdef __CUDACC__
// Loads of the sampling programs go through ZG_LDG (read-only path) and, where a load is written
// in inline PTX, name their address in ZG_NOTE_LOAD.  A translation unit that defines ZG_TOUCH
// before including this header gets a copy of the programs that also counts, per thread, the
// 32-byte sectors its loads touch (a sector equal to the thread's previous one is not counted
// again): the bytes the kernel itself moves, the numerator of its roofline (zg_touch.cu).  Every
// other translation unit compiles both as the plain load.
#ifdef ZG_TOUCH
struct ZgTouch {
  unsigned long long last;  // the previous load's last sector
  unsigned long long sectors;
};
// One slot per thread of a block of at most 256 threads (the touch kernels' block size).
__device__ __forceinline__ ZgTouch& zg_touch_state() {
  __shared__ ZgTouch slots[256];
  return slots[threadIdx.x];
}
__device__ __forceinline__ void zg_touch_note(const void* p, uint32_t bytes) {
  ZgTouch& t = zg_touch_state();
  const unsigned long long a = (unsigned long long)p >> 5, b = ((unsigned long long)p + bytes - 1) >> 5;
  t.sectors += b - a + 1 - (a == t.last ? 1 : 0);
  t.last = b;
}
template <typename T>
__device__ __forceinline__ T zg_touch_ldg(const T* p) {
  zg_touch_note(p, sizeof(T));
  return __ldg(p);
}
// The sectors of every thread of a launch, summed.
__device__ unsigned long long zg_touch_total;
#define ZG_LDG(p) zg_touch_ldg(p)
#define ZG_NOTE_LOAD(p, bytes) zg_touch_note((p), (bytes))
#define ZG_TOUCH_BEGIN() (zg_touch_state().last = ~0ull, zg_touch_state().sectors = 0)
#define ZG_TOUCH_END() atomicAdd(&zg_touch_total, zg_touch_state().sectors)
#else
#define ZG_LDG(p) __ldg(p)
#define ZG_NOTE_LOAD(p, bytes) ((void)0)
#define ZG_TOUCH_BEGIN() ((void)0)
#define ZG_TOUCH_END() ((void)0)
#endif

// A packed record of edge e: q = (src, dst, suf_src, suf_dst), pos = (pos_src, pos_dst).
__device__ __forceinline__ void zg_rec_packed(const ZgDevGraph& g, uint64_t e, uint4& q, uint2& pos) {
  const ulonglong2 w = ZG_LDG(&((const ulonglong2*)g.rec)[e]);
  zg_unpack(g.pk_v, g.pk_s, g.pk_p, w.x, w.y, q.x, q.y, q.z, q.w, pos.x, pos.y);
}
// (src, dst, suf_src, suf_dst) of edge e, in any layout.
__device__ __forceinline__ uint4 zg_rec_e(const ZgDevGraph& g, uint64_t e) {
  if (g.packed) {
    uint4 q;
    uint2 pos;
    zg_rec_packed(g, e, q, pos);
    return q;
  }
  return g.wide ? ZG_LDG(&((const ZgRec*)g.rec)[e].e) : ZG_LDG(&((const uint4*)g.rec)[e]);
}
#endif

// splitmix64 finaliser: the cuckoo table's bucket hashes.
__host__ __device__ __forceinline__ uint64_t zg_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t zg_edge_key(uint32_t x, uint32_t y) {
  return x < y ? ((uint64_t)x << 32) | y : ((uint64_t)y << 32) | x;
}
__host__ __device__ __forceinline__ uint32_t zg_bucket1(uint64_t key, uint64_t seed, uint32_t bits) {
  return (uint32_t)(zg_mix64(key ^ seed) >> (64 - bits));
}
__host__ __device__ __forceinline__ uint32_t zg_bucket2(uint64_t key, uint64_t seed, uint32_t bits) {
  return (uint32_t)(zg_mix64(key ^ (seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull)) >> (64 - bits));
}
// 31 bits, never 0x7FFFFFFF (the fingerprint field of an empty entry); bit 31 of an entry's tag is
// its bucket's overflow flag, kept in slot 0 (ZG_HASH_OVERFLOW).
__host__ __device__ __forceinline__ uint32_t zg_fingerprint(uint64_t key, uint64_t seed) {
  uint32_t f = (uint32_t)(zg_mix64(key + seed + 0xD6E8FEB86659FD93ull) >> 33);
  return f == 0x7FFFFFFFu ? 0x3FFFFFFFu : f;
}
__host__ __device__ __forceinline__ uint32_t zg_entry_fp(unsigned long long x) { return (uint32_t)(x >> 32) & 0x7FFFFFFFu; }

struct zg_graph {
  ZgDevGraph d;
  void* rec;
  uint32_t wide;
  uint32_t packed;
  int64_t* off;
  uint2* adj_e;
  uint2* adj_n;
  uint32_t* w;
  uint32_t* off32;
  unsigned long long* hent;
  void* hot;            // one allocation: adj_e, 8 entries of slack (windowed searches), off32
  uint64_t hot_bytes;
  uint64_t num_edges;   // Graph::num_edges metadata
  uint64_t max_degree;  // Graph::max_degree metadata
  uint64_t bytes;
  // degree statistics of the learned profile's features (zg_graph_features), computed on first use
  mutable bool deg_stats_ready;
  mutable double deg_stats[7];  // s1, s2, s3, emin, esum, non-isolated vertices, max degree
};

// Program descriptor (host copy; device parameters are passed by value).
#define ZG_MAX_PATTERN_V 8
#define ZG_MAX_UNIQUE 40320
struct zg_program {
  int kind;
  uint32_t param;
  uint32_t pv, pe;
  uint32_t pedges[2 * ZG_MAX_LIST];
  uint32_t num_unique;
  uint32_t* d_masks;  // sorted unique relabelled edge masks (pattern programs)
};

struct ZgProgParams {
  int kind;
  uint32_t param;
  uint32_t pv, pe;
  uint32_t num_unique;
  const uint32_t* masks;
  uint32_t den_log2;
};

// Per-block partial of one run; reduced by a single-block finalize kernel.
struct ZgPartial {
  unsigned long long samples, hits, fails, overflow;
  unsigned long long lane[8];  // 32-bit halves of the exact 256-bit sum, carry-saved
  double sum_w4, sum_w2;  // sums of (1/p)^4 and (1/p)^2 in double (the mean's sum is the exact lane[])
};

// ----------------------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11); identical to the CPU oracle's.
__host__ __device__ __forceinline__ void zg_philox4(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                    uint32_t k0, uint32_t k1, uint32_t& o0, uint32_t& o1,
                                                    uint32_t& o2, uint32_t& o3) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
#ifdef __CUDA_ARCH__
    uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  o0 = c0;
  o1 = c1;
  o2 = c2;
  o3 = c3;
}
// Philox4x32-10 round keys of one seed (round r: seed + r * the Weyl constants), computed once per
// launch and passed as a grid-constant kernel parameter, so each round's key is an operand of the
// xor instead of two adds per round.
struct ZgKeys {
  uint32_t k[10][2];
};
__host__ __device__ __forceinline__ ZgKeys zg_round_keys(uint64_t seed) {
  ZgKeys K;
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    K.k[r][0] = k0;
    K.k[r][1] = k1;
  }
  return K;
}
// zg_philox4 with precomputed round keys (the same outputs).
__host__ __device__ __forceinline__ void zg_philox4_k(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                      const ZgKeys& K, uint32_t& o0, uint32_t& o1, uint32_t& o2,
                                                      uint32_t& o3) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
    uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
    uint32_t n0 = hi1 ^ c1 ^ K.k[r][0], n2 = hi0 ^ c3 ^ K.k[r][1];
    c0 = n0;
    c1 = lo1;
    c2 = n2;
    c3 = lo0;
  }
  o0 = c0;
  o1 = c1;
  o2 = c2;
  o3 = c3;
}

// The first two output words.
__host__ __device__ __forceinline__ void zg_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                   uint32_t k0, uint32_t k1, uint32_t& o0, uint32_t& o1) {
  uint32_t o2, o3;
  zg_philox4(c0, c1, c2, c3, k0, k1, o0, o1, o2, o3);
}

__host__ __device__ __forceinline__ uint64_t zg_mulhi64(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// The 64-bit Philox word of draw d of `sample`: counter (sample, d, stream), key seed.
__host__ __device__ __forceinline__ uint64_t zg_draw_word(uint64_t seed, uint32_t stream, uint64_t sample,
                                                          uint32_t d) {
  uint32_t o0, o1;
  zg_philox((uint32_t)sample, (uint32_t)(sample >> 32), d, stream, (uint32_t)seed,
            (uint32_t)(seed >> 32), o0, o1);
  return ((uint64_t)o1 << 32) | o0;
}
// The 64-bit word of an estimator's draw d: two draws per Philox block, counter (sample, d >> 1,
// stream), key seed; draw d takes output words 1:0 (d even) or 3:2 (d odd).  A program's
// consecutive draw pairs cost one Philox evaluation.  (Graph construction keeps zg_draw_word.)
__host__ __device__ __forceinline__ uint64_t zg_sample_word(uint64_t seed, uint32_t stream, uint64_t sample,
                                                            uint32_t d) {
  uint32_t o0, o1, o2, o3;
  zg_philox4((uint32_t)sample, (uint32_t)(sample >> 32), d >> 1, stream, (uint32_t)seed, (uint32_t)(seed >> 32),
             o0, o1, o2, o3);
  return (d & 1) ? (((uint64_t)o3 << 32) | o2) : (((uint64_t)o1 << 32) | o0);
}
// zg_sample_word with the seed's precomputed round keys.
__host__ __device__ __forceinline__ uint64_t zg_sample_word_k(const ZgKeys& K, uint32_t stream, uint64_t sample,
                                                              uint32_t d) {
  uint32_t o0, o1, o2, o3;
  zg_philox4_k((uint32_t)sample, (uint32_t)(sample >> 32), d >> 1, stream, K, o0, o1, o2, o3);
  return (d & 1) ? (((uint64_t)o3 << 32) | o2) : (((uint64_t)o1 << 32) | o0);
}
// A draw's word mapped to [lo, hi] by multiply-high.
__host__ __device__ __forceinline__ uint64_t zg_draw_map(uint64_t r, uint64_t lo, uint64_t hi) {
  uint64_t range = hi - lo + 1;
  if (range == 0) return r;
  return lo + zg_mulhi64(r, range);
}
// Draw d of `sample` in [lo, hi].
__host__ __device__ __forceinline__ uint64_t zg_draw(uint64_t seed, uint32_t stream, uint64_t sample,
                                                     uint32_t d, uint64_t lo, uint64_t hi) {
  return zg_draw_map(zg_draw_word(seed, stream, sample, d), lo, hi);
}

// 192-bit unsigned numerator.
struct ZgU192 {
  uint64_t l[3];
};
__host__ __device__ __forceinline__ void zg_u192_set(ZgU192& a, uint64_t v) {
  a.l[0] = v;
  a.l[1] = 0;
  a.l[2] = 0;
}
// a *= f for a 32-bit factor: per limb two 32 x 32 -> 64-bit multiply-adds, whose sums stay below
// 2^64 ((2^32 - 1)^2 + 2^32 - 1); returns true on overflow beyond 192 bits.
__host__ __device__ __forceinline__ bool zg_u192_mul32(ZgU192& a, uint32_t f) {
  uint64_t c = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const uint64_t lo = (uint64_t)(uint32_t)a.l[i] * f + c;
    const uint64_t hi = (a.l[i] >> 32) * f + (lo >> 32);
    a.l[i] = (hi << 32) | (uint32_t)lo;
    c = hi >> 32;
  }
  return c != 0;
}

const char* zg_set_error(int code, const char* fmt, ...);
int zg_check_cuda(cudaError_t e, const char* what);
#define ZG_CUDA(call)                                   \
  do {                                                  \
    cudaError_t _e = (call);                            \
    if (_e != cudaSuccess) return zg_check_cuda(_e, #call); \
  } while (0)

int zg_num_sms();

// Stream-ordered allocation of per-call scratch from the library's own memory pool on the current
// device.  The pool keeps up to 256 MiB of freed blocks across synchronisations (the device's
// default pool returns them at every synchronisation, and mapping them again cost ~0.1 ms per
// call); free with cudaFreeAsync.
cudaError_t zg_malloc_async(void** p, size_t bytes, cudaStream_t s);

// Learned-profile helpers shared by zg_mlp.cu and zg_batch.cu: the graph's eight degree features
// (f[0..7], the rest zeroed), the program and pilot features (f[8..15]) from a pilot run's
// counters, and the budget for a predicted log2 relative variance.
int zg_degree_features(const zg_graph* g, cudaStream_t s, float* f);
void zg_query_features(const zg_program* p, const zg_counters& c, float* f);
uint64_t zg_learned_n(float pred_log2_cv2, double error, double confidence);
// The graph's largest degree (from its degree statistics, computed once per graph).
int zg_graph_max_degree(const zg_graph* g, cudaStream_t s, uint64_t* out);

// The bound check of a running estimate (zg_elp.cu), shared by zg_query and zg_batch_bounded.
// weight_range: the largest value one estimator of (kind, param, pattern_edges) can return on g.
int zg_weight_range(const zg_graph* g, int kind, uint32_t param, uint32_t pattern_edges, cudaStream_t s,
                    double* range);
// Whether mean +- half lies within error * mean at the confidence: the empirical CLT half-width
// (z sqrt(v / n), used from 30 hits on) or the empirical Bernstein half-width
// (sqrt(2 var x / n) + 3 range x / n, x = ln(3 / (1 - confidence)), valid for any n), whichever is
// smaller where both apply.  var: the empirical (1/n) variance; ew4: the empirical mean of w^4
// (0: unknown); v = zg_variance_bound(mean, var, ew4, n, confidence).  *method: ZG_BOUND_CLT or
// ZG_BOUND_BERNSTEIN, the one that gave *half.
bool zg_bound_check(double mean, double var, double ew4, uint64_t n, uint64_t hits, double error, double confidence,
                    double range, double* half, uint32_t* method);
// An upper confidence bound on the variance, for weights whose variance estimate is itself
// uncertain (heavy tails): var + z sqrt((m4 - var^2) / n), with the fourth central moment bounded
// by ew4 + 2 mean^2 var (nonnegative weights) and z the two-sided quantile of the confidence.
double zg_variance_bound(double mean, double var, double ew4, uint64_t n, double confidence);
// Samples the bound check needs at the variance bound, with headroom 1 + 0.5 / sqrt(hits);
// 2n while hits < 30.
double zg_samples_needed(double mean, double var, double ew4, uint64_t n, uint64_t hits, double error,
                         double confidence);
