/*
 * zg_oracle.c — CPU ORACLE (test infrastructure only; see zg_oracle.h).
 *
 * Restates, in plain C, the reference estimator path of jy-yuan/sampling-graph-mining on a
 * single partition / single socket (the configuration the GPU build replaces the
 * MPI+NUMA partitioning with).  Citations are file:line inside the reference project.
 */
#include "zg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

#define ZGO_STREAM_SHUFFLE   0xFFFFFFF0u
#define ZGO_STREAM_SUBSAMPLE 0xFFFFFFF1u

/* ------------------------------------------------------------------------- */
/* Philox4x32-10, Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy as 1, 2, 3"
 * (SC'11).  Round: (c0,c1,c2,c3) -> (hi(M1*c2)^c1^k0, lo(M1*c2), hi(M0*c0)^c3^k1, lo(M0*c0)),
 * key bumped by the Weyl constants between rounds. */
void zgo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Draw d of sample `sample`: counter (sample_lo, sample_hi, d, stream), key (seed_lo, seed_hi);
 * a 64-bit word r = out1:out0 mapped to [lo, hi] by the multiply-high method. */
uint64_t zgo_draw(uint64_t seed, uint32_t stream, uint64_t sample, uint32_t d, uint64_t lo,
                  uint64_t hi) {
  uint32_t ctr[4] = {(uint32_t)sample, (uint32_t)(sample >> 32), d, stream};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  zgo_philox4x32_10(ctr, key, o);
  uint64_t r = ((uint64_t)o[1] << 32) | o[0];
  uint64_t range = hi - lo + 1;
  if (range == 0) return r;
  return lo + (uint64_t)(((u128)r * range) >> 64);
}

/* Estimator draw d of sample `sample`: two draws per Philox block, counter (sample_lo, sample_hi,
 * d >> 1, stream), key (seed_lo, seed_hi); draw d takes the 64-bit word out1:out0 (d even) or
 * out3:out2 (d odd), mapped to [lo, hi] by the multiply-high method.  (zgo_draw, one draw per
 * block, stays for the graph shuffles and subsamples.) */
uint64_t zgo_sample_draw(uint64_t seed, uint32_t stream, uint64_t sample, uint32_t d, uint64_t lo,
                         uint64_t hi) {
  uint32_t ctr[4] = {(uint32_t)sample, (uint32_t)(sample >> 32), d >> 1, stream};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t o[4];
  zgo_philox4x32_10(ctr, key, o);
  uint64_t r = (d & 1) ? (((uint64_t)o[3] << 32) | o[2]) : (((uint64_t)o[1] << 32) | o[0]);
  uint64_t range = hi - lo + 1;
  if (range == 0) return r;
  return lo + (uint64_t)(((u128)r * range) >> 64);
}

/* ------------------------------------------------------------------------- */
/* Graph: CSRConstructor::construct_bitmap_assisted_csr without its shuffle
 * (src/Graph.cpp:255-311): two half-edges per edge, appended in edge-id order, so every
 * adjacency list is sorted by edge id (the asserts at :324-334).
 * Large graphs are built by several threads with the same result: thread t owns a range of
 * vertices, scans every edge in id order and appends only the half-edges of its own vertices. */
int zgo_graph_build(zgo_graph* g, uint32_t nv, uint64_t m, const uint32_t* edges,
                    const uint32_t* weights) {
  memset(g, 0, sizeof(*g));
  g->nv = nv;
  g->m = m;
  g->num_edges = m;
  g->src = (uint32_t*)malloc(sizeof(uint32_t) * (m ? m : 1));
  g->dst = (uint32_t*)malloc(sizeof(uint32_t) * (m ? m : 1));
  g->off = (uint64_t*)calloc((size_t)nv + 1, sizeof(uint64_t));
  g->adj_nbr = (uint32_t*)malloc(sizeof(uint32_t) * (m ? 2 * m : 1));
  g->adj_eid = (uint64_t*)malloc(sizeof(uint64_t) * (m ? 2 * m : 1));
  if (weights) {
    g->w = (uint32_t*)malloc(sizeof(uint32_t) * (m ? m : 1));
    g->adj_w = (uint32_t*)malloc(sizeof(uint32_t) * (m ? 2 * m : 1));
  }
  if (!g->src || !g->dst || !g->off || !g->adj_nbr || !g->adj_eid || (weights && (!g->w || !g->adj_w)))
    return ZG_ERR_OOM;
  int nt = 1;
#ifdef _OPENMP
  if (m >= (1u << 20)) nt = omp_get_max_threads();
#endif
  int bad = 0;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static) reduction(| : bad)
#endif
  for (uint64_t e = 0; e < m; ++e) {
    uint32_t s = edges[2 * e], d = edges[2 * e + 1];
    if (s >= nv || d >= nv || s == d) bad = 1; /* src/Graph.cpp:454 */
    g->src[e] = s;
    g->dst[e] = d;
    if (weights) g->w[e] = weights[e];
  }
  if (bad) return ZG_ERR_INVALID_GRAPH;
  /* degrees: thread t counts the endpoints in its equal share of the vertex ids */
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    uint32_t vlo = (uint32_t)((uint64_t)nv * t / nt), vhi = (uint32_t)((uint64_t)nv * (t + 1) / nt);
    for (uint64_t e = 0; e < m; ++e) {
      uint32_t s = g->src[e], d = g->dst[e];
      if (s >= vlo && s < vhi) g->off[s + 1]++;
      if (d >= vlo && d < vhi) g->off[d + 1]++;
    }
  }
  for (uint32_t v = 1; v <= nv; ++v) g->off[v] += g->off[v - 1];
  uint64_t* cur = (uint64_t*)malloc(sizeof(uint64_t) * ((size_t)nv + 1));
  uint32_t* cut = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)nt + 1));
  if (!cur || !cut) { free(cur); free(cut); return ZG_ERR_OOM; }
  memcpy(cur, g->off, sizeof(uint64_t) * ((size_t)nv + 1));
  /* scatter: vertex ranges of about equal half-edge counts */
  cut[0] = 0;
  for (int t = 1; t < nt; ++t) {
    uint64_t target = 2 * m / (uint64_t)nt * (uint64_t)t;
    uint32_t lo = cut[t - 1], hi = nv;
    while (lo < hi) { uint32_t mid = lo + (hi - lo) / 2; if (g->off[mid] < target) lo = mid + 1; else hi = mid; }
    cut[t] = lo;
  }
  cut[nt] = nv;
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    uint32_t vlo = cut[t], vhi = cut[t + 1];
    for (uint64_t e = 0; e < m; ++e) {
      uint32_t s = g->src[e], d = g->dst[e];
      if (s >= vlo && s < vhi) {
        uint64_t pos = cur[s]++;
        g->adj_nbr[pos] = d; g->adj_eid[pos] = e;
        if (weights) g->adj_w[pos] = weights[e];
      }
      if (d >= vlo && d < vhi) {
        uint64_t pos = cur[d]++;
        g->adj_nbr[pos] = s; g->adj_eid[pos] = e;
        if (weights) g->adj_w[pos] = weights[e];
      }
    }
  }
  uint64_t maxd = 0;
  for (uint32_t v = 0; v < nv; ++v) {
    uint64_t dv = g->off[v + 1] - g->off[v];
    if (dv > maxd) maxd = dv;
  }
  free(cur);
  free(cut);
  g->max_degree = maxd; /* src/Graph.cpp:467-474 */
  return ZG_OK;
}

void zgo_graph_free(zgo_graph* g) {
  free(g->src); free(g->dst); free(g->w); free(g->off);
  free(g->adj_nbr); free(g->adj_eid); free(g->adj_w);
  memset(g, 0, sizeof(*g));
}

/* ------------------------------------------------------------------------- */
/* Edge / SubGraph (include/ZGraphInstance.hpp:30-105, src/ZGraphInstance.cpp:39-113). */
typedef struct { uint64_t eid; uint32_t src, dst; } zgo_edge;
typedef struct {
  int ne; zgo_edge e[ZG_MAX_LIST];
  int nv; uint32_t v[ZG_MAX_LIST];
  uint64_t min_valid_eid;
} zgo_sub;

static void sub_init(zgo_sub* s) { s->ne = 0; s->nv = 0; s->min_valid_eid = 0; }
static int sub_has_vertex(const zgo_sub* s, uint32_t v) {       /* :45-53 */
  for (int i = 0; i < s->nv; ++i) if (s->v[i] == v) return 1;
  return 0;
}
static void sub_add_vertex(zgo_sub* s, uint32_t v) {             /* :65-73 */
  if (!sub_has_vertex(s, v) && s->nv < ZG_MAX_LIST) s->v[s->nv++] = v;
}
static void sub_add_edge(zgo_sub* s, zgo_edge e) {               /* :55-63 */
  if (s->ne < ZG_MAX_LIST) s->e[s->ne++] = e;
  if (e.eid >= s->min_valid_eid) s->min_valid_eid = e.eid + 1;
  sub_add_vertex(s, e.src);
  sub_add_vertex(s, e.dst);
}
/* SubGraph::operator- : edges of a not present (either orientation) in b (:95-113). */
static void sub_minus(const zgo_sub* a, const zgo_sub* b, zgo_sub* out) {
  sub_init(out);
  for (int i = 0; i < a->ne; ++i) {
    int del = 0;
    for (int j = 0; j < b->ne; ++j) {
      if ((a->e[i].src == b->e[j].src && a->e[i].dst == b->e[j].dst) ||
          (a->e[i].src == b->e[j].dst && a->e[i].dst == b->e[j].src)) { del = 1; break; }
    }
    if (!del) sub_add_edge(out, a->e[i]);
  }
}

/* ------------------------------------------------------------------------- */
/* Sampling context: the replayable Random (src/Random.cpp:11-14) of one estimator. */
typedef struct {
  const zgo_graph* g;
  uint64_t seed, sample;
  uint32_t stream, nd;
  zg_sample_trace* tr;
  int shift;
  u128 num_lo; uint64_t num_hi; /* 192-bit exact numerator */
  int overflow;
  uint32_t sectors; /* 32-byte sector access model (see zgo_model_*) */
  uint32_t closures; /* closure checks of the access model */
  int model;         /* count the access model: only traces report it (an untraced run skips it) */
} zgo_ctx;

/* Access model of the rebuilt kernels, in 32-byte sectors (the roofline's algorithmic bytes):
 * sample_edge 1; a conditional step sum over anchors v with d_v > 0 of 1 + max(1, ceil(log2 d_v) - 2),
 * plus 1 for the chosen entry; a closure edge (x,y) 1 + max(1, ceil(log2 min(d_x,d_y)) - 2) + 1,
 * counted for each edge checked up to the first miss. */
static uint32_t zgo_clog2(uint64_t d) {
  uint32_t b = 0;
  while (((uint64_t)1 << b) < d) ++b;
  return b;
}
static uint32_t zgo_model_search(uint64_t d) {
  uint32_t l = zgo_clog2(d);
  return l > 3 ? l - 2 : 1;
}

static uint64_t ctx_rand(zgo_ctx* c, uint64_t lo, uint64_t hi) {
  uint64_t v = zgo_sample_draw(c->seed, c->stream, c->sample, c->nd, lo, hi);
  if (c->nd < ZG_MAX_DRAWS) {
    c->tr->lo[c->nd] = lo; c->tr->hi[c->nd] = hi; c->tr->val[c->nd] = v;
  }
  c->nd++;
  return v;
}

static void num_mul(zgo_ctx* c, uint64_t f) {
  u128 lo = (c->num_lo & (u128)0xFFFFFFFFFFFFFFFFull) * f;
  u128 mid = (c->num_lo >> 64) * f + (lo >> 64);
  u128 hi = (u128)c->num_hi * f + (mid >> 64);
  c->num_lo = ((u128)(uint64_t)mid << 64) | (uint64_t)lo;
  if (hi >> 64) c->overflow = 1;
  c->num_hi = (uint64_t)hi;
}

/* sample_edge (src/ZGraphInstance.cpp:315-334) */
static double prim_sample_edge(zgo_ctx* c, zgo_edge* out) {
  const zgo_graph* g = c->g;
  if (g->m == 0) return -1.0;
  uint64_t id = ctx_rand(c, 0, g->m - 1);
  out->eid = id; out->src = g->src[id]; out->dst = g->dst[id];
  num_mul(c, g->m);
  c->sectors += 1;
  return 1. / (double)g->m;
}

/* core_conditional_sample_edge (src/ZGraphInstance.cpp:128-222) */
#define ZGO_BS_THRESHOLD 32 /* BINARY_SEARCH_THRESHOLD, :11 */
static double prim_cond_sample(zgo_ctx* c, const zgo_edge* edges, int ne, const uint32_t* verts,
                               int nv, zgo_edge* out) {
  const zgo_graph* g = c->g;
  uint64_t min_valid = 0;
  for (int i = 0; i < ne; ++i) if (edges[i].eid + 1 > min_valid) min_valid = edges[i].eid + 1;
  uint64_t sum = 0, pos[ZG_MAX_LIST];
  int np = 0;
  for (int i = 0; i < nv; ++i) {
    uint32_t v = verts[i];
    uint64_t b = g->off[v], e = g->off[v + 1];
    if (e == b) continue; /* bitmap bit clear */
    if (c->model) c->sectors += 1 + zgo_model_search(e - b);
    if (min_valid <= g->adj_eid[b]) { sum += e - b; pos[np++] = b; }
    else if (min_valid > g->adj_eid[e - 1]) { pos[np++] = e; }
    else if (e - b <= ZGO_BS_THRESHOLD) {
      for (uint64_t idx = b; idx < e; ++idx)
        if (min_valid <= g->adj_eid[idx]) { sum += e - idx; pos[np++] = idx; break; }
    } else {
      uint64_t l = b, r = e - 1;
      while (r - l > 1) {
        uint64_t mid = (l + r) >> 1;
        if (g->adj_eid[mid] < min_valid) l = mid; else r = mid;
      }
      sum += e - r; pos[np++] = r;
    }
  }
  if (sum == 0) return -1.0;
  c->sectors += 1;
  uint64_t rr = ctx_rand(c, 0, sum - 1);
  int pi = 0;
  uint64_t chosen = 0;
  for (int i = 0; i < nv; ++i) {
    uint32_t v = verts[i];
    if (g->off[v + 1] == g->off[v]) continue;
    uint64_t cur = pos[pi++], e = g->off[v + 1];
    if (cur + rr < e) { chosen = cur + rr; out->src = v; break; }
    rr -= e - cur;
  }
  out->eid = g->adj_eid[chosen];
  out->dst = g->adj_nbr[chosen];
  double appear = 0;
  for (int i = 0; i < nv; ++i) {
    if (verts[i] == out->src) ++appear;
    if (verts[i] == out->dst) ++appear;
  }
  num_mul(c, sum);
  if (appear == 2) c->shift++;
  return 1. * appear / (double)sum;
}

/* conditional_close(SubGraph, SubGraph) (src/ZGraphInstance.cpp:372-407): linear scans. */
static int prim_close(zgo_ctx* c, const zgo_sub* sampled, const zgo_sub* wait) {
  const zgo_graph* g = c->g;
  uint64_t min_valid = sampled->min_valid_eid;
  for (int i = 0; i < wait->ne; ++i) {
    uint32_t ws = wait->e[i].src, wd = wait->e[i].dst;
    int found = 0;
    if (c->model) {
      uint64_t dx = g->off[ws + 1] - g->off[ws], dy = g->off[wd + 1] - g->off[wd];
      c->sectors += 2 + zgo_model_search(dx < dy ? dx : dy);
      c->closures++;
    }
    for (int j = 0; j < sampled->nv && !found; ++j) {
      uint32_t v = sampled->v[j];
      for (uint64_t idx = g->off[v]; idx < g->off[v + 1]; ++idx) {
        if (g->adj_eid[idx] < min_valid) continue;
        uint32_t s = v, d = g->adj_nbr[idx];
        if ((s == ws && d == wd) || (d == ws && s == wd)) { found = 1; break; }
      }
    }
    if (!found) return 0;
  }
  return 1;
}

/* Triangle(e0, e1) (applications/Triangle.cpp:17-40) */
static void tri_pattern(zgo_edge e0, zgo_edge e1, zgo_sub* out) {
  sub_init(out);
  sub_add_edge(out, e0);
  sub_add_edge(out, e1);
  zgo_edge e = {0, 0, 0};
  if (e0.src == e1.src) { e.src = e0.dst; e.dst = e1.dst; }
  else if (e0.src == e1.dst) { e.src = e0.dst; e.dst = e1.src; }
  else if (e0.dst == e1.src) { e.src = e0.src; e.dst = e1.dst; }
  else { e.src = e0.src; e.dst = e1.src; }
  sub_add_edge(out, e);
}

/* ------------------------------------------------------------------------- */
/* Programs: the applications' estimate() bodies. Each returns the double estimate(). */

/* applications/Triangle.cpp:48-73 */
static double prog_triangle(zgo_ctx* c) {
  zgo_sub sg; sub_init(&sg);
  double p = 1;
  zgo_edge e0, e1;
  double t0 = prim_sample_edge(c, &e0);
  if (t0 < 0) return -1;
  p *= t0; sub_add_edge(&sg, e0);
  double t1 = prim_cond_sample(c, sg.e, sg.ne, sg.v, sg.nv, &e1);
  if (t1 < 0) return -1;
  p *= t1; sub_add_edge(&sg, e1);
  zgo_sub tri, wait;
  tri_pattern(e0, e1, &tri);
  sub_minus(&tri, &sg, &wait);
  if (prim_close(c, &sg, &wait)) return 1. / p;
  return 0;
}

/* applications/FourClique.cpp:176-191 and 199-234 */
static double prog_four_clique(zgo_ctx* c) {
  zgo_sub sg; sub_init(&sg);
  double p = 1;
  zgo_edge e0, e1, e2;
  double t = prim_sample_edge(c, &e0);
  if (t < 0) return -1;
  p *= t; sub_add_edge(&sg, e0);
  t = prim_cond_sample(c, sg.e, sg.ne, sg.v, sg.nv, &e1);
  if (t < 0) return -1;
  p *= t; sub_add_edge(&sg, e1);
  t = prim_cond_sample(c, sg.e, sg.ne, sg.v, sg.nv, &e2);
  if (t < 0) return -1;
  p *= t; sub_add_edge(&sg, e2);
  if (sg.nv == 3) return 0;
  zgo_sub clique, wait;
  sub_init(&clique);
  for (int i = 0; i < sg.nv; ++i)
    for (int j = i + 1; j < sg.nv; ++j) {
      zgo_edge e = {0, sg.v[i], sg.v[j]};
      sub_add_edge(&clique, e);
    }
  sub_minus(&clique, &sg, &wait);
  if (prim_close(c, &sg, &wait)) return 1. / p;
  return 0;
}

/* The edge id of (x, y), any id, or -1 (a scan of the shorter edge-id-ordered list). */
static int64_t find_edge_id(zgo_ctx* c, uint32_t x, uint32_t y) {
  const zgo_graph* g = c->g;
  uint64_t dx = g->off[x + 1] - g->off[x], dy = g->off[y + 1] - g->off[y];
  if (c->model) {
    c->sectors += 2 + zgo_model_search(dx < dy ? dx : dy);
    c->closures++;
  }
  uint32_t v = dx <= dy ? x : y, t = dx <= dy ? y : x;
  for (uint64_t idx = g->off[v]; idx < g->off[v + 1]; ++idx)
    if (g->adj_nbr[idx] == t) return (int64_t)g->adj_eid[idx];
  return -1;
}

/* The unbiased 4-clique estimator (no counterpart in the reference): FourClique's draws; the three
 * unsampled pairs must be edges (any id), looked up in the order (the other of a and b, c), then the
 * two pairs at d in slot order, up to the first missing one; and the sample must be the clique's
 * canonical path: id0 the smallest of the six ids, id1 the smallest of the four edges joining
 * {a, b} to {c, d}, id2 the smallest id above id1 among the edges at d.  Each 4-clique has exactly
 * one canonical path, which the draws reach with positive probability, so E[estimate] = #4-cliques. */
static double prog_four_clique_unbiased(zgo_ctx* c) {
  zgo_sub sg; sub_init(&sg);
  double p = 1;
  zgo_edge e0, e1, e2;
  double t = prim_sample_edge(c, &e0);
  if (t < 0) return -1;
  p *= t; sub_add_edge(&sg, e0);
  t = prim_cond_sample(c, sg.e, sg.ne, sg.v, sg.nv, &e1);
  if (t < 0) return -1;
  p *= t; sub_add_edge(&sg, e1);
  t = prim_cond_sample(c, sg.e, sg.ne, sg.v, sg.nv, &e2);
  if (t < 0) return -1;
  p *= t; sub_add_edge(&sg, e2);
  if (sg.nv == 3) return 0;
  const uint32_t* v = sg.v; /* a, b, c, d in insertion order */
  int s1 = e1.src == v[0] ? 0 : 1;
  int s2 = e2.src == v[0] ? 0 : (e2.src == v[1] ? 1 : 2);
  int x0 = 1 - s1, x1 = s2 == 0 ? 1 : 0, x2 = s2 == 2 ? 1 : 2;
  int64_t h0 = find_edge_id(c, v[x0], v[2]);
  if (h0 < 0) return 0;
  int64_t h1 = find_edge_id(c, v[x1], v[3]);
  if (h1 < 0) return 0;
  int64_t h2 = find_edge_id(c, v[x2], v[3]);
  if (h2 < 0) return 0;
  uint64_t id0 = e0.eid, id1 = e1.eid, id2 = e2.eid;
  uint64_t d[3];
  d[s2] = id2;
  d[x1] = (uint64_t)h1;
  d[x2] = (uint64_t)h2;
  if ((uint64_t)h0 < id0 || (uint64_t)h1 < id0 || (uint64_t)h2 < id0) return 0;
  if ((uint64_t)h0 < id1 || d[0] < id1 || d[1] < id1) return 0;
  for (int i = 0; i < 3; ++i)
    if (d[i] > id1 && d[i] < id2) return 0;
  return 1. / p;
}

/* applications/ThreeChain.cpp:315-330 */
static double prog_three_chain(zgo_ctx* c) {
  zgo_sub sg; sub_init(&sg);
  double p = 1;
  zgo_edge e0, e1;
  double t = prim_sample_edge(c, &e0);
  if (t < 0) return -1;
  p *= t; sub_add_edge(&sg, e0);
  t = prim_cond_sample(c, sg.e, sg.ne, sg.v, sg.nv, &e1);
  if (t < 0) return -1;
  p *= t;
  return 1. / p;
}

/* the "vertex of e1 not shared with e0" cascade (applications/FourChain.cpp:44-54) */
static uint32_t other_end(zgo_edge e0, zgo_edge e1) {
  if (e0.src == e1.src) return e1.dst;
  if (e0.src == e1.dst) return e1.src;
  if (e0.dst == e1.src) return e1.dst;
  return e1.src;
}

/* applications/FourChain.cpp:24-124 */
static double prog_four_chain(zgo_ctx* c) {
  const int nm = 3;
  uint64_t sel = ctx_rand(c, 1, nm);
  double p = 1. / nm;
  num_mul(c, 3);
  zgo_edge e0, e1, e2, edges[2];
  uint32_t verts[2];
  double t = prim_sample_edge(c, &e0);
  if (t < 0) return -1;
  p *= t;
  edges[0] = e0;
  if (sel == 1) {
    verts[0] = e0.src; verts[1] = e0.dst;
    t = prim_cond_sample(c, edges, 1, verts, 2, &e1);
    if (t < 0) return -1;
    p *= t;
    edges[1] = e1;
    verts[0] = other_end(e0, e1);
    t = prim_cond_sample(c, edges, 2, verts, 1, &e2);
    if (t < 0) return -1;
    p *= t;
    if (e2.src == e0.src || e2.src == e0.dst) return 0;
    if (e2.dst == e0.src || e2.dst == e0.dst) return 0;
    return 1. / p;
  } else if (sel == 2) {
    verts[0] = e0.src; verts[1] = e0.dst;
    t = prim_cond_sample(c, edges, 1, verts, 2, &e1);
    if (t < 0) return -1;
    p *= t;
    verts[0] = other_end(e0, e1);
    t = prim_cond_sample(c, edges, 1, verts, 1, &e2);
    if (t < 0) return -1;
    p *= t;
    if (e2.src == e0.src || e2.src == e0.dst) return 0;
    if (e2.dst == e0.src || e2.dst == e0.dst) return 0;
    if (e2.eid >= e1.eid) return 0;
    return 1. / p;
  } else {
    verts[0] = e0.src;
    t = prim_cond_sample(c, edges, 1, verts, 1, &e1);
    if (t < 0) return -1;
    p *= t;
    verts[0] = e0.dst;
    t = prim_cond_sample(c, edges, 1, verts, 1, &e2);
    if (t < 0) return -1;
    p *= t;
    if (e2.src == e1.src || e2.src == e1.dst) return 0;
    if (e2.dst == e1.src || e2.dst == e1.dst) return 0;
    return 1. / p;
  }
}

/* --- x87 80-bit extended (64-bit mantissa, round to nearest even) in integers ---- */
typedef struct { uint64_t m; int32_t e; } zgo_ext; /* value = m * 2^e, m >= 2^63 */

static zgo_ext ext_from_double(double d) {
  uint64_t b; memcpy(&b, &d, 8);
  int ex = (int)((b >> 52) & 0x7ff);
  uint64_t fr = b & ((1ull << 52) - 1);
  zgo_ext r;
  r.m = (fr | (1ull << 52)) << 11;
  r.e = ex - 1075 - 11;
  return r;
}
static zgo_ext ext_mul(zgo_ext a, zgo_ext b) {
  u128 p = (u128)a.m * b.m;
  uint64_t keep, rem, half = 1ull << 63;
  zgo_ext r;
  if ((uint64_t)(p >> 127)) { keep = (uint64_t)(p >> 64); rem = (uint64_t)p; r.e = a.e + b.e + 64; }
  else { keep = (uint64_t)(p >> 63); rem = (uint64_t)p << 1; r.e = a.e + b.e + 63; }
  if (rem > half || (rem == half && (keep & 1))) {
    keep++;
    if (keep == 0) { keep = 1ull << 63; r.e++; }
  }
  r.m = keep;
  return r;
}
static zgo_ext ext_inv(zgo_ext a) {
  zgo_ext r;
  if (a.m == (1ull << 63)) { r.m = 1ull << 63; r.e = -126 - a.e; return r; }
  u128 num = (u128)1 << 127;
  uint64_t q = (uint64_t)(num / a.m);
  u128 rem = num - (u128)q * a.m;
  r.e = -127 - a.e;
  if (2 * rem > (u128)a.m || (2 * rem == (u128)a.m && (q & 1))) {
    q++;
    if (q == 0) { q = 1ull << 63; r.e++; }
  }
  r.m = q;
  return r;
}
static double ext_to_double(zgo_ext a) {
  uint64_t keep = a.m >> 11, rem = a.m & 0x7ff;
  int e = a.e + 11;
  if (rem > 0x400 || (rem == 0x400 && (keep & 1))) {
    keep++;
    if (keep == (1ull << 53)) { keep >>= 1; e++; }
  }
  return ldexp((double)keep, e);
}
/* 1 / (f0 * f1 * ... ) with `long double p = 1.; p *= f_i; return 1. / p;` semantics. */
double zgo_ext_inv_product(const double* f, int n) {
  zgo_ext p = ext_from_double(1.0);
  for (int i = 0; i < n; ++i) p = ext_mul(p, ext_from_double(f[i]));
  return ext_to_double(ext_inv(p));
}

/* ChainMiningInstance::canonicality_check (applications/ChainMining.cpp:218-235), identical to
 * SamplerGenerator::canonicality_check (src/SamplerGenerator.cpp:368-385). */
static int canonicality_check(const zgo_edge* edges, int ne, zgo_edge e) {
  if (ne <= 1) return 1;
  int found = 0;
  for (int i = 0; i < ne; ++i) {
    if (!found) {
      if (e.src == edges[i].src || e.src == edges[i].dst || e.dst == edges[i].src ||
          e.dst == edges[i].dst)
        found = 1;
    } else if (edges[i].eid >= e.eid) {
      return 0;
    }
  }
  return 1;
}

/* applications/ChainMining.cpp:240-84 (long double p) */
static double prog_chain(zgo_ctx* c, int order) {
  zgo_edge edges[ZG_MAX_LIST], first[1], e0, e;
  double fac[ZG_MAX_LIST + 1];
  int nf = 0, ne = 0;
  uint32_t verts[2];
  zgo_sub sg; sub_init(&sg);
  double t = prim_sample_edge(c, &e0);
  if (t < 0) return -1;
  fac[nf++] = t;
  edges[ne++] = e0; first[0] = e0; sub_add_edge(&sg, e0);
  verts[0] = e0.src; verts[1] = e0.dst;
  for (int i = 0; i < order - 2; ++i) {
    t = prim_cond_sample(c, first, 1, verts, 2, &e);
    if (t < 0) return -1;
    fac[nf++] = t;
    if (!canonicality_check(edges, ne, e)) return 0;
    edges[ne++] = e; sub_add_edge(&sg, e);
    if (sg.nv != i + 3) return 0;
    if (verts[0] == e.src) verts[0] = e.dst;
    else if (verts[0] == e.dst) verts[0] = e.src;
    else if (verts[1] == e.src) verts[1] = e.dst;
    else verts[1] = e.src;
  }
  return zgo_ext_inv_product(fac, nf);
}

/* SamplerGenerator<Empty>::estimate (src/SamplerGenerator.cpp:461-546) */
static int pattern_is_automorphic(const uint32_t* pat, uint32_t pe, const uint32_t* smp) {
  /* Pattern::is_automorphic + is_in_edges_list (:297-320): every sample edge is a pattern edge */
  for (uint32_t i = 0; i < pe; ++i) {
    int in = 0;
    for (uint32_t j = 0; j < pe; ++j) {
      if ((pat[2 * j] == smp[2 * i] && pat[2 * j + 1] == smp[2 * i + 1]) ||
          (pat[2 * j] == smp[2 * i + 1] && pat[2 * j + 1] == smp[2 * i])) { in = 1; break; }
    }
    if (!in) return 0;
  }
  return 1;
}

static double prog_pattern(zgo_ctx* c, const zgo_program* p) {
  zgo_edge sampled[ZG_MAX_LIST], first[1], e;
  int ns = 0;
  zgo_sub sg; sub_init(&sg);
  double pr = 1.;
  double t = prim_sample_edge(c, &e);
  if (t < 0) return -1;
  pr *= t;
  first[0] = e; sampled[ns++] = e; sub_add_edge(&sg, e);
  for (uint32_t k = 1; k < p->pe; ++k) {
    t = prim_cond_sample(c, first, 1, sg.v, sg.nv, &e);
    if (t < 0) return -1;
    pr *= t;
    if (!canonicality_check(sampled, ns, e)) return 0;
    sampled[ns++] = e; sub_add_edge(&sg, e);
    if ((uint32_t)sg.nv > p->pv) return 0;
  }
  if ((uint32_t)sg.nv != p->pv) return 0;
  uint32_t vs[ZG_MAX_LIST];
  for (uint32_t i = 0; i < p->pv; ++i) vs[i] = sg.v[i];
  for (uint32_t i = 0; i < p->pv; ++i)
    for (uint32_t j = i + 1; j < p->pv; ++j)
      if (vs[j] < vs[i]) { uint32_t tmp = vs[j]; vs[j] = vs[i]; vs[i] = tmp; }
  uint32_t rel[2 * ZG_MAX_LIST];
  for (int k = 0; k < ns; ++k) {
    for (uint32_t i = 0; i < p->pv; ++i) if (sampled[k].src == vs[i]) { rel[2 * k] = i; break; }
    for (uint32_t i = 0; i < p->pv; ++i) if (sampled[k].dst == vs[i]) { rel[2 * k + 1] = i; break; }
  }
  for (uint32_t u = 0; u < p->num_unique; ++u)
    if (pattern_is_automorphic(p->unique_edges + (size_t)u * 2 * p->pe, p->pe, rel)) return 1. / pr;
  return 0;
}

/* ------------------------------------------------------------------------- */
/* SamplerGenerator ctor (src/SamplerGenerator.cpp:344-366, 393-445): all pv! relabelings in
 * generate_mapping's lexicographic order, de-duplicated with is_automorphic. */
static void gen_perms(uint32_t pv, uint32_t idx, uint32_t* map, int* used, uint32_t* out,
                      uint32_t* cnt) {
  if (idx == pv) { memcpy(out + (size_t)(*cnt) * pv, map, sizeof(uint32_t) * pv); (*cnt)++; return; }
  for (uint32_t v = 0; v < pv; ++v)
    if (!used[v]) { used[v] = 1; map[idx] = v; gen_perms(pv, idx + 1, map, used, out, cnt); used[v] = 0; }
}

int zgo_program_init(zgo_program* p, int kind, uint32_t param, uint32_t pv, uint32_t pe,
                     const uint32_t* pedges) {
  memset(p, 0, sizeof(*p));
  p->kind = kind;
  p->param = param;
  if (kind == ZG_PROG_CHAIN && (param < 3 || param > ZG_MAX_LIST)) return ZG_ERR_INVALID_ARG;
  if (kind != ZG_PROG_PATTERN) return ZG_OK;
  if (pv < 2 || pv > 8 || pe < 1 || pe > ZG_MAX_LIST - 1) return ZG_ERR_UNSUPPORTED_ESTIMATOR;
  p->pv = pv; p->pe = pe;
  memcpy(p->pedges, pedges, sizeof(uint32_t) * 2 * pe);
  uint32_t nperm = 1;
  for (uint32_t i = 2; i <= pv; ++i) nperm *= i;
  uint32_t* perms = (uint32_t*)malloc(sizeof(uint32_t) * nperm * pv);
  uint32_t map[8]; int used[8] = {0}; uint32_t cnt = 0;
  gen_perms(pv, 0, map, used, perms, &cnt);
  uint32_t* all = (uint32_t*)malloc(sizeof(uint32_t) * nperm * 2 * pe);
  for (uint32_t q = 0; q < nperm; ++q)
    for (uint32_t e = 0; e < pe; ++e) {  /* Pattern::setup_vertex_id_mapping (:326-332) */
      all[(size_t)q * 2 * pe + 2 * e] = perms[(size_t)q * pv + pedges[2 * e]];
      all[(size_t)q * 2 * pe + 2 * e + 1] = perms[(size_t)q * pv + pedges[2 * e + 1]];
    }
  int* dup = (int*)calloc(nperm, sizeof(int));
  p->unique_edges = (uint32_t*)malloc(sizeof(uint32_t) * nperm * 2 * pe);
  for (uint32_t i = 0; i < nperm; ++i) {
    for (uint32_t j = 0; j < i; ++j)
      if (!dup[j] && pattern_is_automorphic(all + (size_t)j * 2 * pe, pe, all + (size_t)i * 2 * pe)) {
        dup[i] = 1; break;
      }
    if (!dup[i]) {
      memcpy(p->unique_edges + (size_t)p->num_unique * 2 * pe, all + (size_t)i * 2 * pe,
             sizeof(uint32_t) * 2 * pe);
      p->num_unique++;
    }
  }
  free(perms); free(all); free(dup);
  return ZG_OK;
}

void zgo_program_free(zgo_program* p) { free(p->unique_edges); memset(p, 0, sizeof(*p)); }

static uint32_t prog_den_log2(const zgo_program* p) {
  switch (p->kind) {
    case ZG_PROG_TRIANGLE: return 1;
    case ZG_PROG_FOUR_CLIQUE: return 2;
    case ZG_PROG_FOUR_CLIQUE_UNBIASED: return 2;
    case ZG_PROG_THREE_CHAIN: return 1;
    case ZG_PROG_FOUR_CHAIN: return 2;
    case ZG_PROG_CHAIN: return p->param - 2;
    case ZG_PROG_PATTERN: return p->pe - 1;
  }
  return 0;
}

/* model = 0: a run that keeps no trace; its scratch record is not cleared (ctx_finish sets every
 * field the counters read) and the access model is not counted. */
static void ctx_init_model(zgo_ctx* c, const zgo_graph* g, uint64_t seed, uint32_t stream,
                           uint64_t sample, zg_sample_trace* tr, int model) {
  c->g = g; c->seed = seed; c->stream = stream; c->sample = sample; c->nd = 0; c->tr = tr;
  c->shift = 0; c->num_lo = 1; c->num_hi = 0; c->overflow = 0; c->sectors = 0; c->closures = 0;
  c->model = model;
  if (model) memset(tr, 0, sizeof(*tr));
}
static void ctx_init(zgo_ctx* c, const zgo_graph* g, uint64_t seed, uint32_t stream,
                     uint64_t sample, zg_sample_trace* tr) {
  ctx_init_model(c, g, seed, stream, sample, tr, 1);
}

static void ctx_finish(zgo_ctx* c, double r) {
  zg_sample_trace* tr = c->tr;
  tr->ndraws = c->nd;
  tr->sectors = c->sectors;
  tr->closures = c->closures;
  tr->fail = 0;
  if (r < 0) { tr->fail = 1; r = 0; }
  tr->w = r;
  tr->hit = r != 0;
  if (tr->hit) {
    tr->shift = (uint32_t)c->shift;
    tr->num[0] = (uint64_t)c->num_lo;
    tr->num[1] = (uint64_t)(c->num_lo >> 64);
    tr->num[2] = c->num_hi;
    if (c->overflow) tr->num[2] = ~0ull;
  }
}

static int sample_one(const zgo_graph* g, const zgo_program* p, uint64_t seed, uint32_t stream,
                      uint64_t sample, zg_sample_trace* tr, int model) {
  zgo_ctx c;
  ctx_init_model(&c, g, seed, stream, sample, tr, model);
  double r = 0;
  switch (p->kind) {
    case ZG_PROG_TRIANGLE: r = prog_triangle(&c); break;
    case ZG_PROG_FOUR_CLIQUE: r = prog_four_clique(&c); break;
    case ZG_PROG_FOUR_CLIQUE_UNBIASED: r = prog_four_clique_unbiased(&c); break;
    case ZG_PROG_THREE_CHAIN: r = prog_three_chain(&c); break;
    case ZG_PROG_FOUR_CHAIN: r = prog_four_chain(&c); break;
    case ZG_PROG_CHAIN: r = prog_chain(&c, (int)p->param); break;
    case ZG_PROG_PATTERN: r = prog_pattern(&c, p); break;
    default: return ZG_ERR_UNSUPPORTED_ESTIMATOR;
  }
  ctx_finish(&c, r);
  return ZG_OK;
}

int zgo_sample(const zgo_graph* g, const zgo_program* p, uint64_t seed, uint32_t stream,
               uint64_t sample, zg_sample_trace* tr) {
  return sample_one(g, p, seed, stream, sample, tr, 1);
}

/* ---- exact accumulation ------------------------------------------------- */
static void acc_add(uint64_t acc[5], const uint64_t num[3], uint32_t lsh) {
  uint64_t v[5] = {num[0], num[1], num[2], 0, 0};
  if (lsh) {
    for (int i = 4; i >= 0; --i) {
      v[i] = (v[i] << lsh) | (i ? (v[i - 1] >> (64 - lsh)) : 0);
    }
  }
  u128 carry = 0;
  for (int i = 0; i < 5; ++i) {
    u128 s = (u128)acc[i] + v[i] + carry;
    acc[i] = (uint64_t)s;
    carry = s >> 64;
  }
}

static double acc_mean(const uint64_t acc[5], uint32_t den_log2, uint64_t n) {
  /* exact Σ/2^den/n: long division to a 128-bit quotient window, then one rounding. */
  if (n == 0) return 0;
  long double v = 0;
  for (int i = 4; i >= 0; --i) v = v * 18446744073709551616.0L + (long double)acc[i];
  return (double)(v / (long double)n / ldexpl(1.0L, (int)den_log2));
}

static void counters_fold(zg_counters* out, const zg_sample_trace* tr, uint32_t den) {
  out->samples++;
  if (tr->fail) out->fails++;
  if (tr->hit) {
    out->hits++;
    if (tr->num[2] == ~0ull) out->overflow = 1;
    acc_add(out->sum_num, tr->num, den - tr->shift);
    out->sum_w += tr->w;
    out->sum_w2 += tr->w * tr->w;
    out->sum_w4 += (tr->w * tr->w) * (tr->w * tr->w);
  }
}

static void counters_merge(zg_counters* a, const zg_counters* b) {
  a->samples += b->samples; a->hits += b->hits; a->fails += b->fails;
  a->overflow |= b->overflow;
  acc_add(a->sum_num, b->sum_num, 0);
  uint64_t hi[3] = {b->sum_num[3], b->sum_num[4], 0};
  /* add the upper limbs at 192-bit offset */
  u128 carry = 0;
  for (int i = 3; i < 5; ++i) {
    u128 s = (u128)a->sum_num[i] + hi[i - 3] + carry;
    a->sum_num[i] = (uint64_t)s; carry = s >> 64;
  }
  a->sum_w += b->sum_w; a->sum_w2 += b->sum_w2; a->sum_w4 += b->sum_w4;
}

int zgo_run(const zgo_graph* g, const zgo_program* p, uint64_t n, uint64_t first,
            uint64_t seed, uint32_t stream, int threads, zg_counters* out,
            zg_sample_trace* traces) {
  memset(out, 0, sizeof(*out));
  uint32_t den = prog_den_log2(p);
  out->den_log2 = den;
  int nt = threads;
#ifdef _OPENMP
  if (nt <= 0) nt = omp_get_max_threads();
#else
  nt = 1;
#endif
  zg_counters* part = (zg_counters*)calloc((size_t)nt, sizeof(zg_counters));
  int err = 0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    uint64_t lo = n / (uint64_t)nt * (uint64_t)t;
    uint64_t hi = (t == nt - 1) ? n : lo + n / (uint64_t)nt;
    zg_sample_trace tr;
    /* each thread folds into its own counters and stores them once: per-sample writes to part[t]
       would share cache lines between neighbouring threads */
    zg_counters acc;
    memset(&acc, 0, sizeof(acc));
    for (uint64_t i = lo; i < hi; ++i) {
      zg_sample_trace* tp = traces ? &traces[i] : &tr;
      if (sample_one(g, p, seed, stream, first + i, tp, traces != NULL) != ZG_OK) { err = 1; break; }
      counters_fold(&acc, tp, den);
    }
    part[t] = acc;
  }
  for (int t = 0; t < nt; ++t) counters_merge(out, &part[t]);
  free(part);
  if (err) return ZG_ERR_UNSUPPORTED_ESTIMATOR;
  out->estimate = acc_mean(out->sum_num, den, out->samples);
  return ZG_OK;
}

/* applications/ThreeMotif.cpp:48-121 with ZGraphInstanceWithCache (src/ZGraphInstance.cpp:
 * 669-833), one thread: estimator i of the triangle instance reuses wedge i of the chain
 * instance when i < n_chain, and samples afresh otherwise. */
int zgo_run_three_motif(const zgo_graph* g, uint64_t n_chain, uint64_t n_tri, uint64_t seed,
                        uint32_t stream_chain, uint32_t stream_tri, zg_counters* out_chain,
                        zg_counters* out_tri, zg_sample_trace* chain_tr,
                        zg_sample_trace* tri_tr) {
  memset(out_chain, 0, sizeof(*out_chain));
  memset(out_tri, 0, sizeof(*out_tri));
  out_chain->den_log2 = 1; out_tri->den_log2 = 1;
  zg_sample_trace ctr, ttr;
  for (uint64_t i = 0; i < (n_chain > n_tri ? n_chain : n_tri); ++i) {
    zg_sample_trace* cp = chain_tr ? &chain_tr[i < n_chain ? i : 0] : &ctr;
    zg_sample_trace* tp = tri_tr ? &tri_tr[i < n_tri ? i : 0] : &ttr;
    if (i < n_chain) {
      /* ThreeChainCountingInstance::estimate (:95-121) keeps the wedge and p */
      zgo_ctx c;
      ctx_init(&c, g, seed, stream_chain, i, cp);
      zgo_sub sg; sub_init(&sg);
      double pr = 1, r;
      zgo_edge e0, e1;
      double t = prim_sample_edge(&c, &e0);
      if (t < 0) r = -1;
      else {
        pr *= t; sub_add_edge(&sg, e0);
        t = prim_cond_sample(&c, sg.e, sg.ne, sg.v, sg.nv, &e1);
        if (t < 0) r = -1;
        else { pr *= t; sub_add_edge(&sg, e1); r = 1. / pr; }
      }
      ctx_finish(&c, r);
      counters_fold(out_chain, cp, 1);
      if (i < n_tri) {
        /* TriangleCoutingInstance::estimate, cached branch (:54-62) */
        zgo_ctx d;
        ctx_init(&d, g, seed, stream_tri, i, tp);
        double rt;
        if (r < 0) rt = 0;
        else {
          zgo_sub tri, wait;
          tri_pattern(sg.e[0], sg.e[1], &tri);
          sub_minus(&tri, &sg, &wait);
          rt = prim_close(&d, &sg, &wait) ? 1. / pr : 0;
        }
        ctx_finish(&d, rt);
        if (rt != 0) {
          tp->shift = (uint32_t)c.shift;
          memcpy(tp->num, cp->num, sizeof(tp->num));
        }
        counters_fold(out_tri, tp, 1);
      }
    } else if (i < n_tri) {
      zgo_ctx d;
      ctx_init(&d, g, seed, stream_tri, i, tp);
      double rt = prog_triangle(&d);
      ctx_finish(&d, rt);
      counters_fold(out_tri, tp, 1);
    }
  }
  out_chain->estimate = acc_mean(out_chain->sum_num, 1, out_chain->samples);
  out_tri->estimate = acc_mean(out_tri->sum_num, 1, out_tri->samples);
  return ZG_OK;
}

/* ------------------------------------------------------------------------- */
/* Edge selections for the derived graphs. */
int zgo_pred(int op, int64_t t0, int64_t t1, uint32_t w) {
  int64_t x = (int64_t)w;
  switch (op) {
    case ZG_PRED_GE: return x >= t0;
    case ZG_PRED_LT: return x < t0;
    case ZG_PRED_GT: return x > t0;
    case ZG_PRED_LE: return x <= t0;
    case ZG_PRED_EQ: return x == t0;
    case ZG_PRED_NE: return x != t0;
    case ZG_PRED_RANGE: return x >= t0 && x < t1;
  }
  return 0;
}

int zgo_subsample_keep(double rate, uint64_t keep_seed, uint64_t e) {
  const unsigned long long max_rand_int = (unsigned long long)1 << 30; /* src/Graph.cpp:652 */
  unsigned long long threshold = rate * max_rand_int;                   /* :653 */
  return zgo_draw(keep_seed, ZGO_STREAM_SUBSAMPLE, e, 0, 1, max_rand_int) <= threshold;
}

typedef struct { uint64_t key, idx; } zgo_kv;
static int kv_cmp(const void* a, const void* b) {
  const zgo_kv* x = (const zgo_kv*)a; const zgo_kv* y = (const zgo_kv*)b;
  if (x->key != y->key) return x->key < y->key ? -1 : 1;
  return x->idx < y->idx ? -1 : (x->idx > y->idx);
}
uint64_t zgo_shuffle_key(uint64_t shuffle_seed, uint64_t i) {
  return zgo_draw(shuffle_seed, ZGO_STREAM_SHUFFLE, i, 0, 0, ~0ull);
}

/* The GPU permutes by sorting (Philox key, position); output edge i comes from perm[i]. */
void zgo_shuffle_perm(uint64_t m, uint64_t shuffle_seed, uint64_t* perm) {
  zgo_kv* kv = (zgo_kv*)malloc(sizeof(zgo_kv) * (m ? m : 1));
  for (uint64_t i = 0; i < m; ++i) {
    kv[i].key = zgo_shuffle_key(shuffle_seed, i);
    kv[i].idx = i;
  }
  qsort(kv, m, sizeof(zgo_kv), kv_cmp);
  for (uint64_t i = 0; i < m; ++i) perm[i] = kv[i].idx;
  free(kv);
}

/* ZGraphInstance::conditional_close(min_valid_edge_id, sampled_vertices, edges_to_wait&)
 * (src/ZGraphInstance.cpp:410-441): each edge to wait in order, searched in every sampled
 * vertex's list (ids below min_valid skipped), its edge id written back when found; returns 0 at
 * the first edge not found.  *found: the edges found before that. */
int zgo_conditional_close_ids(const zgo_graph* g, uint64_t min_valid, const uint32_t* vertices, uint32_t nv,
                              const uint32_t* edges, uint32_t ne, uint64_t* edge_ids, uint32_t* found) {
  *found = 0;
  for (uint32_t i = 0; i < ne; ++i) {
    uint32_t ws = edges[2 * i], wd = edges[2 * i + 1];
    int hit = 0;
    for (uint32_t j = 0; j < nv && !hit; ++j) {
      uint32_t v = vertices[j];
      if (v >= g->nv) continue; /* outgoing_adj_bitmap: no list */
      for (uint64_t idx = g->off[v]; idx < g->off[v + 1]; ++idx) {
        if (g->adj_eid[idx] < min_valid) continue;
        uint32_t s = v, d = g->adj_nbr[idx];
        if ((s == ws && d == wd) || (d == ws && s == wd)) { edge_ids[i] = g->adj_eid[idx]; hit = 1; break; }
      }
    }
    if (!hit) return 0;
    *found = i + 1;
  }
  return 1;
}

/* ------------------------------------------------------------------------- */
/* Exact counts.  u128 results. */
static void put128(uint64_t out[2], u128 v) { out[0] = (uint64_t)v; out[1] = (uint64_t)(v >> 64); }

static int has_edge(const zgo_graph* g, uint32_t a, uint32_t b) {
  for (uint64_t i = g->off[a]; i < g->off[a + 1]; ++i) if (g->adj_nbr[i] == b) return 1;
  return 0;
}

/* naive_implementation/{TriangleCounting,ThreeChain,FourChain,FiveStar,FourClique}.cpp */
int zgo_exact_naive(const zgo_graph* g, int kind, uint64_t out[2]) {
  const uint64_t* off = g->off;
  const uint32_t* nb = g->adj_nbr;
  u128 cnt = 0;
  uint32_t V = g->nv;
  switch (kind) {
    case ZG_EXACT_TRIANGLE:
      for (uint32_t i = 0; i < V; ++i)
        for (uint64_t a = off[i]; a < off[i + 1]; ++a) {
          uint32_t j = nb[a];
          if (j <= i) continue;
          for (uint64_t b = off[j]; b < off[j + 1]; ++b) {
            uint32_t k = nb[b];
            if (k <= j) continue;
            if (has_edge(g, k, i)) cnt++;
          }
        }
      break;
    case ZG_EXACT_WEDGE:
      for (uint32_t v = 0; v < V; ++v) {
        uint64_t d = off[v + 1] - off[v];
        cnt += (u128)(d * (d - 1) / 2);
      }
      break;
    case ZG_EXACT_THREE_PATH:
      for (uint32_t v0 = 0; v0 < V; ++v0)
        for (uint64_t a = off[v0]; a < off[v0 + 1]; ++a) {
          uint32_t v1 = nb[a];
          for (uint64_t b = off[v1]; b < off[v1 + 1]; ++b) {
            uint32_t v2 = nb[b];
            if (v2 == v0) continue;
            for (uint64_t c = off[v2]; c < off[v2 + 1]; ++c) {
              uint32_t v3 = nb[c];
              if (v3 != v0 && v3 != v1) cnt++;
            }
          }
        }
      cnt /= 2;
      break;
    case ZG_EXACT_FIVE_STAR:
      for (uint32_t v = 0; v < V; ++v) {
        uint64_t d = off[v + 1] - off[v];
        if (d >= 4) { uint64_t x = d * (d - 1) * (d - 2) * (d - 3); x /= 24; cnt += x; }
      }
      break;
    case ZG_EXACT_FOUR_CLIQUE:
      for (uint32_t i = 0; i < V; ++i)
        for (uint64_t a = off[i]; a < off[i + 1]; ++a) {
          uint32_t j = nb[a];
          if (j <= i) continue;
          for (uint64_t b = off[j]; b < off[j + 1]; ++b) {
            uint32_t k = nb[b];
            if (k <= j) continue;
            if (!has_edge(g, k, i)) continue;
            for (uint32_t z = k + 1; z < V; ++z) {
              int ct = 0;
              for (uint64_t c = off[z]; c < off[z + 1]; ++c) {
                if (nb[c] == i) ++ct;
                if (nb[c] == j) ++ct;
                if (nb[c] == k) ++ct;
              }
              if (ct == 3) cnt++;
            }
          }
        }
      break;
    case ZG_EXACT_FIVE_HOUSE:
      /* naive_implementation/FiveHouse.cpp:25-49,110-130: every triangle i < j < k, and for each of
       * its edges (left, right) with the third vertex `other`, the pairs (x, y), x a neighbour of
       * left and y one of right, both outside the triangle, x != y, joined by an edge */
      for (uint32_t i = 0; i < V; ++i)
        for (uint64_t a = off[i]; a < off[i + 1]; ++a) {
          uint32_t j = nb[a];
          if (j <= i) continue;
          for (uint64_t b = off[j]; b < off[j + 1]; ++b) {
            uint32_t k = nb[b];
            if (k <= j || !has_edge(g, k, i)) continue;
            const uint32_t tri[3][3] = {{i, j, k}, {i, k, j}, {j, k, i}};
            for (int r = 0; r < 3; ++r) {
              uint32_t l = tri[r][0], rt = tri[r][1], o = tri[r][2];
              for (uint64_t x = off[l]; x < off[l + 1]; ++x) {
                uint32_t vl = nb[x];
                if (vl == l || vl == rt || vl == o) continue;
                for (uint64_t y = off[rt]; y < off[rt + 1]; ++y) {
                  uint32_t vr = nb[y];
                  if (vr == l || vr == rt || vr == o || vr == vl) continue;
                  if (has_edge(g, vr, vl)) cnt++;
                }
              }
            }
          }
        }
      break;
    case ZG_EXACT_FIVE_CHAIN:
      /* naive_implementation/FiveChain.cpp:44-72: walks v0-v1-v2-v3-v4 with v2 != v0,
       * v3 not in {v0, v1}, v4 not in {v0, v1, v2}; each path is walked from both ends */
      for (uint32_t v0 = 0; v0 < V; ++v0)
        for (uint64_t a = off[v0]; a < off[v0 + 1]; ++a) {
          uint32_t v1 = nb[a];
          for (uint64_t b = off[v1]; b < off[v1 + 1]; ++b) {
            uint32_t v2 = nb[b];
            if (v2 == v0) continue;
            for (uint64_t c = off[v2]; c < off[v2 + 1]; ++c) {
              uint32_t v3 = nb[c];
              if (v3 == v0 || v3 == v1) continue;
              for (uint64_t d = off[v3]; d < off[v3 + 1]; ++d) {
                uint32_t v4 = nb[d];
                if (v4 != v0 && v4 != v1 && v4 != v2) cnt++;
              }
            }
          }
        }
      cnt /= 2;
      break;
    default:
      return ZG_ERR_INVALID_ARG;
  }
  put128(out, cnt);
  return ZG_OK;
}

static int cmp_u32(const void* a, const void* b) {
  uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
  return x < y ? -1 : (x > y);
}

/* Faster restatements: sorted neighbour lists, merge intersections; vertices split over the
 * OpenMP threads, per-thread 128-bit partial sums added in thread order. */
static uint64_t merge_count(const uint32_t* s, uint64_t i, uint64_t ie, uint64_t j, uint64_t je) {
  uint64_t c = 0;
  while (i < ie && j < je) {
    if (s[i] < s[j]) ++i;
    else if (s[i] > s[j]) ++j;
    else { ++c; ++i; ++j; }
  }
  return c;
}

/* Houses and 4-edge paths from per-edge counts (the identities the GPU counter uses, checked here
 * against the naive walks above): with t(e) the triangles and c4(e) the 4-cycles through edge
 * e = (a, b), c4(a, b) = sum over x in N(a) \ {b} of (|N(x) ∩ N(b)| - 1),
 *   houses      = sum_e t(e) c4(e) - 2 sum_e t(e)^2 + 6 T
 *   4-edge paths = (sum_v (S1(v)^2 - S2(v)) + 2 sum_e t(e) (3 - d_a - d_b) - 2 sum_e c4(e)) / 2
 * with S1(v) = sum over w in N(v) of (d_w - 1) and S2(v) the sum of the squares. */
static int exact_house_chain(const zgo_graph* g, int kind, const uint32_t* s, uint64_t out[2]) {
  typedef __int128 i128;
  const uint64_t* off = g->off;
  uint32_t V = g->nv;
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#endif
  i128* part = (i128*)calloc((size_t)nt, sizeof(i128));
  if (!part) return ZG_ERR_OOM;
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    i128 acc = 0;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
    for (uint32_t a = 0; a < V; ++a) {
      uint64_t da = off[a + 1] - off[a];
      if (kind == ZG_EXACT_FIVE_CHAIN) {
        i128 s1 = 0, s2 = 0;
        for (uint64_t p = off[a]; p < off[a + 1]; ++p) {
          i128 dw = (i128)(off[s[p] + 1] - off[s[p]]) - 1;
          s1 += dw;
          s2 += dw * dw;
        }
        acc += s1 * s1 - s2;
      }
      for (uint64_t p = off[a]; p < off[a + 1]; ++p) {
        uint32_t b = s[p];
        if (b <= a) continue; /* each undirected edge once */
        uint64_t db = off[b + 1] - off[b];
        i128 te = (i128)merge_count(s, off[a], off[a + 1], off[b], off[b + 1]);
        if (kind == ZG_EXACT_FIVE_HOUSE && te == 0) continue;
        i128 c4 = 0;
        for (uint64_t q = off[a]; q < off[a + 1]; ++q) {
          uint32_t x = s[q];
          if (x == b) continue;
          c4 += (i128)merge_count(s, off[x], off[x + 1], off[b], off[b + 1]) - 1;
        }
        if (kind == ZG_EXACT_FIVE_HOUSE)
          acc += te * c4 - 2 * te * te + 2 * te; /* 6 T = 2 sum_e t(e) */
        else
          acc += 2 * te * (3 - (i128)da - (i128)db) - 2 * c4;
      }
    }
    part[t] = acc;
  }
  i128 tot = 0;
  for (int t = 0; t < nt; ++t) tot += part[t];
  free(part);
  if (kind == ZG_EXACT_FIVE_CHAIN) tot /= 2;
  put128(out, (u128)tot);
  return ZG_OK;
}

int zgo_exact_fast(const zgo_graph* g, int kind, uint64_t out[2]) {
  uint32_t V = g->nv;
  const uint64_t* off = g->off;
  if (kind == ZG_EXACT_WEDGE || kind == ZG_EXACT_FIVE_STAR) return zgo_exact_naive(g, kind, out);
  uint32_t* s = (uint32_t*)malloc(sizeof(uint32_t) * (g->m ? 2 * g->m : 1));
  if (!s) return ZG_ERR_OOM;
  memcpy(s, g->adj_nbr, sizeof(uint32_t) * 2 * g->m);
  int nt = 1;
#ifdef _OPENMP
  nt = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nt)
#endif
  for (uint32_t v = 0; v < V; ++v) qsort(s + off[v], off[v + 1] - off[v], sizeof(uint32_t), cmp_u32);
  if (kind == ZG_EXACT_FIVE_HOUSE || kind == ZG_EXACT_FIVE_CHAIN) {
    int rc = exact_house_chain(g, kind, s, out);
    free(s);
    return rc;
  }
  u128* part = (u128*)calloc((size_t)nt * 3, sizeof(u128)); /* tri3, paths, cliques per thread */
  if (!part) { free(s); return ZG_ERR_OOM; }
#ifdef _OPENMP
#pragma omp parallel num_threads(nt)
#endif
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    u128 tri3 = 0, paths = 0, cnt = 0;
    uint32_t* com = NULL;
    uint64_t com_cap = 0;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
    for (uint32_t u = 0; u < V; ++u)
      for (uint64_t a = off[u]; a < off[u + 1]; ++a) {
        uint32_t v = s[a];
        if (v <= u) continue;
        uint64_t du = off[u + 1] - off[u], dv = off[v + 1] - off[v];
        paths += (u128)(du - 1) * (dv - 1);
        if (kind == ZG_EXACT_THREE_PATH || kind == ZG_EXACT_TRIANGLE) {
          /* triangles per edge (u<v): |N(u) ∩ N(v)| */
          uint64_t i = off[u], j = off[v];
          while (i < off[u + 1] && j < off[v + 1]) {
            if (s[i] < s[j]) ++i;
            else if (s[i] > s[j]) ++j;
            else { if (kind == ZG_EXACT_TRIANGLE) { if (s[i] > v) tri3++; } else tri3++; ++i; ++j; }
          }
        } else if (kind == ZG_EXACT_FOUR_CLIQUE) {
          /* common neighbours w > v, then pairs (w,x) with w<x both common and adjacent */
          uint64_t need = (du < dv ? du : dv) + 4;
          if (need > com_cap) { free(com); com_cap = need; com = (uint32_t*)malloc(sizeof(uint32_t) * com_cap); }
          uint64_t nc = 0, i = off[u], j = off[v];
          while (i < off[u + 1] && j < off[v + 1]) {
            if (s[i] < s[j]) ++i;
            else if (s[i] > s[j]) ++j;
            else { if (s[i] > v) com[nc++] = s[i]; ++i; ++j; }
          }
          for (uint64_t x = 0; x < nc; ++x) {
            uint32_t w = com[x];
            /* count com[y] (y > x) adjacent to w: merge N(w) with com[x+1..] */
            uint64_t p = off[w], q = x + 1;
            while (p < off[w + 1] && q < nc) {
              if (s[p] < com[q]) ++p;
              else if (s[p] > com[q]) ++q;
              else { cnt++; ++p; ++q; }
            }
          }
        }
      }
    free(com);
    part[3 * t] = tri3; part[3 * t + 1] = paths; part[3 * t + 2] = cnt;
  }
  u128 tri3 = 0, paths = 0, cnt = 0;
  for (int t = 0; t < nt; ++t) { tri3 += part[3 * t]; paths += part[3 * t + 1]; cnt += part[3 * t + 2]; }
  free(part);
  if (kind == ZG_EXACT_TRIANGLE) cnt = tri3;
  else if (kind == ZG_EXACT_THREE_PATH) cnt = paths - tri3; /* tri3 here = 3 * triangles */
  free(s);
  put128(out, cnt);
  return ZG_OK;
}

/* naive_implementation/WeightedTriangleCounting.cpp (all three edges >= t) and
 * AtLeastOneWeightedTriangleCounting.cpp (at least one edge >= t). */
int zgo_exact_weighted_triangle(const zgo_graph* g, uint32_t t, int at_least_one,
                                uint64_t out[2]) {
  if (!g->w) return ZG_ERR_INVALID_ARG;
  const uint64_t* off = g->off;
  u128 cnt = 0;
  for (uint32_t i = 0; i < g->nv; ++i)
    for (uint64_t a = off[i]; a < off[i + 1]; ++a) {
      uint32_t j = g->adj_nbr[a];
      if (j <= i) continue;
      if (!at_least_one && g->adj_w[a] < t) continue;
      for (uint64_t b = off[j]; b < off[j + 1]; ++b) {
        uint32_t k = g->adj_nbr[b];
        if (k <= j) continue;
        if (!at_least_one && g->adj_w[b] < t) continue;
        for (uint64_t c = off[k]; c < off[k + 1]; ++c) {
          if (g->adj_nbr[c] != i) continue;
          int ok = at_least_one ? (g->adj_w[a] >= t || g->adj_w[b] >= t || g->adj_w[c] >= t)
                                : (g->adj_w[c] >= t);
          if (ok) { cnt++; break; }
        }
      }
    }
  put128(out, cnt);
  return ZG_OK;
}

/* ------------------------------------------------------------------------- */
double zgo_calculate_bound(double epsilon, double delta, double nse, double ncse,
                           double estimation, uint64_t max_degree, uint64_t num_edges) {
  double factor_0 = 1. / pow(epsilon, 2.);
  double factor_1 = pow((double)max_degree, ncse) * pow((double)num_edges, nse) / estimation;
  double factor_2 = log(2. / delta);
  return factor_0 * factor_1 * factor_2;
}

double zgo_regression_k(const double* x, const double* y, uint32_t len) {
  long double t0 = 0, t1 = 0;
  for (uint32_t i = 0; i < len; ++i) t0 += (long double)x[i] * (long double)y[i];
  for (uint32_t i = 0; i < len; ++i) t1 += (long double)x[i] * (long double)x[i];
  return (double)(t0 / t1);
}
