/*
 * Driver around one reference application, compiled into oracle/_ref/ by
 * oracle/build_ref.sh.  Each app_*.cpp includes the reference application source (its main
 * renamed), defines ZGREF_E and zgref_make(), then includes this file.
 *
 * The graph is built with the reference's own CSRConstructor (src/Graph.cpp:215-377) from
 * the given edge order (its shuffle is replayed as the identity), and estimate() is called
 * per sample with the recorded draws queued in the replaying Random.  Test infrastructure.
 */
#ifndef ZGREF_DRIVER_HPP
#define ZGREF_DRIVER_HPP

#include <stdint.h>
#include <string.h>
#include <type_traits>
#include <vector>

#include <numa.h>

#include "Graph.hpp"
#include "NetworkInterface.hpp"
#include "SharedMemSys.hpp"
#include "ZGraphInstance.hpp"
#include "ErrorLatencyProfile.hpp"
#include "zgref_replay.hpp"
#include "../../include/zgraph_gpu.h"
#include "../zg_oracle.h"

#define ZGREF_API extern "C" __attribute__((visibility("default")))

static void zgref_boot() {
  static bool booted = false;
  if (booted) return;
  booted = true;
  static int argc = 1;
  static char arg0[] = "zgref";
  static char* argv_[] = {arg0, nullptr};
  static char** argv = argv_;
  NetworkInterface::init_network_interface(&argc, &argv);
  SharedMemSys::init_shared_mem_sys();
}

template <typename E>
static void zgref_fill_edge_data(EdgeUnit<E>& u, const uint32_t* w, uint64_t e) {
  if (w) memcpy(&u.edge_data, &w[e], sizeof(E));
}
template <>
void zgref_fill_edge_data<Empty>(EdgeUnit<Empty>&, const uint32_t*, uint64_t) {}

/* Graph<E> in the loader's end state for one partition / one socket, edge ids = positions. */
template <typename E>
static void zgref_build_graph(Graph<E>& g, const uint32_t* edges, uint64_t m, uint32_t nv,
                              const uint32_t* w) {
  UniformGraphPartitioner part(nv);
  part.partition_graph(g.p);
  g.edge_data_size = std::is_same<E, Empty>::value ? 0 : sizeof(E);
  g.edge_unit_size = g.edge_data_size + sizeof(VertexId) * 2;
  g.num_vertices = nv;
  g.num_edges = m;
  g.degree = (EdgeId*)numa_alloc_interleaved(sizeof(EdgeId) * nv);
  for (uint64_t e = 0; e < m; ++e) { g.degree[edges[2 * e]]++; g.degree[edges[2 * e + 1]]++; }
  g.max_degree = 0;
  for (uint32_t v = 0; v < nv; ++v) if (g.degree[v] > g.max_degree) g.max_degree = g.degree[v];
  EdgeId* nle = new EdgeId[1];
  nle[0] = m;
  EdgeUnit<E>** le = new EdgeUnit<E>*[1];
  le[0] = (EdgeUnit<E>*)numa_alloc_onnode(sizeof(EdgeUnit<E>) * (m ? m : 1), 0);
  for (uint64_t e = 0; e < m; ++e) {
    le[0][e].src = edges[2 * e];
    le[0][e].dst = edges[2 * e + 1];
    zgref_fill_edge_data<E>(le[0][e], w, e);
  }
  zgref_replay.raw_script = zgref_shuffle_script(nullptr, m); /* identity shuffle */
  zgref_replay.raw_pos = 0;
  CSRConstructor<E> csr;
  csr.construct_bitmap_assisted_csr(le, nle, g);
  g.num_local_edges = nle;
  g.local_edges = le;
}

struct ZgrefHandle {
  Graph<ZGREF_E> graph;
  ZGraphInstance<ZGREF_E>* inst = nullptr;
};

static ZGraphInstance<ZGREF_E>* zgref_make(Graph<ZGREF_E>* g, uint32_t param,
                                           const uint32_t* pattern, uint32_t pv, uint32_t pe);

static void zgref_queue(const zg_sample_trace& t) {
  for (uint32_t d = 0; d < t.ndraws && d < ZG_MAX_DRAWS; ++d)
    zgref_replay.q.push_back(ZgrefDraw{t.lo[d], t.hi[d], t.val[d]});
}

/* filter_perm: permutation the derived (filtered) graph's shuffle must realise (AllPredicate). */
ZGREF_API void* zgref_open(const uint32_t* edges, uint64_t m, uint32_t nv, const uint32_t* w,
                           uint32_t param, const uint64_t* filter_perm, uint64_t filter_m,
                           const uint32_t* pattern, uint32_t pv, uint32_t pe) {
  zgref_boot();
  ZgrefHandle* h = new ZgrefHandle();
  zgref_build_graph<ZGREF_E>(h->graph, edges, m, nv, w);
  zgref_replay.raw_script = zgref_shuffle_script(filter_perm, filter_perm ? filter_m : 0);
  zgref_replay.raw_pos = 0;
  zgref_replay.reset_counts();
  h->inst = zgref_make(&h->graph, param, pattern, pv, pe);
  return h;
}

/* estimate() per sample: out[i] its result, consumed[i] draws taken; returns #mismatches. */
ZGREF_API uint64_t zgref_estimates(void* hv, uint64_t n, const zg_sample_trace* tr, double* out,
                                   uint32_t* consumed) {
  ZgrefHandle* h = (ZgrefHandle*)hv;
  uint64_t bad = 0;
  for (uint64_t i = 0; i < n; ++i) {
    zgref_replay.q.clear();
    zgref_replay.reset_counts();
    zgref_queue(tr[i]);
    out[i] = h->inst->estimate();
    consumed[i] = (uint32_t)zgref_replay.consumed;
    bad += zgref_replay.mismatches + zgref_replay.overruns + zgref_replay.q.size();
  }
  zgref_replay.q.clear();
  return bad;
}

/* calculate(n, k, Estimation) with all draws queued in sample order (one thread). */
ZGREF_API double zgref_calculate(void* hv, uint64_t n, uint32_t k, const zg_sample_trace* tr,
                                 uint64_t* bad) {
  ZgrefHandle* h = (ZgrefHandle*)hv;
  zgref_replay.q.clear();
  zgref_replay.reset_counts();
  for (uint64_t i = 0; i < n; ++i) zgref_queue(tr[i]);
  Estimation est;
  double r = h->inst->calculate(n, k, est);
  *bad = zgref_replay.mismatches + zgref_replay.overruns + zgref_replay.q.size();
  zgref_replay.q.clear();
  return r;
}

/* ErrorProfile<E>::get_num_estimators run by the reference itself, its Random replaying, in the
 * order the reference consumes them: 1024 probe estimators on the original graph (oracle stream
 * probe_stream), one keep draw per edge for GraphSampler, the shuffle of the kept edges, then the
 * 2^14 x 16 + 2^23 estimators on the subsample (oracle, stream ZG_ELP_STREAM, indices from 0) —
 * the draw plan of zg_elp_plain.  Returns n_required; *bad counts replay mismatches. */
ZGREF_API void zgref_close(void* hv);

struct ZgrefElpFeed {
  const zgo_graph* orig;
  zgo_graph sub;
  zgo_program prog;
  uint64_t seed, m, next_probe, next_keep, next_sample, total_samples;
  uint32_t probe_stream;
};

static bool zgref_elp_refill(void* vctx) {
  ZgrefElpFeed* f = (ZgrefElpFeed*)vctx;
  zg_sample_trace t;
  if (f->next_probe < 1024) {
    for (int k = 0; k < 256 && f->next_probe < 1024; ++k, ++f->next_probe) {
      zgo_sample(f->orig, &f->prog, f->seed, f->probe_stream, f->next_probe, &t);
      zgref_queue(t);
    }
    return true;
  }
  if (f->next_keep < f->m) {
    for (int k = 0; k < 65536 && f->next_keep < f->m; ++k, ++f->next_keep) {
      uint64_t v = zgo_draw(f->seed + ZG_ELP_KEEP_OFFSET, 0xFFFFFFF1u, f->next_keep, 0, 1, 1ull << 30);
      zgref_replay.q.push_back(ZgrefDraw{1, 1ull << 30, v});
    }
    return true;
  }
  if (f->next_sample < f->total_samples) {
    for (int k = 0; k < 4096 && f->next_sample < f->total_samples; ++k, ++f->next_sample) {
      zgo_sample(&f->sub, &f->prog, f->seed, ZG_ELP_STREAM, f->next_sample, &t);
      zgref_queue(t);
    }
    return true;
  }
  return false;
}

ZGREF_API uint64_t zgref_elp(const uint32_t* edges, uint64_t m, uint32_t nv, int kind, uint32_t param,
                             const uint32_t* pattern, uint32_t pv, uint32_t pe, uint64_t seed, uint32_t probe_stream,
                             double eps, double conf, uint64_t* bad) {
  zgref_boot();
  ZgrefHandle* h = (ZgrefHandle*)zgref_open(edges, m, nv, nullptr, param, nullptr, 0, pattern, pv, pe);
  ZgrefElpFeed f;
  zgo_graph orig;
  zgo_graph_build(&orig, nv, m, edges, nullptr);
  f.orig = &orig;
  zgo_program_init(&f.prog, kind, param, pv, pe, pattern);
  f.seed = seed;
  f.m = m;
  f.probe_stream = probe_stream;
  f.next_probe = f.next_keep = f.next_sample = 0;
  f.total_samples = (1ull << 18) + (1ull << 23);
  // the subsample our device builds: kept edges in order, then permuted
  std::vector<uint64_t> kept;
  for (uint64_t e = 0; e < m; ++e)
    if (zgo_subsample_keep(0.1, seed + ZG_ELP_KEEP_OFFSET, e)) kept.push_back(e);
  std::vector<uint64_t> perm(kept.size() ? kept.size() : 1);
  zgo_shuffle_perm(kept.size(), seed + ZG_ELP_SHUFFLE_OFFSET, perm.data());
  std::vector<uint32_t> sub_edges(2 * kept.size());
  for (size_t i = 0; i < kept.size(); ++i) {
    sub_edges[2 * i] = edges[2 * kept[perm[i]]];
    sub_edges[2 * i + 1] = edges[2 * kept[perm[i]] + 1];
  }
  zgo_graph_build(&f.sub, nv, kept.size(), sub_edges.data(), nullptr);
  zgref_replay.q.clear();
  zgref_replay.reset_counts();
  zgref_replay.raw_script = zgref_shuffle_script(perm.data(), kept.size());
  zgref_replay.raw_pos = 0;
  zgref_replay.refill = zgref_elp_refill;
  zgref_replay.refill_ctx = &f;
  ErrorProfile<ZGREF_E> ep;
  unsigned long long n = ep.get_num_estimators(*h->inst, 3, eps, conf);
  *bad = zgref_replay.mismatches + zgref_replay.overruns + zgref_replay.q.size() + zgref_replay.raw_overruns +
         (f.next_sample != f.total_samples);
  zgref_replay.refill = nullptr;
  zgref_replay.q.clear();
  zgo_graph_free(&f.sub);
  zgo_graph_free(&orig);
  zgo_program_free(&f.prog);
  zgref_close(h);
  return n;
}

ZGREF_API void zgref_close(void* hv) {
  ZgrefHandle* h = (ZgrefHandle*)hv;
  delete h->inst;
  NumaAwareGraphDestroyer<ZGREF_E> d;
  d.destroy_graph(h->graph);
  delete h;
}

#endif
