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
#include "zgref_replay.hpp"
#include "../../include/zgraph_gpu.h"

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

ZGREF_API void zgref_close(void* hv) {
  ZgrefHandle* h = (ZgrefHandle*)hv;
  delete h->inst;
  NumaAwareGraphDestroyer<ZGREF_E> d;
  d.destroy_graph(h->graph);
  delete h;
}

#endif
