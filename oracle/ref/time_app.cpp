/*
 * Times the reference's own ZGraphInstance::calculate (its own mt19937 Random and OpenMP
 * threads, src/ZGraphInstance.cpp:257-297) for one application on a given edge list: a CPU
 * measurement of the unmodified estimator path, next to the oracle port.  Compiled by
 * oracle/build_ref.sh with ZGREF_APP_FILE / ZGREF_APP_CLASS set, or with ZGREF_PATTERN for
 * SamplerGenerator<Empty> on a pattern given at run time (as applications/FiveStar.cpp:18-26 and
 * FiveHouse.cpp:18-27 build theirs).  Test infrastructure.
 */
#ifdef ZGREF_PATTERN
#include <vector>
#include "SamplerGenerator.hpp"
#else
#define main zgref_app_main
#include ZGREF_APP_FILE
#undef main
#endif

#include <stdint.h>
#include <chrono>
#include <type_traits>

#include <numa.h>

#include "Graph.hpp"
#include "NetworkInterface.hpp"
#include "SharedMemSys.hpp"
#include "ZGraphInstance.hpp"

int zgref_num_cpus = 1;

/* Graph<Empty> in the loader's end state for one partition / one socket; the reference's
 * CSRConstructor shuffles the edges with its own Random (src/Graph.cpp:215-377). */
static void zgref_time_graph(Graph<Empty>& g, const uint32_t* edges, uint64_t m, uint32_t nv) {
  UniformGraphPartitioner part(nv);
  part.partition_graph(g.p);
  g.edge_data_size = 0;
  g.edge_unit_size = sizeof(VertexId) * 2;
  g.num_vertices = nv;
  g.num_edges = m;
  g.degree = (EdgeId*)numa_alloc_interleaved(sizeof(EdgeId) * nv);
  for (uint32_t v = 0; v < nv; ++v) g.degree[v] = 0;
  for (uint64_t e = 0; e < m; ++e) { g.degree[edges[2 * e]]++; g.degree[edges[2 * e + 1]]++; }
  g.max_degree = 0;
  for (uint32_t v = 0; v < nv; ++v) if (g.degree[v] > g.max_degree) g.max_degree = g.degree[v];
  EdgeId* nle = new EdgeId[1];
  nle[0] = m;
  EdgeUnit<Empty>** le = new EdgeUnit<Empty>*[1];
  le[0] = (EdgeUnit<Empty>*)numa_alloc_onnode(sizeof(EdgeUnit<Empty>) * (m ? m : 1), 0);
  for (uint64_t e = 0; e < m; ++e) {
    le[0][e].src = edges[2 * e];
    le[0][e].dst = edges[2 * e + 1];
  }
  CSRConstructor<Empty> csr;
  csr.construct_bitmap_assisted_csr(le, nle, g);
  g.num_local_edges = nle;
  g.local_edges = le;
}

static void zgref_boot(int threads) {
  static bool booted = false;
  zgref_num_cpus = threads > 0 ? threads : 1;
  if (!booted) {
    booted = true;
    static int argc = 1;
    static char arg0[] = "zgref";
    static char* argv_[] = {arg0, nullptr};
    static char** argv = argv_;
    NetworkInterface::init_network_interface(&argc, &argv);
    SharedMemSys::init_shared_mem_sys();
  }
}

/* calculate(n / 16) once untimed, then calculate(n) timed; returns seconds, *estimate the result. */
static double zgref_time_instance(ZGraphInstance<Empty>* inst, uint64_t n, double* estimate) {
  Estimation warm;
  inst->calculate(n / 16 + 1, 3, warm);
  Estimation est;
  auto t0 = std::chrono::steady_clock::now();
  double r = inst->calculate(n, 3, est);
  auto t1 = std::chrono::steady_clock::now();
  *estimate = r;
  return std::chrono::duration<double>(t1 - t0).count();
}

#ifdef ZGREF_PATTERN
/* SamplerGenerator<Empty> for the pattern of pv vertices and pe edges (pedges: (src, dst) pairs,
 * edge_id = index), timed with `threads` OpenMP threads. */
extern "C" __attribute__((visibility("default"))) double zgref_time_pattern(const uint32_t* edges, uint64_t m,
                                                                             uint32_t nv, uint32_t pv, uint32_t pe,
                                                                             const uint32_t* pedges, uint64_t n,
                                                                             int threads, double* estimate) {
  zgref_boot(threads);
  Graph<Empty> g;
  zgref_time_graph(g, edges, m, nv);
  std::vector<Edge<Empty>> es(pe);
  for (uint32_t i = 0; i < pe; ++i) {
    es[i].src = pedges[2 * i];
    es[i].dst = pedges[2 * i + 1];
    es[i].edge_id = i;
  }
  Pattern pattern(pv, pe, es.data());
  SamplerGenerator<Empty>* inst = new SamplerGenerator<Empty>(&g, &pattern);
  return zgref_time_instance(inst, n, estimate);
}
#else
/* Builds the graph and times the application's instance with `threads` OpenMP threads. */
extern "C" __attribute__((visibility("default"))) double zgref_time_calculate(const uint32_t* edges, uint64_t m,
                                                                               uint32_t nv, uint64_t n, int threads,
                                                                               double* estimate) {
  zgref_boot(threads);
  Graph<Empty> g;
  zgref_time_graph(g, edges, m, nv);
  ZGREF_APP_CLASS<Empty>* inst = new ZGREF_APP_CLASS<Empty>(&g);
  return zgref_time_instance(inst, n, estimate);
}
#endif
