/* Oracle driver around applications/ThreeMotif.cpp (ZGraphInstanceWithCache 3-chain + triangle).
 * Test infrastructure. */
#define main zgref_app_main
#include "applications/ThreeMotif.cpp"
#undef main
#define ZGREF_E Empty
#include "zgref_driver.hpp"
static ZGraphInstance<Empty>* zgref_make(Graph<Empty>* g, uint32_t, const uint32_t*, uint32_t,
                                         uint32_t) {
  return new TriangleCoutingInstance<Empty>(g);
}

/* ThreeMotif.cpp:149-196 without the ELP: chain calculate(n_chain), export its cache, triangle
 * calculate(n_tri) importing it.  Chain draws for samples [0,n_chain); triangle draws only for
 * the fresh samples [n_chain, n_tri). */
ZGREF_API uint64_t zgref_motif(const uint32_t* edges, uint64_t m, uint32_t nv, uint64_t n_chain,
                               uint64_t n_tri, const zg_sample_trace* chain_tr,
                               const zg_sample_trace* tri_tr, double* est_chain, double* est_tri) {
  zgref_boot();
  Graph<Empty> g;
  zgref_build_graph<Empty>(g, edges, m, nv, nullptr);
  ThreeChainCountingInstance<Empty>* chain = new ThreeChainCountingInstance<Empty>(&g);
  TriangleCoutingInstance<Empty>* tri = new TriangleCoutingInstance<Empty>(&g);
  uint64_t bad = 0;
  zgref_replay.q.clear();
  zgref_replay.reset_counts();
  for (uint64_t i = 0; i < n_chain; ++i) zgref_queue(chain_tr[i]);
  Estimation e1;
  *est_chain = chain->calculate(n_chain, 3, e1);
  bad += zgref_replay.mismatches + zgref_replay.overruns + zgref_replay.q.size();
  tri->set_cached_sub_patterns(chain->get_cached_sub_patterns());
  zgref_replay.q.clear();
  zgref_replay.reset_counts();
  for (uint64_t i = n_chain; i < n_tri; ++i) zgref_queue(tri_tr[i]);
  Estimation e2;
  *est_tri = tri->calculate(n_tri, 3, e2);
  bad += zgref_replay.mismatches + zgref_replay.overruns + zgref_replay.q.size();
  zgref_replay.q.clear();
  delete chain;
  delete tri;
  NumaAwareGraphDestroyer<Empty> d;
  d.destroy_graph(g);
  return bad;
}
