// zgh_gpu_check.cpp — end-to-end check of the C++ host layer on the GPU.
//
// Writes a synthetic graph in the reference's file formats (.biedgelist + .csv), loads it the way
// an application does, and runs the estimator applications of zgh_apps.hpp through calculate(),
// ErrorProfile, TimeProfile, the AllPredicate filter, the 3-motif cache and SamplerGenerator.
// Every estimate is compared with the C ABI run on the same Philox draws (bit-equal doubles and
// 320-bit sums), and the profiles with zg_elp_plain (the same estimator count).
//
// usage: zgh_gpu_check <scratch dir>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "SharedMemSys.hpp"
#include "Time.hpp"
#include "Utilities.hpp"
#include "zgh_apps.hpp"

static int failures = 0;
#define CHECK(cond, ...)                         \
  do {                                           \
    if (!(cond)) {                               \
      printf("FAIL %s:%d ", __FILE__, __LINE__); \
      printf(__VA_ARGS__);                       \
      printf("\n");                              \
      ++failures;                                \
    }                                            \
  } while (0)

static void ok(int rc, const char* what) {
  if (rc != ZG_OK) throw std::runtime_error(std::string(what) + ": " + zg_last_error());
}

static bool same_counters(const zg_counters& a, const zg_counters& b) {
  return a.samples == b.samples && a.hits == b.hits && a.fails == b.fails && a.den_log2 == b.den_log2 &&
         memcmp(a.sum_num, b.sum_num, sizeof(a.sum_num)) == 0 && memcmp(&a.estimate, &b.estimate, 8) == 0;
}

// calculate() of an application against zg_run of the named program on the same draws.
template <typename E>
static void compare_run(const char* name, ZGraphInstance<E>& inst, Graph<E>& g, int kind, uint32_t param,
                        unsigned long long n, uint64_t seed, uint32_t stream) {
  inst.set_sampling_seed(seed, stream);
  Estimation est;
  double got = inst.calculate(n, 3, est);
  zg_program* p = nullptr;
  ok(zg_program_create(kind, param, &p), "zg_program_create");
  zg_counters want;
  ok(zg_run(zgh_device_graph(g), p, n, 0, seed, stream, nullptr, &want), "zg_run");
  zg_program_free(p);
  printf("%-14s n=%llu estimate %.6e (hits %llu)\n", name, n, got, (unsigned long long)want.hits);
  CHECK(memcmp(&got, &want.estimate, 8) == 0, "%s: calculate %.17g vs zg_run %.17g", name, got, want.estimate);
  CHECK(same_counters(inst.get_last_counters(), want), "%s: counters differ", name);
  // a second calculate continues with fresh sample indices
  Estimation est2;
  inst.calculate(n, 3, est2);
  zg_counters next;
  ok(zg_program_create(kind, param, &p), "zg_program_create");
  ok(zg_run(zgh_device_graph(g), p, n, n, seed, stream, nullptr, &next), "zg_run");
  zg_program_free(p);
  CHECK(same_counters(inst.get_last_counters(), next), "%s: second calculate is not the next sample range", name);
}

static void write_graph(const std::string& dir, const std::vector<uint32_t>& coo, const uint32_t* w, VertexId nv,
                        const char* stem) {
  const uint64_t m = coo.size() / 2;
  FILE* f = fopen((dir + "/" + stem + ".biedgelist").c_str(), "wb");
  for (uint64_t e = 0; e < m; ++e) {
    fwrite(&coo[2 * e], 4, 2, f);
    if (w) fwrite(&w[e], 4, 1, f);
  }
  fclose(f);
  f = fopen((dir + "/" + stem + ".csv").c_str(), "w");
  fprintf(f, "num_vertices,num_edges\n%u,%llu\n", nv, (unsigned long long)m);
  fclose(f);
}

int main(int argc, char** argv) {
  if (argc != 2) {
    fprintf(stderr, "usage: %s <dir>\n", argv[0]);
    return 2;
  }
  NetworkInterface::init_network_interface(&argc, &argv);
  SharedMemSys::init_shared_mem_sys();
  std::string dir = argv[1];

  // R-MAT scale 12, edge factor 16; edge data uniform in [0, 100)
  uint64_t m = 0;
  ok(zg_gen_rmat(12, 16, 0.57, 0.19, 0.19, 5, 0, nullptr, &m), "zg_gen_rmat");
  std::vector<uint32_t> coo(2 * m), w(m);
  ok(zg_gen_rmat(12, 16, 0.57, 0.19, 0.19, 5, m, coo.data(), &m), "zg_gen_rmat");
  ok(zg_gen_weights(m, 100, 9, w.data()), "zg_gen_weights");
  write_graph(dir, coo, nullptr, 1 << 12, "g");
  write_graph(dir, coo, w.data(), 1 << 12, "w");

  VertexId nv = 0;
  load_graph_meta_data(dir + "/g.csv", nv);
  CHECK(nv == 4096, "meta data");
  UniformGraphPartitioner part(nv);
  IdenticalMapping ident;
  CSRConstructor<Empty> csr;
  NumaAwareGraphDestroyer<Empty> destroyer;
  DistGraphLoader<Empty> loader(&part, &ident, &csr, &destroyer);
  Graph<Empty> g;
  g.shuffle_seed = 1234;
  loader.load_graph(dir + "/g.biedgelist", nv, g);  // first device use: zg_init happens here
  CHECK(g.num_edges == m && g.num_local_edges[0] == m && g.device != nullptr, "loaded graph");
  {
    // host arrays and device copy share one edge order
    std::vector<uint32_t> dev(2 * m);
    ok(zg_graph_download(g.device, dev.data(), nullptr, nullptr, nullptr, nullptr, nullptr), "download");
    bool same = true;
    for (uint64_t e = 0; e < m && same; ++e)
      same = dev[2 * e] == g.local_edges[0][e].src && dev[2 * e + 1] == g.local_edges[0][e].dst;
    CHECK(same, "host and device edge orders differ");
    std::vector<uint32_t> perm(2 * m);
    zg_graph* ref = nullptr;
    ok(zg_graph_permuted(coo.data(), m, nv, nullptr, 1234, nullptr, nullptr, &ref), "zg_graph_permuted");
    ok(zg_graph_download(ref, perm.data(), nullptr, nullptr, nullptr, nullptr, nullptr), "download");
    zg_graph_free(ref);
    CHECK(perm == dev, "loader shuffle is not zg_graph_permuted with the graph's seed");
  }
  uint64_t exact_tri[2];
  ok(zg_exact_count(g.device, ZG_EXACT_TRIANGLE, nullptr, exact_tri), "zg_exact_count");
  const double tri_count = (double)exact_tri[0];

  // ---- calculate() of every application against zg_run -------------------------------------
  const unsigned long long n = 1ull << 22;
  {
    TriangleApp<Empty> a(&g);
    compare_run("triangle", a, g, ZG_PROG_TRIANGLE, 0, n, 11, 1);
    FourCliqueApp<Empty> b(&g);
    compare_run("four_clique", b, g, ZG_PROG_FOUR_CLIQUE, 0, n, 12, 2);
    ThreeChainApp<Empty> c(&g);
    compare_run("three_chain", c, g, ZG_PROG_THREE_CHAIN, 0, n, 13, 3);
    FourChainApp<Empty> d(&g);
    compare_run("four_chain", d, g, ZG_PROG_FOUR_CHAIN, 0, n, 14, 4);
    ChainApp<Empty> e(&g, 5);
    compare_run("chain5", e, g, ZG_PROG_CHAIN, 5, n, 15, 5);
    ChainApp<Empty> f(&g, 7);
    compare_run("chain7", f, g, ZG_PROG_CHAIN, 7, n, 16, 6);
  }
  // ---- SamplerGenerator -------------------------------------------------------------------------
  {
    std::unique_ptr<Pattern> star(star_pattern()), tp(triangle_pattern());
    SamplerGenerator<Empty> s(&g, star.get()), t(&g, tp.get());
    uint32_t nu = 0;
    ok(zg_program_info(s.device_program(), &nu, nullptr, nullptr), "zg_program_info");
    CHECK(nu == 5, "five-star unique patterns %u", nu);
    for (auto* inst : {&s, &t}) {
      inst->set_sampling_seed(21, 7);
      Estimation est;
      double got = inst->calculate(n, 5, est);
      zg_counters want;
      ok(zg_run(g.device, inst->device_program(), n, 0, 21, 7, nullptr, &want), "zg_run");
      CHECK(memcmp(&got, &want.estimate, 8) == 0, "pattern estimate %.17g vs %.17g", got, want.estimate);
    }
    std::unique_ptr<Pattern> house(house_pattern());
    SamplerGenerator<Empty> h(&g, house.get());
    ok(zg_program_info(h.device_program(), &nu, nullptr, nullptr), "zg_program_info");
    CHECK(nu == 60, "house unique patterns %u", nu);
    // triangles by the pattern sampler agree with the exact count
    Estimation est;
    t.set_sampling_seed(22, 8);
    double tri_est = t.calculate(1ull << 26, 3, est);
    printf("pattern triangle %.6e exact %.6e\n", tri_est, tri_count);
    CHECK(fabs(tri_est / tri_count - 1) < 0.02, "pattern triangle estimate off");
  }
  // ---- unsupported estimator --------------------------------------------------------------------
  {
    VertexPairApp<Empty> v(&g);
    bool threw = false;
    try {
      Estimation est;
      v.calculate(1000, 2, est);
    } catch (const std::runtime_error& e) {
      threw = strstr(e.what(), "no device program") != nullptr;
    }
    CHECK(threw, "an unsupported estimator was not refused");
  }
  // ---- ErrorProfile / TimeProfile ---------------------------------------------------------------
  {
    TriangleApp<Empty> a(&g);
    a.set_sampling_seed(31, 9);
    ErrorProfile<Empty> ep;
    unsigned long long need = ep.get_num_estimators(a, 3, 0.05, 0.95);
    zg_elp_result r;
    ok(zg_elp_plain(g.device, a.device_program(), 0, 0, 0, 0.05, 0.95, 31, nullptr, &r, nullptr), "zg_elp_plain");
    printf("ErrorProfile n %llu, zg_elp_plain n %llu\n", need, (unsigned long long)r.n_required);
    CHECK(need == r.n_required, "ErrorProfile %llu vs zg_elp_plain %llu", need, (unsigned long long)r.n_required);
    CHECK(a.get_graph() == &g, "instance graph restored");
    Estimation est;
    double cnt = ep.run(a, 3, 0.05, 0.95, est);
    printf("ErrorProfile::run %.6e exact %.6e\n", cnt, tri_count);
    CHECK(fabs(cnt / tri_count - 1) < 0.05, "ErrorProfile::run estimate off");
    TimeProfile<Empty> tp;
    double t0 = get_time();
    double tc = tp.run(a, 3, 300);
    double dt = get_time() - t0;
    printf("TimeProfile(300 ms) %.6e in %.0f ms\n", tc, dt * 1000);
    CHECK(fabs(tc / tri_count - 1) < 0.05, "TimeProfile estimate off");
    CHECK(dt < 3.0, "TimeProfile overran its budget: %.2f s", dt);
  }
  // ---- the 3-motif cache ------------------------------------------------------------------------
  {
    CachedChainApp<Empty> chain(&g);
    CachedTriangleApp<Empty> tri(&g);
    chain.set_sampling_seed(41, 0x100);
    tri.set_sampling_seed(41, 0x200);
    const unsigned long long nc = 1ull << 16, nt = 1ull << 20;
    Estimation e1, e2;
    double c3 = chain.calculate(nc, 3, e1);
    CachedSubPatterns<Empty>* cache = chain.get_cached_sub_patterns();
    CHECK(cache && cache->get_num_patterns(0, 0) == nc, "exported cache");
    tri.set_cached_sub_patterns(cache);
    double c_tri = tri.calculate(nt, 3, e2);
    zg_counters oc, ot;
    ok(zg_run_three_motif(g.device, nc, nt, 41, 0x100, 0x200, nullptr, &oc, &ot), "zg_run_three_motif");
    CHECK(memcmp(&c3, &oc.estimate, 8) == 0, "cached chain %.17g vs %.17g", c3, oc.estimate);
    CHECK(memcmp(&c_tri, &ot.estimate, 8) == 0, "cached triangle %.17g vs %.17g", c_tri, ot.estimate);
    unsigned long long np = 0;
    auto all = cache->get_all(0, 0, np);
    double s = 0;
    for (unsigned long long i = 0; i < np; ++i)
      if (all.second[i] > 0) {
        s += 1. / all.second[i];
        CHECK(all.first[i].get_edges().list_size == 2, "materialised wedge %llu", i);
      }
    CHECK(np == nc && fabs(s / nc / c3 - 1) < 1e-12, "materialised wedges: mean %.17g vs %.17g", s / nc, c3);
    printf("3-motif: chains %.6e triangles %.6e (exact %.6e)\n", c3, c_tri, tri_count);
  }
  // ---- AllPredicate on edge data ------------------------------------------------------------------
  {
    CSRConstructor<VertexId> wcsr;
    NumaAwareGraphDestroyer<VertexId> wd;
    DistGraphLoader<VertexId> wl(&part, &ident, &wcsr, &wd);
    Graph<VertexId> wg;
    wl.load_graph(dir + "/w.biedgelist", nv, wg);
    std::function<bool(VertexId)> pred = [](VertexId x) { return x >= 50; };
    PredicateTriangleApp<VertexId> a(&wg, pred);
    CHECK(a.get_graph() == &wg, "predicate instance reports the original graph");
    uint64_t ex[2];
    zg_graph* fg = nullptr;
    uint64_t fm = 0;
    ok(zg_graph_filter(wg.device, ZG_PRED_GE, 50, 0, 77, nullptr, nullptr, &fm, &fg), "zg_graph_filter");
    ok(zg_exact_count(fg, ZG_EXACT_TRIANGLE, nullptr, ex), "zg_exact_count");
    zg_graph_free(fg);
    a.set_sampling_seed(51, 3);
    Estimation est;
    double got = a.calculate(1ull << 26, 3, est);
    printf("AllPredicate triangles %.6e exact %.6e\n", got, (double)ex[0]);
    CHECK(fabs(got / (double)ex[0] - 1) < 0.03, "predicate estimate off");
    ErrorProfile<VertexId> ep;
    unsigned long long need = ep.get_num_estimators(a, 3, 0.05, 0.95);
    zg_elp_result r;
    ok(zg_elp_plain(wg.device, a.device_program(), ZG_PRED_GE, 50, 0, 0.05, 0.95, 51, nullptr, &r, nullptr),
       "zg_elp_plain");
    printf("AllPredicate ErrorProfile n %llu, zg_elp_plain n %llu\n", need, (unsigned long long)r.n_required);
    CHECK(need == r.n_required, "predicate ErrorProfile %llu vs %llu", need, (unsigned long long)r.n_required);
    wl.destroy_graph(wg);
  }
  // ---- GraphSampler ----------------------------------------------------------------------------------
  {
    GraphSampler<Empty> sampler(&csr, &destroyer, 0.1);
    sampler.set_seeds(61, 62);
    Graph<Empty> sg;
    sampler.sample_graph(g, sg);
    zg_graph* want = nullptr;
    uint64_t km = 0;
    ok(zg_graph_subsample(g.device, 0.1, 61, 62, nullptr, nullptr, &km, &want), "zg_graph_subsample");
    zg_graph_meta a, b;
    ok(zg_graph_get_meta(sg.device, &a), "meta");
    ok(zg_graph_get_meta(want, &b), "meta");
    CHECK(sg.num_local_edges[0] == km && a.num_edges == b.num_edges && a.max_degree == b.max_degree &&
              sg.num_edges == b.num_edges && sg.max_degree == b.max_degree,
          "subsample meta: host %llu/%llu device %llu/%llu", (unsigned long long)sg.num_edges,
          (unsigned long long)sg.max_degree, (unsigned long long)b.num_edges, (unsigned long long)b.max_degree);
    zg_graph_free(want);
    sampler.destroy_graph(sg);
  }
  loader.destroy_graph(g);
  Timer::report_timers();
  NetworkInterface::finalize_instance();
  printf(failures ? "FAILED %d\n" : "PASS\n", failures);
  return failures ? 1 : 0;
}
