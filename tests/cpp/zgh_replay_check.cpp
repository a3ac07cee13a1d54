// zgh_replay_check.cpp — CPU check of the C++ host layer (no GPU needed).
//
// Reads a graph and per-sample traces of the CPU oracle (the same records zg_run_debug writes),
// builds the graph's host arrays in the reference's layout, and replays every trace through the
// estimator applications of zgh_apps.hpp with ZGraphInstance::replay_trace: draw ranges, draw
// counts and returned doubles must agree bit for bit.  Also checks the host-only pieces
// (Estimation, SubGraph difference, RandomMapping, regression, meta data reader, Pattern).
//
// usage: zgh_replay_check <dir>   (dir holds graph.bin and <app>.tr files)
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include "Regression.hpp"
#include "Utilities.hpp"
#include "zgh_apps.hpp"

static int failures = 0;
#define CHECK(cond, ...)                      \
  do {                                        \
    if (!(cond)) {                            \
      printf("FAIL %s:%d ", __FILE__, __LINE__); \
      printf(__VA_ARGS__);                    \
      printf("\n");                           \
      ++failures;                             \
    }                                         \
  } while (0)

// Host arrays of a graph in the given edge order (edge id = position), the layout
// CSRConstructor produces, without a device copy.
template <typename E>
void host_graph(Graph<E>& g, const std::vector<uint32_t>& coo, VertexId nv) {
  UniformGraphPartitioner part(nv);
  part.partition_graph(g.p);
  const EdgeId m = coo.size() / 2;
  g.num_vertices = nv;
  g.num_edges = m;
  g.edge_data_size = 0;
  g.edge_unit_size = 8;
  g.local_edges = new EdgeUnit<E>*[1];
  g.local_edges[0] = (EdgeUnit<E>*)malloc(sizeof(EdgeUnit<E>) * (m ? m : 1));
  g.num_local_edges = new EdgeId[1]{m};
  for (EdgeId e = 0; e < m; ++e) {
    g.local_edges[0][e].src = coo[2 * e];
    g.local_edges[0][e].dst = coo[2 * e + 1];
  }
  g.degree = new EdgeId[nv]();
  EdgeId* idx = new EdgeId[nv + 1]();
  for (EdgeId e = 0; e < m; ++e) {
    g.degree[coo[2 * e]]++;
    g.degree[coo[2 * e + 1]]++;
    idx[coo[2 * e] + 1]++;
    idx[coo[2 * e + 1] + 1]++;
  }
  g.max_degree = 0;
  for (VertexId v = 0; v < nv; ++v) g.max_degree = std::max(g.max_degree, g.degree[v]);
  for (VertexId v = 1; v <= nv; ++v) idx[v] += idx[v - 1];
  AdjUnit<E>* adj = (AdjUnit<E>*)malloc(sizeof(AdjUnit<E>) * (m ? 2 * m : 1));
  std::vector<EdgeId> pos(idx, idx + nv + 1);
  Bitmap* bm = new Bitmap(nv);
  bm->clear();
  for (EdgeId e = 0; e < m; ++e) {
    VertexId s = coo[2 * e], d = coo[2 * e + 1];
    bm->set_bit(s);
    bm->set_bit(d);
    AdjUnit<E>& a = adj[pos[s]++];
    a.edge_id = e;
    a.src = s;
    a.dst = d;
    AdjUnit<E>& b = adj[pos[d]++];
    b.edge_id = e;
    b.src = d;
    b.dst = s;
  }
  g.outgoing_adj_bitmap = new Bitmap*[1]{bm};
  g.outgoing_adj_index = new EdgeId*[1]{idx};
  g.outgoing_adj_list = new AdjUnit<E>*[1]{adj};
}

static void read_graph(const std::string& dir, Graph<Empty>& g) {
  std::ifstream f(dir + "/graph.bin", std::ios::binary);
  uint64_t m = 0;
  uint32_t nv = 0;
  f.read((char*)&m, 8);
  f.read((char*)&nv, 4);
  std::vector<uint32_t> coo(2 * m);
  f.read((char*)coo.data(), 8 * m);
  CHECK(f.good() && m > 0, "%s/graph.bin", dir.c_str());
  host_graph(g, coo, nv);
}

static std::vector<zg_sample_trace> read_traces(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  std::vector<zg_sample_trace> out;
  if (!f) return out;
  f.seekg(0, std::ios::end);
  size_t bytes = f.tellg();
  f.seekg(0);
  out.resize(bytes / sizeof(zg_sample_trace));
  f.read((char*)out.data(), out.size() * sizeof(zg_sample_trace));
  return out;
}

static void replay(const char* name, ZGraphInstance<Empty>& inst, const std::string& dir) {
  std::vector<zg_sample_trace> tr = read_traces(dir + "/" + name + ".tr");
  CHECK(!tr.empty(), "%s: no traces", name);
  uint64_t counts[3] = {0, 0, 0}, hits = 0;
  for (auto& t : tr) {
    double v;
    int r = inst.replay_trace(t, &v);
    counts[r]++;
    hits += t.hit;
    if (r == 2 && counts[2] <= 3)
      printf("  %s mismatch: ndraws %u hit %u w %.17g host %.17g\n", name, t.ndraws, t.hit, t.w, v);
  }
  printf("%s samples %zu exact %llu near %llu mismatch %llu hits %llu\n", name, tr.size(),
         (unsigned long long)counts[0], (unsigned long long)counts[1], (unsigned long long)counts[2],
         (unsigned long long)hits);
  CHECK(counts[1] == 0 && counts[2] == 0, "%s: not bit-exact", name);
  CHECK(hits > 0, "%s: no hits in the traces", name);
}

static void host_units(const std::string& dir) {
  Estimation est;
  est.update(10, 4.0);
  est.update(30, 8.0);
  CHECK(est.get_num_finished_estimators() == 40, "estimation count");
  CHECK(est.get_currnet_estimation() == (1. * 10 / 40) * 4.0 + (1. * 30 / 40) * 8.0, "estimation mean");

  SubGraph<Empty> a, b;
  Edge<Empty> e;
  e.edge_id = 5;
  e.src = 1;
  e.dst = 2;
  a.add_edge(e);
  e.edge_id = 9;
  e.src = 3;
  e.dst = 2;
  a.add_edge(e);
  e.src = 2;
  e.dst = 1;
  b.add_edge(e);
  SubGraph<Empty> d = a - b;
  CHECK(d.get_edges().list_size == 1 && d.get_edges().list[0].src == 3, "subgraph difference");
  CHECK(a.get_min_valid_edge_id() == 10 && a.get_vertices().list_size == 3 && a.get_min_valid_vertex_id() == 4,
        "subgraph bookkeeping");

  RandomMapping rm(7, 1000);
  std::vector<int> seen(1000, 0);
  for (VertexId v = 0; v < 1000; ++v) {
    seen[rm.get_mapping(v)]++;
    CHECK(rm.get_inv_mapping(rm.get_mapping(v)) == v, "inverse mapping");
  }
  for (int c : seen) CHECK(c == 1, "mapping is a permutation");

  long double x[3] = {1, 2, 3}, y[3] = {2, 4, 6.5};
  UnbiasedLinearRegression reg;
  reg.solve(x, y, 3);
  CHECK(reg.get_k() == (2.0L + 8 + 19.5L) / 14, "regression slope");

  std::string csv = dir + "/meta.csv";
  FILE* f = fopen(csv.c_str(), "w");
  fprintf(f, "vertices,edges\nnum_vertices: 12345, 99\n");
  fclose(f);
  VertexId nv = 0;
  load_graph_meta_data(csv, nv);
  CHECK(nv == 12345, "meta data reader");

  std::unique_ptr<Pattern> house(house_pattern()), star(star_pattern());
  CHECK(house->get_num_vertices() == 5 && house->get_num_edges() == 6, "pattern sizes");
  Edge<Empty> rel[6];
  VertexId perm[5] = {4, 3, 2, 1, 0};
  for (int i = 0; i < 6; ++i) {
    rel[i].src = perm[house->get_edges()[i].src];
    rel[i].dst = perm[house->get_edges()[i].dst];
  }
  // the reversed labelling of the house is a different labelled graph unless it is an automorphism
  bool same = house->is_automorphic(5, 6, rel);
  CHECK(!same, "house relabelling");
  CHECK(house->is_automorphic(*house), "pattern equals itself");
  CHECK(!star->is_automorphic(*house), "different patterns");
}

int main(int argc, char** argv) {
  if (argc != 2) {
    fprintf(stderr, "usage: %s <dir>\n", argv[0]);
    return 2;
  }
  std::string dir = argv[1];
  host_units(dir);

  Graph<Empty> g, dense;
  read_graph(dir, g);
  read_graph(dir + "/house", dense);

  {
    TriangleApp<Empty> tri(&g);
    replay("triangle", tri, dir);
    FourCliqueApp<Empty> fc(&g);
    replay("four_clique", fc, dir);
    ThreeChainApp<Empty> c3(&g);
    replay("three_chain", c3, dir);
    FourChainApp<Empty> c4(&g);
    replay("four_chain", c4, dir);
    ChainApp<Empty> c5(&g, 5);
    replay("chain5", c5, dir);
    ChainApp<Empty> c3b(&g, 3);
    replay("chain3", c3b, dir);
    CachedChainApp<Empty> cc(&g);
    replay("three_chain", cc, dir);
    CachedTriangleApp<Empty> ct(&g);
    replay("triangle", ct, dir);
    std::unique_ptr<Pattern> star(star_pattern()), house(house_pattern()), tp(triangle_pattern());
    SamplerGenerator<Empty> gs(&g, star.get()), gh(&dense, house.get()), gt(&g, tp.get());
    replay("pattern_star", gs, dir);
    replay("pattern_house", gh, dir + "/house");
    replay("pattern_triangle", gt, dir);
    // a triangle estimator replayed on 3-chain traces must be told apart
    std::vector<zg_sample_trace> tr = read_traces(dir + "/three_chain.tr");
    int worst = 0;
    for (auto& t : tr) worst = std::max(worst, tri.replay_trace(t));
    CHECK(worst == 2, "triangle estimator accepted 3-chain traces");
  }
  NumaAwareGraphDestroyer<Empty> destroyer;
  destroyer.destroy_graph(g);
  destroyer.destroy_graph(dense);
  printf(failures ? "FAILED %d\n" : "PASS\n", failures);
  return failures ? 1 : 0;
}
