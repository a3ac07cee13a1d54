// zgh_graph.cpp — the graph store of the host layer.  Every graph built here gets its device copy
// at construction: the edge shuffle, the subsample and the adjacency builds run on the GPU
// (zg_graph_permuted / zg_graph_subsample), and the host arrays of the reference's layout are
// filled from the device's edge order, so that host and device agree on every edge id.
//
// Reference behaviour followed: src/Graph.cpp:174-210 (destroyer), :215-377 (CSR constructor),
// :383-627 (loader), :629-780 (sampler), src/GraphFilters.cpp:17-177 (filter).
#include <fcntl.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <type_traits>
#include <vector>

#include "../include/Graph.hpp"
#include "../include/GraphFilters.hpp"
#include "../include/Time.hpp"
#include "../include/Utilities.hpp"
#include "zgh_internal.hpp"

namespace {

static_assert(sizeof(EdgeUnit<Empty>) == 8 && sizeof(EdgeUnit<VertexId>) == 12, "EdgeUnit layout");

// Edge weights of the device graph: the VertexId edge data, or none.
template <typename E>
struct EdgeWeights {
  static_assert(std::is_same<E, Empty>::value || std::is_same<E, VertexId>::value,
                "the device graph carries Empty or VertexId edge data");
  static bool present() { return std::is_same<E, VertexId>::value; }
  static uint32_t get(const EdgeUnit<E>& e) { return *(const uint32_t*)((const char*)&e + 8); }
  static void set(EdgeUnit<E>& e, uint32_t w) { *(uint32_t*)((char*)&e + 8) = w; }
};

template <typename E>
void pack(const EdgeUnit<E>* edges, EdgeId m, std::vector<uint32_t>& coo, std::vector<uint32_t>& w) {
  coo.resize(2 * m);
  w.resize(EdgeWeights<E>::present() ? m : 0);
  for (EdgeId e = 0; e < m; ++e) {
    coo[2 * e] = edges[e].src;
    coo[2 * e + 1] = edges[e].dst;
    if (EdgeWeights<E>::present()) w[e] = EdgeWeights<E>::get(edges[e]);
  }
}

// Host arrays (local_edges[0] in the device's edge-id order, bitmap, index, adjacency) from the
// device copy: the adjacency of v lists its edges in increasing edge id with src = v
// (src/Graph.cpp:288-307), the order the device's edge-id-ordered adjacency has.
template <typename E>
void fill_host_from_device(Graph<E>& g, EdgeUnit<E>** local_edges, EdgeId* num_local_edges) {
  zg_graph_meta meta;
  zgh::check(zg_graph_get_meta(g.device, &meta), "zg_graph_get_meta");
  const EdgeId m = meta.num_local_edges;
  const VertexId nv = g.num_vertices;
  std::vector<uint32_t> coo(2 * m + 2), w(EdgeWeights<E>::present() ? m + 1 : 0);
  zgh::check(zg_graph_download(g.device, coo.data(), EdgeWeights<E>::present() ? w.data() : nullptr, nullptr,
                               nullptr, nullptr, nullptr),
             "zg_graph_download");
  if (local_edges[0] == nullptr || num_local_edges[0] != m) {
    free(local_edges[0]);
    local_edges[0] = (EdgeUnit<E>*)malloc(sizeof(EdgeUnit<E>) * (m ? m : 1));
    if (!local_edges[0]) throw std::runtime_error("host allocation of the edge list failed");
    num_local_edges[0] = m;
  }
  EdgeUnit<E>* le = local_edges[0];
  for (EdgeId e = 0; e < m; ++e) {
    le[e].src = coo[2 * e];
    le[e].dst = coo[2 * e + 1];
    if (EdgeWeights<E>::present()) EdgeWeights<E>::set(le[e], w[e]);
  }
  Bitmap* bm = new Bitmap(nv);
  bm->clear();
  EdgeId* idx = new EdgeId[(size_t)nv + 1]();
  for (EdgeId e = 0; e < m; ++e) {
    idx[le[e].src + 1]++;
    idx[le[e].dst + 1]++;
  }
  for (VertexId v = 1; v <= nv; ++v) idx[v] += idx[v - 1];
  AdjUnit<E>* adj = (AdjUnit<E>*)malloc(sizeof(AdjUnit<E>) * (m ? 2 * m : 1));
  if (!adj) throw std::runtime_error("host allocation of the adjacency failed");
  std::vector<EdgeId> pos(idx, idx + nv + 1);
  for (EdgeId e = 0; e < m; ++e) {
    VertexId s = le[e].src, d = le[e].dst;
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
    if (EdgeWeights<E>::present()) {
      uint32_t x = EdgeWeights<E>::get(le[e]);
      memcpy((char*)&a + 16, &x, 4);
      memcpy((char*)&b + 16, &x, 4);
    }
  }
  g.outgoing_adj_bitmap = new Bitmap*[1]{bm};
  g.outgoing_adj_index = new EdgeId*[1]{idx};
  g.outgoing_adj_list = new AdjUnit<E>*[1]{adj};
}

template <typename E>
void compute_degree(Graph<E>& g, const EdgeUnit<E>* le, EdgeId m, EdgeId& max_degree) {
  g.degree = new EdgeId[g.num_vertices ? g.num_vertices : 1]();
  for (EdgeId e = 0; e < m; ++e) {
    g.degree[le[e].src]++;
    g.degree[le[e].dst]++;
  }
  max_degree = 0;
  for (VertexId v = 0; v < g.num_vertices; ++v)
    if (g.degree[v] > max_degree) max_degree = g.degree[v];
}

}  // namespace

// ---- device copy ---------------------------------------------------------------------------------
template <typename E>
zg_graph* zgh_device_graph(Graph<E>& graph) {
  if (graph.device) return graph.device;
  zgh::ensure_init();
  std::vector<uint32_t> coo, w;
  EdgeId m = graph.num_local_edges ? graph.num_local_edges[0] : 0;
  pack<E>(m ? graph.local_edges[0] : nullptr, m, coo, w);
  zgh::check(zg_graph_create(coo.data(), m, graph.num_vertices, w.empty() ? nullptr : w.data(), nullptr, &graph.device),
             "zg_graph_create");
  zgh::check(zg_graph_set_meta(graph.device, graph.num_edges, graph.max_degree), "zg_graph_set_meta");
  return graph.device;
}

// ---- NumaAwareGraphDestroyer -----------------------------------------------------------------------
template <typename E>
void NumaAwareGraphDestroyer<E>::destroy_graph(Graph<E>& graph) {
  delete[] graph.degree;
  graph.degree = nullptr;
  if (graph.outgoing_adj_bitmap) {
    delete graph.outgoing_adj_bitmap[0];
    delete[] graph.outgoing_adj_bitmap;
  }
  if (graph.outgoing_adj_list) {
    free(graph.outgoing_adj_list[0]);
    delete[] graph.outgoing_adj_list;
  }
  if (graph.outgoing_adj_index) {
    delete[] graph.outgoing_adj_index[0];
    delete[] graph.outgoing_adj_index;
  }
  if (graph.local_edges) {
    free(graph.local_edges[0]);
    delete[] graph.local_edges;
  }
  delete[] graph.num_local_edges;
  graph.outgoing_adj_bitmap = nullptr;
  graph.outgoing_adj_list = nullptr;
  graph.outgoing_adj_index = nullptr;
  graph.local_edges = nullptr;
  graph.num_local_edges = nullptr;
  if (graph.device) zg_graph_free(graph.device);
  graph.device = nullptr;
  graph.shuffle_seed = 0;
}

// ---- CSRConstructor --------------------------------------------------------------------------------
template <typename E>
void CSRConstructor<E>::construct_bitmap_assisted_csr(EdgeUnit<E>** local_edges, EdgeId* num_local_edges,
                                                      Graph<E>& graph) {
  zgh::ensure_init();
  const EdgeId m = num_local_edges[0];
  std::vector<uint32_t> coo, w;
  pack<E>(local_edges[0], m, coo, w);
  if (graph.shuffle_seed == 0) graph.shuffle_seed = zgh::next_seed() | 1;
  if (graph.device) zg_graph_free(graph.device);
  graph.device = nullptr;
  zgh::check(zg_graph_permuted(coo.data(), m, graph.num_vertices, w.empty() ? nullptr : w.data(), graph.shuffle_seed,
                               nullptr, nullptr, &graph.device),
             "zg_graph_permuted");
  zgh::check(zg_graph_set_meta(graph.device, graph.num_edges ? graph.num_edges : m, graph.max_degree),
             "zg_graph_set_meta");
  fill_host_from_device(graph, local_edges, num_local_edges);
}

// ---- DistGraphLoader: .biedgelist = packed (u32 src, u32 dst[, edge data]) records ----------------
template <typename E>
DistGraphLoader<E>::DistGraphLoader(GraphPartitioner* partitioner_, Mapping* mapping_,
                                    CSRConstructor<E>* csr_constructor_, GraphDestroyer<E>* destroyer_)
    : partitioner(partitioner_), mapping(mapping_), csr_constructor(csr_constructor_), destroyer(destroyer_) {}

template <typename E>
void DistGraphLoader<E>::load_graph(std::string graph_path, VertexId num_vertices, Graph<E>& graph) {
  Timer::timer_start("load_graph");
  partitioner->partition_graph(graph.p);
  graph.edge_data_size = std::is_same<E, Empty>::value ? 0 : sizeof(E);
  graph.edge_unit_size = graph.edge_data_size + sizeof(VertexId) * 2;
  graph.num_vertices = num_vertices;
  long total_bytes = file_size(graph_path);
  if (total_bytes % (long)graph.edge_unit_size != 0)
    throw std::runtime_error(graph_path + ": size is not a multiple of the edge record size");
  const EdgeId m = total_bytes / graph.edge_unit_size;
  graph.num_edges = m;
  EdgeUnit<E>* le = (EdgeUnit<E>*)malloc(sizeof(EdgeUnit<E>) * (m ? m : 1));
  if (!le) throw std::runtime_error("host allocation of the edge list failed");
  int fd = open(graph_path.c_str(), O_RDONLY);
  if (fd < 0) throw std::runtime_error("cannot open " + graph_path);
  size_t want = sizeof(EdgeUnit<E>) * m, got = 0;
  while (got < want) {
    ssize_t r = read(fd, (char*)le + got, want - got);
    if (r <= 0) {
      close(fd);
      free(le);
      throw std::runtime_error("short read of " + graph_path);
    }
    got += (size_t)r;
  }
  close(fd);
  for (EdgeId e = 0; e < m; ++e) {
    if (le[e].src >= num_vertices || le[e].dst >= num_vertices) {
      free(le);
      throw std::runtime_error(graph_path + ": vertex id out of range");
    }
    le[e].src = mapping->get_mapping(le[e].src);
    le[e].dst = mapping->get_mapping(le[e].dst);
    if (le[e].src == le[e].dst) {  // src/Graph.cpp:447
      free(le);
      throw std::runtime_error(graph_path + ": self-loops are not allowed in the input graph file");
    }
  }
  EdgeId max_degree;
  compute_degree(graph, le, m, max_degree);
  graph.max_degree = max_degree;
  EdgeUnit<E>** local_edges = new EdgeUnit<E>*[1]{le};
  EdgeId* num_local_edges = new EdgeId[1]{m};
  csr_constructor->construct_bitmap_assisted_csr(local_edges, num_local_edges, graph);
  graph.num_local_edges = num_local_edges;
  graph.local_edges = local_edges;
  Timer::timer_stop("load_graph");
}

template <typename E>
void DistGraphLoader<E>::destroy_graph(Graph<E>& graph) {
  destroyer->destroy_graph(graph);
}

// ---- GraphSampler ------------------------------------------------------------------------------------
template <typename E>
GraphSampler<E>::GraphSampler(CSRConstructor<E>* csr_constructor_, GraphDestroyer<E>* destroyer_, double sample_rate_)
    : csr_constructor(csr_constructor_), destroyer(destroyer_), sample_rate(sample_rate_), keep_seed_(0),
      shuffle_seed_(0) {}

template <typename E>
void GraphSampler<E>::set_seeds(uint64_t keep_seed, uint64_t shuffle_seed) {
  keep_seed_ = keep_seed;
  shuffle_seed_ = shuffle_seed;
}

// Metadata as src/Graph.cpp:704-749: num_edges and max_degree are rescaled by the input's
// local/global edge ratio (1 on one partition).
template <typename E>
static void derived_meta(const Graph<E>& in, Graph<E>& out, EdgeId kept) {
  double rate = in.num_edges ? (double)in.num_local_edges[0] / (double)in.num_edges : 1.0;
  out.num_edges = (EdgeId)(1. * kept / rate);
  EdgeId max_degree;
  compute_degree(out, out.local_edges[0], kept, max_degree);
  out.max_degree = (EdgeId)(max_degree / rate);
}

template <typename E>
void GraphSampler<E>::sample_graph(const Graph<E>& input_graph, Graph<E>& output_graph) {
  zg_graph* din = zgh_device_graph(const_cast<Graph<E>&>(input_graph));
  output_graph.p = input_graph.p;
  output_graph.edge_data_size = input_graph.edge_data_size;
  output_graph.edge_unit_size = input_graph.edge_unit_size;
  output_graph.num_vertices = input_graph.num_vertices;
  uint64_t keep = keep_seed_ ? keep_seed_ : zgh::next_seed();
  uint64_t shuf = shuffle_seed_ ? shuffle_seed_ : (zgh::next_seed() | 1);
  uint64_t kept = 0;
  output_graph.device = nullptr;
  zgh::check(zg_graph_subsample(din, sample_rate, keep, shuf, nullptr, nullptr, &kept, &output_graph.device),
             "zg_graph_subsample");
  output_graph.shuffle_seed = shuf;
  output_graph.local_edges = new EdgeUnit<E>*[1]{nullptr};
  output_graph.num_local_edges = new EdgeId[1]{0};
  fill_host_from_device(output_graph, output_graph.local_edges, output_graph.num_local_edges);
  derived_meta(input_graph, output_graph, kept);
  zgh::check(zg_graph_set_meta(output_graph.device, output_graph.num_edges, output_graph.max_degree),
             "zg_graph_set_meta");
}

template <typename E>
void GraphSampler<E>::destroy_graph(Graph<E>& graph) {
  destroyer->destroy_graph(graph);
}

// ---- GraphFilter -------------------------------------------------------------------------------------
template <typename E>
GraphFilter<E>::GraphFilter(CSRConstructor<E>* csr_constructor_, GraphDestroyer<E>* destroyer_,
                            std::function<bool(E)> predicate_)
    : csr_constructor(csr_constructor_), destroyer(destroyer_), predicate(predicate_) {}

// The predicate is an arbitrary host function, so it is evaluated here; the kept edges (input
// order) are then shuffled and rebuilt on the device with output_graph.shuffle_seed (fresh when 0),
// which gives the same graph as zg_graph_filter with that seed.
template <typename E>
void GraphFilter<E>::generate_graph(const Graph<E>& input_graph, Graph<E>& output_graph) {
  output_graph.p = input_graph.p;
  output_graph.edge_data_size = input_graph.edge_data_size;
  output_graph.edge_unit_size = input_graph.edge_unit_size;
  output_graph.num_vertices = input_graph.num_vertices;
  const EdgeId m = input_graph.num_local_edges[0];
  const EdgeUnit<E>* in = input_graph.local_edges[0];
  EdgeId kept = 0;
  for (EdgeId e = 0; e < m; ++e) kept += predicate(in[e].edge_data) ? 1 : 0;
  EdgeUnit<E>* le = (EdgeUnit<E>*)malloc(sizeof(EdgeUnit<E>) * (kept ? kept : 1));
  if (!le) throw std::runtime_error("host allocation of the edge list failed");
  EdgeId k = 0;
  for (EdgeId e = 0; e < m; ++e)
    if (predicate(in[e].edge_data)) le[k++] = in[e];
  output_graph.local_edges = new EdgeUnit<E>*[1]{le};
  output_graph.num_local_edges = new EdgeId[1]{kept};
  derived_meta(input_graph, output_graph, kept);
  output_graph.device = nullptr;
  csr_constructor->construct_bitmap_assisted_csr(output_graph.local_edges, output_graph.num_local_edges, output_graph);
}

template <typename E>
void GraphFilter<E>::destroy_graph(Graph<E>& graph) {
  destroyer->destroy_graph(graph);
}

template zg_graph* zgh_device_graph<Empty>(Graph<Empty>&);
template zg_graph* zgh_device_graph<VertexId>(Graph<VertexId>&);
template class NumaAwareGraphDestroyer<Empty>;
template class NumaAwareGraphDestroyer<VertexId>;
template class CSRConstructor<Empty>;
template class CSRConstructor<VertexId>;
template class DistGraphLoader<Empty>;
template class DistGraphLoader<VertexId>;
template class GraphSampler<Empty>;
template class GraphSampler<VertexId>;
template class GraphFilter<Empty>;
template class GraphFilter<VertexId>;
