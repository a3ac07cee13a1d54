// zgh_instance.cpp — estimator instances, profiles and the pattern sampler of the host layer.
//
// The ASAP primitives (sample_edge, conditional_sample_edge, conditional_close, sample_interger)
// are kept on the host exactly as the reference states them; they serve estimate() calls made
// directly by an application and the identification replay.  calculate() never runs estimate()
// to produce a number: it runs the device program that reproduces estimate(), identified on first
// use by replaying device traces (zg_run_debug) through the application's own estimate() and
// requiring every draw range, draw count and returned double to agree bit for bit.
//
// Reference behaviour followed: src/ZGraphInstance.cpp:38-113 (SubGraph), :115-455 (instance and
// primitives), :493-525 (AllPredicate), :596-833 (cache), src/ErrorLatencyProfile.cpp:25-207,
// src/SamplerGenerator.cpp:287-546.
#include <string.h>

#include <algorithm>
#include <atomic>
#include <memory>
#include <stdexcept>

#include "../include/ErrorLatencyProfile.hpp"
#include "../include/SamplerGenerator.hpp"
#include "../include/SharedMemSys.hpp"
#include "../include/ZGraphInstance.hpp"
#include "zgh_internal.hpp"

#define BINARY_SEARCH_THRESHOLD 32
#define BASIC_NUM_ESTIMATORS_PER_THREAD 64

namespace {

// Identification replays: stream of the traces, sample budget, and hits wanted before adopting.
const uint32_t kValidationStream = 0x56414C00u;
const uint64_t kValidationSeed = 0x7A67685F76616CULL;
const uint64_t kValidationBatch = 512;
const uint64_t kValidationMaxSamples = 1ull << 16;
const uint64_t kValidationHits = 64;

// Default Philox streams: one block of 256 per instance, so instances never share a stream.
std::atomic<uint32_t> g_instances{0};

uint64_t bits_of(double x) {
  uint64_t b;
  memcpy(&b, &x, 8);
  return b;
}

}  // namespace

// ---- SubGraph -------------------------------------------------------------------------------------
template <typename E>
SubGraph<E>::SubGraph() {
  min_valid_edge_id = 0;
  min_valid_vertex_id = 0;
}

template <typename E>
bool SubGraph<E>::is_in_vertices_list(VertexId vertex) {
  for (int i = 0; i < vertices.list_size; ++i)
    if (vertices.list[i] == vertex) return true;
  return false;
}

template <typename E>
void SubGraph<E>::add_edge(const Edge<E>& edge) {
  edges.push_back(edge);
  if (edge.edge_id >= min_valid_edge_id) min_valid_edge_id = edge.edge_id + 1;
  add_vertex(edge.src);
  add_vertex(edge.dst);
}

template <typename E>
void SubGraph<E>::add_vertex(VertexId vertex) {
  if (!is_in_vertices_list(vertex)) {
    vertices.push_back(vertex);
    if (vertex >= min_valid_vertex_id) min_valid_vertex_id = vertex + 1;
  }
}

template <typename E>
const MyList<Edge<E>>& SubGraph<E>::get_edges() const {
  return edges;
}

template <typename E>
const MyList<VertexId>& SubGraph<E>::get_vertices() const {
  return vertices;
}

template <typename E>
EdgeId SubGraph<E>::get_min_valid_edge_id() const {
  return min_valid_edge_id;
}

template <typename E>
VertexId SubGraph<E>::get_min_valid_vertex_id() const {
  return min_valid_vertex_id;
}

// The edges of *this that are not in sub_graph (either orientation).
template <typename E>
SubGraph<E> SubGraph<E>::operator-(const SubGraph<E>& sub_graph) {
  SubGraph<E> result;
  for (int i = 0; i < edges.list_size; ++i) {
    const Edge<E>& a = edges.list[i];
    bool drop = false;
    for (int j = 0; j < sub_graph.edges.list_size && !drop; ++j) {
      const Edge<E>& b = sub_graph.edges.list[j];
      drop = (a.src == b.src && a.dst == b.dst) || (a.src == b.dst && a.dst == b.src);
    }
    if (!drop) result.add_edge(a);
  }
  return result;
}

// ---- ZGraphInstance ----------------------------------------------------------------------------------
template <typename E>
ZGraphInstance<E>::ZGraphInstance() : ZGraphInstance(nullptr) {}

template <typename E>
ZGraphInstance<E>::ZGraphInstance(Graph<E>* graph_) : graph(graph_) {
  randoms = new Random[SharedMemSys::get_instance()->get_num_threads()];
  is_counting_sample_edge_calls = false;
  is_counting_conditional_edge_calls = false;
  cnt = 0;
  program_ = nullptr;
  program_kind_ = 0;
  validating_ = false;
  seed_ = zgh::next_seed();
  stream_id_ = g_instances.fetch_add(1) << 8;
  next_sample_ = 0;
  memset(&last_counters_, 0, sizeof(last_counters_));
}

template <typename E>
ZGraphInstance<E>::~ZGraphInstance() {
  delete[] randoms;
  if (program_) zg_program_free(program_);
}

template <typename E>
Graph<E>* ZGraphInstance<E>::get_graph() {
  return graph;
}

template <typename E>
void ZGraphInstance<E>::set_graph(Graph<E>* graph_) {
  graph = graph_;
}

template <typename E>
double ZGraphInstance<E>::get_scaling_factor(VertexId num_vertices_in_pattern) {
  double factor = 1.;
  double num_workers = (double)graph->p.num_sockets * graph->p.num_partitions;
  for (VertexId i = 1; i < num_vertices_in_pattern; ++i) factor *= num_workers;
  return factor;
}

template <typename E>
void ZGraphInstance<E>::set_sampling_seed(uint64_t seed, uint32_t stream_id) {
  seed_ = seed;
  stream_id_ = stream_id;
  next_sample_ = 0;
}

template <typename E>
std::vector<std::pair<int, zg_program*>> ZGraphInstance<E>::program_candidates() {
  std::vector<std::pair<int, uint32_t>> kinds = {
      {ZG_PROG_TRIANGLE, 0}, {ZG_PROG_THREE_CHAIN, 0}, {ZG_PROG_FOUR_CLIQUE, 0}, {ZG_PROG_FOUR_CHAIN, 0}};
  for (uint32_t k = 4; k <= ZG_MAX_LIST; ++k) kinds.push_back({ZG_PROG_CHAIN, k});
  kinds.push_back({ZG_PROG_CHAIN, 3});
  std::vector<std::pair<int, zg_program*>> out;
  for (auto& k : kinds) {
    zg_program* p = nullptr;
    zgh::check(zg_program_create(k.first, k.second, &p), "zg_program_create");
    out.push_back({k.first, p});
  }
  return out;
}

template <typename E>
int ZGraphInstance<E>::replay_trace(const zg_sample_trace& t, double* value) {
  Random::Draw d[ZG_MAX_DRAWS];
  uint32_t n = t.ndraws < ZG_MAX_DRAWS ? t.ndraws : ZG_MAX_DRAWS;
  for (uint32_t k = 0; k < n; ++k) d[k] = {t.lo[k], t.hi[k], t.val[k]};
  bool was = validating_;
  validating_ = true;
  randoms[0].replay(d, (int)n);
  double r;
  try {
    r = estimate();
  } catch (...) {
    randoms[0].stop_replay();
    validating_ = was;
    throw;
  }
  bool draws_ok = randoms[0].mismatches() == 0 && randoms[0].pending() == 0 && n == t.ndraws;
  randoms[0].stop_replay();
  validating_ = was;
  if (value) *value = r;
  if (!draws_ok) return 2;
  uint64_t a = bits_of(r), b = bits_of(t.w);
  if (a == b) return 0;
  if (r == 0 || t.w == 0 || (a >> 63) != (b >> 63)) return 2;
  uint64_t ulps = a > b ? a - b : b - a;
  return ulps <= 4 ? 1 : 2;
}

// Each candidate is replayed until kValidationHits device hits were seen (or kValidationMaxSamples
// samples); a candidate whose every sample agrees bit for bit is adopted, else the first whose
// samples agree within 4 ulps.
template <typename E>
zg_program* ZGraphInstance<E>::identify_program() {
  zg_graph* dg = zgh_device_graph(*graph);
  std::vector<std::pair<int, zg_program*>> cands = program_candidates();
  std::vector<zg_sample_trace> tr(kValidationBatch);
  int exact = -1, near = -1;
  try {
    for (size_t c = 0; c < cands.size() && exact < 0; ++c) {
      int worst = 0;
      uint64_t hits = 0;
      for (uint64_t done = 0; worst < 2 && done < kValidationMaxSamples && hits < kValidationHits;
           done += kValidationBatch) {
        zgh::check(zg_run_debug(dg, cands[c].second, kValidationBatch, done, kValidationSeed, kValidationStream, tr.data()),
                   "zg_run_debug");
        for (uint64_t i = 0; worst < 2 && i < kValidationBatch; ++i) {
          worst = std::max(worst, replay_trace(tr[i]));
          hits += tr[i].hit;
        }
      }
      if (worst == 0) exact = (int)c;
      if (worst == 1 && near < 0) near = (int)c;
    }
  } catch (...) {
    for (auto& c : cands) zg_program_free(c.second);
    throw;
  }
  int chosen = exact >= 0 ? exact : near;
  for (size_t c = 0; c < cands.size(); ++c)
    if ((int)c != chosen) zg_program_free(cands[c].second);
  if (chosen < 0)
    throw std::runtime_error(
        "ZGraphInstance::calculate: no device program reproduces this estimate() "
        "(status " + std::to_string(ZG_ERR_UNSUPPORTED_ESTIMATOR) + "); there is no CPU execution path");
  program_kind_ = cands[chosen].first;
  return cands[chosen].second;
}

template <typename E>
zg_program* ZGraphInstance<E>::device_program() {
  if (!program_) {
    zgh::ensure_init();
    program_ = identify_program();
  }
  return program_;
}

template <typename E>
zg_counters ZGraphInstance<E>::device_run(unsigned long long n) {
  zg_program* p = device_program();
  zg_graph* dg = zgh_device_graph(*graph);
  zg_counters c;
  zgh::check(zg_run(dg, p, n, next_sample_, seed_, stream_id_, nullptr, &c), "zg_run");
  next_sample_ += n;
  last_counters_ = c;
  return c;
}

// src/ZGraphInstance.cpp:257-297, with the estimators on the device and their mean exact.
template <typename E>
double ZGraphInstance<E>::calculate(unsigned long long num_estmators, VertexId num_vertices_in_pattern,
                                    Estimation& init_estimation) {
  if (init_estimation.get_num_finished_estimators() >= num_estmators) return init_estimation.get_currnet_estimation();
  num_estmators -= init_estimation.get_num_finished_estimators();
  zg_counters c = device_run(num_estmators);
  double estimation = c.estimate * get_scaling_factor(num_vertices_in_pattern);
  init_estimation.update(num_estmators, estimation);
  return init_estimation.get_currnet_estimation();
}

template <typename E>
void ZGraphInstance<E>::require_replay(const char* primitive) const {
  if (!validating_)
    throw std::runtime_error(std::string(primitive) +
                             ": the ASAP primitives run on the host only to replay a device trace; estimates come "
                             "from calculate() on the GPU (no host execution path, ZG_ERR_UNSUPPORTED_ESTIMATOR)");
}

template <typename E>
std::pair<VertexId, double> ZGraphInstance<E>::sample_vertex() {
  require_replay("sample_vertex");
  if (graph->p.local_partition_offset[0] == graph->p.local_partition_offset[1])
    return std::make_pair((VertexId)0, (double)-1);
  VertexId min_v = graph->p.local_partition_offset[0];
  VertexId max_v = graph->p.local_partition_offset[1] - 1;
  return std::make_pair((VertexId)randoms[0].rand_int(min_v, max_v), 1. / (max_v - min_v + 1));
}

template <typename E>
std::pair<Edge<E>, double> ZGraphInstance<E>::sample_edge() {
  require_replay("sample_edge");
  if (is_counting_sample_edge_calls) ++cnt;
  Edge<E> edge;
  EdgeId m = graph->num_local_edges[0];
  if (m == 0) return std::make_pair(edge, (double)-1);
  EdgeId id = randoms[0].rand_int(0, m - 1);
  const EdgeUnit<E>& u = graph->local_edges[0][id];
  edge.edge_id = id;
  edge.src = u.src;
  edge.dst = u.dst;
  if (!std::is_same<E, Empty>::value) edge.edge_data = u.edge_data;
  return std::make_pair(edge, 1. / m);
}

template <typename E>
std::pair<VertexId, double> ZGraphInstance<E>::conditional_sample_vertex(const SubGraph<E>& sub_graph) {
  require_replay("conditional_sample_vertex");
  VertexId lo = sub_graph.get_min_valid_vertex_id();
  VertexId end = graph->p.local_partition_offset[1];
  if (lo >= end) return std::make_pair((VertexId)0, (double)-1);
  VertexId v = randoms[0].rand_int(lo, end - 1);
  return std::make_pair(v, 1. / (end - lo));
}

// src/ZGraphInstance.cpp:128-222: the suffix of each anchor's edge-id-ordered list past the
// largest given edge id; one draw over their total; p = (anchors the edge touches) / total.
template <typename E>
std::pair<Edge<E>, double> ZGraphInstance<E>::core_conditional_sample_edge(const MyList<Edge<E>>& sampled_edges,
                                                                         const MyList<VertexId>& sampled_vertices) {
  require_replay("conditional_sample_edge");
  EdgeId min_valid = 0;
  for (int i = 0; i < sampled_edges.list_size; ++i)
    if (sampled_edges.list[i].edge_id + 1 > min_valid) min_valid = sampled_edges.list[i].edge_id + 1;
  Edge<E> sampled_edge;
  Bitmap* bm = graph->outgoing_adj_bitmap[0];
  const EdgeId* idx = graph->outgoing_adj_index[0];
  const AdjUnit<E>* adj = graph->outgoing_adj_list[0];
  EdgeId sum = 0;
  MyList<EdgeId> start;
  for (int i = 0; i < sampled_vertices.list_size; ++i) {
    VertexId v = sampled_vertices.list[i];
    if (!bm->get_bit(v)) continue;
    EdgeId b = idx[v], e = idx[v + 1];
    if (min_valid <= adj[b].edge_id) {
      sum += e - b;
      start.push_back(b);
    } else if (min_valid > adj[e - 1].edge_id) {
      start.push_back(e);
    } else if (e - b <= BINARY_SEARCH_THRESHOLD) {
      for (EdgeId k = b; k < e; ++k)
        if (min_valid <= adj[k].edge_id) {
          sum += e - k;
          start.push_back(k);
          break;
        }
    } else {
      EdgeId l = b, r = e - 1;  // adj[l].edge_id < min_valid <= adj[r].edge_id
      while (r - l > 1) {
        EdgeId mid = (l + r) >> 1;
        if (adj[mid].edge_id < min_valid)
          l = mid;
        else
          r = mid;
      }
      sum += e - r;
      start.push_back(r);
    }
  }
  if (sum == 0) return std::make_pair(sampled_edge, (double)-1);
  EdgeId r = randoms[0].rand_int(0, sum - 1);
  int si = 0;
  bool found = false;
  for (int i = 0; i < sampled_vertices.list_size && !found; ++i) {
    VertexId v = sampled_vertices.list[i];
    if (!bm->get_bit(v)) continue;
    EdgeId cur = start.list[si++], e = idx[v + 1];
    if (cur + r < e) {
      const AdjUnit<E>& a = adj[cur + r];
      sampled_edge.edge_id = a.edge_id;
      sampled_edge.src = a.src;
      sampled_edge.dst = a.dst;
      if (!std::is_same<E, Empty>::value) sampled_edge.edge_data = a.edge_data;
      found = true;
    } else {
      r -= e - cur;
    }
  }
  double appear = 0;
  for (int i = 0; i < sampled_vertices.list_size; ++i) {
    if (sampled_vertices.list[i] == sampled_edge.src) ++appear;
    if (sampled_vertices.list[i] == sampled_edge.dst) ++appear;
  }
  assert(found);
  assert(appear == 1 || appear == 2);
  return std::make_pair(sampled_edge, 1. * appear / sum);
}

template <typename E>
std::pair<Edge<E>, double> ZGraphInstance<E>::conditional_sample_edge(const SubGraph<E>& sub_graph) {
  if (is_counting_conditional_edge_calls) ++cnt;
  return core_conditional_sample_edge(sub_graph.get_edges(), sub_graph.get_vertices());
}

template <typename E>
std::pair<Edge<E>, double> ZGraphInstance<E>::conditional_sample_edge(const MyList<Edge<E>>& edges,
                                                                     const MyList<VertexId>& vertices) {
  if (is_counting_conditional_edge_calls) ++cnt;
  return core_conditional_sample_edge(edges, vertices);
}

// src/ZGraphInstance.cpp:372-407: each edge to wait must appear, with an id past the sample's
// largest, in the adjacency of one of the sampled vertices.
template <typename E>
bool ZGraphInstance<E>::conditional_close(const SubGraph<E>& sampled_subgraph, const SubGraph<E>& subgraph_to_wait) {
  MyList<Edge<E>> wait = subgraph_to_wait.get_edges();
  return conditional_close(sampled_subgraph.get_min_valid_edge_id(), sampled_subgraph.get_vertices(), wait);
}

template <typename E>
bool ZGraphInstance<E>::conditional_close(EdgeId min_valid_edge_id, const MyList<VertexId>& sampled_vertices,
                                          MyList<Edge<E>>& edges_to_wait) {
  require_replay("conditional_close");
  Bitmap* bm = graph->outgoing_adj_bitmap[0];
  const EdgeId* idx = graph->outgoing_adj_index[0];
  const AdjUnit<E>* adj = graph->outgoing_adj_list[0];
  for (int i = 0; i < edges_to_wait.list_size; ++i) {
    Edge<E>& w = edges_to_wait.list[i];
    bool found = false;
    for (int j = 0; j < sampled_vertices.list_size && !found; ++j) {
      VertexId v = sampled_vertices.list[j];
      if (!bm->get_bit(v)) continue;
      for (EdgeId k = idx[v]; k < idx[v + 1]; ++k) {
        const AdjUnit<E>& a = adj[k];
        if (a.edge_id < min_valid_edge_id) continue;
        if ((a.src == w.src && a.dst == w.dst) || (a.dst == w.src && a.src == w.dst)) {
          w.edge_id = a.edge_id;
          found = true;
          break;
        }
      }
    }
    if (!found) return false;
  }
  return true;
}

template <typename E>
unsigned long long ZGraphInstance<E>::sample_interger(unsigned long long min_int, unsigned long long max_int) {
  require_replay("sample_interger");
  return randoms[0].rand_int(min_int, max_int);
}

// The reference returns 1 here (src/ZGraphInstance.cpp:449-450).
template <typename E>
double ZGraphInstance<E>::get_num_sample_edge_calls() {
  return 1;
}

// The reference counts conditional_sample_edge calls over the successful estimates of 1024
// estimate() runs (src/ZGraphInstance.cpp:471-490); every successful estimate of a program makes
// the same number of calls, which the identified device program states.
template <typename E>
double ZGraphInstance<E>::get_num_conditional_sample_edge_calls() {
  uint32_t cc = 0;
  zgh::check(zg_program_info(device_program(), nullptr, &cc, nullptr), "zg_program_info");
  return (double)cc;
}

// ---- AllPredicateZGraphInstance (src/ZGraphInstance.cpp:493-525) -------------------------------------
template <typename E>
AllPredicateZGraphInstance<E>::AllPredicateZGraphInstance(Graph<E>* graph_, std::function<bool(E)> predicate_)
    : original_graph(graph_), predicate(predicate_), next_filter_seed_(0) {
  csr_constructor = new CSRConstructor<E>();
  destroyer = new NumaAwareGraphDestroyer<E>();
  graph_filter = new GraphFilter<E>(csr_constructor, destroyer, predicate);
  graph_filter->generate_graph(*original_graph, filtered_graph);
  ZGraphInstance<E>::set_graph(&filtered_graph);
}

template <typename E>
AllPredicateZGraphInstance<E>::~AllPredicateZGraphInstance() {
  graph_filter->destroy_graph(filtered_graph);
  delete graph_filter;
  delete csr_constructor;
  delete destroyer;
}

template <typename E>
Graph<E>* AllPredicateZGraphInstance<E>::get_graph() {
  return original_graph;
}

template <typename E>
void AllPredicateZGraphInstance<E>::set_graph(Graph<E>* graph_) {
  graph_filter->destroy_graph(filtered_graph);
  original_graph = graph_;
  filtered_graph.shuffle_seed = next_filter_seed_;
  next_filter_seed_ = 0;
  graph_filter->generate_graph(*original_graph, filtered_graph);
  ZGraphInstance<E>::set_graph(&filtered_graph);
}

template <typename E>
double AllPredicateZGraphInstance<E>::calculate(unsigned long long num_estmators, VertexId num_vertices_in_pattern,
                                                Estimation& init_estimation) {
  return ZGraphInstance<E>::calculate(num_estmators, num_vertices_in_pattern, init_estimation);
}

// ---- CachedSubPatterns ---------------------------------------------------------------------------------
template <typename E>
CachedSubPatterns<E>::CachedSubPatterns(unsigned long long num_estmators_, unsigned long long** num_saved_sub_patterns_)
    : num_estmators(num_estmators_), num_saved_sub_patterns(num_saved_sub_patterns_), saved_sub_patterns(nullptr),
      saved_probability(nullptr), source_(nullptr), device_graph_(nullptr), seed_(0), stream_(0), pure_chain_(false) {}

template <typename E>
CachedSubPatterns<E>::~CachedSubPatterns() {
  if (saved_sub_patterns) {
    delete[] saved_sub_patterns[0][0];
    delete[] saved_probability[0][0];
    delete[] saved_sub_patterns[0];
    delete[] saved_probability[0];
    delete[] saved_sub_patterns;
    delete[] saved_probability;
  }
  delete[] num_saved_sub_patterns[0];
  delete[] num_saved_sub_patterns;
}

// The wedges on the host: the device traces of the three-chain estimators, replayed through the
// source instance's sample_edge and conditional_sample_edge (what the reference's 3-chain estimate
// stores, applications/ThreeMotif.cpp:96-121; p = -1 marks a failed estimator).
template <typename E>
void CachedSubPatterns<E>::materialise() {
  if (saved_sub_patterns) return;
  if (!source_ || !pure_chain_)
    throw std::runtime_error("CachedSubPatterns: these wedges are not stored on the host (only a 3-chain run's are)");
  if (source_->graph == nullptr || source_->graph->device != device_graph_)
    throw std::runtime_error("CachedSubPatterns: the graph of the 3-chain run has changed");
  const unsigned long long n = num_saved_sub_patterns[0][0];
  if (n > (1ull << 22)) throw std::runtime_error("CachedSubPatterns: more than 2^22 wedges to materialise");
  SubGraph<E>* sg = new SubGraph<E>[n ? n : 1];
  double* pr = new double[n ? n : 1];
  std::vector<zg_sample_trace> tr(n ? n : 1);
  if (n) zgh::check(zg_run_debug(device_graph_, source_->device_program(), n, 0, seed_, stream_, tr.data()), "zg_run_debug");
  Random& rnd = source_->randoms[0];
  // a replay: the primitives below run on the device trace's draws
  struct ReplayScope {
    bool& flag;
    bool was;
    explicit ReplayScope(bool& f) : flag(f), was(f) { flag = true; }
    ~ReplayScope() { flag = was; }
  } scope(source_->validating_);
  for (unsigned long long i = 0; i < n; ++i) {
    Random::Draw d[ZG_MAX_DRAWS];
    for (uint32_t k = 0; k < tr[i].ndraws && k < ZG_MAX_DRAWS; ++k) d[k] = {tr[i].lo[k], tr[i].hi[k], tr[i].val[k]};
    rnd.replay(d, (int)tr[i].ndraws);
    double p = 1;
    auto e0 = source_->ZGraphInstance<E>::sample_edge();
    if (e0.second < 0) {
      p = -1;
    } else {
      p *= e0.second;
      sg[i].add_edge(e0.first);
      auto e1 = source_->ZGraphInstance<E>::conditional_sample_edge(sg[i]);
      if (e1.second < 0) {
        p = -1;
      } else {
        p *= e1.second;
        sg[i].add_edge(e1.first);
      }
    }
    pr[i] = p;
  }
  rnd.stop_replay();
  saved_sub_patterns = new SubGraph<E>**[1]{new SubGraph<E>*[1]{sg}};
  saved_probability = new double**[1]{new double*[1]{pr}};
}

template <typename E>
void CachedSubPatterns<E>::add(int socket_id, int socket_offset, unsigned long long estimator_id, SubGraph<E>& sub_graph,
                               double probability) {
  materialise();
  saved_sub_patterns[socket_id][socket_offset][estimator_id] = sub_graph;
  saved_probability[socket_id][socket_offset][estimator_id] = probability;
  pure_chain_ = false;  // host-edited wedges are no longer the device's
}

template <typename E>
void CachedSubPatterns<E>::get(int socket_id, int socket_offset, unsigned long long estimator_id, SubGraph<E>*& subgraph,
                               double*& probability) {
  materialise();
  subgraph = &saved_sub_patterns[socket_id][socket_offset][estimator_id];
  probability = &saved_probability[socket_id][socket_offset][estimator_id];
}

template <typename E>
std::pair<SubGraph<E>*, double*> CachedSubPatterns<E>::get_all(int socket_id, int socket_offset,
                                                              unsigned long long& num_patterns) {
  materialise();
  num_patterns = num_saved_sub_patterns[socket_id][socket_offset];
  return std::make_pair(saved_sub_patterns[socket_id][socket_offset], saved_probability[socket_id][socket_offset]);
}

template <typename E>
unsigned long long CachedSubPatterns<E>::get_num_patterns(int socket_id, int socket_offset) {
  return num_saved_sub_patterns[socket_id][socket_offset];
}

// ---- ZGraphInstanceWithCache (src/ZGraphInstance.cpp:674-833) ---------------------------------------
template <typename E>
ZGraphInstanceWithCache<E>::ZGraphInstanceWithCache(Graph<E>* graph_) : ZGraphInstance<E>(graph_) {
  imported_cached_sub_patterns = nullptr;
  exported_cached_sub_patterns = nullptr;
  curr_estimator_id = new unsigned long long*[1]{new unsigned long long[1]{0}};
  fake_p = 0;
  calls_ = 0;
}

template <typename E>
ZGraphInstanceWithCache<E>::~ZGraphInstanceWithCache() {
  delete exported_cached_sub_patterns;
  delete[] curr_estimator_id[0];
  delete[] curr_estimator_id;
}

// On the host, estimate() always takes the uncached branch: the cached branch runs on the device
// inside the fused 3-motif kernel.
template <typename E>
void ZGraphInstanceWithCache<E>::get_subgraph(bool& is_cached_pattern, SubGraph<E>*& subgraph, double*& p) {
  is_cached_pattern = false;
  subgraph = &fake_subgraph;
  subgraph->edges.list_size = 0;
  subgraph->vertices.list_size = 0;
  subgraph->min_valid_edge_id = 0;
  subgraph->min_valid_vertex_id = 0;
  p = &fake_p;
}

template <typename E>
CachedSubPatterns<E>* ZGraphInstanceWithCache<E>::get_cached_sub_patterns() {
  return exported_cached_sub_patterns;
}

template <typename E>
void ZGraphInstanceWithCache<E>::set_cached_sub_patterns(CachedSubPatterns<E>* cached_sub_patterns_) {
  imported_cached_sub_patterns = cached_sub_patterns_;
}

// A run without an imported cache samples afresh (estimators [0, n) on a stream of their own) and
// exports their description.  A run with one must be the triangle closure of a 3-chain run's
// wedges on the same graph: the first min(n_chain, n) estimators close the cached wedges, the rest
// sample afresh, all in one fused launch (zg_run_three_motif).
template <typename E>
double ZGraphInstanceWithCache<E>::calculate(unsigned long long num_estmators, VertexId num_vertices_in_pattern,
                                             Estimation& init_estimation) {
  if (init_estimation.get_num_finished_estimators() >= num_estmators) return init_estimation.get_currnet_estimation();
  num_estmators -= init_estimation.get_num_finished_estimators();
  zg_program* prog = this->device_program();
  zg_graph* dg = zgh_device_graph(*this->get_graph());
  const uint32_t stream = this->stream_id_ + (calls_++ & 0xff);
  zg_counters c;
  CachedSubPatterns<E>* imp = imported_cached_sub_patterns;
  imported_cached_sub_patterns = nullptr;
  unsigned long long** counts = new unsigned long long*[1]{new unsigned long long[1]{num_estmators}};
  CachedSubPatterns<E>* exp = new CachedSubPatterns<E>(num_estmators, counts);
  if (imp == nullptr) {
    zgh::check(zg_run(dg, prog, num_estmators, 0, this->seed_, stream, nullptr, &c), "zg_run");
    exp->source_ = this;
    exp->device_graph_ = dg;
    exp->seed_ = this->seed_;
    exp->stream_ = stream;
    exp->pure_chain_ = this->program_kind_ == ZG_PROG_THREE_CHAIN;
  } else {
    if (this->program_kind_ != ZG_PROG_TRIANGLE || !imp->pure_chain_ || imp->device_graph_ != dg) {
      delete exp;
      throw std::runtime_error(
          "ZGraphInstanceWithCache::calculate: an imported cache is closed on the device only by a triangle "
          "estimator over the wedges of a 3-chain run on the same graph");
    }
    zg_counters chain;
    zgh::check(zg_run_three_motif(dg, imp->num_saved_sub_patterns[0][0], num_estmators, imp->seed_, imp->stream_, stream,
                                  nullptr, &chain, &c),
               "zg_run_three_motif");
  }
  delete exported_cached_sub_patterns;
  exported_cached_sub_patterns = exp;
  this->last_counters_ = c;
  double estimation = c.estimate * this->get_scaling_factor(num_vertices_in_pattern);
  init_estimation.update(num_estmators, estimation);
  return init_estimation.get_currnet_estimation();
}

// ---- TimeProfile (src/ErrorLatencyProfile.cpp:12-47) ---------------------------------------------------
template <typename E>
void TimeProfile<E>::reset() {
  num_finished_estimators = 0;
  current_estimation = 0;
}

template <typename E>
void TimeProfile<E>::update(unsigned long long new_num_estimators, double new_estimation) {
  current_estimation =
      current_estimation * double(num_finished_estimators) / double(num_finished_estimators + new_num_estimators) +
      new_estimation * double(new_num_estimators) / double(num_finished_estimators + new_num_estimators);
  num_finished_estimators += new_num_estimators;
}

template <typename E>
double TimeProfile<E>::run(ZGraphInstance<E>& zgraph_instance, VertexId num_vertices_in_pattern, unsigned int time_limit) {
  reset();
  zgraph_instance.device_program();  // identification is set-up, not part of the budget
  unsigned int used_time = 0, curr_used_time = 0;
  unsigned long long next = BASIC_NUM_ESTIMATORS_PER_THREAD * SharedMemSys::get_instance()->get_num_threads_per_socket();
  while (used_time + curr_used_time * 2 <= time_limit) {
    double t = -get_time();
    Estimation init;
    double e = zgraph_instance.calculate(next, num_vertices_in_pattern, init);
    t += get_time();
    update(next, e);
    next <<= 1;
    curr_used_time = (unsigned int)(t * 1000);
    used_time += curr_used_time;
  }
  Estimation init;
  unsigned long long remained = next * (time_limit - used_time) / (curr_used_time * 2);
  if (remained) {
    double e = zgraph_instance.calculate(remained, num_vertices_in_pattern, init);
    update(remained, e);
  }
  return current_estimation;
}

// ---- ErrorProfile (src/ErrorLatencyProfile.cpp:52-207) --------------------------------------------------
template <typename E>
double ErrorProfile<E>::calculate_bound(double epsilon, double delta, double nse, double ncse, double estimation,
                                        EdgeId max_degree, EdgeId num_edges) {
  return zg_calculate_bound(epsilon, delta, nse, ncse, estimation, max_degree, num_edges);
}

template <typename E>
double ErrorProfile<E>::run(ZGraphInstance<E>& zgraph_instance, VertexId num_vertices_in_pattern,
                            double required_error_rate, double required_confidence, Estimation& init_estimation) {
  unsigned long long n = get_num_estimators(zgraph_instance, num_vertices_in_pattern, required_error_rate, required_confidence);
  return zgraph_instance.calculate(n, num_vertices_in_pattern, init_estimation);
}

// The reference's procedure with its 2^14 calculate(16) calls and the calculate(2^23) follow-up
// batched into two device launches.  Draw plan for the instance's seed s: subsample keep draws
// s+1, shuffle s+2, predicate filter shuffle s+3; estimators on stream ZG_ELP_STREAM — the plan of
// zg_elp_plain, which gives the same number for a threshold predicate.
template <typename E>
unsigned long long ErrorProfile<E>::get_num_estimators(ZGraphInstance<E>& zgraph_instance, VertexId,
                                                       double required_error_rate, double required_confidence) {
  zg_program* prog = zgraph_instance.device_program();
  double nse = zgraph_instance.get_num_sample_edge_calls();
  double ncse = zgraph_instance.get_num_conditional_sample_edge_calls();
  const uint64_t seed = zgraph_instance.seed_;
  CSRConstructor<E> csr;
  NumaAwareGraphDestroyer<E> destroyer;
  GraphSampler<E> sampler(&csr, &destroyer, 0.1);
  sampler.set_seeds(seed + ZG_ELP_KEEP_OFFSET, seed + ZG_ELP_SHUFFLE_OFFSET);
  Graph<E>& original = *zgraph_instance.get_graph();
  Graph<E> sampled;
  sampler.sample_graph(original, sampled);
  if (auto* ap = dynamic_cast<AllPredicateZGraphInstance<E>*>(&zgraph_instance))
    ap->next_filter_seed_ = seed + ZG_ELP_FILTER_OFFSET;
  zgraph_instance.set_graph(&sampled);
  zg_elp_result res;
  int rc = ZG_OK;
  try {
    zg_graph* dg = zgh_device_graph(*zgraph_instance.graph);
    const uint64_t n_groups = 1ull << 14, big_n = 1ull << 23;
    const uint32_t group = 16;
    std::vector<double> groups(n_groups);
    zgh::check(zg_run_groups(dg, prog, n_groups, group, 0, seed, ZG_ELP_STREAM, nullptr, groups.data()), "zg_run_groups");
    zg_counters big;
    zgh::check(zg_run(dg, prog, big_n, n_groups * group, seed, ZG_ELP_STREAM, nullptr, &big), "zg_run");
    rc = zg_elp_solve(groups.data(), n_groups, group, big.estimate, big_n, nse, ncse, sampled.num_edges,
                      sampled.max_degree, original.num_edges, original.max_degree, required_error_rate,
                      required_confidence, &res);
  } catch (...) {
    sampler.destroy_graph(sampled);
    zgraph_instance.set_graph(&original);
    throw;
  }
  sampler.destroy_graph(sampled);
  zgraph_instance.set_graph(&original);
  zgh::check(rc, "zg_elp_solve");
  Debug::get_instance()->print("num_estimators required: ", res.n_required_f);
  return res.n_required;
}

// ---- SamplerGenerator (src/SamplerGenerator.cpp:287-546) -------------------------------------------------
template <typename E>
void SamplerGenerator<E>::generate_mapping(VertexId idx) {
  if (idx == num_vertices) {
    patterns[curr_pos++]->setup_vertex_id_mapping(mapping);
    return;
  }
  for (VertexId v = 0; v < num_vertices; ++v)
    if (!is_used[v]) {
      is_used[v] = true;
      mapping[idx] = v;
      generate_mapping(idx + 1);
      is_used[v] = false;
    }
}

// A new edge must not precede, in edge id, an edge listed after its first neighbour in the list.
template <typename E>
bool SamplerGenerator<E>::canonicality_check(const MyList<Edge<E>>& edges, const Edge<E> new_edge) {
  if (edges.list_size <= 1) return true;
  bool found_neighbour = false;
  for (int i = 0; i < edges.list_size; ++i) {
    if (!found_neighbour) {
      const Edge<E>& x = edges.list[i];
      found_neighbour = new_edge.src == x.src || new_edge.src == x.dst || new_edge.dst == x.src || new_edge.dst == x.dst;
    } else if (edges.list[i].edge_id >= new_edge.edge_id) {
      return false;
    }
  }
  return true;
}

template <typename E>
void SamplerGenerator<E>::set_predicate_fun(std::function<bool(SubGraph<E>)> predicate_fun_) {
  used_predicate_fun = true;
  predicate_fun = predicate_fun_;
}

template <typename E>
SamplerGenerator<E>::SamplerGenerator(Graph<E>* graph_, Pattern* pattern_) : ZGraphInstance<E>(graph_) {
  pattern = new Pattern(pattern_->get_num_vertices(), pattern_->get_num_edges(), pattern_->get_edges());
  assert(pattern->get_num_vertices() >= 1);
  assert(pattern->get_num_edges() >= 1);
  num_vertices = pattern->get_num_vertices();
  num_edges = pattern->get_num_edges();
  num_patterns = 1;
  for (VertexId v = 1; v <= num_vertices; ++v) num_patterns *= v;
  patterns = new Pattern*[num_patterns];
  for (VertexId p = 0; p < num_patterns; ++p) patterns[p] = new Pattern(num_vertices, num_edges, pattern->get_edges());
  mapping = new VertexId[num_vertices];
  is_used = new bool[num_vertices]();
  curr_pos = 0;
  generate_mapping(0);
  is_duplicated = new bool[num_patterns]();
  num_unique_patterns = 0;
  for (VertexId p = 0; p < num_patterns; ++p) {
    for (VertexId q = 0; q < p; ++q)
      if (!is_duplicated[q] && patterns[q]->is_automorphic(*patterns[p])) {
        is_duplicated[p] = true;
        break;
      }
    if (!is_duplicated[p]) ++num_unique_patterns;
  }
  unique_patterns = new Pattern*[num_unique_patterns];
  VertexId k = 0;
  for (VertexId p = 0; p < num_patterns; ++p)
    if (!is_duplicated[p]) unique_patterns[k++] = patterns[p];
  used_predicate_fun = false;
}

template <typename E>
SamplerGenerator<E>::~SamplerGenerator() {
  delete pattern;
  for (VertexId p = 0; p < num_patterns; ++p) delete patterns[p];
  delete[] patterns;
  delete[] mapping;
  delete[] is_used;
  delete[] is_duplicated;
  delete[] unique_patterns;
}

template <typename E>
std::vector<std::pair<int, zg_program*>> SamplerGenerator<E>::program_candidates() {
  if (used_predicate_fun) return {};
  std::vector<uint32_t> pairs;
  Edge<Empty>* pe = pattern->get_edges();
  for (EdgeId e = 0; e < num_edges; ++e) {
    pairs.push_back(pe[e].src);
    pairs.push_back(pe[e].dst);
  }
  zg_program* p = nullptr;
  zgh::check(zg_program_create_pattern(num_vertices, (uint32_t)num_edges, pairs.data(), &p), "zg_program_create_pattern");
  return {{ZG_PROG_PATTERN, p}};
}

template <typename E>
double SamplerGenerator<E>::estimate() {
  MyList<Edge<E>> sampled_edges;
  SubGraph<E> sampled_subgraph;
  const MyList<VertexId>& sampled_vertices = sampled_subgraph.get_vertices();
  double p = 1.;
  MyList<Edge<E>> first_edge;
  std::pair<Edge<E>, double> t0 = this->sample_edge();
  if (t0.second < 0) return 0;
  p *= t0.second;
  first_edge.push_back(t0.first);
  sampled_edges.push_back(t0.first);
  sampled_subgraph.add_edge(t0.first);
  for (EdgeId e = 1; e < num_edges; ++e) {
    std::pair<Edge<E>, double> t = this->conditional_sample_edge(first_edge, sampled_vertices);
    if (t.second < 0) return 0;
    p *= t.second;
    if (!canonicality_check(sampled_edges, t.first)) return 0;
    sampled_edges.push_back(t.first);
    sampled_subgraph.add_edge(t.first);
    if ((VertexId)sampled_vertices.list_size > num_vertices) return 0;
  }
  if ((VertexId)sampled_vertices.list_size != num_vertices) return 0;
  VertexId vs[MAX_LIST_SIZE];
  for (VertexId i = 0; i < num_vertices; ++i) vs[i] = sampled_vertices.list[i];
  std::sort(vs, vs + num_vertices);
  Edge<Empty> rel[MAX_LIST_SIZE];
  for (int e = 0; e < sampled_edges.list_size; ++e) {
    rel[e].src = (VertexId)(std::find(vs, vs + num_vertices, sampled_edges.list[e].src) - vs);
    rel[e].dst = (VertexId)(std::find(vs, vs + num_vertices, sampled_edges.list[e].dst) - vs);
  }
  if (used_predicate_fun && !predicate_fun(sampled_subgraph)) return 0;
  for (VertexId q = 0; q < num_unique_patterns; ++q)
    if (unique_patterns[q]->is_automorphic(num_vertices, num_edges, rel)) return 1. / p;
  return 0;
}

template <typename E>
double SamplerGenerator<E>::get_num_sample_edge_calls() {
  return 1;
}

template <typename E>
double SamplerGenerator<E>::get_num_conditional_sample_edge_calls() {
  return num_edges - 1;
}

template struct SubGraph<Empty>;
template struct SubGraph<VertexId>;
template class ZGraphInstance<Empty>;
template class ZGraphInstance<VertexId>;
template class AllPredicateZGraphInstance<Empty>;
template class AllPredicateZGraphInstance<VertexId>;
template class CachedSubPatterns<Empty>;
template class CachedSubPatterns<VertexId>;
template class ZGraphInstanceWithCache<Empty>;
template class ZGraphInstanceWithCache<VertexId>;
template class TimeProfile<Empty>;
template class TimeProfile<VertexId>;
template class ErrorProfile<Empty>;
template class ErrorProfile<VertexId>;
template class SamplerGenerator<Empty>;
template class SamplerGenerator<VertexId>;
