// ZGraphInstance.hpp — the estimator interface of ZGraph (class names and signatures of the
// reference's include/ZGraphInstance.hpp), executed on the GPU.
//
// An application subclasses ZGraphInstance<E> and writes estimate() with the ASAP primitives, as
// before.  calculate() runs the estimators on the device: the first call identifies the device
// program that reproduces this estimate() (zg_run_debug traces of each candidate program are
// replayed through the application's own estimate() on the host, bit for bit, on a few hundred
// samples), then every calculate() is one device run of fresh Philox sample indices.  If no
// device program reproduces estimate(), calculate() throws: there is no CPU execution path.
#ifndef ZGRAPH_INSTANCE_HPP
#define ZGRAPH_INSTANCE_HPP

#include <assert.h>
#include <stdint.h>

#include <functional>
#include <iostream>
#include <utility>
#include <vector>

#include "Graph.hpp"
#include "GraphFilters.hpp"
#include "Random.hpp"
#include "Type.hpp"
#include "../../../include/zgraph_gpu.h"

#define MAX_LIST_SIZE 16

class Estimation {
 private:
  unsigned long long num_finished_estimators;
  double current_estimation;

 public:
  Estimation();
  void reset();
  void update(unsigned long long new_num_estimators, double new_estimation);
  unsigned long long get_num_finished_estimators();
  double get_currnet_estimation();
};

template <typename EdgeData>
struct Edge {
  EdgeId edge_id;
  VertexId src;
  VertexId dst;
  EdgeData edge_data;
};

template <>
struct Edge<Empty> {
  EdgeId edge_id;
  VertexId src;
  union {
    VertexId dst;
    Empty edge_data;
  };
};

template <typename Data>
struct MyList {
  int list_size;
  Data list[MAX_LIST_SIZE];
  MyList() { list_size = 0; }
  inline void push_back(const Data& data) {
    assert(list_size < MAX_LIST_SIZE);
    list[list_size++] = data;
  }
};

template <typename Data>
struct VectorList {
  int list_size;
  std::vector<Data> list;
  VectorList() { list_size = 0; }
  inline void push_back(const Data& data) {
    list.push_back(data);
    list_size += 1;
  }
};

template <typename EdgeData>
struct SubGraph {
  MyList<Edge<EdgeData>> edges;
  MyList<VertexId> vertices;
  EdgeId min_valid_edge_id;
  VertexId min_valid_vertex_id;

  SubGraph();
  bool is_in_vertices_list(VertexId vertex);
  void add_edge(const Edge<EdgeData>& edge);
  void add_vertex(VertexId vertex);
  const MyList<Edge<EdgeData>>& get_edges() const;
  const MyList<VertexId>& get_vertices() const;
  EdgeId get_min_valid_edge_id() const;
  VertexId get_min_valid_vertex_id() const;
  SubGraph<EdgeData> operator-(const SubGraph<EdgeData>& sub_graph);

  friend std::ostream& operator<<(std::ostream& os, const SubGraph& g) {
    os << "SubGraph: ";
    for (int i = 0; i < g.edges.list_size; ++i)
      os << "(" << "[" << g.edges.list[i].edge_id << "]: " << g.edges.list[i].src << "<->" << g.edges.list[i].dst << ") ";
    return os;
  }
};

template <typename EdgeData>
class ErrorProfile;
template <typename EdgeData>
class CachedSubPatterns;

template <typename EdgeData>
class ZGraphInstance {
 private:
  Graph<EdgeData>* graph;  // the graph the estimators sample (the filtered one for a predicate instance)

 protected:
  Random* randoms;
  bool is_counting_sample_edge_calls;
  bool is_counting_conditional_edge_calls;
  int cnt;

  double get_scaling_factor(VertexId num_vertices_in_pattern);
  std::pair<Edge<EdgeData>, double> core_conditional_sample_edge(const MyList<Edge<EdgeData>>& sampled_edges,
                                                                 const MyList<VertexId>& sampled_vertices);

  // ---- device binding (no counterpart in the reference) ----
  zg_program* program_;      // device program reproducing estimate(), identified on first use
  bool program_owned_;
  bool validating_;          // estimate() is being replayed against device traces
  // The ASAP primitives run on the host only while estimate() replays a device trace (program
  // identification, replay_trace, CachedSubPatterns); outside a replay they throw: estimates come
  // from calculate() on the GPU, and there is no host execution path.
  void require_replay(const char* primitive) const;
  uint64_t seed_;            // Philox key of this instance's estimators
  uint32_t stream_id_;       // Philox stream of this instance's estimators
  uint64_t next_sample_;     // first sample index of the next calculate()
  zg_counters last_counters_;
  // Device programs tried by identification, as (ZG_PROG_* kind, program) in order of
  // preference; identify_program() keeps the one it adopts and frees the others.
  virtual std::vector<std::pair<int, zg_program*>> program_candidates();
  int program_kind_;
  zg_program* identify_program();
  // Runs n estimators of this instance on the device: fresh sample indices every call.
  zg_counters device_run(unsigned long long n);
  template <typename> friend class ErrorProfile;
  template <typename> friend class CachedSubPatterns;

 public:
  ZGraphInstance();  // set_graph must be called before use
  ZGraphInstance(Graph<EdgeData>* graph_);
  virtual ~ZGraphInstance();
  virtual Graph<EdgeData>* get_graph();
  virtual void set_graph(Graph<EdgeData>* graph_);
  virtual double calculate(unsigned long long num_estmators, VertexId num_vertices_in_pattern,
                           Estimation& init_estimation);

  virtual std::pair<VertexId, double> sample_vertex();
  virtual std::pair<Edge<EdgeData>, double> sample_edge();
  virtual std::pair<VertexId, double> conditional_sample_vertex(const SubGraph<EdgeData>& sub_graph);
  virtual std::pair<Edge<EdgeData>, double> conditional_sample_edge(const SubGraph<EdgeData>& sub_graph);
  virtual std::pair<Edge<EdgeData>, double> conditional_sample_edge(const MyList<Edge<EdgeData>>& edges,
                                                                    const MyList<VertexId>& vertices);
  virtual bool conditional_close(const SubGraph<EdgeData>& sampled_subgraph,
                                 const SubGraph<EdgeData>& subgraph_to_wait);
  virtual bool conditional_close(EdgeId min_valid_edge_id, const MyList<VertexId>& sampled_vertices,
                                 MyList<Edge<EdgeData>>& edges_to_wait);
  virtual unsigned long long sample_interger(unsigned long long min_int, unsigned long long max_int);

  virtual double get_num_sample_edge_calls();
  virtual double get_num_conditional_sample_edge_calls();

  virtual double estimate() = 0;

  // ---- additions of the GPU build ----
  // The device program reproducing estimate() (identified on first use; throws if none does).
  zg_program* device_program();
  // Fixes the Philox key and stream of this instance's estimators and restarts its sample indices.
  void set_sampling_seed(uint64_t seed, uint32_t stream_id);
  uint64_t get_sampling_seed() const { return seed_; }
  uint32_t get_sampling_stream() const { return stream_id_; }
  // Exact counters of the last device run.
  const zg_counters& get_last_counters() const { return last_counters_; }
  // Runs estimate() on the host with the draws of one device trace (zg_run_debug) and compares:
  // returns 0 when every draw range, the draw count and the returned double agree bit for bit,
  // 1 when they agree but the double differs by at most 4 units in the last place (a long double
  // estimator on a host whose long double is not the x87 format), 2 otherwise.
  int replay_trace(const zg_sample_trace& trace, double* value = nullptr);
};

template <typename EdgeData>
class AllPredicateZGraphInstance : public ZGraphInstance<EdgeData> {
 private:
  Graph<EdgeData>* original_graph;
  Graph<EdgeData> filtered_graph;
  GraphFilter<EdgeData>* graph_filter;
  CSRConstructor<EdgeData>* csr_constructor;
  GraphDestroyer<EdgeData>* destroyer;
  std::function<bool(EdgeData)> predicate;
  uint64_t next_filter_seed_;  // shuffle seed of the next filtered graph (0: fresh)
  template <typename> friend class ErrorProfile;

 public:
  AllPredicateZGraphInstance(Graph<EdgeData>* graph_, std::function<bool(EdgeData)> predicate_);
  ~AllPredicateZGraphInstance();
  Graph<EdgeData>* get_graph();
  void set_graph(Graph<EdgeData>* graph_);
  double calculate(unsigned long long num_estmators, VertexId num_vertices_in_pattern, Estimation& init_estimation);
};

// The wedges of a 3-chain run as a triangle run re-reads them (ThreeMotif).  On the device a
// wedge is a deterministic function of its Philox key, stream and sample index, so the cache is
// that description; the triangle run closes the same wedges in one fused kernel
// (zg_run_three_motif).  get()/get_all() materialise wedges on the host on request.
template <typename EdgeData>
class CachedSubPatterns {
 private:
  unsigned long long num_estmators;
  unsigned long long** num_saved_sub_patterns;
  SubGraph<EdgeData>*** saved_sub_patterns;  // host copies, materialised on first get()
  double*** saved_probability;
  // device description
  ZGraphInstance<EdgeData>* source_;  // the instance whose estimators drew the wedges
  zg_graph* device_graph_;
  uint64_t seed_;
  uint32_t stream_;
  bool pure_chain_;  // wedges of the three-chain program alone, closable by zg_run_three_motif
  void materialise();
  template <typename> friend class ZGraphInstanceWithCache;

 public:
  CachedSubPatterns(unsigned long long num_estmators_, unsigned long long** num_saved_sub_patterns_);
  ~CachedSubPatterns();
  void add(int socket_id, int socket_offset, unsigned long long estimator_id, SubGraph<EdgeData>& sub_graph,
           double probability);
  void get(int socket_id, int socket_offset, unsigned long long estimator_id, SubGraph<EdgeData>*& subgraph,
           double*& probability);
  std::pair<SubGraph<EdgeData>*, double*> get_all(int socket_id, int socket_offset, unsigned long long& num_patterns);
  unsigned long long get_num_patterns(int socket_id, int socket_offset);
};

template <typename EdgeData>
class ZGraphInstanceWithCache : public ZGraphInstance<EdgeData> {
 private:
  CachedSubPatterns<EdgeData>* imported_cached_sub_patterns;
  CachedSubPatterns<EdgeData>* exported_cached_sub_patterns;
  unsigned long long** curr_estimator_id;
  SubGraph<EdgeData> fake_subgraph;
  double fake_p;
  uint32_t calls_;

 protected:
  void get_subgraph(bool& is_cached_pattern, SubGraph<EdgeData>*& subgraph, double*& p);

 public:
  ZGraphInstanceWithCache(Graph<EdgeData>* graph_);
  ~ZGraphInstanceWithCache();
  CachedSubPatterns<EdgeData>* get_cached_sub_patterns();
  void set_cached_sub_patterns(CachedSubPatterns<EdgeData>* cached_sub_patterns_);
  double calculate(unsigned long long num_estmators, VertexId num_vertices_in_pattern, Estimation& init_estimation);
};

#endif
