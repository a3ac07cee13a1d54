// SamplerGenerator.hpp — a generic estimator from a small pattern graph (the reference's
// include/SamplerGenerator.hpp interface); on the device it is one program with a lookup table of
// the pattern's unique relabellings.
#ifndef SAMPLER_GENERATOR_HPP
#define SAMPLER_GENERATOR_HPP

#include <iostream>

#include "Debug.hpp"
#include "ZGraphInstance.hpp"

class Pattern {
 private:
  EdgeId* csr_idx;
  Edge<Empty>* csr_list;
  Edge<Empty>* edges;
  VertexId num_vertices;
  EdgeId num_edges;
  void construct_csr();
  EdgeId get_idx_by_edge_id(EdgeId edge_id) const;
  bool is_vertex_mapping_correct(VertexId* vertex_mapping, const Pattern& pattern);
  bool core_has_same_edge_ordering(VertexId src, VertexId dst, const Pattern& pattern);

 public:
  Pattern(VertexId num_vertices_, EdgeId num_edges_, Edge<Empty>* edges);
  ~Pattern();
  EdgeId* get_csr_idx();
  Edge<Empty>* get_csr_list();
  Edge<Empty>* get_edges();
  VertexId get_num_vertices();
  EdgeId get_num_edges();
  bool has_same_edge_ordering(const Pattern& pattern);
  void setup_edge_id_mapping(EdgeId* mapping);
  bool is_in_edges_list(Edge<Empty> edge);
  bool is_automorphic(VertexId num_vertices_, EdgeId num_edges_, const Edge<Empty>* edges_);
  bool is_automorphic(const Pattern& pattern);
  void setup_vertex_id_mapping(VertexId* mapping);

  friend std::ostream& operator<<(std::ostream& os, const Pattern& pattern) {
    os << "Pattern: num_vertices: " << pattern.num_vertices << ", num_edges: " << pattern.num_edges << ", ";
    for (EdgeId e = 0; e < pattern.num_edges; ++e)
      os << "(" << pattern.edges[e].edge_id << "):" << pattern.edges[e].src << "<->" << pattern.edges[e].dst << " ";
    return os;
  }
};

template <typename EdgeData>
class SamplerGenerator : public ZGraphInstance<EdgeData> {
 private:
  VertexId num_vertices;
  EdgeId num_edges;
  VertexId num_patterns;
  VertexId curr_pos;
  VertexId num_unique_patterns;

  Pattern* pattern;
  Pattern** patterns;
  VertexId* mapping;
  bool* is_used;
  bool* is_duplicated;
  Pattern** unique_patterns;

  std::function<bool(SubGraph<EdgeData>)> predicate_fun;
  bool used_predicate_fun;

  void generate_mapping(VertexId idx);
  bool canonicality_check(const MyList<Edge<EdgeData>>& edges, const Edge<EdgeData> new_edge);
  void set_predicate_fun(std::function<bool(SubGraph<EdgeData>)> predicate_fun_);

 protected:
  // The one device program: the pattern's unique relabellings as a lookup table.
  std::vector<std::pair<int, zg_program*>> program_candidates();

 public:
  SamplerGenerator(Graph<EdgeData>* graph_, Pattern* pattern_);
  ~SamplerGenerator();
  double estimate();

  double get_num_sample_edge_calls();
  double get_num_conditional_sample_edge_calls();
};

#endif
