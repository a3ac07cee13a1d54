// Graph.hpp — the graph store: Graph<E> (host arrays in the reference's layout, plus a lazily
// created device copy), the loader, the uniform partitioner (one partition here), vertex
// mappings, the CSR constructor and the edge subsampler.  Interfaces follow the reference's
// include/Graph.hpp so that applications compile unchanged.
#ifndef GRAPH_HPP
#define GRAPH_HPP

#include <assert.h>

#include <string>

#include "Bitmap.hpp"
#include "Debug.hpp"
#include "Type.hpp"

struct zg_graph;

struct GraphPartition {
  int partition_id;
  int num_partitions;
  int num_sockets;
  VertexId owned_num_vertices;
  VertexId* partition_offset;              // [num_partitions + 1]
  VertexId* local_partition_offset;        // [num_sockets + 1]
  VertexId** all_local_partition_offset;   // [num_partitions][num_sockets + 1]

  GraphPartition();
  ~GraphPartition();
  GraphPartition(const GraphPartition& o);
  GraphPartition& operator=(const GraphPartition& o);
  int get_partition_id(VertexId v_i);
  int get_local_partition_id(VertexId v_i);
  int get_local_partition_id(int p_i, VertexId v_i);
};

class GraphPartitioner {
 public:
  virtual ~GraphPartitioner() {}
  virtual void partition_graph(GraphPartition& partition) = 0;
};

class UniformGraphPartitioner : public GraphPartitioner {
 private:
  VertexId num_vertices;

 public:
  ~UniformGraphPartitioner() {}
  UniformGraphPartitioner(VertexId num_vertices_);
  void partition_graph(GraphPartition& partition);
};

template <typename EdgeData>
struct Graph {
  GraphPartition p;
  size_t edge_data_size = 0;
  size_t edge_unit_size = 0;
  VertexId num_vertices = 0;
  EdgeId num_edges = 0;
  EdgeId* degree = nullptr;
  EdgeId max_degree = 0;
  EdgeId* num_local_edges = nullptr;               // [num_sockets]
  EdgeUnit<EdgeData>** local_edges = nullptr;      // [num_sockets][...], edge id = position
  Bitmap** outgoing_adj_bitmap = nullptr;
  EdgeId** outgoing_adj_index = nullptr;
  AdjUnit<EdgeData>** outgoing_adj_list = nullptr;
  // device copy, created from local_edges[0] on first use by an estimator and freed with the graph
  zg_graph* device = nullptr;
  uint64_t shuffle_seed = 0;
};

class Mapping {
 public:
  virtual ~Mapping() {}
  virtual VertexId get_mapping(VertexId vtx) = 0;
  virtual VertexId get_inv_mapping(VertexId vtx) = 0;
};

class IdenticalMapping : public Mapping {
 public:
  ~IdenticalMapping() {}
  VertexId get_mapping(VertexId vtx);
  VertexId get_inv_mapping(VertexId vtx);
};

// Seeded random relabelling of the vertex ids (Fisher-Yates over Philox draws).
class RandomMapping : public Mapping {
 private:
  VertexId* mapping;
  VertexId* inv_mapping;

 public:
  RandomMapping(unsigned int seed, VertexId num_vertices);
  ~RandomMapping();
  VertexId get_mapping(VertexId vtx);
  VertexId get_inv_mapping(VertexId vtx);
};

template <typename EdgeData>
class GraphDestroyer {
 public:
  virtual ~GraphDestroyer() {}
  virtual void destroy_graph(Graph<EdgeData>& graph) = 0;
};

template <typename EdgeData>
class NumaAwareGraphDestroyer : public GraphDestroyer<EdgeData> {
 public:
  void destroy_graph(Graph<EdgeData>& graph);
};

// Shuffles the local edges with a seeded permutation (edge id = new position; the seed is
// graph.shuffle_seed when non-zero, else fresh) on the device, creates the graph's device copy,
// and builds the host edge-id-ordered adjacency lists of the same order.
template <typename EdgeData>
class CSRConstructor {
 public:
  void construct_bitmap_assisted_csr(EdgeUnit<EdgeData>** local_edges, EdgeId* num_local_edges,
                                     Graph<EdgeData>& graph);
};

template <typename EdgeData>
class GraphLoader {
 public:
  virtual ~GraphLoader() {}
  virtual void load_graph(std::string graph_path, VertexId num_vertices, Graph<EdgeData>& graph) = 0;
  virtual void destroy_graph(Graph<EdgeData>& graph) = 0;
};

// Reads a .biedgelist (binary (src, dst[, data]) uint32 records).
template <typename EdgeData>
class DistGraphLoader : public GraphLoader<EdgeData> {
 private:
  GraphPartitioner* partitioner;
  Mapping* mapping;
  CSRConstructor<EdgeData>* csr_constructor;
  GraphDestroyer<EdgeData>* destroyer;

 public:
  DistGraphLoader(GraphPartitioner* partitioner_, Mapping* mapping_, CSRConstructor<EdgeData>* csr_constructor_,
                  GraphDestroyer<EdgeData>* destroyer_);
  ~DistGraphLoader() {}
  void load_graph(std::string graph_path, VertexId num_vertices, Graph<EdgeData>& graph);
  void destroy_graph(Graph<EdgeData>& graph);
};

// Keeps edge e iff its draw in [1, 2^30] is <= sample_rate * 2^30, then reshuffles and rebuilds
// (the error profile's subsample), on the device.
template <typename EdgeData>
class GraphSampler {
 private:
  CSRConstructor<EdgeData>* csr_constructor;
  GraphDestroyer<EdgeData>* destroyer;
  double sample_rate;
  uint64_t keep_seed_, shuffle_seed_;  // 0: fresh per call

 public:
  GraphSampler(CSRConstructor<EdgeData>* csr_constructor_, GraphDestroyer<EdgeData>* destroyer_,
               double sample_rate_ = 0.05);
  // Fixes the Philox keys of the keep draws and of the shuffle (addition of the GPU build).
  void set_seeds(uint64_t keep_seed, uint64_t shuffle_seed);
  void sample_graph(const Graph<EdgeData>& input_graph, Graph<EdgeData>& output_graph);
  void destroy_graph(Graph<EdgeData>& graph);
};

// The device copy of a graph (uploads local_edges[0] in its current order on first call when the
// graph was not built by CSRConstructor).
template <typename EdgeData>
zg_graph* zgh_device_graph(Graph<EdgeData>& graph);

#endif
