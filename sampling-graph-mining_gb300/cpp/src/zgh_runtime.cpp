// zgh_runtime.cpp — the non-template parts of the host layer: process set-up singletons
// (NetworkInterface, SharedMemSys, Debug, Timer), Bitmap, Random, the regression, file helpers,
// partitioning, vertex mappings, Estimation and Pattern.
//
// Reference behaviour followed: src/NetworkInterface.cpp, src/SharedMemSys.cpp, src/Debug.cpp,
// src/Time.cpp, src/Bitmap.cpp, src/Random.cpp, src/Regression.cpp:17-28, src/Utilities.cpp,
// src/Graph.cpp:17-170 (partition, mappings), src/ZGraphInstance.cpp:15-35 (Estimation),
// src/SamplerGenerator.cpp:11-285 (Pattern).
#include <assert.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/time.h>
#include <unistd.h>
#include <time.h>

#include <atomic>
#include <fstream>
#include <mutex>

#include "../include/Bitmap.hpp"
#include "../include/Debug.hpp"
#include "../include/Graph.hpp"
#include "../include/NetworkInterface.hpp"
#include "../include/Random.hpp"
#include "../include/Regression.hpp"
#include "../include/SamplerGenerator.hpp"
#include "../include/SharedMemSys.hpp"
#include "../include/Time.hpp"
#include "../include/Utilities.hpp"
#include "../include/ZGraphInstance.hpp"
#include "zgh_internal.hpp"

// ---- helpers -------------------------------------------------------------------------------
namespace zgh {

void check(int rc, const char* what) {
  if (rc == ZG_OK) return;
  throw std::runtime_error(std::string(what) + ": " + zg_last_error() + " (status " + std::to_string(rc) + ")");
}

void ensure_init() {
  static std::once_flag once;
  static int rc = ZG_OK;
  std::call_once(once, [] {
    const char* d = getenv("ZGRAPH_DEVICE");
    rc = zg_init(d ? atoi(d) : 0);
  });
  check(rc, "zg_init");
}

uint64_t philox64(uint64_t counter, uint32_t c2, uint32_t c3, uint64_t key) {
  uint32_t c0 = (uint32_t)counter, c1 = (uint32_t)(counter >> 32);
  uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    c0 = n0;
    c1 = (uint32_t)p1;
    c2 = n2;
    c3 = (uint32_t)p0;
  }
  return ((uint64_t)c1 << 32) | c0;
}

uint64_t next_seed() {
  static std::atomic<uint64_t> calls{0};
  static uint64_t base = []() -> uint64_t {
    const char* s = getenv("ZGRAPH_SEED");
    if (s) return (uint64_t)strtoull(s, nullptr, 0);  // deterministic runs
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    return (uint64_t)tv.tv_sec * 1000003ull ^ (uint64_t)tv.tv_usec ^ ((uint64_t)getpid() << 32);
  }();
  uint64_t k = calls.fetch_add(1);
  return philox64(k, 0x5EED, 0, base);
}

}  // namespace zgh

// ---- NetworkInterface (src/NetworkInterface.cpp): one partition -------------------------------
NetworkInterface* NetworkInterface::instance = nullptr;

NetworkInterface::NetworkInterface(int*, char***) : partition_id(0), partitions(1) {}
NetworkInterface::~NetworkInterface() {}

void NetworkInterface::init_network_interface(int* argc, char*** argv) {
  if (instance == nullptr) instance = new NetworkInterface(argc, argv);
}

NetworkInterface* NetworkInterface::get_instance(int* argc, char*** argv) {
  if (instance == nullptr) instance = new NetworkInterface(argc, argv);
  return instance;
}

void NetworkInterface::finalize_instance() {
  delete instance;
  instance = nullptr;
}

void NetworkInterface::pause() {}
int NetworkInterface::get_partition_id() { return partition_id; }
int NetworkInterface::get_num_partitions() { return partitions; }

// ---- SharedMemSys (src/SharedMemSys.cpp): one socket, one host thread -------------------------
SharedMemSys* SharedMemSys::instance = nullptr;

SharedMemSys::SharedMemSys() : num_threads(1), num_sockets(1), num_threads_per_socket(1) {}

void SharedMemSys::init_shared_mem_sys() {
  if (instance == nullptr) instance = new SharedMemSys();
}

SharedMemSys* SharedMemSys::get_instance() {
  if (instance == nullptr) instance = new SharedMemSys();
  return instance;
}

int SharedMemSys::get_socket_id(int thread_id) { return thread_id / num_threads_per_socket; }
int SharedMemSys::get_socket_offset(int thread_id) { return thread_id % num_threads_per_socket; }
int SharedMemSys::get_num_sockets() { return num_sockets; }
int SharedMemSys::get_num_threads() { return num_threads; }
int SharedMemSys::get_num_threads_per_socket() { return num_threads_per_socket; }
int SharedMemSys::get_current_thread_id() { return 0; }
int SharedMemSys::get_current_socket_id() { return 0; }
int SharedMemSys::get_current_socket_offset() { return 0; }

// ---- Debug / Timer -------------------------------------------------------------------------------
Debug* Debug::instance = nullptr;

Debug* Debug::get_instance() {
  if (instance == nullptr) instance = new Debug();
  return instance;
}

void Debug::enter_function(std::string func_name) { log(">>> entering function ", func_name, "..."); }
void Debug::leave_function(std::string func_name) { log("<<< leaving function ", func_name, "..."); }

std::vector<std::pair<std::string, double>> Timer::timers;

double get_time() {
  struct timeval tv;
  gettimeofday(&tv, nullptr);
  return tv.tv_sec + (tv.tv_usec / 1e6);
}

void Timer::timer_start(std::string timer_name) {
  for (auto& t : timers)
    if (t.first == timer_name) {
      t.second -= get_time();
      return;
    }
  timers.push_back(std::make_pair(timer_name, -get_time()));
}

void Timer::timer_stop(std::string timer_name) {
  for (auto& t : timers)
    if (t.first == timer_name) {
      t.second += get_time();
      return;
    }
  assert(false);
}

void Timer::report_timers() {
  Debug::get_instance()->print("timer_name,\t\ttime(ms)");
  for (auto& t : timers) Debug::get_instance()->print(t.first, ",\t\t", int(t.second * 1000));
}

// ---- Bitmap ------------------------------------------------------------------------------------
Bitmap::Bitmap() : size(0), data(nullptr) {}
Bitmap::Bitmap(size_t size_) : size(size_) { data = new unsigned long[WORD_OFFSET(size) + 1]; }
Bitmap::~Bitmap() { delete[] data; }
void Bitmap::clear() { memset(data, 0, sizeof(unsigned long) * (WORD_OFFSET(size) + 1)); }
void Bitmap::fill() { memset(data, 0xff, sizeof(unsigned long) * (WORD_OFFSET(size) + 1)); }
unsigned long Bitmap::get_bit(size_t i) { return data[WORD_OFFSET(i)] & (1ul << BIT_OFFSET(i)); }
void Bitmap::set_bit(size_t i) { __sync_fetch_and_or(data + WORD_OFFSET(i), 1ul << BIT_OFFSET(i)); }

// ---- Random ------------------------------------------------------------------------------------
Random::Random() : seed_(zgh::next_seed()), counter_(0), replaying_(false), mismatches_(0), consumed_(0) {}

unsigned long long Random::rand_int() {
  if (replaying_) return rand_int(0, ~0ull);
  return zgh::philox64(counter_++, 0x484F5354u, 0, seed_);
}

unsigned long long Random::rand_int(unsigned long long min, unsigned long long max) {
  if (replaying_) {
    if (queue_.empty()) {
      ++mismatches_;
      return min;
    }
    Draw d = queue_.front();
    queue_.pop_front();
    ++consumed_;
    if (d.lo != min || d.hi != max) ++mismatches_;
    return (d.val >= min && d.val <= max) ? d.val : min;
  }
  return zgh::map_range(zgh::philox64(counter_++, 0x484F5354u, 0, seed_), min, max);
}

void Random::replay(const Draw* draws, int n) {
  replaying_ = true;
  queue_.clear();
  for (int i = 0; i < n; ++i) queue_.push_back(draws[i]);
  mismatches_ = 0;
  consumed_ = 0;
}

void Random::stop_replay() {
  replaying_ = false;
  queue_.clear();
}

// ---- UnbiasedLinearRegression (src/Regression.cpp:17-28): y = k x through the origin ---------
UnbiasedLinearRegression::UnbiasedLinearRegression() : is_solved(false), k(0) {}

void UnbiasedLinearRegression::solve(long double* x, long double* y, unsigned int len) {
  long double sxy = 0, sxx = 0;
  for (unsigned int i = 0; i < len; ++i) {
    sxy += x[i] * y[i];
    sxx += x[i] * x[i];
  }
  k = sxy / sxx;
  is_solved = true;
}

long double UnbiasedLinearRegression::get_k() {
  assert(is_solved);
  return k;
}

// ---- Utilities (src/Utilities.cpp) -----------------------------------------------------------
bool file_exists(std::string filename) {
  struct stat st;
  return stat(filename.c_str(), &st) == 0;
}

long file_size(std::string filename) {
  struct stat st;
  if (stat(filename.c_str(), &st) != 0) throw std::runtime_error("cannot stat " + filename);
  return st.st_size;
}

// The second line of the .csv holds the vertex count (first run of digits).
void load_graph_meta_data(std::string meta_path, VertexId& num_vertices) {
  std::ifstream fin(meta_path);
  if (!fin) throw std::runtime_error("cannot open " + meta_path);
  std::string str;
  getline(fin, str);
  getline(fin, str);
  size_t pos = 0;
  while (pos < str.size() && (str[pos] < '0' || str[pos] > '9')) ++pos;
  std::string digits;
  while (pos < str.size() && str[pos] >= '0' && str[pos] <= '9') digits += str[pos++];
  if (digits.empty()) throw std::runtime_error("no vertex count in " + meta_path);
  num_vertices = (VertexId)std::stoul(digits);
}

unsigned int get_globally_consistent_seed() {
  const char* s = getenv("ZGRAPH_SEED");
  if (s) return (unsigned int)strtoul(s, nullptr, 0);
  return (unsigned int)time(nullptr);
}

// ---- GraphPartition / UniformGraphPartitioner: one partition, one socket ----------------------
GraphPartition::GraphPartition()
    : partition_id(0), num_partitions(0), num_sockets(0), owned_num_vertices(0), partition_offset(nullptr),
      local_partition_offset(nullptr), all_local_partition_offset(nullptr) {}

static void free_partition(GraphPartition& p) {
  delete[] p.partition_offset;
  delete[] p.local_partition_offset;
  if (p.all_local_partition_offset) {
    for (int i = 0; i < p.num_partitions; ++i) delete[] p.all_local_partition_offset[i];
    delete[] p.all_local_partition_offset;
  }
  p.partition_offset = nullptr;
  p.local_partition_offset = nullptr;
  p.all_local_partition_offset = nullptr;
}

static void copy_partition(GraphPartition& d, const GraphPartition& o) {
  d.partition_id = o.partition_id;
  d.num_partitions = o.num_partitions;
  d.num_sockets = o.num_sockets;
  d.owned_num_vertices = o.owned_num_vertices;
  if (o.partition_offset) {
    d.partition_offset = new VertexId[o.num_partitions + 1];
    memcpy(d.partition_offset, o.partition_offset, sizeof(VertexId) * (o.num_partitions + 1));
  }
  if (o.local_partition_offset) {
    d.local_partition_offset = new VertexId[o.num_sockets + 1];
    memcpy(d.local_partition_offset, o.local_partition_offset, sizeof(VertexId) * (o.num_sockets + 1));
  }
  if (o.all_local_partition_offset) {
    d.all_local_partition_offset = new VertexId*[o.num_partitions];
    for (int i = 0; i < o.num_partitions; ++i) {
      d.all_local_partition_offset[i] = new VertexId[o.num_sockets + 1];
      memcpy(d.all_local_partition_offset[i], o.all_local_partition_offset[i], sizeof(VertexId) * (o.num_sockets + 1));
    }
  }
}

GraphPartition::~GraphPartition() { free_partition(*this); }
GraphPartition::GraphPartition(const GraphPartition& o)
    : partition_offset(nullptr), local_partition_offset(nullptr), all_local_partition_offset(nullptr) {
  copy_partition(*this, o);
}
GraphPartition& GraphPartition::operator=(const GraphPartition& o) {
  if (this != &o) {
    free_partition(*this);
    copy_partition(*this, o);
  }
  return *this;
}

int GraphPartition::get_partition_id(VertexId v_i) {
  for (int p = 0; p < num_partitions; ++p)
    if (v_i >= partition_offset[p] && v_i < partition_offset[p + 1]) return p;
  return -1;
}

int GraphPartition::get_local_partition_id(VertexId v_i) { return get_local_partition_id(partition_id, v_i); }

int GraphPartition::get_local_partition_id(int p_i, VertexId v_i) {
  for (int s = 0; s < num_sockets; ++s)
    if (v_i >= all_local_partition_offset[p_i][s] && v_i < all_local_partition_offset[p_i][s + 1]) return s;
  return -1;
}

UniformGraphPartitioner::UniformGraphPartitioner(VertexId num_vertices_) : num_vertices(num_vertices_) {}

void UniformGraphPartitioner::partition_graph(GraphPartition& p) {
  free_partition(p);
  p.partition_id = 0;
  p.num_partitions = 1;
  p.num_sockets = 1;
  p.owned_num_vertices = num_vertices;
  p.partition_offset = new VertexId[2]{0, num_vertices};
  p.local_partition_offset = new VertexId[2]{0, num_vertices};
  p.all_local_partition_offset = new VertexId*[1];
  p.all_local_partition_offset[0] = new VertexId[2]{0, num_vertices};
}

// ---- mappings (src/Graph.cpp:115-170) ----------------------------------------------------------
VertexId IdenticalMapping::get_mapping(VertexId vtx) { return vtx; }
VertexId IdenticalMapping::get_inv_mapping(VertexId vtx) { return vtx; }

RandomMapping::RandomMapping(unsigned int seed, VertexId num_vertices) {
  mapping = new VertexId[num_vertices];
  inv_mapping = new VertexId[num_vertices];
  for (VertexId v = 0; v < num_vertices; ++v) mapping[v] = v;
  for (VertexId v = num_vertices ? num_vertices - 1 : 0; v; --v) {
    VertexId pos = (VertexId)zgh::map_range(zgh::philox64(v, 0x4D415050u, 0, seed), 0, v);
    VertexId t = mapping[v];
    mapping[v] = mapping[pos];
    mapping[pos] = t;
  }
  for (VertexId v = 0; v < num_vertices; ++v) inv_mapping[mapping[v]] = v;
}

RandomMapping::~RandomMapping() {
  delete[] mapping;
  delete[] inv_mapping;
}

VertexId RandomMapping::get_mapping(VertexId vtx) { return mapping[vtx]; }
VertexId RandomMapping::get_inv_mapping(VertexId vtx) { return inv_mapping[vtx]; }

// ---- Estimation (src/ZGraphInstance.cpp:15-35) --------------------------------------------------
Estimation::Estimation() { reset(); }

void Estimation::reset() {
  num_finished_estimators = 0;
  current_estimation = 0;
}

void Estimation::update(unsigned long long new_num_estimators, double new_estimation) {
  current_estimation =
      (1. * num_finished_estimators / (num_finished_estimators + new_num_estimators)) * current_estimation +
      (1. * new_num_estimators / (num_finished_estimators + new_num_estimators)) * new_estimation;
  num_finished_estimators += new_num_estimators;
}

unsigned long long Estimation::get_num_finished_estimators() { return num_finished_estimators; }
double Estimation::get_currnet_estimation() { return current_estimation; }

// ---- Pattern (src/SamplerGenerator.cpp:11-285) ---------------------------------------------------
void Pattern::construct_csr() {
  for (VertexId v = 0; v <= num_vertices; ++v) csr_idx[v] = 0;
  for (EdgeId e = 0; e < num_edges; ++e) {
    csr_idx[edges[e].src + 1]++;
    csr_idx[edges[e].dst + 1]++;
  }
  for (VertexId v = 1; v <= num_vertices; ++v) csr_idx[v] += csr_idx[v - 1];
  std::vector<EdgeId> pos(csr_idx, csr_idx + num_vertices + 1);
  for (EdgeId e = 0; e < num_edges; ++e) {
    VertexId s = edges[e].src, d = edges[e].dst;
    EdgeId a = pos[s]++;
    csr_list[a].src = s;
    csr_list[a].dst = d;
    csr_list[a].edge_id = edges[e].edge_id;
    EdgeId b = pos[d]++;
    csr_list[b].src = d;
    csr_list[b].dst = s;
    csr_list[b].edge_id = edges[e].edge_id;
  }
}

Pattern::Pattern(VertexId num_vertices_, EdgeId num_edges_, Edge<Empty>* edges_)
    : num_vertices(num_vertices_), num_edges(num_edges_) {
  csr_idx = new EdgeId[num_vertices + 1];
  csr_list = new Edge<Empty>[num_edges * 2];
  edges = new Edge<Empty>[num_edges];
  memcpy((void*)edges, (const void*)edges_, sizeof(Edge<Empty>) * num_edges);
  construct_csr();
}

Pattern::~Pattern() {
  delete[] csr_idx;
  delete[] csr_list;
  delete[] edges;
}

EdgeId Pattern::get_idx_by_edge_id(EdgeId edge_id) const {
  for (EdgeId e = 0; e < num_edges; ++e)
    if (edges[e].edge_id == edge_id) return e;
  assert(false);
  return num_edges;
}

bool Pattern::is_vertex_mapping_correct(VertexId* vertex_mapping, const Pattern& pattern) {
  if (num_edges != pattern.num_edges || num_vertices != pattern.num_vertices) return false;
  for (EdgeId e = 0; e < num_edges; ++e) {
    const Edge<Empty>& q = pattern.edges[pattern.get_idx_by_edge_id(edges[e].edge_id)];
    VertexId a = vertex_mapping[edges[e].src], b = vertex_mapping[edges[e].dst];
    if (!((a == q.src && b == q.dst) || (a == q.dst && b == q.src))) return false;
  }
  return true;
}

// Breadth-first extension of the mapping fixed by edge id 0, following edge ids.
bool Pattern::core_has_same_edge_ordering(VertexId src, VertexId dst, const Pattern& pattern) {
  std::vector<VertexId> map(num_vertices), queue;
  std::vector<char> matched(num_vertices, 0), matched_p(num_vertices, 0);
  const Edge<Empty>& first = pattern.edges[pattern.get_idx_by_edge_id(0)];
  map[src] = first.src;
  map[dst] = first.dst;
  matched[src] = matched[dst] = 1;
  matched_p[first.src] = matched_p[first.dst] = 1;
  queue.push_back(src);
  queue.push_back(dst);
  bool ok = true;
  for (size_t h = 0; ok && h < queue.size(); ++h) {
    VertexId v = queue[h];
    for (EdgeId e = csr_idx[v]; e < csr_idx[v + 1]; ++e) {
      VertexId u = csr_list[e].dst;
      if (matched[u]) continue;
      const Edge<Empty>& q = pattern.edges[pattern.get_idx_by_edge_id(csr_list[e].edge_id)];
      VertexId other;
      if (q.src == map[v])
        other = q.dst;
      else if (q.dst == map[v])
        other = q.src;
      else {
        ok = false;
        break;
      }
      if (matched_p[other]) {
        ok = false;
        break;
      }
      map[u] = other;
      matched[u] = 1;
      matched_p[other] = 1;
      queue.push_back(u);
    }
  }
  for (VertexId v = 0; ok && v < num_vertices; ++v)
    if (!matched[v] || !matched_p[v]) ok = false;
  if (ok && !is_vertex_mapping_correct(map.data(), pattern)) ok = false;
  return ok;
}

EdgeId* Pattern::get_csr_idx() { return csr_idx; }
Edge<Empty>* Pattern::get_csr_list() { return csr_list; }
Edge<Empty>* Pattern::get_edges() { return edges; }
VertexId Pattern::get_num_vertices() { return num_vertices; }
EdgeId Pattern::get_num_edges() { return num_edges; }

bool Pattern::has_same_edge_ordering(const Pattern& pattern) {
  if (num_vertices != pattern.num_vertices || num_edges != pattern.num_edges) return false;
  const Edge<Empty>& e0 = edges[get_idx_by_edge_id(0)];
  return core_has_same_edge_ordering(e0.src, e0.dst, pattern) || core_has_same_edge_ordering(e0.dst, e0.src, pattern);
}

void Pattern::setup_edge_id_mapping(EdgeId* mapping) {
  for (EdgeId e = 0; e < num_edges; ++e) edges[e].edge_id = mapping[edges[e].edge_id];
  for (EdgeId e = 0; e < num_edges * 2; ++e) csr_list[e].edge_id = mapping[csr_list[e].edge_id];
}

bool Pattern::is_in_edges_list(Edge<Empty> edge) {
  for (EdgeId e = 0; e < num_edges; ++e)
    if ((edges[e].src == edge.src && edges[e].dst == edge.dst) || (edges[e].src == edge.dst && edges[e].dst == edge.src))
      return true;
  return false;
}

bool Pattern::is_automorphic(VertexId num_vertices_, EdgeId num_edges_, const Edge<Empty>* edges_) {
  if (num_vertices_ != num_vertices || num_edges_ != num_edges) return false;
  for (EdgeId e = 0; e < num_edges; ++e)
    if (!is_in_edges_list(edges_[e])) return false;
  return true;
}

bool Pattern::is_automorphic(const Pattern& pattern) { return is_automorphic(pattern.num_vertices, pattern.num_edges, pattern.edges); }

void Pattern::setup_vertex_id_mapping(VertexId* mapping) {
  for (EdgeId e = 0; e < num_edges; ++e) {
    edges[e].src = mapping[edges[e].src];
    edges[e].dst = mapping[edges[e].dst];
  }
  construct_csr();
}
