// zgh_apps.hpp — estimator applications written against the ZGraph class interface, the way an
// application of the library writes them (estimate() bodies built from the ASAP primitives).
// Used by the C++ tests of the host layer: each one must be identified as its device program and
// reproduce the device's per-sample outcomes bit for bit.
#ifndef ZGH_APPS_HPP
#define ZGH_APPS_HPP

#include <assert.h>

#include "ErrorLatencyProfile.hpp"
#include "SamplerGenerator.hpp"
#include "ZGraphInstance.hpp"

// The edge closing the wedge a-b (they share exactly one endpoint).
template <typename E>
Edge<E> wedge_closer(const Edge<E>& a, const Edge<E>& b) {
  Edge<E> c;
  c.edge_id = 0;
  if (a.src == b.src) {
    c.src = a.dst;
    c.dst = b.dst;
  } else if (a.src == b.dst) {
    c.src = a.dst;
    c.dst = b.src;
  } else if (a.dst == b.src) {
    c.src = a.src;
    c.dst = b.dst;
  } else {
    assert(a.dst == b.dst);
    c.src = a.src;
    c.dst = b.src;
  }
  return c;
}

// Every vertex pair of the sample as an edge list.
template <typename E>
SubGraph<E> all_pairs(const MyList<VertexId>& vs) {
  SubGraph<E> out;
  for (int i = 0; i < vs.list_size; ++i)
    for (int j = i + 1; j < vs.list_size; ++j) {
      Edge<E> e;
      e.edge_id = 0;
      e.src = vs.list[i];
      e.dst = vs.list[j];
      out.add_edge(e);
    }
  return out;
}

template <typename E>
class TriangleApp : public ZGraphInstance<E> {
 public:
  explicit TriangleApp(Graph<E>* g) : ZGraphInstance<E>(g) {}
  double estimate() {
    SubGraph<E> s;
    double p = 1;
    auto a = this->sample_edge();
    if (a.second < 0) return 0;
    p *= a.second;
    s.add_edge(a.first);
    auto b = this->conditional_sample_edge(s);
    if (b.second < 0) return 0;
    p *= b.second;
    s.add_edge(b.first);
    SubGraph<E> closing;
    closing.add_edge(wedge_closer(a.first, b.first));
    return this->conditional_close(s, closing) ? 1. / p : 0;
  }
};

template <typename E>
class PredicateTriangleApp : public AllPredicateZGraphInstance<E> {
 public:
  PredicateTriangleApp(Graph<E>* g, std::function<bool(E)> pred) : AllPredicateZGraphInstance<E>(g, pred) {}
  double estimate() {
    SubGraph<E> s;
    double p = 1;
    auto a = this->sample_edge();
    if (a.second < 0) return 0;
    p *= a.second;
    s.add_edge(a.first);
    auto b = this->conditional_sample_edge(s);
    if (b.second < 0) return 0;
    p *= b.second;
    s.add_edge(b.first);
    SubGraph<E> closing;
    closing.add_edge(wedge_closer(a.first, b.first));
    return this->conditional_close(s, closing) ? 1. / p : 0;
  }
};

template <typename E>
class FourCliqueApp : public ZGraphInstance<E> {
 public:
  explicit FourCliqueApp(Graph<E>* g) : ZGraphInstance<E>(g) {}
  double estimate() {
    SubGraph<E> s;
    double p = 1;
    auto a = this->sample_edge();
    if (a.second < 0) return 0;
    p *= a.second;
    s.add_edge(a.first);
    for (int k = 0; k < 2; ++k) {
      auto b = this->conditional_sample_edge(s);
      if (b.second < 0) return 0;
      p *= b.second;
      s.add_edge(b.first);
    }
    if (s.get_vertices().list_size == 3) return 0;
    SubGraph<E> rest = all_pairs<E>(s.get_vertices()) - s;
    return this->conditional_close(s, rest) ? 1. / p : 0;
  }
};

template <typename E>
class ThreeChainApp : public ZGraphInstance<E> {
 public:
  explicit ThreeChainApp(Graph<E>* g) : ZGraphInstance<E>(g) {}
  double estimate() {
    SubGraph<E> s;
    double p = 1;
    auto a = this->sample_edge();
    if (a.second < 0) return 0;
    p *= a.second;
    s.add_edge(a.first);
    auto b = this->conditional_sample_edge(s);
    if (b.second < 0) return 0;
    p *= b.second;
    return 1. / p;
  }
};

// Three-edge paths, one of three sampling orders chosen uniformly: the middle edge first, an end
// edge first with the path grown from its far end, or an end edge first grown from the other.
template <typename E>
class FourChainApp : public ZGraphInstance<E> {
  static VertexId far_end(const Edge<E>& first, const Edge<E>& second) {
    if (first.src == second.src || first.dst == second.src) return second.dst;
    return second.src;
  }
  static bool touches(const Edge<E>& e, const Edge<E>& f) {
    return e.src == f.src || e.src == f.dst || e.dst == f.src || e.dst == f.dst;
  }

 public:
  explicit FourChainApp(Graph<E>* g) : ZGraphInstance<E>(g) {}
  double estimate() {
    int order = (int)this->sample_interger(1, 3);
    double p = 1. / 3;
    MyList<Edge<E>> es;
    MyList<VertexId> vs;
    auto a = this->sample_edge();
    if (a.second < 0) return 0;
    p *= a.second;
    es.push_back(a.first);
    if (order == 3) {
      vs.push_back(a.first.src);
      auto b = this->conditional_sample_edge(es, vs);
      if (b.second < 0) return 0;
      p *= b.second;
      vs.list[0] = a.first.dst;
      auto c = this->conditional_sample_edge(es, vs);
      if (c.second < 0) return 0;
      p *= c.second;
      if (touches(c.first, b.first)) return 0;
      return 1. / p;
    }
    vs.push_back(a.first.src);
    vs.push_back(a.first.dst);
    auto b = this->conditional_sample_edge(es, vs);
    if (b.second < 0) return 0;
    p *= b.second;
    if (order == 1) es.push_back(b.first);
    vs.list_size = 1;
    vs.list[0] = far_end(a.first, b.first);
    auto c = this->conditional_sample_edge(es, vs);
    if (c.second < 0) return 0;
    p *= c.second;
    if (touches(c.first, a.first)) return 0;
    if (order == 2 && c.first.edge_id >= b.first.edge_id) return 0;
    return 1. / p;
  }
};

// Paths of k vertices grown from both ends of the first edge, canonical in edge-id order.
template <typename E>
class ChainApp : public ZGraphInstance<E> {
  int k;
  static bool canonical(const MyList<Edge<E>>& es, const Edge<E>& e) {
    if (es.list_size <= 1) return true;
    bool seen = false;
    for (int i = 0; i < es.list_size; ++i) {
      const Edge<E>& x = es.list[i];
      if (!seen)
        seen = e.src == x.src || e.src == x.dst || e.dst == x.src || e.dst == x.dst;
      else if (x.edge_id >= e.edge_id)
        return false;
    }
    return true;
  }

 public:
  ChainApp(Graph<E>* g, int k_) : ZGraphInstance<E>(g), k(k_) {}
  double estimate() {
    MyList<Edge<E>> es, first;
    MyList<VertexId> ends;
    SubGraph<E> s;
    long double p = 1.;
    auto a = this->sample_edge();
    if (a.second < 0) return 0;
    p *= a.second;
    es.push_back(a.first);
    first.push_back(a.first);
    s.add_edge(a.first);
    ends.push_back(a.first.src);
    ends.push_back(a.first.dst);
    for (int i = 0; i < k - 2; ++i) {
      auto b = this->conditional_sample_edge(first, ends);
      if (b.second < 0) return 0;
      p *= b.second;
      if (!canonical(es, b.first)) return 0;
      es.push_back(b.first);
      s.add_edge(b.first);
      if (s.get_vertices().list_size != i + 3) return 0;
      for (int j = 0; j < 2; ++j) {
        if (ends.list[j] == b.first.src) {
          ends.list[j] = b.first.dst;
          break;
        }
        if (ends.list[j] == b.first.dst) {
          ends.list[j] = b.first.src;
          break;
        }
      }
    }
    return 1. / p;
  }
};

// The 3-motif pair sharing wedges through the cache.
template <typename E>
class CachedChainApp : public ZGraphInstanceWithCache<E> {
 public:
  explicit CachedChainApp(Graph<E>* g) : ZGraphInstanceWithCache<E>(g) {}
  double estimate() {
    SubGraph<E>* s;
    double* p;
    bool cached;
    this->get_subgraph(cached, s, p);
    *p = 1;
    auto a = this->sample_edge();
    if (a.second < 0) {
      *p = -1;
      return 0;
    }
    *p *= a.second;
    s->add_edge(a.first);
    auto b = this->conditional_sample_edge(*s);
    if (b.second < 0) {
      *p = -1;
      return 0;
    }
    *p *= b.second;
    s->add_edge(b.first);
    return 1. / *p;
  }
};

template <typename E>
class CachedTriangleApp : public ZGraphInstanceWithCache<E> {
 public:
  explicit CachedTriangleApp(Graph<E>* g) : ZGraphInstanceWithCache<E>(g) {}
  double estimate() {
    SubGraph<E>* s;
    double* p;
    bool cached;
    this->get_subgraph(cached, s, p);
    if (cached) {
      if (*p < 0) return 0;
      const MyList<Edge<E>>& es = s->get_edges();
      SubGraph<E> closing;
      closing.add_edge(wedge_closer(es.list[0], es.list[1]));
      return this->conditional_close(*s, closing) ? 1. / *p : 0;
    }
    *p = 1;
    auto a = this->sample_edge();
    if (a.second < 0) return 0;
    *p *= a.second;
    s->add_edge(a.first);
    auto b = this->conditional_sample_edge(*s);
    if (b.second < 0) return 0;
    *p *= b.second;
    s->add_edge(b.first);
    SubGraph<E> closing;
    closing.add_edge(wedge_closer(a.first, b.first));
    return this->conditional_close(*s, closing) ? 1. / *p : 0;
  }
};

// An estimator no device program reproduces (it samples vertices): calculate() must refuse it.
template <typename E>
class VertexPairApp : public ZGraphInstance<E> {
 public:
  explicit VertexPairApp(Graph<E>* g) : ZGraphInstance<E>(g) {}
  double estimate() {
    auto v = this->sample_vertex();
    if (v.second < 0) return 0;
    return 1. / v.second;
  }
};

inline Pattern* make_pattern(VertexId nv, const std::vector<std::pair<VertexId, VertexId>>& edges) {
  std::vector<Edge<Empty>> es(edges.size());
  for (size_t i = 0; i < edges.size(); ++i) {
    es[i].edge_id = i;
    es[i].src = edges[i].first;
    es[i].dst = edges[i].second;
  }
  return new Pattern(nv, (EdgeId)edges.size(), es.data());
}

inline Pattern* star_pattern() { return make_pattern(5, {{0, 1}, {0, 2}, {0, 3}, {0, 4}}); }
inline Pattern* house_pattern() { return make_pattern(5, {{0, 1}, {0, 2}, {1, 2}, {1, 3}, {2, 4}, {3, 4}}); }
inline Pattern* triangle_pattern() { return make_pattern(3, {{0, 1}, {0, 2}, {1, 2}}); }

#endif
