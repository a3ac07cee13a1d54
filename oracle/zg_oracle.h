/*
 * zg_oracle.h — CPU ORACLE (test infrastructure only).
 *
 * A plain-C restatement of jy-yuan/sampling-graph-mining's neighbour-sampling estimator
 * path, used to check libzgraph_gpu.so.  Only tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline / --impl reference legs may load it, and only to check results or
 * as the timed CPU baseline; the product path never calls it.
 *
 * Parity is pinned: tests/golden/ holds per-sample outcomes produced by the reference's own
 * sources (compiled by oracle/build_ref.sh against a replaying Random), and this restatement
 * must reproduce them bit for bit (tests/test_oracle_golden.py).
 *
 * Every function cites the reference file:line it restates.
 */
#ifndef ZG_ORACLE_H
#define ZG_ORACLE_H

#include <stdint.h>
#include "../include/zgraph_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Graph<E> restated for one partition and one socket (include/Graph.hpp:148-166):
 * local_edges in edge-id order, outgoing_adj_index (off) and outgoing_adj_list
 * (adj_nbr = AdjUnit.dst, adj_eid = AdjUnit.edge_id, adj_w = AdjUnit.edge_data),
 * each list sorted by edge id (src/Graph.cpp:287-334). */
typedef struct zgo_graph {
  uint32_t nv;
  uint64_t m;            /* num_local_edges[0] */
  uint64_t num_edges;    /* Graph::num_edges (metadata, rescaled by filters)  */
  uint64_t max_degree;   /* Graph::max_degree (metadata)                      */
  uint32_t* src;
  uint32_t* dst;
  uint32_t* w;           /* NULL for Graph<Empty> */
  uint64_t* off;         /* nv + 1 */
  uint32_t* adj_nbr;     /* 2m */
  uint64_t* adj_eid;     /* 2m */
  uint32_t* adj_w;       /* 2m or NULL */
} zgo_graph;

typedef struct zgo_program {
  int kind;
  uint32_t param;
  /* SamplerGenerator state (src/SamplerGenerator.cpp:393-445) */
  uint32_t pv, pe;
  uint32_t pedges[2 * ZG_MAX_LIST];
  uint32_t num_unique;
  uint32_t* unique_edges; /* num_unique * pe * 2 (src,dst) after relabelling */
} zgo_program;

int  zgo_graph_build(zgo_graph* g, uint32_t nv, uint64_t m, const uint32_t* edges,
                     const uint32_t* weights);
void zgo_graph_free(zgo_graph* g);

int  zgo_program_init(zgo_program* p, int kind, uint32_t param, uint32_t pv, uint32_t pe,
                      const uint32_t* pedges);
void zgo_program_free(zgo_program* p);

/* Philox4x32-10 (Salmon et al., SC'11) and the draw mapping shared with the GPU. */
void     zgo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
uint64_t zgo_draw(uint64_t seed, uint32_t stream, uint64_t sample, uint32_t d,
                  uint64_t lo, uint64_t hi);
uint64_t zgo_sample_draw(uint64_t seed, uint32_t stream, uint64_t sample, uint32_t d,
                         uint64_t lo, uint64_t hi);

/* One estimate() call for sample index `sample`; fills *tr (never NULL). Returns 0. */
int zgo_sample(const zgo_graph* g, const zgo_program* p, uint64_t seed, uint32_t stream,
               uint64_t sample, zg_sample_trace* tr);

/* n estimators [first, first+n) with `threads` OpenMP threads (<=0: all).  traces may be NULL.
 * Exact sums are filled as in zg_counters; sum_w/sum_w2 are summed in sample order per
 * thread and are not bit-comparable with the GPU's. */
int zgo_run(const zgo_graph* g, const zgo_program* p, uint64_t n, uint64_t first,
            uint64_t seed, uint32_t stream, int threads, zg_counters* out,
            zg_sample_trace* traces);

/* ThreeMotif with the sub-pattern cache (applications/ThreeMotif.cpp:48-121). */
int zgo_run_three_motif(const zgo_graph* g, uint64_t n_chain, uint64_t n_tri, uint64_t seed,
                        uint32_t stream_chain, uint32_t stream_tri, zg_counters* out_chain,
                        zg_counters* out_tri, zg_sample_trace* chain_tr,
                        zg_sample_trace* tri_tr);

/* Deterministic edge selections used by the filtered / subsampled graphs.
 * zgo_filter_keep: GraphFilter predicate (src/GraphFilters.cpp:48-53).
 * zgo_subsample_keep: GraphSampler draw rand_int(1, 2^30) <= rate*2^30 (src/Graph.cpp:651-668). */
int zgo_pred(int op, int64_t t0, int64_t t1, uint32_t w);
int zgo_subsample_keep(double rate, uint64_t keep_seed, uint64_t e);
/* The permutation applied by a shuffle seed: perm[i] = input position of output edge i. */
void zgo_shuffle_perm(uint64_t m, uint64_t shuffle_seed, uint64_t* perm);
/* The sort key of input position i under a shuffle seed: output edges are the inputs in ascending
 * (key, i) order. */
uint64_t zgo_shuffle_key(uint64_t shuffle_seed, uint64_t i);
/* The subsample GraphSampler::sample_graph keeps (src/Graph.cpp:629-780), with the device's draw
 * plan (zg_graph_subsample): edge e of the m (src, dst) pairs is kept when
 * zgo_subsample_keep(rate, keep_seed, e), and the kept edges are permuted as
 * zgo_shuffle_perm(k, shuffle_seed) orders them.  out: room for `capacity` pairs; *k_out: pairs
 * kept.  Parallel (OpenMP) and m < 2^32: the ELP subsample of the largest benchmark graph. */
int zgo_subsample_edges(const uint32_t* edges, uint64_t m, double rate, uint64_t keep_seed, uint64_t shuffle_seed,
                        uint64_t capacity, uint32_t* out, uint64_t* k_out);

/* conditional_close with the found edge ids written back (src/ZGraphInstance.cpp:410-441).
 * Returns 1 when every edge was found; *found = edges found before the first miss. */
int zgo_conditional_close_ids(const zgo_graph* g, uint64_t min_valid, const uint32_t* vertices, uint32_t nv,
                              const uint32_t* edges, uint32_t ne, uint64_t* edge_ids, uint32_t* found);

/* Exact counts, restating naive_implementation/<Counter>.cpp (out: 128-bit). */
int zgo_exact_naive(const zgo_graph* g, int kind, uint64_t out[2]);
/* Faster CPU restatements of the same counts (checked against the naive ones). */
int zgo_exact_fast(const zgo_graph* g, int kind, uint64_t out[2]);
/* naive_implementation/WeightedTriangleCounting.cpp and AtLeastOneWeightedTriangleCounting.cpp */
int zgo_exact_weighted_triangle(const zgo_graph* g, uint32_t threshold, int at_least_one,
                                uint64_t out[2]);

/* ErrorProfile::calculate_bound (src/ErrorLatencyProfile.cpp:52-59). */
double zgo_calculate_bound(double epsilon, double delta, double nse, double ncse,
                           double estimation, uint64_t max_degree, uint64_t num_edges);
/* UnbiasedLinearRegression::solve (src/Regression.cpp:17-28), long double as the reference. */
double zgo_regression_k(const double* x, const double* y, uint32_t len);

/* Seeded R-MAT edge list on the host (oracle/zgo_gen.c), edge for edge the library's
 * zg_gen_rmat output: the CPU arm's input.  edges == NULL only reports *m_out. */
int zgo_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                 uint64_t capacity, uint32_t* edges, uint64_t* m_out);

/* x87 80-bit extended arithmetic restated in integers (used by ChainMining's long double p). */
double zgo_ext_inv_product(const double* factors, int n);

#ifdef __cplusplus
}
#endif
#endif
