/*
 * zgraph_gpu.h — C ABI of libzgraph_gpu.so, the GB300 (sm_103a) implementation of
 * ZGraph's ASAP neighbour-sampling estimator hot path.
 *
 * Every entry point returns an int status (ZG_OK == 0); none aborts, throws or
 * falls back to the CPU.  Pointers are plain host pointers unless a parameter is
 * named `cuda_stream` (a cudaStream_t passed as void*, NULL = legacy stream).
 *
 * Reference interfaces replaced (paths inside jy-yuan/sampling-graph-mining):
 *   Graph<E> + CSRConstructor       include/Graph.hpp:148-166, src/Graph.cpp:215-377
 *   GraphFilter (AllPredicate)      include/GraphFilters.hpp:9-18, src/GraphFilters.cpp:17-177
 *   GraphSampler (ELP subsample)    include/Graph.hpp:234-244, src/Graph.cpp:629-780
 *   ZGraphInstance::calculate       include/ZGraphInstance.hpp:125, src/ZGraphInstance.cpp:257-297
 *   estimate() bodies               applications/<App>.cpp, src/SamplerGenerator.cpp:461-546
 *   ZGraphInstanceWithCache         include/ZGraphInstance.hpp:196-214, src/ZGraphInstance.cpp:749-833
 *   naive exact counters            naive_implementation/<Counter>.cpp
 */
#ifndef ZGRAPH_GPU_H
#define ZGRAPH_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define ZG_OK                         0
#define ZG_ERR_INVALID_ARG            1
#define ZG_ERR_OOM                    2
#define ZG_ERR_CUDA                   3
#define ZG_ERR_INVALID_GRAPH          4  /* self-loop, duplicate edge, id out of range */
#define ZG_ERR_UNSUPPORTED_ESTIMATOR  5
#define ZG_ERR_TIMEOUT                6  /* a bounded device wait gave up */
#define ZG_ERR_BOUND_NOT_MET          7
#define ZG_ERR_NO_DEVICE              8
#define ZG_ERR_OVERFLOW               9  /* an exact weight left the 192-bit range */
#define ZG_ERR_TOO_LARGE             10  /* a size beyond a documented maximum */

/* ---- estimator programs: the applications' estimate() bodies ------------- */
#define ZG_PROG_TRIANGLE      1  /* applications/Triangle.cpp:48-73 (also the predicate apps) */
#define ZG_PROG_FOUR_CLIQUE   2  /* applications/FourClique.cpp:199-234                         */
#define ZG_PROG_THREE_CHAIN   3  /* applications/ThreeChain.cpp:315-330                         */
#define ZG_PROG_FOUR_CHAIN    4  /* applications/FourChain.cpp:24-124                           */
#define ZG_PROG_CHAIN         5  /* applications/ChainMining.cpp:240-84 (param = order k)       */
#define ZG_PROG_PATTERN       6  /* SamplerGenerator<Empty>::estimate, src/SamplerGenerator.cpp */
/* No counterpart in the reference: FourClique's draws, but a sample counts only if it followed the
 * clique's canonical path (e0 the smallest of the six edge ids; e1 the smallest edge joining e0's
 * endpoints to the other two vertices; e2 the smallest edge id above e1 at the fourth vertex), so
 * every 4-clique is counted exactly once: unbiased, where the reference's estimator counts only
 * cliques whose three smallest edges grow connectedly (60 % of them for random edge ids). */
#define ZG_PROG_FOUR_CLIQUE_UNBIASED 7

/* ---- exact counters: naive_implementation/<Counter>.cpp --------------------------- */
#define ZG_EXACT_TRIANGLE     1  /* TriangleCounting.cpp            */
#define ZG_EXACT_WEDGE        2  /* ThreeChain.cpp  (sum C(d,2))    */
#define ZG_EXACT_THREE_PATH   3  /* FourChain.cpp   (3-edge paths)  */
#define ZG_EXACT_FIVE_STAR    4  /* FiveStar.cpp    (sum C(d,4))    */
#define ZG_EXACT_FOUR_CLIQUE  5  /* FourClique.cpp                  */
#define ZG_EXACT_FIVE_HOUSE   6  /* FiveHouse.cpp   (house subgraphs: a triangle on one side of a 4-cycle) */
#define ZG_EXACT_FIVE_CHAIN   7  /* FiveChain.cpp   (4-edge paths)  */
/* Predicate-weighted triangles, zg_exact_count_weighted (threshold T; the naive programs use 50): */
#define ZG_EXACT_WEIGHTED_TRIANGLE      8  /* WeightedTriangleCounting.cpp: every edge's data >= T */
#define ZG_EXACT_AT_LEAST_ONE_TRIANGLE  9  /* AtLeastOneWeightedTriangleCounting.cpp: some edge >= T */

/* ---- edge predicates for GraphFilter (std::function<bool(VertexId)>) ------ */
#define ZG_PRED_GE            1  /* w >= t0       (AllPredicateWeightedTriangle.cpp:101-103) */
#define ZG_PRED_LT            2  /* w <  t0       (AtLeastOnePredicateWeightedTriangle.cpp:138-140) */
#define ZG_PRED_GT            3
#define ZG_PRED_LE            4
#define ZG_PRED_EQ            5
#define ZG_PRED_NE            6
#define ZG_PRED_RANGE         7  /* t0 <= w < t1  */

#define ZG_NO_SHUFFLE         0xffffffffffffffffull

/* Per-sample draw capacity and list capacity (MAX_LIST_SIZE, include/ZGraphInstance.hpp:16). */
#define ZG_MAX_DRAWS          16
#define ZG_MAX_LIST           16

typedef struct zg_graph zg_graph;     /* device-resident graph (opaque)   */
typedef struct zg_program zg_program; /* estimator program (opaque)       */
typedef struct zg_mlp zg_mlp;         /* learned-profile network (opaque) */

/* Graph metadata.  num_edges / max_degree are the reference's Graph<E>::num_edges and
 * ::max_degree (include/Graph.hpp:155-158), which GraphSampler/GraphFilter rescale; the
 * sampler itself always uses the local edge count (num_local_edges). */
typedef struct zg_graph_meta {
  uint32_t num_vertices;
  uint32_t weighted;
  uint64_t num_local_edges;
  uint64_t num_edges;
  uint64_t max_degree;
  uint64_t device_bytes;
  uint32_t record_bytes;   /* bytes per edge record: 16 (compact, packed) or 32 (wide)    */
  uint32_t record_layout;  /* ZG_RECORDS_COMPACT, ZG_RECORDS_WIDE or ZG_RECORDS_PACKED       */
} zg_graph_meta;

/* Result of one calculate()-style run.  The exact estimate is
 *   sum_num / 2^den_log2 / samples
 * where sum_num is a 320-bit little-endian integer: every sample's 1/p is
 * numerator / 2^shift with numerator = m * prod(S_i) (* 3 for the four-chain program)
 * and shift = #(conditional steps whose edge appeared twice among the anchors). */
typedef struct zg_counters {
  uint64_t samples;
  uint64_t hits;           /* estimate() returned a non-zero weight                 */
  uint64_t fails;          /* a primitive returned probability < 0 (no valid edge)   */
  uint32_t den_log2;
  uint32_t overflow;       /* non-zero: some numerator exceeded 192 bits            */
  uint64_t sum_num[5];
  double   sum_w;          /* sum of 1/p: the exact sum, rounded once to double     */
  double   sum_w2;         /* sum of (1/p)^2 in double (fixed block order); each 1/p
                              truncated to 53 bits first: the variance term          */
  double   estimate;       /* exact mean, rounded once to double                    */
  double   sum_w4;         /* sum of (1/p)^4 in double (fixed block order): the
                              uncertainty of the variance term                     */
} zg_counters;

/* Per-sample trace written by zg_run_debug: the draws a replayed Random::rand_int(min,max)
 * (src/Random.cpp:11-14) must return, and the outcome the estimator must produce. */
typedef struct zg_sample_trace {
  uint32_t ndraws;
  uint32_t hit;
  uint32_t fail;
  uint32_t shift;
  uint32_t sectors;        /* 32-byte sectors of the access model (algorithmic bytes / 32) */
  uint32_t closures;       /* closure checks of the access model (conditional_close edge
                              look-ups, up to the first missing edge)                   */
  double   w;              /* bit-exact reference value of estimate()               */
  uint64_t num[3];         /* 192-bit exact numerator                               */
  uint64_t lo[ZG_MAX_DRAWS];
  uint64_t hi[ZG_MAX_DRAWS];
  uint64_t val[ZG_MAX_DRAWS];
} zg_sample_trace;

/* ---- library / device --------------------------------------------------- */
/* Returns the ABI version (monotonic). */
int zg_version(void);
/* Selects and checks the device (replaces NetworkInterface/SharedMemSys set-up,
 * src/NetworkInterface.cpp:5-10, src/SharedMemSys.cpp:13-46). */
int zg_init(int device);
/* Human-readable text of the last error on this thread. */
const char* zg_last_error(void);
/* The current device's L2 fetch granularity hint (cudaLimitMaxL2FetchGranularity: 32, 64 or 128
 * bytes fetched from memory per L2 miss; 0 leaves it as it is), for this process's context only.
 * *previous (may be NULL) receives the value before the call.  No counterpart in the reference. */
int zg_set_l2_fetch_granularity(uint32_t bytes, uint32_t* previous);

/* ---- graph store -------------------------------------------------------- */
/* Uploads a COO edge list in edge-id order (edge id == position, src/Graph.cpp:295-306) and
 * builds, on the device, the edge-id-ordered adjacency, the neighbour-sorted adjacency and
 * per-edge ranks.  edges: 2*m uint32 (src,dst) pairs; weights: m uint32 or NULL.
 * Replaces CSRConstructor::construct_bitmap_assisted_csr (src/Graph.cpp:215-377) minus its
 * shuffle (the caller's order is kept; see zg_graph_permuted for a device shuffle). */
int zg_graph_create(const uint32_t* edges, uint64_t m, uint32_t num_vertices,
                    const uint32_t* weights, void* cuda_stream, zg_graph** out);
/* Same as zg_graph_create after a seeded device permutation of the edge order, the
 * rebuild's counterpart of the Fisher-Yates shuffle at src/Graph.cpp:218-231.
 * parent_index (m entries, may be NULL) receives, for every new edge id, its input position. */
int zg_graph_permuted(const uint32_t* edges, uint64_t m, uint32_t num_vertices,
                      const uint32_t* weights, uint64_t shuffle_seed, void* cuda_stream,
                      uint64_t* parent_index, zg_graph** out);
int zg_graph_free(zg_graph* g);
/* Layout of the per-edge records of graphs built after this call (every graph constructor,
 * filters and subsamples included); process-wide, not to be changed while another thread builds.
 * AUTO (the default): packed (else compact) while the graph's sampling working set is within
 * twice the GPU's L2, wide beyond.  COMPACT: (src, dst, suffix sizes), 16 bytes; the steps also
 * read vertex offsets.  WIDE: adds each edge's slot and predecessor count in both endpoint lists,
 * 32 bytes (one sector); a step then needs no offset read.  PACKED: src, dst, both suffix sizes
 * and both slots as bit fields of 16 bytes, where they fit (2 x vertex bits + suffix bits <= 64
 * and suffix bits + 2 x slot bits <= 64; else compact); a step needs no offset read.  Every
 * estimate is identical under each layout.  No counterpart in the reference (its layout is fixed:
 * src/Graph.cpp:215-377). */
#define ZG_RECORDS_AUTO 0
#define ZG_RECORDS_COMPACT 1
#define ZG_RECORDS_WIDE 2
#define ZG_RECORDS_PACKED 3
int zg_set_record_layout(int layout);
int zg_graph_get_meta(const zg_graph* g, zg_graph_meta* out);
int zg_graph_set_meta(zg_graph* g, uint64_t num_edges, uint64_t max_degree);
/* Copies the device arrays back (test/inspection).  Any pointer may be NULL.
 *   edges   : 2*m (src,dst) in edge-id order     weights: m
 *   offsets : V+1 int64                          adj_e  : 2*2m (nbr, edge_id) edge-id order
 *   adj_n   : 2*2m (nbr, edge_id) neighbour order
 *   suffix  : 2*m (entries after the edge in its src list, in its dst list) */
int zg_graph_download(const zg_graph* g, uint32_t* edges, uint32_t* weights, int64_t* offsets,
                      uint32_t* adj_e, uint32_t* adj_n, uint32_t* suffix);
/* GraphFilter::generate_graph (src/GraphFilters.cpp:17-177): keeps the edges whose weight
 * satisfies the predicate, in order, then permutes them with shuffle_seed (ZG_NO_SHUFFLE keeps
 * the order) and rebuilds the adjacency.  num_edges/max_degree follow :90-135.
 * parent_index (may be NULL, capacity m of the input) receives the input edge id of every
 * output edge; *out_m its length. */
int zg_graph_filter(const zg_graph* g, int pred_op, int64_t t0, int64_t t1,
                    uint64_t shuffle_seed, void* cuda_stream, uint64_t* parent_index,
                    uint64_t* out_m, zg_graph** out);
/* GraphSampler::sample_graph (src/Graph.cpp:629-780): keeps edge e iff its draw in
 * [1, 2^30] is <= floor(rate * 2^30), draws from keep_seed; then as zg_graph_filter. */
int zg_graph_subsample(const zg_graph* g, double rate, uint64_t keep_seed,
                       uint64_t shuffle_seed, void* cuda_stream, uint64_t* parent_index,
                       uint64_t* out_m, zg_graph** out);

/* ---- estimator programs -------------------------------------------------- */
/* kind: ZG_PROG_*; param: chain order for ZG_PROG_CHAIN (3..16), else 0. */
int zg_program_create(int kind, uint32_t param, zg_program** out);
/* SamplerGenerator(graph, Pattern) (src/SamplerGenerator.cpp:393-445): pattern with
 * num_vertices (<= 8) vertices and num_edges (<= 15) edges given as (src,dst) pairs. */
int zg_program_create_pattern(uint32_t num_vertices, uint32_t num_edges,
                              const uint32_t* edges, zg_program** out);
int zg_program_free(zg_program* p);
/* num_unique: number of unique relabelled patterns (SamplerGenerator's num_unique_patterns);
 * cond_calls: conditional_sample_edge calls of a successful estimate (the ELP's probe);
 * vertices: num_vertices_in_pattern. */
int zg_program_info(const zg_program* p, uint32_t* num_unique, uint32_t* cond_calls,
                    uint32_t* vertices);

/* ---- sampling ------------------------------------------------------------ */
/* Runs n estimators, sample indices [first_sample, first_sample+n), on Philox stream
 * (seed, stream_id); the device counterpart of ZGraphInstance::calculate
 * (src/ZGraphInstance.cpp:257-297) without the Estimation fold, which the host does. */
int zg_run(const zg_graph* g, const zg_program* p, uint64_t n, uint64_t first_sample,
           uint64_t seed, uint32_t stream_id, void* cuda_stream, zg_counters* out);
/* Asynchronous zg_run: enqueues the sampling and reduction kernels on cuda_stream and returns.
 * The reduced result (ZG_RESULT_BYTES bytes) lands in device memory at d_result; copy it to the
 * host after the stream completes and convert it with zg_result_to_counters.  Stream-ordered,
 * so several runs can be queued back to back. */
#define ZG_RESULT_BYTES 112
int zg_run_async(const zg_graph* g, const zg_program* p, uint64_t n, uint64_t first_sample,
                 uint64_t seed, uint32_t stream_id, void* cuda_stream, void* d_result);
int zg_result_to_counters(const void* h_result, const zg_program* p, zg_counters* out);

/* zg_run_async that allocates nothing, for callers that cannot allocate device memory while they
 * serve queries: a process whose memory manager reserves all device memory up front, or a
 * latency-critical path where cudaMalloc/cudaFree could synchronise the device.  It has no
 * counterpart in the reference.  The per-block scratch is one fixed device array of
 * ZG_NOALLOC_MAX_BLOCKS x ZG_RESULT_BYTES bytes (1.75 MiB) that every GPU loading the library keeps
 * until the process exits; a launch that would need more blocks is rejected with ZG_ERR_TOO_LARGE
 * (the library's sampling grids never do: at most 8 resident blocks per SM, 24 times the resident
 * blocks on wide-record graphs, and never more than ZG_NOALLOC_MAX_BLOCKS).  The array used is the
 * current device's: g must have been built on the current device (a graph on another device is
 * refused with ZG_ERR_INVALID_ARG).  The first call on each device looks up the array's device
 * address (cudaGetSymbolAddress), so make that first call before any stream capture.  All calls share the array: calls whose
 * executions overlap on the GPU race and must be serialised by the caller.  d_result: device
 * memory of ZG_RESULT_BYTES bytes provided by the caller; read it as for zg_run_async. */
#define ZG_NOALLOC_MAX_BLOCKS 16384
int zg_run_noalloc(const zg_graph* g, const zg_program* p, uint64_t n, uint64_t first_sample,
                   uint64_t seed, uint32_t stream_id, void* cuda_stream, void* d_result);
/* Autotuner (no counterpart in the reference, whose thread count comes from libnuma).  Each
 * program kind has ZG_VARIANTS launch shapes: the sampling kernel compiled for
 * min-blocks-per-SM 1, 2, 3, 4, 5, 6, 8 (register caps 255/128/80/64/48/40/32) with a grid of
 * occupancy x SM count (24 times that on wide-record graphs, whose SMs progress at different
 * rates: the block scheduler then balances them; at most ZG_NOALLOC_MAX_BLOCKS); the 4-chain's shapes with at most 3 blocks per SM interleave two samples
 * per thread (more registers, two load chains in flight), the others run one.  zg_tune times every
 * variant on g (probe_samples estimators, best of 3) and keeps the fastest for this device and
 * kind; ms_per_variant (may be NULL) receives ZG_VARIANTS timings.  zg_set_variant /
 * zg_get_variant fix or read the choice (zg_get_variant's grid: the compact- and packed-record one). */
#define ZG_VARIANTS 7
int zg_tune(const zg_graph* g, const zg_program* p, uint64_t probe_samples, void* cuda_stream,
            int* best_variant, float* ms_per_variant);
int zg_set_variant(int kind, int variant);
int zg_get_variant(int kind, int* variant, int* min_blocks, int* grid);
/* As zg_run, one trace per sample (n <= 2^22). */
int zg_run_debug(const zg_graph* g, const zg_program* p, uint64_t n, uint64_t first_sample,
                 uint64_t seed, uint32_t stream_id, zg_sample_trace* traces);
/* ThreeMotif (applications/ThreeMotif.cpp:43-122,149-196): n_chain 3-chain estimators
 * (stream_chain) whose wedges are cached; the first min(n_chain, n_tri) triangle estimators
 * close the cached wedges, the rest sample afresh on stream_tri. */
int zg_run_three_motif(const zg_graph* g, uint64_t n_chain, uint64_t n_tri, uint64_t seed,
                       uint32_t stream_chain, uint32_t stream_tri, void* cuda_stream,
                       zg_counters* out_chain, zg_counters* out_tri);
int zg_run_three_motif_debug(const zg_graph* g, uint64_t n_chain, uint64_t n_tri,
                             uint64_t seed, uint32_t stream_chain, uint32_t stream_tri,
                             zg_sample_trace* chain_traces, zg_sample_trace* tri_traces);

/* ---- the closure primitive on its own ------------------------------------------------- */
/* ZGraphInstance::conditional_close(min_valid_edge_id, sampled_vertices, edges_to_wait&)
 * (src/ZGraphInstance.cpp:410-441, include/ZGraphInstance.hpp:131), one query per thread: for each
 * edge to wait in order, look for it in the lists of the sampled vertices, at an edge id >=
 * min_valid_edge_id; a found edge's id is written back (the reference stores it in
 * edge_to_wait.edge_id), and the first edge not found ends the query with closed = 0.  An edge is
 * found only in the list of a sampled vertex, so an edge none of whose endpoints is sampled is not
 * found, as in the reference.  The estimator programs answer the same question with a cuckoo-table
 * look-up (the edges they wait for always join sampled vertices). */
typedef struct zg_close_query {
  uint64_t min_valid_edge_id;
  uint32_t num_vertices;             /* <= ZG_MAX_LIST */
  uint32_t num_edges;                /* <= ZG_MAX_LIST */
  uint32_t vertices[ZG_MAX_LIST];
  uint32_t edges[2 * ZG_MAX_LIST];   /* (src, dst) of each edge to wait */
} zg_close_query;
typedef struct zg_close_result {
  uint32_t closed;                   /* every edge was found: conditional_close's return value */
  uint32_t found;                    /* edges found before the first miss (their ids are valid) */
  uint64_t edge_ids[ZG_MAX_LIST];
} zg_close_result;
/* queries and results: host arrays of n entries (copied in and out on cuda_stream; synchronous). */
int zg_conditional_close(const zg_graph* g, const zg_close_query* queries, uint32_t n, void* cuda_stream,
                         zg_close_result* results);

/* ---- batched mixed queries ----------------------------------------------------- */
/* Many estimator queries of uneven program, predicate and budget in one persistent launch (no
 * counterpart in the reference, whose applications run one calculate() at a time).  A query runs
 * n estimators of `kind` (ZG_PROG_TRIANGLE .. ZG_PROG_CHAIN with param = chain order, or
 * ZG_PROG_PATTERN with a program from zg_program_create_pattern) with sample indices
 * [first_sample, first_sample + n) on Philox stream (seed, stream_id), on the batch's base graph or, when pred_op
 * != 0, on the base graph filtered by (pred_op, t0, t1) as AllPredicateZGraphInstance does
 * (src/ZGraphInstance.cpp:492-525).  ZG_QUERY_THREE_MOTIF runs ThreeMotif's pair: n 3-chain
 * estimators and the triangle estimators that close their wedges (zg_run_three_motif with
 * n_chain = n_tri = n).  Results equal zg_run's (zg_run_three_motif's) on the same draws, exactly,
 * except sum_w2, which is summed in a different (fixed) order. */
#define ZG_QUERY_THREE_MOTIF   16
#define ZG_BATCH_MAX_QUERIES   65536
#define ZG_BATCH_MAX_CHUNKS    65536   /* work items of 2^k samples, k >= 12 chosen per batch */
typedef struct zg_batch_query {
  int32_t  kind;
  uint32_t param;
  int32_t  pred_op;        /* 0: base graph; else ZG_PRED_* */
  uint32_t stream_id;
  int64_t  t0, t1;
  uint64_t n;
  uint64_t seed;
  uint64_t first_sample;   /* sample indices [first_sample, first_sample + n) */
  const zg_program* program; /* ZG_PROG_PATTERN: the pattern program (must outlive zg_batch_wait) */
} zg_batch_query;
typedef struct zg_batch zg_batch;
/* A batch engine over base (which must outlive it): capacity max_queries per submit; filtered
 * graphs are cached up to cache_bytes of device memory (least recently used first out), each
 * shuffled with a seed derived from filter_seed and its predicate.  A filtered graph whose build
 * runs out of device memory first frees cached graphs the submit does not use, least recently
 * used first, and is built again. */
int zg_batch_create(const zg_graph* base, uint32_t max_queries, uint64_t cache_bytes, uint64_t filter_seed,
                    zg_batch** out);
int zg_batch_free(zg_batch* b);
/* Enqueues the batch on cuda_stream (one CUDA graph launch after any filtered graphs it needs
 * are built) and returns; a second submit first waits for the previous batch. */
int zg_batch_submit(zg_batch* b, const zg_batch_query* queries, uint32_t nq, void* cuda_stream);
/* Waits for the submitted batch; out[2i] receives query i's counters (ZG_QUERY_THREE_MOTIF:
 * out[2i] the 3-chain, out[2i+1] the triangle). */
int zg_batch_wait(zg_batch* b, zg_counters* out);
/* Learned sizing for a batch (no counterpart in the reference): every query with n == 0 gets the
 * learned profile's budget for (error, confidence), from pilot batches (pilot_samples per query, 0:
 * adaptive as in zg_graph_features, on the pilot stream zg_graph_features uses: first sample 0,
 * stream ZG_ELP_STREAM + 1, the query's seed), the degree statistics of its graph (base or filtered) and one prediction for
 * all of them; n as zg_elp_learned computes it.  Queries with n > 0 are left as they are; a 3-motif
 * query needs its n.  Runs the batch (so not while one of its batches is pending). */
int zg_batch_size_learned(zg_batch* b, const zg_mlp* net, zg_batch_query* queries, uint32_t nq,
                          double error, double confidence, uint64_t pilot_samples, void* cuda_stream);
/* The batch counterpart of zg_query_learned (no counterpart in the reference): learned sizing of
 * the queries without a sample count (zg_batch_size_learned), one batch, then further batches for
 * the answers whose half-width (as zg_query checks it: empirical CLT or Bernstein, with the base
 * graph's weight range) is still above error * estimate, each topped up to what its observed
 * variance needs (headroom 1 + 0.5 / sqrt(hits)) on fresh sample indices and merged
 * exactly (an answer equals one run over all its samples), for at most max_rounds batches (0: 4)
 * and max_samples per query (0: 2^40).  3-motif queries run their given budgets once.  out: two
 * zg_counters per query as zg_batch_wait; bound_met: one flag per query; *rounds_run may be NULL. */
int zg_batch_bounded(zg_batch* b, const zg_mlp* net, const zg_batch_query* queries, uint32_t nq,
                     double error, double confidence, uint32_t max_rounds, uint64_t max_samples,
                     void* cuda_stream, zg_counters* out, uint32_t* bound_met, uint32_t* rounds_run);
/* Device time of the last waited batch (CUDA events around its graph launch), in ms. */
int zg_batch_elapsed_ms(const zg_batch* b, float* ms);
/* Bytes one submit copies host -> device (header, query descriptors, work list) and one wait
 * copies device -> host (the per-query results), for end-to-end accounting. */
int zg_batch_copy_bytes(const zg_batch* b, uint64_t* h2d, uint64_t* d2h);
/* The cached filtered graph of a predicate (built if missing): what a filtered query samples. */
int zg_batch_filtered_graph(zg_batch* b, int pred_op, int64_t t0, int64_t t1, void* cuda_stream,
                            const zg_graph** out);
/* Autotuner of the batch kernel's launch shape (resident blocks 2, 3 or 4 of 256 threads): runs
 * the batch three times per shape and keeps the fastest; ms_per_variant (may be NULL) gets 3. */
int zg_batch_tune(zg_batch* b, const zg_batch_query* queries, uint32_t nq, void* cuda_stream, int* best_variant,
                  float* ms_per_variant);

/* ---- error-latency profiles and bounded queries ------------------------------ */
/* Draw plan of zg_elp_plain for a given seed: the subsample keeps edge e iff
 * zg_draw(seed + ZG_ELP_KEEP_OFFSET, subsample stream, e) <= 0.1 * 2^30 and is permuted with
 * seed + ZG_ELP_SHUFFLE_OFFSET; a predicate filter on it uses seed + ZG_ELP_FILTER_OFFSET; the
 * 2^14 x 16 grouped estimators take sample indices [0, 2^18) and the 2^23 follow-up estimators
 * [2^18, 2^18 + 2^23), all on stream ZG_ELP_STREAM. */
#define ZG_ELP_KEEP_OFFSET    1
#define ZG_ELP_SHUFFLE_OFFSET 2
#define ZG_ELP_FILTER_OFFSET  3
#define ZG_ELP_STREAM         0x454C5000u

typedef struct zg_elp_result {
  uint64_t n_required;        /* (unsigned long long) of the bound, as get_num_estimators returns */
  double   n_required_f;
  double   K;                 /* regression slope (src/Regression.cpp:17-28) */
  double   estimate_sampled;  /* estimate on the 10 % subsample */
  double   big_estimate;      /* mean of the 2^23 follow-up estimators */
  double   rough_estimate;    /* estimate_sampled / 0.1^(nse + ncse) */
  double   nse, ncse;         /* sample_edge / conditional_sample_edge calls per estimate */
  uint64_t sampled_edges, sampled_max_degree;
  double   profile_ms;        /* wall time of the whole profile */
} zg_elp_result;

/* ErrorProfile<E>::calculate_bound (src/ErrorLatencyProfile.cpp:52-59). */
double zg_calculate_bound(double epsilon, double delta, double nse, double ncse, double estimation,
                          uint64_t max_degree, uint64_t num_edges);
/* Standard normal quantile (Acklam's approximation, one Halley refinement). */
double zg_normal_quantile(double p);
/* n_groups consecutive groups of group_size estimators: per-group mean of estimate() summed in
 * sample order in double, what a one-threaded calculate(group_size) returns
 * (src/ZGraphInstance.cpp:273-292).  group_estimates: host array of n_groups. */
int zg_run_groups(const zg_graph* g, const zg_program* p, uint64_t n_groups, uint32_t group_size,
                  uint64_t first_sample, uint64_t seed, uint32_t stream_id, void* cuda_stream,
                  double* group_estimates);
/* The host half of ErrorProfile::get_num_estimators (src/ErrorLatencyProfile.cpp:115-206). */
int zg_elp_solve(const double* group_estimates, uint64_t n_groups, uint32_t group_size,
                 double big_estimate, uint64_t big_n, double nse, double ncse, uint64_t sampled_m,
                 uint64_t sampled_max_degree, uint64_t orig_m, uint64_t orig_max_degree, double eps,
                 double conf, zg_elp_result* out);
/* ErrorProfile<E>::get_num_estimators (src/ErrorLatencyProfile.cpp:72-207) on the device.
 * pred_op != 0 profiles an AllPredicate instance: the predicate filters the subsample, as
 * AllPredicateZGraphInstance::set_graph does (src/ZGraphInstance.cpp:514-520).
 * group_estimates (may be NULL) receives the 2^14 group means. */
int zg_elp_plain(const zg_graph* g, const zg_program* p, int pred_op, int64_t t0, int64_t t1,
                 double error, double confidence, uint64_t seed, void* cuda_stream,
                 zg_elp_result* out, double* group_estimates);
/* TimeProfile<E>::run (src/ErrorLatencyProfile.cpp:25-47): doubling calculate() calls from 64
 * estimators while the next one fits the budget, then a final call sized to the remaining time. */
int zg_time_profile(const zg_graph* g, const zg_program* p, uint32_t time_limit_ms, uint64_t seed,
                    uint32_t stream_id, void* cuda_stream, double* estimate, uint64_t* samples_used);

#define ZG_BOUND_CLT        1  /* empirical CLT: z * sqrt(var / n), from 30 hits on          */
#define ZG_BOUND_BERNSTEIN  2  /* empirical Bernstein: sqrt(2 var x / n) + 3 R x / n         */
typedef struct zg_query_result {
  double   estimate;          /* exact mean over all samples taken */
  double   half_width;        /* the half-width of the bound below at the requested confidence */
  double   rel_half_width;
  uint64_t samples, hits;
  uint32_t bound_met, rounds;
  uint64_t n_sized;           /* the initial budget */
  double   ms_total;
  uint32_t bound_method;      /* ZG_BOUND_CLT or ZG_BOUND_BERNSTEIN: the bound half_width is from */
  uint32_t reserved;
  double   weight_range;      /* R: the largest value one estimator can return on the graph */
} zg_query_result;
/* A bounded query (no counterpart in the reference, whose ErrorProfile::run trusts its bound; the
 * stop rule of its sampling/IEStop.cpp is a CLT interval): run n_initial estimators and keep
 * sampling fresh estimators until the running estimate's half-width at the requested confidence is
 * <= error * estimate, or max_samples (0: 2^40) is reached (then bound_met = 0).  The half-width is
 * the empirical CLT one, z * sqrt(var / n) (from 30 hits on), or the empirical Bernstein one
 * (Audibert, Munos, Szepesvari 2009: for values in [0, R], with probability >= 1 - delta,
 * |mean - mu| <= sqrt(2 var ln(3/delta) / n) + 3 R ln(3/delta) / n, var the empirical variance),
 * whichever is smaller; below 30 hits only the Bernstein one.  The CLT one takes an upper
 * confidence bound on the variance from the fourth moment (zg_bound_half_width).  R bounds one
 * estimator's weight:
 * m * prod over the conditional steps i = 1.. of min((i + 1) * max_degree, 2m) (x 3 for the
 * 4-chain).  Each further round runs what the observed variance needs, with headroom
 * 1 + 0.5 / sqrt(hits).  A round whose exact weights overflowed 192 bits (zg_counters.overflow;
 * only programs with more than six weight factors can) ends the query with ZG_ERR_OVERFLOW. */
int zg_query(const zg_graph* g, const zg_program* p, double error, double confidence,
             uint64_t n_initial, uint64_t max_samples, uint64_t seed, uint32_t stream_id,
             void* cuda_stream, zg_query_result* out);
/* The check zg_query applies to a running estimate (host arithmetic only, no device): mean,
 * empirical (1/n) variance and empirical mean of w^4 (fourth_moment; 0: unknown) of n estimators
 * with `hits` non-zero ones, each in [0, weight_range].  *half_width gets the half-width at
 * `confidence` (CLT from 30 hits on, or Bernstein, whichever is smaller; Bernstein alone below 30
 * hits), *method the bound it came from, *met whether half_width <= error * mean.  The CLT
 * half-width uses an upper confidence bound on the variance, var + z sqrt((m4 - var^2) / n) with
 * m4 <= fourth_moment + 2 mean^2 var, so that heavy-tailed weights, whose variance estimate runs
 * low in most runs, keep their coverage.  A fourth moment that overflowed (infinite: weights
 * beyond about 1e77) counts as unknown. */
int zg_bound_half_width(double mean, double var, double fourth_moment, uint64_t n, uint64_t hits, double error,
                        double confidence, double weight_range, double* half_width, uint32_t* method, uint32_t* met);

/* ---- learned error-latency profile (no counterpart in the reference) ------------------- */
/* A 16 -> 64 -> 64 (GELU) -> 2 MLP predicting, for a (graph, program) query, log2 of the
 * per-sample relative variance Var(1/p)/E(1/p)^2 and log2 of the per-sample latency in ns.
 * BF16 weights with FP32 accumulation; FP32 master weights and Adam moments; trained and run by
 * this library's own CUDA kernels.  Parameters: ZG_MLP_PARAMS floats in the order W1[64][16],
 * b1[64], W2[64][64], b2[64], W3[2][64], b3[2]; norm: 36 floats (feature mean[16], std[16],
 * target mean[2], std[2]). */
#define ZG_MLP_FEATURES 16
#define ZG_MLP_OUTPUTS  2
#define ZG_MLP_PARAMS   5378
int zg_mlp_num_params(void);
int zg_mlp_create(uint64_t seed, zg_mlp** out);
int zg_mlp_free(zg_mlp* net);
int zg_mlp_get_params(const zg_mlp* net, float* params, float* norm);
int zg_mlp_set_params(zg_mlp* net, const float* params, const float* norm);
/* epochs over n_rows raw rows (normalisation statistics are taken from them), minibatches of
 * batch <= 64 rows in a seeded order, Adam(lr, 0.9, 0.999, 1e-8); loss_history gets one MSE per
 * step (epochs * n_rows / batch entries), may be NULL. */
int zg_mlp_train(zg_mlp* net, const float* X, const float* Y, uint32_t n_rows, uint32_t epochs,
                 uint32_t batch, float lr, uint64_t seed, float* loss_history);
/* Gradient of the MSE over n_rows <= 64 already-normalised rows at the current weights. */
int zg_mlp_grad(const zg_mlp* net, const float* X, const float* Y, uint32_t n_rows, float* grads,
                float* loss);
/* Predictions for raw features, de-normalised: Y[n_rows][2]. */
int zg_mlp_predict(const zg_mlp* net, const float* X, uint32_t n_rows, float* Y);
/* The 16 features of a query: degree statistics of g (one device pass on the first call for g,
 * then kept with the graph), the program's pattern class, and a pilot run of pilot_samples
 * estimators (0: adaptive, 2^16 and then 2^18, 2^20, 2^22 from the same first sample until the
 * pilot has 8 hits; the shipped network is trained on adaptive pilots).  Not to be called for the
 * same graph from two threads at once. */
int zg_graph_features(const zg_graph* g, const zg_program* p, uint64_t pilot_samples,
                      uint64_t seed, void* cuda_stream, float* features);
/* Learned sizing (the learned counterpart of ErrorProfile::get_num_estimators,
 * src/ErrorLatencyProfile.cpp:52-59): the query's features (zg_graph_features with pilot_samples),
 * the network's prediction, and n = z^2 * 2^pred_cv2 / error^2, z the two-sided normal quantile
 * of confidence, at least 2^16.  prediction (may be NULL) gets the network's two outputs. */
int zg_elp_learned(const zg_mlp* net, const zg_graph* g, const zg_program* p, double error,
                   double confidence, uint64_t pilot_samples, uint64_t seed, void* cuda_stream,
                   uint64_t* n_required, float* prediction);
/* zg_elp_learned (adaptive pilot from feature_seed), then zg_query from query_seed.  A budget
 * above 2^30 samples runs in two looks: half of it first, then what the bound check still needs, so an
 * over-predicted budget costs at most half of it in extra samples.  n_required may be NULL. */
int zg_query_learned(const zg_mlp* net, const zg_graph* g, const zg_program* p, double error,
                     double confidence, uint64_t max_samples, uint64_t feature_seed, uint64_t query_seed,
                     uint32_t stream_id, void* cuda_stream, uint64_t* n_required, zg_query_result* out);

/* ---- measurement ------------------------------------------------------------ */
/* Read bandwidth (GB/s) of a device buffer of `bytes` read `reps` times by one persistent grid,
 * timed with CUDA events: below the 129 MB L2 it measures L2, well above it HBM.  The L2 view of
 * the roofline for graphs that nearly fit in L2 (no counterpart in the reference). */
int zg_read_bandwidth(uint64_t bytes, uint32_t reps, void* cuda_stream, double* gbs);
/* Random 32-byte sector reads per second over g's edge records and edge-id-ordered adjacency
 * (every sector of the two arrays equally likely; each thread of one full-occupancy grid keeps 8
 * independent loads in flight, `iters` rounds of them; CUDA events after a warm-up launch): the
 * rate at which the memory system serves isolated sectors of the arrays the sampling kernels
 * read, the ceiling of kernels whose loads are random sectors (no counterpart in the reference). */
int zg_random_sector_rate(const zg_graph* g, uint32_t iters, void* cuda_stream, double* sectors_per_s);
/* The bytes zg_run's sampling kernel moves (no counterpart in the reference): the same kernel,
 * compiled a second time with every global load also counting the 32-byte sectors it spans (a
 * sector equal to the thread's previous load's last sector is counted once), run on n estimators
 * (sample indices [first_sample, first_sample + n), 1 <= n <= 2^32); *sectors gets the total over
 * all threads.  sectors * 32 / n is the kernel's bytes per sample: the numerator of its roofline.
 * Synchronous; allocates its per-block scratch. */
int zg_touch_sectors(const zg_graph* g, const zg_program* p, uint64_t n, uint64_t first_sample, uint64_t seed,
                     uint32_t stream_id, void* cuda_stream, uint64_t* sectors);

/* ---- exact counts ---------------------------------------------------------- */
/* out[0..1]: 128-bit little-endian count.  kind: ZG_EXACT_*. */
int zg_exact_count(const zg_graph* g, int kind, void* cuda_stream, uint64_t out[2]);
/* The predicate-weighted triangle counts of a graph with edge data (out as zg_exact_count):
 * ZG_EXACT_WEIGHTED_TRIANGLE counts the triangles whose three edges all have data >= threshold
 * (naive_implementation/WeightedTriangleCounting.cpp:46-75, threshold 50 there),
 * ZG_EXACT_AT_LEAST_ONE_TRIANGLE those with at least one such edge
 * (naive_implementation/AtLeastOneWeightedTriangleCounting.cpp). */
int zg_exact_count_weighted(const zg_graph* g, int kind, uint32_t threshold, void* cuda_stream, uint64_t out[2]);

/* ---- synthetic inputs (host) ------------------------------------------------ */
/* The reference reads SNAP files prepared by datasets/toolkits/edgelist_to_biedgelist.cpp;
 * these seeded generators stand in for them.  Output: undirected, no self-loops or duplicates,
 * random order and orientation.  edges == NULL only reports *m_out; otherwise capacity is the
 * number of (src,dst) pairs edges can hold. */
int zg_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                uint64_t capacity, uint32_t* edges, uint64_t* m_out);
int zg_gen_chung_lu(uint32_t num_vertices, double exponent, double avg_degree, uint64_t seed,
                    uint64_t capacity, uint32_t* edges, uint64_t* m_out);
/* Edge data uniform in [0, max_value) (datasets/toolkits/get_weighted_datasets.cpp:28-43). */
int zg_gen_weights(uint64_t m, uint32_t max_value, uint64_t seed, uint32_t* weights);
/* The same generators on the device, built straight into a device graph: the graph equals
 * zg_graph_create() of zg_gen_rmat / zg_gen_chung_lu's output (edge for edge, in that order), with
 * zg_gen_weights(m, max_weight, weight_seed) as edge data when max_weight > 0.  flags:
 * ZG_GRAPH_SAMPLING_ONLY leaves out the neighbour-ordered adjacency (zg_graph_download's adj_n),
 * which only exports use: a third less memory for the largest graphs. */
#define ZG_GRAPH_SAMPLING_ONLY 1u
int zg_graph_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                      uint32_t max_weight, uint64_t weight_seed, uint32_t flags, void* cuda_stream,
                      zg_graph** out);
int zg_graph_gen_chung_lu(uint32_t num_vertices, double exponent, double avg_degree, uint64_t seed,
                          uint32_t max_weight, uint64_t weight_seed, uint32_t flags, void* cuda_stream,
                          zg_graph** out);

#ifdef __cplusplus
}
#endif
#endif /* ZGRAPH_GPU_H */
