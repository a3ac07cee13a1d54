"""Python binding of libzgraph_gpu.so (ctypes over include/zgraph_gpu.h) and a host-side mirror of
the reference's estimator interface (jy-yuan/sampling-graph-mining):

  Graph                     Graph<E> + DistGraphLoader/CSRConstructor (include/Graph.hpp:148-246)
  Estimation                include/ZGraphInstance.hpp:18-28, src/ZGraphInstance.cpp:15-35
  ZGraphInstance.calculate  src/ZGraphInstance.cpp:257-297
  TriangleCountingInstance, FourCliqueCountingInstance, ThreeChainCountingInstance,
  FourChainCountingInstance, ChainMiningInstance       applications/<App>.cpp estimate() bodies
  Pattern, SamplerGenerator                            include/SamplerGenerator.hpp:9-80
  AllPredicateZGraphInstance                           include/ZGraphInstance.hpp:143-157
  ThreeMotif (ZGraphInstanceWithCache pair)            applications/ThreeMotif.cpp:149-196

Every estimate runs on the GPU through the C ABI; there is no CPU path.  Loading fails loudly
when the library has not been built.
"""
import ctypes as C
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libzgraph_gpu.so")

ZG_OK = 0
(ZG_ERR_INVALID_ARG, ZG_ERR_OOM, ZG_ERR_CUDA, ZG_ERR_INVALID_GRAPH, ZG_ERR_UNSUPPORTED_ESTIMATOR, ZG_ERR_TIMEOUT,
 ZG_ERR_BOUND_NOT_MET, ZG_ERR_NO_DEVICE, ZG_ERR_OVERFLOW, ZG_ERR_TOO_LARGE) = range(1, 11)
ERRORS = {1: "INVALID_ARG", 2: "OOM", 3: "CUDA", 4: "INVALID_GRAPH", 5: "UNSUPPORTED_ESTIMATOR",
          6: "TIMEOUT", 7: "BOUND_NOT_MET", 8: "NO_DEVICE", 9: "OVERFLOW", 10: "TOO_LARGE"}

PROG_TRIANGLE, PROG_FOUR_CLIQUE, PROG_THREE_CHAIN, PROG_FOUR_CHAIN, PROG_CHAIN, PROG_PATTERN = 1, 2, 3, 4, 5, 6
PROG_FOUR_CLIQUE_UNBIASED = 7  # canonical-path 4-clique estimator (no counterpart in the reference)
EXACT_TRIANGLE, EXACT_WEDGE, EXACT_THREE_PATH, EXACT_FIVE_STAR, EXACT_FOUR_CLIQUE = 1, 2, 3, 4, 5
EXACT_FIVE_HOUSE, EXACT_FIVE_CHAIN, EXACT_WEIGHTED_TRIANGLE, EXACT_AT_LEAST_ONE_TRIANGLE = 6, 7, 8, 9
PRED_GE, PRED_LT, PRED_GT, PRED_LE, PRED_EQ, PRED_NE, PRED_RANGE = 1, 2, 3, 4, 5, 6, 7
QUERY_THREE_MOTIF = 16
BOUND_CLT, BOUND_BERNSTEIN = 1, 2
RESULT_BYTES = 112  # ZG_RESULT_BYTES: one reduced result of zg_run_async
GRAPH_SAMPLING_ONLY = 1
RECORDS_AUTO, RECORDS_COMPACT, RECORDS_WIDE, RECORDS_PACKED = 0, 1, 2, 3
BATCH_MAX_QUERIES, BATCH_MAX_CHUNKS = 65536, 65536
NO_SHUFFLE = 0xFFFFFFFFFFFFFFFF
MAX_DRAWS = 16
VARIANTS = 7  # ZG_VARIANTS: launch shapes per program kind


class ZgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code


class GraphMeta(C.Structure):
    _fields_ = [("num_vertices", C.c_uint32), ("weighted", C.c_uint32), ("num_local_edges", C.c_uint64),
                ("num_edges", C.c_uint64), ("max_degree", C.c_uint64), ("device_bytes", C.c_uint64),
                ("record_bytes", C.c_uint32), ("record_layout", C.c_uint32)]


class Counters(C.Structure):
    _fields_ = [("samples", C.c_uint64), ("hits", C.c_uint64), ("fails", C.c_uint64),
                ("den_log2", C.c_uint32), ("overflow", C.c_uint32), ("sum_num", C.c_uint64 * 5),
                ("sum_w", C.c_double), ("sum_w2", C.c_double), ("estimate", C.c_double),
                ("sum_w4", C.c_double)]

    def exact_sum(self):
        """Exact sum of 1/p over the samples as a Python Fraction."""
        from fractions import Fraction
        v = 0
        for i in range(5):
            v |= int(self.sum_num[i]) << (64 * i)
        return Fraction(v, 1 << self.den_log2)

    def as_dict(self):
        return {"samples": self.samples, "hits": self.hits, "fails": self.fails,
                "den_log2": self.den_log2, "overflow": self.overflow,
                "sum_num": [int(x) for x in self.sum_num], "sum_w": self.sum_w,
                "sum_w2": self.sum_w2, "estimate": self.estimate}


class BatchQuery(C.Structure):
    _fields_ = [("kind", C.c_int32), ("param", C.c_uint32), ("pred_op", C.c_int32), ("stream_id", C.c_uint32),
                ("t0", C.c_int64), ("t1", C.c_int64), ("n", C.c_uint64), ("seed", C.c_uint64),
                ("first_sample", C.c_uint64), ("program", C.c_void_p)]


class ElpResult(C.Structure):
    _fields_ = [("n_required", C.c_uint64), ("n_required_f", C.c_double), ("K", C.c_double),
                ("estimate_sampled", C.c_double), ("big_estimate", C.c_double), ("rough_estimate", C.c_double),
                ("nse", C.c_double), ("ncse", C.c_double), ("sampled_edges", C.c_uint64),
                ("sampled_max_degree", C.c_uint64), ("profile_ms", C.c_double)]


class CloseQuery(C.Structure):
    _fields_ = [("min_valid_edge_id", C.c_uint64), ("num_vertices", C.c_uint32), ("num_edges", C.c_uint32),
                ("vertices", C.c_uint32 * 16), ("edges", C.c_uint32 * 32)]


class CloseResult(C.Structure):
    _fields_ = [("closed", C.c_uint32), ("found", C.c_uint32), ("edge_ids", C.c_uint64 * 16)]


class QueryResult(C.Structure):
    _fields_ = [("estimate", C.c_double), ("half_width", C.c_double), ("rel_half_width", C.c_double),
                ("samples", C.c_uint64), ("hits", C.c_uint64), ("bound_met", C.c_uint32), ("rounds", C.c_uint32),
                ("n_sized", C.c_uint64), ("ms_total", C.c_double), ("bound_method", C.c_uint32),
                ("reserved", C.c_uint32), ("weight_range", C.c_double)]


ELP_KEEP_OFFSET, ELP_SHUFFLE_OFFSET, ELP_FILTER_OFFSET, ELP_STREAM = 1, 2, 3, 0x454C5000

TRACE_DTYPE = np.dtype([("ndraws", "<u4"), ("hit", "<u4"), ("fail", "<u4"), ("shift", "<u4"),
                        ("sectors", "<u4"), ("closures", "<u4"), ("w", "<f8"), ("num", "<u8", (3,)), ("lo", "<u8", (MAX_DRAWS,)),
                        ("hi", "<u8", (MAX_DRAWS,)), ("val", "<u8", (MAX_DRAWS,))])

_lib = None
_lock = threading.Lock()


def lib():
    """Loads libzgraph_gpu.so (raises if it is missing: no fallback exists)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libzgraph_gpu.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        P, U32, U64, I64, I32, D = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int64, C.c_int, C.c_double
        sig = {
            "zg_version": ([], I32), "zg_init": ([I32], I32), "zg_last_error": ([], C.c_char_p),
            "zg_graph_create": ([P, U64, U32, P, P, C.POINTER(P)], I32),
            "zg_graph_permuted": ([P, U64, U32, P, U64, P, P, C.POINTER(P)], I32),
            "zg_graph_free": ([P], I32), "zg_set_record_layout": ([I32], I32),
            "zg_graph_get_meta": ([P, C.POINTER(GraphMeta)], I32),
            "zg_graph_set_meta": ([P, U64, U64], I32),
            "zg_graph_download": ([P, P, P, P, P, P, P], I32),
            "zg_graph_filter": ([P, I32, I64, I64, U64, P, P, C.POINTER(U64), C.POINTER(P)], I32),
            "zg_graph_subsample": ([P, D, U64, U64, P, P, C.POINTER(U64), C.POINTER(P)], I32),
            "zg_program_create": ([I32, U32, C.POINTER(P)], I32),
            "zg_program_create_pattern": ([U32, U32, P, C.POINTER(P)], I32),
            "zg_program_free": ([P], I32),
            "zg_program_info": ([P, C.POINTER(U32), C.POINTER(U32), C.POINTER(U32)], I32),
            "zg_run": ([P, P, U64, U64, U64, U32, P, C.POINTER(Counters)], I32),
            "zg_run_async": ([P, P, U64, U64, U64, U32, P, P], I32),
            "zg_result_to_counters": ([P, P, C.POINTER(Counters)], I32),
            "zg_run_noalloc": ([P, P, U64, U64, U64, U32, P, P], I32),
            "zg_tune": ([P, P, U64, P, C.POINTER(I32), P], I32),
            "zg_set_variant": ([I32, I32], I32),
            "zg_get_variant": ([I32, C.POINTER(I32), C.POINTER(I32), C.POINTER(I32)], I32),
            "zg_run_debug": ([P, P, U64, U64, U64, U32, P], I32),
            "zg_run_three_motif": ([P, U64, U64, U64, U32, U32, P, C.POINTER(Counters), C.POINTER(Counters)], I32),
            "zg_run_three_motif_debug": ([P, U64, U64, U64, U32, U32, P, P], I32),
            "zg_exact_count": ([P, I32, P, P], I32),
            "zg_calculate_bound": ([D, D, D, D, D, U64, U64], D),
            "zg_normal_quantile": ([D], D),
            "zg_run_groups": ([P, P, U64, U32, U64, U64, U32, P, P], I32),
            "zg_elp_solve": ([P, U64, U32, D, U64, D, D, U64, U64, U64, U64, D, D, C.POINTER(ElpResult)], I32),
            "zg_elp_plain": ([P, P, I32, I64, I64, D, D, U64, P, C.POINTER(ElpResult), P], I32),
            "zg_time_profile": ([P, P, U32, U64, U32, P, C.POINTER(D), C.POINTER(U64)], I32),
            "zg_query": ([P, P, D, D, U64, U64, U64, U32, P, C.POINTER(QueryResult)], I32),
            "zg_mlp_num_params": ([], I32),
            "zg_mlp_create": ([U64, C.POINTER(P)], I32),
            "zg_mlp_free": ([P], I32),
            "zg_mlp_get_params": ([P, P, P], I32),
            "zg_mlp_set_params": ([P, P, P], I32),
            "zg_mlp_train": ([P, P, P, U32, U32, U32, C.c_float, U64, P], I32),
            "zg_mlp_grad": ([P, P, P, U32, P, P], I32),
            "zg_mlp_predict": ([P, P, U32, P], I32),
            "zg_graph_features": ([P, P, U64, U64, P, P], I32),
            "zg_elp_learned": ([P, P, P, D, D, U64, U64, P, C.POINTER(U64), P], I32),
            "zg_query_learned": ([P, P, P, D, D, U64, U64, U64, U32, P, C.POINTER(U64), C.POINTER(QueryResult)],
                                 I32),
            "zg_gen_rmat": ([U32, U32, D, D, D, U64, U64, P, C.POINTER(U64)], I32),
            "zg_gen_chung_lu": ([U32, D, D, U64, U64, P, C.POINTER(U64)], I32),
            "zg_gen_weights": ([U64, U32, U64, P], I32),
            "zg_graph_gen_rmat": ([U32, U32, D, D, D, U64, U32, U64, U32, P, C.POINTER(P)], I32),
            "zg_graph_gen_chung_lu": ([U32, D, D, U64, U32, U64, U32, P, C.POINTER(P)], I32),
            "zg_batch_create": ([P, U32, U64, U64, C.POINTER(P)], I32),
            "zg_batch_free": ([P], I32),
            "zg_batch_submit": ([P, P, U32, P], I32),
            "zg_batch_wait": ([P, P], I32),
            "zg_batch_size_learned": ([P, P, P, U32, D, D, U64, P], I32),
            "zg_batch_bounded": ([P, P, P, U32, D, D, U32, U64, P, P, P, C.POINTER(U32)], I32),
            "zg_batch_filtered_graph": ([P, I32, I64, I64, P, C.POINTER(P)], I32),
            "zg_batch_tune": ([P, P, U32, P, C.POINTER(I32), P], I32),
            "zg_batch_elapsed_ms": ([P, C.POINTER(C.c_float)], I32),
            "zg_read_bandwidth": ([U64, U32, P, C.POINTER(D)], I32),
            "zg_random_sector_rate": ([P, U32, P, C.POINTER(D)], I32),
            "zg_touch_sectors": ([P, P, U64, U64, U64, U32, P, C.POINTER(U64)], I32),
            "zg_set_l2_fetch_granularity": ([U32, C.POINTER(U32)], I32),
            "zg_exact_count_weighted": ([P, I32, U32, P, P], I32),
            "zg_conditional_close": ([P, P, U32, P, P], I32),
            "zg_bound_half_width": ([D, D, D, U64, U64, D, D, D, C.POINTER(D), C.POINTER(U32), C.POINTER(U32)], I32),
            "zg_batch_copy_bytes": ([P, C.POINTER(U64), C.POINTER(U64)], I32),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
        return _lib


def check(rc):
    if rc != ZG_OK:
        raise ZgError(rc, lib().zg_last_error().decode(errors="replace"))


_init_done = set()


def init(device=0):
    """zg_init: select and check the sm_103 device (NetworkInterface/SharedMemSys set-up)."""
    if device not in _init_done:
        check(lib().zg_init(device))
        _init_done.add(device)


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


# ---- synthetic inputs ---------------------------------------------------------------------
def gen_rmat(scale, edge_factor, a=0.57, b=0.19, c=0.19, seed=1):
    """Undirected simplified R-MAT edge list, (m, 2) uint32 in a seeded random order."""
    L = lib()
    m = C.c_uint64(0)
    check(L.zg_gen_rmat(scale, edge_factor, a, b, c, seed, 0, None, C.byref(m)))
    out = np.empty((m.value, 2), dtype=np.uint32)
    check(L.zg_gen_rmat(scale, edge_factor, a, b, c, seed, m.value, _ptr(out), C.byref(m)))
    return out


def gen_chung_lu(n, exponent, avg_degree, seed=1):
    L = lib()
    m = C.c_uint64(0)
    check(L.zg_gen_chung_lu(n, exponent, avg_degree, seed, 0, None, C.byref(m)))
    out = np.empty((m.value, 2), dtype=np.uint32)
    check(L.zg_gen_chung_lu(n, exponent, avg_degree, seed, m.value, _ptr(out), C.byref(m)))
    return out


def gen_weights(m, max_value=100, seed=1):
    w = np.empty(m, dtype=np.uint32)
    check(lib().zg_gen_weights(m, max_value, seed, _ptr(w)))
    return w


# ---- graph --------------------------------------------------------------------------------
class Graph:
    """Device-resident Graph<E>: COO in edge-id order + both adjacency orders (zg_graph_create)."""

    def __init__(self, handle, num_vertices, parent_index=None):
        self._h = handle
        self.num_vertices = num_vertices
        self.parent_index = parent_index

    @classmethod
    def from_edges(cls, edges, num_vertices, weights=None, shuffle_seed=None, stream=None):
        init()
        e = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1, 2)
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.uint32)
        h = C.c_void_p()
        L = lib()
        if shuffle_seed is None:
            check(L.zg_graph_create(_ptr(e), e.shape[0], num_vertices, _ptr(w), stream, C.byref(h)))
            return cls(h, num_vertices)
        parent = np.empty(e.shape[0], dtype=np.uint64)
        check(L.zg_graph_permuted(_ptr(e), e.shape[0], num_vertices, _ptr(w), shuffle_seed, stream,
                                  _ptr(parent), C.byref(h)))
        return cls(h, num_vertices, parent)

    @classmethod
    def gen_rmat(cls, scale, edge_factor, a=0.57, b=0.19, c=0.19, seed=1, max_weight=0, weight_seed=1,
                 sampling_only=False):
        """zg_graph_gen_rmat: the seeded R-MAT graph generated and built on the device."""
        init()
        h = C.c_void_p()
        check(lib().zg_graph_gen_rmat(scale, edge_factor, a, b, c, seed, max_weight, weight_seed,
                                      GRAPH_SAMPLING_ONLY if sampling_only else 0, None, C.byref(h)))
        return cls(h, 1 << scale)

    @classmethod
    def gen_chung_lu(cls, num_vertices, exponent, avg_degree, seed=1, max_weight=0, weight_seed=1,
                     sampling_only=False):
        """zg_graph_gen_chung_lu: the seeded Chung-Lu graph generated and built on the device."""
        init()
        h = C.c_void_p()
        check(lib().zg_graph_gen_chung_lu(num_vertices, exponent, avg_degree, seed, max_weight, weight_seed,
                                          GRAPH_SAMPLING_ONLY if sampling_only else 0, None, C.byref(h)))
        return cls(h, num_vertices)

    @classmethod
    def load(cls, path, weighted=False, shuffle_seed=None):
        """Reads the reference's binary .biedgelist (+ .csv vertex count, src/Utilities.cpp:24-35)."""
        raw = np.fromfile(path + ".biedgelist", dtype=np.uint32)
        rec = raw.reshape(-1, 3 if weighted else 2)
        with open(path + ".csv") as f:
            f.readline()
            line = f.readline()
        digits = ""
        for ch in line:
            if ch.isdigit():
                digits += ch
            elif digits:
                break
        nv = int(digits)
        return cls.from_edges(rec[:, :2], nv, rec[:, 2] if weighted else None, shuffle_seed=shuffle_seed)

    @property
    def handle(self):
        if not self._h:
            raise ValueError("graph was freed")
        return self._h

    def meta(self):
        m = GraphMeta()
        check(lib().zg_graph_get_meta(self.handle, C.byref(m)))
        return m

    @property
    def num_local_edges(self):
        return self.meta().num_local_edges

    @property
    def num_edges(self):
        return self.meta().num_edges

    @property
    def max_degree(self):
        return self.meta().max_degree

    def set_meta(self, num_edges, max_degree):
        check(lib().zg_graph_set_meta(self.handle, num_edges, max_degree))

    def download_edges(self):
        """The COO edge list in edge-id order, (m, 2) uint32 (unpacked on the device)."""
        e = np.empty((self.num_local_edges, 2), np.uint32)
        check(lib().zg_graph_download(self.handle, _ptr(e), None, None, None, None, None))
        return e

    def download(self, neighbour_order=True):
        """Device arrays on the host; neighbour_order=False skips adj_n (absent from the graphs a
        batch caches)."""
        m = self.num_local_edges
        nv = self.num_vertices
        out = {"edges": np.empty((m, 2), np.uint32), "offsets": np.empty(nv + 1, np.int64),
               "adj_e": np.empty((2 * m, 2), np.uint32),
               "adj_n": np.empty((2 * m, 2), np.uint32) if neighbour_order else None,
               "suffix": np.empty((m, 2), np.uint32)}
        w = np.empty(m, np.uint32) if self.meta().weighted else None
        check(lib().zg_graph_download(self.handle, _ptr(out["edges"]), _ptr(w), _ptr(out["offsets"]),
                                      _ptr(out["adj_e"]), _ptr(out["adj_n"]), _ptr(out["suffix"])))
        out["weights"] = w
        return out

    def filter(self, op, t0, t1=0, shuffle_seed=NO_SHUFFLE):
        """GraphFilter::generate_graph (src/GraphFilters.cpp:17-177)."""
        parent = np.empty(max(1, self.num_local_edges), np.uint64)
        mo = C.c_uint64(0)
        h = C.c_void_p()
        check(lib().zg_graph_filter(self.handle, op, t0, t1, shuffle_seed, None, _ptr(parent), C.byref(mo),
                                    C.byref(h)))
        return Graph(h, self.num_vertices, parent[:mo.value].copy())

    def subsample(self, rate, keep_seed, shuffle_seed=NO_SHUFFLE):
        """GraphSampler::sample_graph (src/Graph.cpp:629-780)."""
        parent = np.empty(max(1, self.num_local_edges), np.uint64)
        mo = C.c_uint64(0)
        h = C.c_void_p()
        check(lib().zg_graph_subsample(self.handle, rate, keep_seed, shuffle_seed, None, _ptr(parent),
                                       C.byref(mo), C.byref(h)))
        return Graph(h, self.num_vertices, parent[:mo.value].copy())

    def exact_count(self, kind, stream=None):
        out = (C.c_uint64 * 2)()
        check(lib().zg_exact_count(self.handle, kind, stream, out))
        return int(out[0]) | (int(out[1]) << 64)

    def exact_count_weighted(self, kind, threshold, stream=None):
        """zg_exact_count_weighted: EXACT_WEIGHTED_TRIANGLE (all edges' data >= threshold) or
        EXACT_AT_LEAST_ONE_TRIANGLE (some edge's data >= threshold)."""
        out = (C.c_uint64 * 2)()
        check(lib().zg_exact_count_weighted(self.handle, kind, threshold, stream, out))
        return int(out[0]) | (int(out[1]) << 64)

    def free(self):
        if self._h:
            if not getattr(self, "_borrowed", False):  # a batch's cached graph belongs to the batch
                lib().zg_graph_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def set_record_layout(layout):
    """zg_set_record_layout: per-edge record layout of the graphs built from now on
    (RECORDS_AUTO, RECORDS_COMPACT, RECORDS_WIDE or RECORDS_PACKED); estimates are identical under
    each."""
    check(lib().zg_set_record_layout(layout))


def set_l2_fetch_granularity(nbytes):
    """zg_set_l2_fetch_granularity: the bytes the L2 fetches per miss on the current device (0: keep);
    returns the previous value."""
    prev = C.c_uint32()
    check(lib().zg_set_l2_fetch_granularity(nbytes, C.byref(prev)))
    return prev.value


def random_sector_rate(graph, iters=64, cuda_stream=None):
    """zg_random_sector_rate: random 32-byte sector reads per second over graph's records and adjacency."""
    out = C.c_double(0)
    check(lib().zg_random_sector_rate(graph.handle, iters, cuda_stream, C.byref(out)))
    return out.value


def read_bandwidth(nbytes, reps=200, cuda_stream=None):
    """zg_read_bandwidth: GB/s of repeated reads of an nbytes device buffer (L2 below 129 MB)."""
    init()
    out = C.c_double(0)
    check(lib().zg_read_bandwidth(nbytes, reps, cuda_stream, C.byref(out)))
    return out.value


# ---- batched mixed queries ----------------------------------------------------------------
class Batch:
    """zg_batch_*: many queries (program, optional predicate filter, budget, Philox stream) in one
    persistent launch replayed through a CUDA graph; filtered graphs are cached on the device."""

    def __init__(self, graph, max_queries=1024, cache_bytes=16 << 30, filter_seed=1):
        init()
        self.graph = graph  # the base graph must outlive the batch
        h = C.c_void_p()
        check(lib().zg_batch_create(graph.handle, max_queries, cache_bytes, filter_seed, C.byref(h)))
        self._h = h
        self.max_queries = max_queries
        self._nq = 0

    @staticmethod
    def queries(qs):
        """qs: iterable of dicts with kind, n, seed and optional param, pred_op, t0, t1, stream_id,
        first_sample and program (a Program, for PROG_PATTERN)."""
        qs = list(qs)
        arr = (BatchQuery * max(1, len(qs)))()
        keep = []
        for i, q in enumerate(qs):
            arr[i].kind = q["kind"]
            arr[i].param = q.get("param", 0)
            arr[i].pred_op = q.get("pred_op", 0)
            arr[i].stream_id = q.get("stream_id", 0)
            arr[i].t0 = q.get("t0", 0)
            arr[i].t1 = q.get("t1", 0)
            arr[i].n = q.get("n", 0)
            arr[i].seed = q["seed"]
            arr[i].first_sample = q.get("first_sample", 0)
            prog = q.get("program")
            if prog is not None:
                arr[i].program = prog._h
                keep.append(prog)
        return arr, len(qs), keep

    def submit(self, qs, cuda_stream=None):
        arr, nq, keep = self.queries(qs)
        check(lib().zg_batch_submit(self._h, arr, nq, cuda_stream))
        self._nq = nq
        self._keep = keep  # pattern programs stay alive until the batch completes

    def wait(self):
        """Counters per query: [(c, None) or (chain, triangle) for 3-motif queries]."""
        out = (Counters * max(2, 2 * self._nq))()
        check(lib().zg_batch_wait(self._h, out))
        self._keep = []
        return [(out[2 * i], out[2 * i + 1]) for i in range(self._nq)]

    def run(self, qs, cuda_stream=None):
        self.submit(qs, cuda_stream)
        return self.wait()

    def size_learned(self, mlp, qs, eps, conf, pilot_samples=0, cuda_stream=None):
        """zg_batch_size_learned: the learned budget of every query without an "n" (one pilot
        batch, one prediction); returns the queries with "n" filled in."""
        qs = [dict(q) for q in qs]
        arr, nq, keep = self.queries(qs)
        check(lib().zg_batch_size_learned(self._h, mlp._h, arr, nq, eps, conf, pilot_samples, cuda_stream))
        for i, q in enumerate(qs):
            q["n"] = int(arr[i].n)
        return qs

    def bounded(self, mlp, qs, eps, conf, max_rounds=4, max_samples=1 << 40, cuda_stream=None):
        """zg_batch_bounded, the batch counterpart of zg_query_learned: learned sizing of every
        query without an "n", one batch, then further batches for the answers whose empirical CLT
        half-width is still above eps * estimate, topped up on fresh sample indices and merged
        exactly.  Returns (counters per query (a pair for 3-motif queries), bound met per query,
        rounds)."""
        qs = list(qs)
        arr, nq, keep = self.queries(qs)
        out = (Counters * max(2, 2 * nq))()
        met = (C.c_uint32 * max(1, nq))()
        rounds = C.c_uint32(0)
        check(lib().zg_batch_bounded(self._h, mlp._h, arr, nq, eps, conf, max_rounds, max_samples, cuda_stream,
                                     out, met, C.byref(rounds)))
        total = [(out[2 * i], out[2 * i + 1]) if qs[i]["kind"] == QUERY_THREE_MOTIF else out[2 * i]
                 for i in range(nq)]
        return total, [bool(met[i]) for i in range(nq)], int(rounds.value)

    def copy_bytes(self):
        """zg_batch_copy_bytes: (host->device bytes per submit, device->host bytes per wait)."""
        a, b = C.c_uint64(), C.c_uint64()
        check(lib().zg_batch_copy_bytes(self._h, C.byref(a), C.byref(b)))
        return int(a.value), int(b.value)

    def elapsed_ms(self):
        """Device time of the last waited batch (CUDA events around its graph launch)."""
        ms = C.c_float(0)
        check(lib().zg_batch_elapsed_ms(self._h, C.byref(ms)))
        return ms.value

    def filtered_graph(self, op, t0, t1=0):
        """The cached filtered graph a predicate query samples (owned by the batch)."""
        h = C.c_void_p()
        check(lib().zg_batch_filtered_graph(self._h, op, t0, t1, None, C.byref(h)))
        g = Graph(h, self.graph.num_vertices)
        g._borrowed = True
        return g

    def tune(self, qs, cuda_stream=None):
        arr, nq, keep = self.queries(qs)
        best = C.c_int(0)
        ms = (C.c_float * 3)()
        check(lib().zg_batch_tune(self._h, arr, nq, cuda_stream, C.byref(best), ms))
        return best.value, [float(x) for x in ms]

    def free(self):
        if getattr(self, "_h", None):
            lib().zg_batch_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# ---- programs -----------------------------------------------------------------------------
class Program:
    def __init__(self, kind, param=0, pattern=None):
        h = C.c_void_p()
        if kind == PROG_PATTERN:
            nv, edges = pattern
            e = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1, 2)
            check(lib().zg_program_create_pattern(nv, e.shape[0], _ptr(e), C.byref(h)))
        else:
            check(lib().zg_program_create(kind, param, C.byref(h)))
        self._h = h
        self.kind = kind
        self.param = param

    @property
    def handle(self):
        return self._h

    def info(self):
        u, c, v = C.c_uint32(), C.c_uint32(), C.c_uint32()
        check(lib().zg_program_info(self._h, C.byref(u), C.byref(c), C.byref(v)))
        return {"num_unique": u.value, "cond_calls": c.value, "vertices": v.value}

    def run(self, graph, n, seed, stream_id=0, first_sample=0, cuda_stream=None):
        out = Counters()
        check(lib().zg_run(graph.handle, self._h, n, first_sample, seed, stream_id, cuda_stream, C.byref(out)))
        return out

    def run_async(self, graph, n, seed, d_result, stream_id=0, first_sample=0, cuda_stream=None):
        """Enqueues the run on cuda_stream; the 112-byte result lands at device address d_result."""
        check(lib().zg_run_async(graph.handle, self._h, n, first_sample, seed, stream_id, cuda_stream,
                                 C.c_void_p(d_result)))

    def result_to_counters(self, host_bytes):
        out = Counters()
        buf = (C.c_char * len(host_bytes)).from_buffer_copy(host_bytes)
        check(lib().zg_result_to_counters(buf, self._h, C.byref(out)))
        return out

    def tune(self, graph, probe_samples=1 << 22, cuda_stream=None):
        """zg_tune: time every launch variant on graph, keep the fastest; returns (best, ms list)."""
        best = C.c_int(0)
        ms = (C.c_float * 8)()
        check(lib().zg_tune(graph.handle, self._h, probe_samples, cuda_stream, C.byref(best), ms))
        return best.value, [float(ms[i]) for i in range(VARIANTS)]

    def set_variant(self, variant):
        """zg_set_variant: fix this program kind's launch shape (0..ZG_VARIANTS-1)."""
        check(lib().zg_set_variant(self.kind, int(variant)))

    def variant(self):
        v, mb, g = C.c_int(), C.c_int(), C.c_int()
        check(lib().zg_get_variant(self.kind, C.byref(v), C.byref(mb), C.byref(g)))
        return {"variant": v.value, "min_blocks": mb.value, "grid": g.value}

    def touch_bytes_per_sample(self, graph, n, seed, stream_id=0, first_sample=0):
        """zg_touch_sectors: 32-byte sectors the production kernel's loads touch, x 32 / n."""
        out = C.c_uint64()
        check(lib().zg_touch_sectors(graph.handle, self._h, n, first_sample, seed, stream_id, None, C.byref(out)))
        return 32.0 * out.value / n

    def run_debug(self, graph, n, seed, stream_id=0, first_sample=0):
        tr = np.zeros(n, dtype=TRACE_DTYPE)
        check(lib().zg_run_debug(graph.handle, self._h, n, first_sample, seed, stream_id, _ptr(tr)))
        return tr

    def __del__(self):
        try:
            if self._h:
                lib().zg_program_free(self._h)
                self._h = None
        except Exception:
            pass


def elp_solve(groups, group_size, big_estimate, big_n, nse, ncse, sampled_m, sampled_max_degree, orig_m,
              orig_max_degree, eps, conf):
    """zg_elp_solve: the host half of ErrorProfile::get_num_estimators (no GPU needed)."""
    g = np.ascontiguousarray(groups, dtype=np.float64)
    out = ElpResult()
    check(lib().zg_elp_solve(_ptr(g), len(g), group_size, big_estimate, big_n, nse, ncse, sampled_m,
                             sampled_max_degree, orig_m, orig_max_degree, eps, conf, C.byref(out)))
    return out


def elp_plain(graph, program, eps, conf, seed, predicate=None, cuda_stream=None, want_groups=False):
    """zg_elp_plain: ErrorProfile::get_num_estimators on the device."""
    out = ElpResult()
    groups = np.zeros(1 << 14, np.float64) if want_groups else None
    op, t0, t1 = (0, 0, 0) if predicate is None else (predicate[0], predicate[1],
                                                      predicate[2] if len(predicate) > 2 else 0)
    check(lib().zg_elp_plain(graph.handle, program.handle, op, t0, t1, eps, conf, seed, cuda_stream, C.byref(out),
                             _ptr(groups)))
    return (out, groups) if want_groups else out


def run_groups(graph, program, n_groups, group_size, seed, stream_id=0, first_sample=0):
    out = np.zeros(n_groups, np.float64)
    check(lib().zg_run_groups(graph.handle, program.handle, n_groups, group_size, first_sample, seed, stream_id,
                              None, _ptr(out)))
    return out


def time_profile(graph, program, time_limit_ms, seed, stream_id=0):
    """zg_time_profile: TimeProfile::run."""
    est, used = C.c_double(), C.c_uint64()
    check(lib().zg_time_profile(graph.handle, program.handle, time_limit_ms, seed, stream_id, None, C.byref(est),
                                C.byref(used)))
    return est.value, used.value


def query(graph, program, eps, conf, n_initial, seed, stream_id=0, max_samples=0, cuda_stream=None):
    """zg_query: budgeted run checked against its empirical CLT bound, extended until the bound holds."""
    out = QueryResult()
    check(lib().zg_query(graph.handle, program.handle, eps, conf, n_initial, max_samples, seed, stream_id,
                         cuda_stream, C.byref(out)))
    return out


def conditional_close(graph, queries, cuda_stream=None):
    """zg_conditional_close: conditional_close(min_valid, vertices, edges&) (src/ZGraphInstance.cpp:
    410-441) for a list of (min_valid, vertices, edges) queries on the device; returns
    [(closed, found, edge ids of the found edges)]."""
    qs = list(queries)
    arr = (CloseQuery * max(1, len(qs)))()
    for i, (mv, verts, edges) in enumerate(qs):
        edges = [tuple(x) for x in edges]
        arr[i].min_valid_edge_id = mv
        arr[i].num_vertices = len(verts)
        arr[i].num_edges = len(edges)
        for j, v in enumerate(verts[:16]):  # longer lists are rejected by the library
            arr[i].vertices[j] = v
        for j, (a, b) in enumerate(edges[:16]):
            arr[i].edges[2 * j] = a
            arr[i].edges[2 * j + 1] = b
    res = (CloseResult * max(1, len(qs)))()
    check(lib().zg_conditional_close(graph.handle, arr, len(qs), cuda_stream, res))
    return [(bool(r.closed), int(r.found), [int(r.edge_ids[j]) for j in range(r.found)]) for r in res[:len(qs)]]


def bound_half_width(mean, var, n, hits, eps, conf, weight_range, fourth_moment=0.0):
    """zg_bound_half_width: (half-width, BOUND_CLT or BOUND_BERNSTEIN, met) of a running estimate."""
    h, m, ok = C.c_double(), C.c_uint32(), C.c_uint32()
    check(lib().zg_bound_half_width(mean, var, fourth_moment, n, hits, eps, conf, weight_range, C.byref(h),
                                    C.byref(m), C.byref(ok)))
    return h.value, m.value, bool(ok.value)


def merge_counters(parts):
    """Exact merge of runs over disjoint sample ranges (the multi-GPU shards): 320-bit sums add,
    hit/fail counts add, the mean is re-rounded once from the exact total."""
    from fractions import Fraction
    parts = list(parts)
    out = Counters()
    den = max(p.den_log2 for p in parts)
    total = 0
    for p in parts:
        v = sum(int(p.sum_num[i]) << (64 * i) for i in range(5))
        total += v << (den - p.den_log2)
        out.samples += p.samples
        out.hits += p.hits
        out.fails += p.fails
        out.overflow |= p.overflow
        out.sum_w += p.sum_w
        out.sum_w2 += p.sum_w2
    out.den_log2 = den
    for i in range(5):
        out.sum_num[i] = (total >> (64 * i)) & 0xFFFFFFFFFFFFFFFF
    out.estimate = float(Fraction(total, (1 << den) * out.samples)) if out.samples else 0.0
    return out


def allgather_counters(c, group=None):
    """torch.distributed all-gather of one rank's Counters as integer limbs, merged exactly on every
    rank (no floating-point reduction of the estimate)."""
    import torch
    import torch.distributed as dist
    words = [c.samples, c.hits, c.fails, c.den_log2, c.overflow] + [int(x) for x in c.sum_num]
    t = torch.tensor([w - (1 << 64) if w >= (1 << 63) else w for w in words], dtype=torch.int64)
    f = torch.tensor([c.sum_w, c.sum_w2], dtype=torch.float64)
    backend = dist.get_backend(group)
    if backend == "nccl":
        t, f = t.cuda(), f.cuda()
    ts = [torch.zeros_like(t) for _ in range(dist.get_world_size(group))]
    fs = [torch.zeros_like(f) for _ in range(dist.get_world_size(group))]
    dist.all_gather(ts, t, group=group)
    dist.all_gather(fs, f, group=group)
    parts = []
    for tt, ff in zip(ts, fs):
        w = [int(x) & 0xFFFFFFFFFFFFFFFF for x in tt.cpu().tolist()]
        p = Counters()
        p.samples, p.hits, p.fails, p.den_log2, p.overflow = w[0], w[1], w[2], w[3], w[4]
        for i in range(5):
            p.sum_num[i] = w[5 + i]
        p.sum_w, p.sum_w2 = [float(x) for x in ff.cpu().tolist()]
        parts.append(p)
    return merge_counters(parts)


MLP_FEATURES, MLP_OUTPUTS, MLP_PARAMS = 16, 2, 5378


def features(graph, program, pilot_samples=0, seed=1, cuda_stream=None):
    """zg_graph_features: 16 features of a (graph, program) query."""
    f = np.zeros(MLP_FEATURES, np.float32)
    check(lib().zg_graph_features(graph.handle, program.handle, pilot_samples, seed, cuda_stream, _ptr(f)))
    return f


class Mlp:
    """The learned ELP's network (zg_mlp_*): trained and evaluated by the library's CUDA kernels."""

    def __init__(self, seed=1):
        init()
        h = C.c_void_p()
        check(lib().zg_mlp_create(seed, C.byref(h)))
        self._h = h

    def params(self):
        p = np.zeros(MLP_PARAMS, np.float32)
        nrm = np.zeros(36, np.float32)
        check(lib().zg_mlp_get_params(self._h, _ptr(p), _ptr(nrm)))
        return p, nrm

    def set_params(self, params=None, norm=None):
        pp = None if params is None else np.ascontiguousarray(params, np.float32)
        nn = None if norm is None else np.ascontiguousarray(norm, np.float32)
        check(lib().zg_mlp_set_params(self._h, _ptr(pp), _ptr(nn)))

    def train(self, X, Y, epochs=200, batch=64, lr=3e-3, seed=7):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.ascontiguousarray(Y, np.float32)
        steps = max(1, epochs * len(X) // batch)
        loss = np.zeros(steps, np.float32)
        check(lib().zg_mlp_train(self._h, _ptr(X), _ptr(Y), len(X), epochs, batch, lr, seed, _ptr(loss)))
        return loss

    def grad(self, Xn, Yn):
        Xn = np.ascontiguousarray(Xn, np.float32)
        Yn = np.ascontiguousarray(Yn, np.float32)
        g = np.zeros(MLP_PARAMS, np.float32)
        loss = np.zeros(1, np.float32)
        check(lib().zg_mlp_grad(self._h, _ptr(Xn), _ptr(Yn), len(Xn), _ptr(g), _ptr(loss)))
        return g, float(loss[0])

    def predict(self, X):
        X = np.ascontiguousarray(X, np.float32).reshape(-1, MLP_FEATURES)
        Y = np.zeros((len(X), MLP_OUTPUTS), np.float32)
        check(lib().zg_mlp_predict(self._h, _ptr(X), len(X), _ptr(Y)))
        return Y

    def save(self, path):
        p, n = self.params()
        np.savez(path, params=p, norm=n)

    @classmethod
    def load(cls, path):
        d = np.load(path)
        m = cls()
        m.set_params(d["params"], d["norm"])
        return m

    def __del__(self):
        try:
            if self._h:
                lib().zg_mlp_free(self._h)
                self._h = None
        except Exception:
            pass


def learned_budget(mlp, graph, program, eps, conf, seed=1, pilot_samples=0):
    """zg_elp_learned: predicted per-sample relative variance -> n = z^2 * cv2 / eps^2.
    Returns (n, features, prediction)."""
    f = features(graph, program, pilot_samples, seed)
    n = C.c_uint64(0)
    y = np.zeros(2, np.float32)
    check(lib().zg_elp_learned(mlp._h, graph.handle, program.handle, eps, conf, pilot_samples, seed, None,
                               C.byref(n), _ptr(y)))
    return int(n.value), f, y


def learned_query(mlp, graph, program, eps, conf, seed, query_seed, stream_id=0, max_samples=0, cuda_stream=None):
    """zg_query_learned: learned sizing (adaptive pilot from seed), then the bound check from query_seed;
    a budget above 2^30 samples runs in two looks (half first).  Returns (QueryResult, budget)."""
    n = C.c_uint64(0)
    out = QueryResult()
    check(lib().zg_query_learned(mlp._h, graph.handle, program.handle, eps, conf, max_samples, seed, query_seed,
                                 stream_id, cuda_stream, C.byref(n), C.byref(out)))
    return out, int(n.value)


def run_three_motif(graph, n_chain, n_tri, seed, stream_chain=0, stream_tri=1, cuda_stream=None):
    a, b = Counters(), Counters()
    check(lib().zg_run_three_motif(graph.handle, n_chain, n_tri, seed, stream_chain, stream_tri, cuda_stream,
                                   C.byref(a), C.byref(b)))
    return a, b


def run_three_motif_debug(graph, n_chain, n_tri, seed, stream_chain=0, stream_tri=1):
    tc = np.zeros(max(1, n_chain), dtype=TRACE_DTYPE)
    tt = np.zeros(max(1, n_tri), dtype=TRACE_DTYPE)
    check(lib().zg_run_three_motif_debug(graph.handle, n_chain, n_tri, seed, stream_chain, stream_tri,
                                         _ptr(tc), _ptr(tt)))
    return tc[:n_chain], tt[:n_tri]


# ---- the reference's estimator interface --------------------------------------------------
class Estimation:
    """Running mean of finished estimators (src/ZGraphInstance.cpp:15-35)."""

    def __init__(self):
        self.reset()

    def reset(self):
        self.num_finished_estimators = 0
        self.current_estimation = 0.0

    def update(self, new_num_estimators, new_estimation):
        n, k = self.num_finished_estimators, new_num_estimators
        self.current_estimation = (1.0 * n / (n + k)) * self.current_estimation + (1.0 * k / (n + k)) * new_estimation
        self.num_finished_estimators = n + k

    def get_num_finished_estimators(self):
        return self.num_finished_estimators

    def get_currnet_estimation(self):
        return self.current_estimation


class ZGraphInstance:
    """ZGraphInstance<E> (include/ZGraphInstance.hpp:107-140) bound to one device program.

    calculate(n, k, init) runs n estimators on the GPU and folds their mean into init exactly as
    src/ZGraphInstance.cpp:257-297 does (one partition, one socket: scaling factor 1).  Each call
    consumes fresh sample indices of this instance's Philox stream.
    """

    program_kind = None
    program_param = 0

    def __init__(self, graph, seed=None, stream_id=0):
        init()
        self._graph = graph
        self.seed = int.from_bytes(os.urandom(8), "little") if seed is None else int(seed)
        self.stream_id = stream_id
        self.next_sample = 0
        self.program = self._make_program()
        self.last_counters = None

    def _make_program(self):
        return Program(self.program_kind, self.program_param)

    def get_graph(self):
        return self._graph

    def set_graph(self, graph):
        self._graph = graph

    def _sampling_graph(self):
        return self._graph

    def run(self, n, cuda_stream=None):
        """n estimators -> Counters (exact sums); advances the sample cursor."""
        c = self.program.run(self._sampling_graph(), n, self.seed, self.stream_id, self.next_sample, cuda_stream)
        self.next_sample += n
        self.last_counters = c
        return c

    def calculate(self, num_estimators, num_vertices_in_pattern, init_estimation):
        if init_estimation.get_num_finished_estimators() >= num_estimators:
            return init_estimation.get_currnet_estimation()
        n = num_estimators - init_estimation.get_num_finished_estimators()
        c = self.run(n)
        init_estimation.update(n, c.estimate)
        return init_estimation.get_currnet_estimation()

    def get_num_sample_edge_calls(self):
        return 1.0  # src/ZGraphInstance.cpp:450-452 returns 1 before measuring

    def get_num_conditional_sample_edge_calls(self):
        return float(self.program.info()["cond_calls"])


class TriangleCountingInstance(ZGraphInstance):
    """applications/Triangle.cpp:42-74."""
    program_kind = PROG_TRIANGLE


class FourCliqueCountingInstance(ZGraphInstance):
    """applications/FourClique.cpp:193-235."""
    program_kind = PROG_FOUR_CLIQUE


class ThreeChainCountingInstance(ZGraphInstance):
    """applications/ThreeChain.cpp:309-331."""
    program_kind = PROG_THREE_CHAIN


class FourChainCountingInstance(ZGraphInstance):
    """applications/FourChain.cpp:18-125."""
    program_kind = PROG_FOUR_CHAIN


class ChainMiningInstance(ZGraphInstance):
    """applications/ChainMining.cpp:213-85 (order k)."""
    program_kind = PROG_CHAIN

    def __init__(self, graph, order, seed=None, stream_id=0):
        self.program_param = int(order)
        super().__init__(graph, seed, stream_id)


class Pattern:
    """Pattern (include/SamplerGenerator.hpp:9-49): num_vertices, edges as (src, dst) pairs."""

    def __init__(self, num_vertices, num_edges, edges):
        self.num_vertices = int(num_vertices)
        self.edges = [(int(s), int(d)) for s, d in edges][:num_edges]
        if len(self.edges) != num_edges:
            raise ValueError("pattern lists %d edges, expected %d" % (len(self.edges), num_edges))

    def get_num_vertices(self):
        return self.num_vertices

    def get_num_edges(self):
        return len(self.edges)

    def is_in_edges_list(self, e):
        return any((a, b) == (e[0], e[1]) or (a, b) == (e[1], e[0]) for a, b in self.edges)

    def is_automorphic(self, other):
        """Pattern::is_automorphic (src/SamplerGenerator.cpp:307-324)."""
        if other.num_vertices != self.num_vertices or len(other.edges) != len(self.edges):
            return False
        return all(self.is_in_edges_list(e) for e in other.edges)

    def relabelled(self, mapping):
        return Pattern(self.num_vertices, len(self.edges), [(mapping[s], mapping[d]) for s, d in self.edges])


class SamplerGenerator(ZGraphInstance):
    """SamplerGenerator<Empty>(graph, pattern) (src/SamplerGenerator.cpp:393-546)."""
    program_kind = PROG_PATTERN

    def __init__(self, graph, pattern, seed=None, stream_id=0):
        self.pattern = pattern
        super().__init__(graph, seed, stream_id)
        self.num_unique_patterns = self.program.info()["num_unique"]

    def _make_program(self):
        return Program(PROG_PATTERN, pattern=(self.pattern.num_vertices, self.pattern.edges))

    def get_num_sample_edge_calls(self):
        return 1.0

    def get_num_conditional_sample_edge_calls(self):
        return float(self.pattern.get_num_edges() - 1)


class AllPredicateZGraphInstance(ZGraphInstance):
    """AllPredicateZGraphInstance<VertexId> (src/ZGraphInstance.cpp:492-525) running the triangle
    estimator of applications/AllPredicateWeightedTriangle.cpp:42-72 on the filtered graph.
    predicate = (op, t0[, t1]) with op one of PRED_*.
    """
    program_kind = PROG_TRIANGLE

    def __init__(self, graph, predicate, seed=None, stream_id=0, shuffle_seed=None):
        self.predicate = tuple(predicate)
        self.shuffle_seed = shuffle_seed
        self._filtered = None
        super().__init__(graph, seed, stream_id)
        self.set_graph(graph)

    def set_graph(self, graph):
        self._graph = graph
        op, t0 = self.predicate[0], self.predicate[1]
        t1 = self.predicate[2] if len(self.predicate) > 2 else 0
        sh = self.seed ^ 0x5A5A5A5A if self.shuffle_seed is None else self.shuffle_seed
        if self._filtered is not None:
            self._filtered.free()
        self._filtered = graph.filter(op, t0, t1, sh)

    def get_filtered_graph(self):
        return self._filtered

    def _sampling_graph(self):
        return self._filtered


class ThreeMotif:
    """applications/ThreeMotif.cpp:149-196: a 3-chain run whose wedges a triangle run re-closes
    (ZGraphInstanceWithCache), fused into one kernel."""

    def __init__(self, graph, seed=None):
        init()
        self.graph = graph
        self.seed = int.from_bytes(os.urandom(8), "little") if seed is None else int(seed)

    def calculate(self, n_chain, n_tri):
        a, b = run_three_motif(self.graph, n_chain, n_tri, self.seed)
        return a.estimate, b.estimate, a, b
