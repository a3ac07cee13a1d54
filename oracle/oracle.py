"""ctypes wrapper of the CPU ORACLE (oracle/zg_oracle.c) — test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may import this module;
the product path (libzgraph_gpu.so and its binding) never does.  Also wraps the drivers that
oracle/build_ref.sh builds from the reference's own sources (oracle/_ref/), when present.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "_build", "libzgoracle.so")
REF_DIR = os.path.join(HERE, "_ref")

MAX_DRAWS = 16
TRACE_DTYPE = np.dtype([("ndraws", "<u4"), ("hit", "<u4"), ("fail", "<u4"), ("shift", "<u4"),
                        ("sectors", "<u4"), ("closures", "<u4"), ("w", "<f8"), ("num", "<u8", (3,)), ("lo", "<u8", (MAX_DRAWS,)),
                        ("hi", "<u8", (MAX_DRAWS,)), ("val", "<u8", (MAX_DRAWS,))])


class _Graph(C.Structure):
    _fields_ = [("nv", C.c_uint32), ("m", C.c_uint64), ("num_edges", C.c_uint64), ("max_degree", C.c_uint64),
                ("src", C.c_void_p), ("dst", C.c_void_p), ("w", C.c_void_p), ("off", C.c_void_p),
                ("adj_nbr", C.c_void_p), ("adj_eid", C.c_void_p), ("adj_w", C.c_void_p)]


class _Program(C.Structure):
    _fields_ = [("kind", C.c_int), ("param", C.c_uint32), ("pv", C.c_uint32), ("pe", C.c_uint32),
                ("pedges", C.c_uint32 * 32), ("num_unique", C.c_uint32), ("unique_edges", C.c_void_p)]


class Counters(C.Structure):
    _fields_ = [("samples", C.c_uint64), ("hits", C.c_uint64), ("fails", C.c_uint64),
                ("den_log2", C.c_uint32), ("overflow", C.c_uint32), ("sum_num", C.c_uint64 * 5),
                ("sum_w", C.c_double), ("sum_w2", C.c_double), ("estimate", C.c_double),
                ("sum_w4", C.c_double)]

    def exact_sum(self):
        from fractions import Fraction
        v = 0
        for i in range(5):
            v |= int(self.sum_num[i]) << (64 * i)
        return Fraction(v, 1 << self.den_log2)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_LIB):
            raise RuntimeError("oracle library not built: %s" % ORACLE_LIB)
        L = C.CDLL(ORACLE_LIB)
        P, U32, U64, I64, I32, D = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int64, C.c_int, C.c_double
        sig = {
            "zgo_graph_build": ([C.POINTER(_Graph), U32, U64, P, P], I32),
            "zgo_graph_free": ([C.POINTER(_Graph)], None),
            "zgo_program_init": ([C.POINTER(_Program), I32, U32, U32, U32, P], I32),
            "zgo_program_free": ([C.POINTER(_Program)], None),
            "zgo_philox4x32_10": ([P, P, P], None),
            "zgo_draw": ([U64, U32, U64, U32, U64, U64], U64),
            "zgo_sample": ([C.POINTER(_Graph), C.POINTER(_Program), U64, U32, U64, P], I32),
            "zgo_run": ([C.POINTER(_Graph), C.POINTER(_Program), U64, U64, U64, U32, I32, C.POINTER(Counters), P],
                        I32),
            "zgo_run_three_motif": ([C.POINTER(_Graph), U64, U64, U64, U32, U32, C.POINTER(Counters),
                                     C.POINTER(Counters), P, P], I32),
            "zgo_pred": ([I32, I64, I64, U32], I32),
            "zgo_subsample_keep": ([D, U64, U64], I32),
            "zgo_shuffle_perm": ([U64, U64, P], None),
            "zgo_shuffle_key": ([U64, U64], U64),
            "zgo_subsample_edges": ([P, U64, D, U64, U64, U64, P, C.POINTER(C.c_uint64)], I32),
            "zgo_exact_naive": ([C.POINTER(_Graph), I32, P], I32),
            "zgo_exact_fast": ([C.POINTER(_Graph), I32, P], I32),
            "zgo_exact_weighted_triangle": ([C.POINTER(_Graph), U32, I32, P], I32),
            "zgo_calculate_bound": ([D, D, D, D, D, U64, U64], D),
            "zgo_regression_k": ([P, P, U32], D),
            "zgo_ext_inv_product": ([P, I32], D),
            "zgo_gen_rmat": ([U32, U32, D, D, D, U64, U64, P, C.POINTER(C.c_uint64)], I32),
            "zgo_conditional_close_ids": ([C.POINTER(_Graph), U64, P, U32, P, U32, P, C.POINTER(C.c_uint32)], I32),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class OracleGraph:
    """Graph<E> restated on the host (one partition, one socket), edge ids = positions."""

    def __init__(self, edges, num_vertices, weights=None):
        self.edges = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1, 2)
        self.weights = None if weights is None else np.ascontiguousarray(weights, dtype=np.uint32)
        self.num_vertices = int(num_vertices)
        self.g = _Graph()
        rc = lib().zgo_graph_build(C.byref(self.g), self.num_vertices, self.edges.shape[0], _p(self.edges),
                                   _p(self.weights))
        if rc != 0:
            lib().zgo_graph_free(C.byref(self.g))
            raise ValueError("oracle graph build failed (%d)" % rc)

    @property
    def m(self):
        return self.g.m

    @property
    def max_degree(self):
        return self.g.max_degree

    def arrays(self):
        m, nv = self.g.m, self.g.nv
        def arr(ptr, n, dt):
            if not ptr or n == 0:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dt))), (n,)).copy()
        return {"off": arr(self.g.off, nv + 1, np.uint64), "adj_nbr": arr(self.g.adj_nbr, 2 * m, np.uint32),
                "adj_eid": arr(self.g.adj_eid, 2 * m, np.uint64)}

    def conditional_close(self, min_valid, vertices, edges):
        """conditional_close(min_valid, vertices, edges&) (src/ZGraphInstance.cpp:410-441):
        (closed, found, edge ids of the found edges)."""
        v = np.ascontiguousarray(vertices, dtype=np.uint32)
        e = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1, 2)
        ids = np.zeros(max(1, len(e)), np.uint64)
        found = C.c_uint32(0)
        closed = lib().zgo_conditional_close_ids(C.byref(self.g), min_valid, _p(v), len(v), _p(e), len(e), _p(ids),
                                                 C.byref(found))
        return bool(closed), int(found.value), ids[:found.value].copy()

    def exact_naive(self, kind):
        out = (C.c_uint64 * 2)()
        rc = lib().zgo_exact_naive(C.byref(self.g), kind, out)
        assert rc == 0
        return int(out[0]) | (int(out[1]) << 64)

    def exact_fast(self, kind):
        out = (C.c_uint64 * 2)()
        rc = lib().zgo_exact_fast(C.byref(self.g), kind, out)
        assert rc == 0
        return int(out[0]) | (int(out[1]) << 64)

    def exact_weighted_triangle(self, threshold, at_least_one):
        out = (C.c_uint64 * 2)()
        rc = lib().zgo_exact_weighted_triangle(C.byref(self.g), threshold, int(at_least_one), out)
        assert rc == 0
        return int(out[0]) | (int(out[1]) << 64)

    def __del__(self):
        try:
            lib().zgo_graph_free(C.byref(self.g))
        except Exception:
            pass


class OracleProgram:
    def __init__(self, kind, param=0, pattern=None):
        self.p = _Program()
        if pattern is not None:
            nv, edges = pattern
            e = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1, 2)
            rc = lib().zgo_program_init(C.byref(self.p), kind, param, nv, e.shape[0], _p(e))
        else:
            rc = lib().zgo_program_init(C.byref(self.p), kind, param, 0, 0, None)
        if rc != 0:
            raise ValueError("oracle program init failed (%d)" % rc)

    @property
    def num_unique(self):
        return self.p.num_unique

    def __del__(self):
        try:
            lib().zgo_program_free(C.byref(self.p))
        except Exception:
            pass


def traces(graph, prog, n, seed, stream=0, first=0, threads=0):
    """Per-sample traces (and the run's counters) of samples [first, first + n); each sample's trace
    is independent of the thread that computes it."""
    tr = np.zeros(n, dtype=TRACE_DTYPE)
    c = Counters()
    rc = lib().zgo_run(C.byref(graph.g), C.byref(prog.p), n, first, seed, stream, threads, C.byref(c), _p(tr))
    assert rc == 0
    return tr, c


def run(graph, prog, n, seed, stream=0, first=0, threads=0):
    c = Counters()
    rc = lib().zgo_run(C.byref(graph.g), C.byref(prog.p), n, first, seed, stream, threads, C.byref(c), None)
    assert rc == 0
    return c


def three_motif(graph, n_chain, n_tri, seed, stream_chain=0, stream_tri=1):
    tc = np.zeros(max(1, n_chain), dtype=TRACE_DTYPE)
    tt = np.zeros(max(1, n_tri), dtype=TRACE_DTYPE)
    a, b = Counters(), Counters()
    rc = lib().zgo_run_three_motif(C.byref(graph.g), n_chain, n_tri, seed, stream_chain, stream_tri, C.byref(a),
                                   C.byref(b), _p(tc), _p(tt))
    assert rc == 0
    return tc[:n_chain], tt[:n_tri], a, b


def gen_rmat(scale, edge_factor, a=0.57, b=0.19, c=0.19, seed=1):
    """Seeded R-MAT edge list built on the host (oracle/zgo_gen.c): the library's zg_gen_rmat
    graph, edge for edge, without loading the GPU library.  Returns an (m, 2) uint32 array."""
    cap = edge_factor << scale  # every draw kept: an upper bound on the edge count
    out = np.empty((cap, 2), dtype=np.uint32)
    m = C.c_uint64(0)
    rc = lib().zgo_gen_rmat(scale, edge_factor, a, b, c, seed, cap, _p(out), C.byref(m))
    if rc != 0:
        raise ValueError("zgo_gen_rmat failed (%d)" % rc)
    return out[:m.value]


def draw(seed, stream, sample, d, lo, hi):
    return lib().zgo_draw(seed, stream, sample, d, lo, hi)


def philox(ctr, key):
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    lib().zgo_philox4x32_10(_p(c), _p(k), _p(o))
    return [int(x) for x in o]


def shuffle_perm(m, seed):
    p = np.zeros(max(1, m), dtype=np.uint64)
    lib().zgo_shuffle_perm(m, seed, _p(p))
    return p[:m]


def subsample_edges(edges, rate, keep_seed, shuffle_seed):
    """GraphSampler::sample_graph's kept edges in the device's draw plan (zgo_subsample_edges): the
    edge list zg_graph_subsample(rate, keep_seed, shuffle_seed) builds its graph from."""
    e = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1, 2)
    out = np.empty((max(1, e.shape[0]), 2), np.uint32)  # pages past the kept edges are never touched
    k = C.c_uint64(0)
    rc = lib().zgo_subsample_edges(_p(e), e.shape[0], rate, keep_seed, shuffle_seed, e.shape[0], _p(out), C.byref(k))
    if rc != 0:
        raise ValueError("zgo_subsample_edges failed (%d)" % rc)
    return out[:k.value]


# zg_elp_plain's draw plan (ZG_ELP_* in include/zgraph_gpu.h), so that the CPU arm needs no GPU library
ELP_KEEP_OFFSET, ELP_SHUFFLE_OFFSET, ELP_FILTER_OFFSET, ELP_STREAM = 1, 2, 3, 0x454C5000


def elp_solve(groups, group_size, big_estimate, big_n, nse, ncse, sampled_m, sampled_max_degree, orig_m,
              orig_max_degree, eps, conf):
    """The host half of ErrorProfile::get_num_estimators (src/ErrorLatencyProfile.cpp:115-206) with
    its long double intermediates: the running estimate after each group (Estimation::update,
    src/ZGraphInstance.cpp:24-27), the moving average of the scaled error, the regression
    through the origin (UnbiasedLinearRegression::solve, src/Regression.cpp:17-28) and the bound
    on the original graph.  Returns the estimator count as a float (the reference truncates it)."""
    LD = np.longdouble
    n, cur = 0, 0.0
    running = []
    for v in groups:
        cur = (1.0 * n / (n + group_size)) * cur + (1.0 * group_size / (n + group_size)) * float(v)
        n += group_size
        running.append(cur)
    est = (1.0 * n / (n + big_n)) * cur + (1.0 * big_n / (n + big_n)) * float(big_estimate)
    ema, alpha = LD(100), 0.04
    t0, t1 = LD(0), LD(0)
    xs, ys = [], []
    for i, r in enumerate(running):
        err = (LD(r) - LD(est)) / LD(est) * LD(5)
        if err < 0:
            err = -err
        ema = ema * LD(1 - alpha) + err * LD(alpha)
        x_tmp = float(LD(calculate_bound(float(ema), 1 - conf, nse, ncse, est, sampled_max_degree, sampled_m)) *
                      (ema * ema))
        xs.append(LD(np.sqrt(x_tmp / ((i + 1) * group_size))))
        ys.append(ema)
    for x, y in zip(xs, ys):
        t0 += x * y
    for x in xs:
        t1 += x * x
    k = float(t0 / t1)
    rough = float(LD(est) / LD(0.1) ** LD(nse + ncse))
    return calculate_bound(eps, 1 - conf, nse, ncse, rough, orig_max_degree, orig_m) * (k * k)


def plain_elp(edges, num_vertices, program, ncse, seed, eps, conf, orig_m, orig_max_degree, threads=0):
    """ErrorProfile::get_num_estimators (src/ErrorLatencyProfile.cpp:72-207) on the host with
    zg_elp_plain's draw plan: the 10 % edge subsample, 2^14 groups of 16 estimators (each group's
    mean summed in sample order, as a one-threaded calculate(16) does) and 2^23 more estimators on
    it, then the regression and the bound.  Returns the estimator count (truncated)."""
    sub = subsample_edges(edges, 0.1, seed + ELP_KEEP_OFFSET, seed + ELP_SHUFFLE_OFFSET)
    og = OracleGraph(sub, num_vertices)
    tr, _ = traces(og, program, 1 << 18, seed, stream=ELP_STREAM, threads=threads)
    w = tr["w"].reshape(-1, 16)
    acc = np.zeros(w.shape[0])
    for j in range(16):  # sample order within each group
        acc = acc + w[:, j]
    big = run(og, program, 1 << 23, seed, ELP_STREAM, 1 << 18, threads)
    n = elp_solve(acc / 16.0, 16, float(big.exact_sum() / big.samples), 1 << 23, 1.0, float(ncse), og.m,
                  og.max_degree, orig_m, orig_max_degree, eps, conf)
    return int(n)


def pred(op, t0, t1, w):
    return bool(lib().zgo_pred(op, t0, t1, w))


def subsample_keep(rate, seed, e):
    return bool(lib().zgo_subsample_keep(rate, seed, e))


def calculate_bound(eps, delta, nse, ncse, est, maxdeg, m):
    return lib().zgo_calculate_bound(eps, delta, nse, ncse, est, maxdeg, m)


def regression_k(x, y):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    return lib().zgo_regression_k(_p(x), _p(y), len(x))


def ext_inv_product(factors):
    f = np.ascontiguousarray(factors, dtype=np.float64)
    return lib().zgo_ext_inv_product(_p(f), len(f))


# ---- drivers around the reference's own sources (built here only) -------------------------
REF_APPS = ("triangle", "four_clique", "three_chain", "four_chain", "chain", "pred_triangle", "three_motif",
            "pattern")


def ref_available():
    return all(os.path.exists(os.path.join(REF_DIR, "libzgref_%s.so" % a)) for a in REF_APPS)


_ref = {}


def ref_lib(app):
    if app not in _ref:
        path = os.path.join(REF_DIR, "libzgref_%s.so" % app)
        L = C.CDLL(path, mode=C.RTLD_LOCAL)
        P, U32, U64, D = C.c_void_p, C.c_uint32, C.c_uint64, C.c_double
        L.zgref_open.argtypes = [P, U64, U32, P, U32, P, U64, P, U32, U32]
        L.zgref_open.restype = P
        L.zgref_estimates.argtypes = [P, U64, P, P, P]
        L.zgref_estimates.restype = U64
        L.zgref_calculate.argtypes = [P, U64, U32, P, C.POINTER(U64)]
        L.zgref_calculate.restype = D
        L.zgref_close.argtypes = [P]
        L.zgref_close.restype = None
        if app == "three_motif":
            L.zgref_motif.argtypes = [P, U64, U32, U64, U64, P, P, C.POINTER(D), C.POINTER(D)]
            L.zgref_motif.restype = U64
        L.zgref_elp.argtypes = [P, U64, U32, C.c_int, U32, P, U32, U32, U64, U32, D, D, C.POINTER(U64)]
        L.zgref_elp.restype = U64
        if app == "pattern":
            L.zgref_regression_k.argtypes = [P, P, U32]
            L.zgref_regression_k.restype = D
            L.zgref_calculate_bound.argtypes = [D, D, D, D, D, U64, U64]
            L.zgref_calculate_bound.restype = D
            L.zgref_estimation_fold.argtypes = [P, P, U32]
            L.zgref_estimation_fold.restype = D
        _ref[app] = L
    return _ref[app]


class RefInstance:
    """One reference application instance on a graph in the given edge order."""

    def __init__(self, app, edges, num_vertices, weights=None, param=0, filter_perm=None, pattern=None):
        self.L = ref_lib(app)
        self.edges = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1, 2)
        self.weights = None if weights is None else np.ascontiguousarray(weights, dtype=np.uint32)
        fp = None if filter_perm is None else np.ascontiguousarray(filter_perm, dtype=np.uint64)
        pv, pe, pedges = 0, 0, None
        if pattern is not None:
            pv, pedges = pattern
            pedges = np.ascontiguousarray(pedges, dtype=np.uint32).reshape(-1, 2)
            pe = pedges.shape[0]
        self.h = self.L.zgref_open(_p(self.edges), self.edges.shape[0], num_vertices, _p(self.weights), param,
                                   _p(fp), 0 if fp is None else len(fp), _p(pedges), pv, pe)

    def estimates(self, tr):
        out = np.zeros(len(tr), dtype=np.float64)
        used = np.zeros(len(tr), dtype=np.uint32)
        bad = self.L.zgref_estimates(self.h, len(tr), _p(tr), _p(out), _p(used))
        return out, used, int(bad)

    def calculate(self, tr, k=3):
        bad = C.c_uint64(0)
        r = self.L.zgref_calculate(self.h, len(tr), k, _p(tr), C.byref(bad))
        return r, int(bad.value)

    def close(self):
        if self.h:
            self.L.zgref_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ref_elp(app, edges, num_vertices, kind, param=0, pattern=None, seed=1, probe_stream=0x50524F42, eps=0.05,
            conf=0.95):
    """The reference's ErrorProfile::get_num_estimators, replaying the zg_elp_plain draw plan."""
    L = ref_lib(app)
    e = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1, 2)
    pv, pe, pedges = 0, 0, None
    if pattern is not None:
        pv, pedges = pattern
        pedges = np.ascontiguousarray(pedges, dtype=np.uint32).reshape(-1, 2)
        pe = pedges.shape[0]
    bad = C.c_uint64(0)
    n = L.zgref_elp(_p(e), e.shape[0], num_vertices, kind, param, _p(pedges), pv, pe, seed, probe_stream, eps, conf,
                    C.byref(bad))
    return int(n), int(bad.value)


def ref_motif(edges, num_vertices, n_chain, n_tri, chain_tr, tri_tr):
    L = ref_lib("three_motif")
    e = np.ascontiguousarray(edges, dtype=np.uint32).reshape(-1, 2)
    a, b = C.c_double(), C.c_double()
    bad = L.zgref_motif(_p(e), e.shape[0], num_vertices, n_chain, n_tri, _p(chain_tr), _p(tri_tr), C.byref(a),
                        C.byref(b))
    return a.value, b.value, int(bad)
