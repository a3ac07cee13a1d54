"""GPU parity: libzgraph_gpu.so (through its C ABI) against the CPU oracle on the same seeded inputs.

Bit-exact for everything: per-sample draws (value and requested range), outcomes, 192-bit
numerators, the reference double 1/p, the access-model sector counts, the exact 320-bit sums,
the device-built adjacency arrays, derived (filtered / subsampled) graphs and exact counts.
"""
import numpy as np
import pytest

import oracle as O
import zgraph as Z

pytestmark = pytest.mark.gpu

FIELDS = ("ndraws", "hit", "fail", "shift", "sectors", "closures", "num", "lo", "hi", "val")

STAR = (5, [(0, 1), (0, 2), (0, 3), (0, 4)])                     # applications/FiveStar.cpp:18-26
HOUSE = (5, [(0, 1), (0, 2), (1, 2), (1, 3), (2, 4), (3, 4)])     # applications/FiveHouse.cpp:18-27
TRI = (3, [(0, 1), (0, 2), (1, 2)])                               # applications/Triangle2.cpp:18-24
CYCLE4 = (4, [(0, 1), (1, 2), (2, 3), (3, 0)])
CHAIN5 = (5, [(0, 1), (1, 2), (2, 3), (3, 4)])
CLIQUE4 = (4, [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)])

PROGRAMS = [
    ("triangle", Z.PROG_TRIANGLE, 0, None),
    ("four_clique", Z.PROG_FOUR_CLIQUE, 0, None),
    ("three_chain", Z.PROG_THREE_CHAIN, 0, None),
    ("four_chain", Z.PROG_FOUR_CHAIN, 0, None),
    ("chain3", Z.PROG_CHAIN, 3, None),
    ("chain4", Z.PROG_CHAIN, 4, None),
    ("chain6", Z.PROG_CHAIN, 6, None),
    ("chain9", Z.PROG_CHAIN, 9, None),
    ("star", Z.PROG_PATTERN, 0, STAR),
    ("house", Z.PROG_PATTERN, 0, HOUSE),
    ("tri_pattern", Z.PROG_PATTERN, 0, TRI),
    ("cycle4", Z.PROG_PATTERN, 0, CYCLE4),
    ("chain5_pattern", Z.PROG_PATTERN, 0, CHAIN5),
    ("clique4_pattern", Z.PROG_PATTERN, 0, CLIQUE4),
    ("four_clique_unbiased", Z.PROG_FOUR_CLIQUE_UNBIASED, 0, None),
]


def _graphs():
    out = {}
    e = Z.gen_rmat(10, 8, seed=3)
    out["rmat10"] = (e, 1 << 10)
    e = Z.gen_rmat(12, 16, seed=5)
    out["rmat12"] = (e, 1 << 12)
    e = Z.gen_chung_lu(3000, 2.3, 12.0, seed=9)
    out["chunglu3k"] = (e, 3000)
    # dense small graph so that the house and 4-clique programs hit often
    e = Z.gen_rmat(7, 30, a=0.45, b=0.2, c=0.2, seed=2)
    out["dense7"] = (e, 1 << 7)
    return out


@pytest.fixture(scope="module")
def graphs():
    Z.init(0)
    return _graphs()


def _assert_traces(gt, ot, label):
    for f in FIELDS:
        if not np.array_equal(gt[f], ot[f]):
            bad = np.nonzero(np.any((gt[f] != ot[f]).reshape(len(gt), -1), axis=1))[0]
            i = int(bad[0])
            raise AssertionError("%s: field %s differs at sample %d of %d: gpu=%s oracle=%s"
                                 % (label, f, i, len(bad), gt[i], ot[i]))
    assert np.array_equal(gt["w"].view(np.uint64), ot["w"].view(np.uint64)), label + ": reference doubles differ"


def _sums(c):
    return [int(x) for x in c.sum_num]


@pytest.mark.parametrize("gname", ["rmat10", "rmat12", "chunglu3k", "dense7"])
def test_graph_build_matches_oracle(graphs, gname):
    e, nv = graphs[gname]
    g = Z.Graph.from_edges(e, nv)
    d = g.download()
    og = O.OracleGraph(e, nv)
    a = og.arrays()
    assert np.array_equal(d["edges"], e)
    assert np.array_equal(d["offsets"].astype(np.uint64), a["off"])
    assert np.array_equal(d["adj_e"][:, 0], a["adj_nbr"])
    assert np.array_equal(d["adj_e"][:, 1].astype(np.uint64), a["adj_eid"])
    off = d["offsets"]
    deg = np.diff(off)
    owner = np.repeat(np.arange(nv), deg)
    # neighbour order: sorted by (vertex, nbr, edge id)
    key = owner.astype(np.uint64) << np.uint64(32) | d["adj_n"][:, 0].astype(np.uint64)
    assert np.all(np.diff(key.astype(np.int64)) > 0)
    same = np.lexsort((d["adj_e"][:, 1], d["adj_e"][:, 0], owner))
    assert np.array_equal(d["adj_n"], d["adj_e"][same])
    # suffix counts: entries after the edge in each endpoint's edge-id-ordered list
    pos = np.arange(len(owner))
    suf = off[owner + 1] - 1 - pos
    eid = d["adj_e"][:, 1]
    is_src = d["edges"][eid, 0] == owner
    assert np.array_equal(d["suffix"][eid[is_src], 0], suf[is_src])
    assert np.array_equal(d["suffix"][eid[~is_src], 1], suf[~is_src])
    assert g.max_degree == og.max_degree == deg.max()


@pytest.mark.parametrize("gname", ["rmat10", "chunglu3k", "dense7"])
@pytest.mark.parametrize("name,kind,param,pattern", PROGRAMS, ids=[p[0] for p in PROGRAMS])
def test_traces_bit_exact(graphs, gname, name, kind, param, pattern):
    e, nv = graphs[gname]
    g = Z.Graph.from_edges(e, nv)
    og = O.OracleGraph(e, nv)
    n, seed = 20000, 77
    gp = Z.Program(kind, param, pattern)
    op = O.OracleProgram(kind, param, pattern)
    if kind == Z.PROG_PATTERN:
        assert gp.info()["num_unique"] == op.num_unique
    gt = gp.run_debug(g, n, seed, stream_id=3, first_sample=1000)
    ot, oc = O.traces(og, op, n, seed, stream=3, first=1000)
    _assert_traces(gt, ot, "%s/%s" % (gname, name))
    c = gp.run(g, n, seed, stream_id=3, first_sample=1000)
    assert (c.samples, c.hits, c.fails) == (oc.samples, oc.hits, oc.fails)
    assert _sums(c) == _sums(oc)
    assert c.den_log2 == oc.den_log2


@pytest.mark.parametrize("name,kind,param,pattern", PROGRAMS[:8], ids=[p[0] for p in PROGRAMS[:8]])
def test_counters_exact_at_scale(graphs, name, kind, param, pattern):
    e, nv = graphs["rmat12"]
    g = Z.Graph.from_edges(e, nv)
    og = O.OracleGraph(e, nv)
    n = 1 << 20
    c = Z.Program(kind, param, pattern).run(g, n, 99)
    oc = O.run(og, O.OracleProgram(kind, param, pattern), n, 99)
    assert (c.samples, c.hits, c.fails) == (oc.samples, oc.hits, oc.fails)
    assert _sums(c) == _sums(oc)
    # the exact mean, rounded once
    ex = c.exact_sum() / c.samples
    assert c.estimate == float(ex)


def test_three_motif_matches_oracle(graphs):
    e, nv = graphs["rmat10"]
    g = Z.Graph.from_edges(e, nv)
    og = O.OracleGraph(e, nv)
    for n_chain, n_tri in ((5000, 8000), (8000, 5000), (0, 3000), (3000, 0)):
        tc, tt = Z.run_three_motif_debug(g, n_chain, n_tri, 31, 4, 5)
        oc_, ot_, a, b = O.three_motif(og, n_chain, n_tri, 31, 4, 5)
        if n_chain:
            _assert_traces(tc, oc_, "motif chain")
        if n_tri:
            _assert_traces(tt, ot_, "motif triangle")
        ca, cb = Z.run_three_motif(g, n_chain, n_tri, 31, 4, 5)
        assert _sums(ca) == _sums(a) and _sums(cb) == _sums(b)
        assert (ca.hits, cb.hits) == (a.hits, b.hits)


def test_filter_and_subsample_match_oracle(graphs):
    e, nv = graphs["chunglu3k"]
    w = Z.gen_weights(len(e), 100, seed=4)
    g = Z.Graph.from_edges(e, nv, weights=w)
    for op, t0, t1 in ((Z.PRED_GE, 50, 0), (Z.PRED_LT, 50, 0), (Z.PRED_RANGE, 10, 90), (Z.PRED_EQ, 7, 0)):
        for sh in (Z.NO_SHUFFLE, 12345):
            f = g.filter(op, t0, t1, sh)
            keep = np.array([O.pred(op, t0, t1, int(x)) for x in w], dtype=bool)
            idx = np.nonzero(keep)[0]
            if sh != Z.NO_SHUFFLE:
                idx = idx[O.shuffle_perm(len(idx), sh).astype(np.int64)]
            assert np.array_equal(f.parent_index, idx.astype(np.uint64))
            d = f.download()
            assert np.array_equal(d["edges"], e[idx])
            assert np.array_equal(d["weights"], w[idx])
            assert f.num_edges == len(idx)  # one partition: sample_rate_after_partition == 1
            # the triangle program on the filtered graph
            og = O.OracleGraph(e[idx], nv)
            gt = Z.Program(Z.PROG_TRIANGLE).run_debug(f, 4000, 5)
            ot, _ = O.traces(og, O.OracleProgram(Z.PROG_TRIANGLE), 4000, 5)
            _assert_traces(gt, ot, "filtered triangle")
    s = g.subsample(0.1, keep_seed=8, shuffle_seed=9)
    keep = np.array([O.subsample_keep(0.1, 8, i) for i in range(len(e))], dtype=bool)
    idx = np.nonzero(keep)[0]
    idx = idx[O.shuffle_perm(len(idx), 9).astype(np.int64)]
    assert np.array_equal(s.parent_index, idx.astype(np.uint64))
    assert np.array_equal(s.download()["edges"], e[idx])


def test_permuted_graph_matches_oracle(graphs):
    e, nv = graphs["rmat10"]
    g = Z.Graph.from_edges(e, nv, shuffle_seed=606)
    perm = O.shuffle_perm(len(e), 606).astype(np.int64)
    assert np.array_equal(g.parent_index, perm.astype(np.uint64))
    assert np.array_equal(g.download()["edges"], e[perm])


@pytest.mark.parametrize("gname", ["rmat10", "chunglu3k", "dense7"])
def test_exact_counts_match_oracle(graphs, gname):
    e, nv = graphs[gname]
    g = Z.Graph.from_edges(e, nv)
    og = O.OracleGraph(e, nv)
    for kind in (Z.EXACT_TRIANGLE, Z.EXACT_WEDGE, Z.EXACT_THREE_PATH, Z.EXACT_FIVE_STAR, Z.EXACT_FOUR_CLIQUE,
                 Z.EXACT_FIVE_HOUSE, Z.EXACT_FIVE_CHAIN):
        assert g.exact_count(kind) == og.exact_fast(kind), kind
    if gname != "chunglu3k":
        for kind in (Z.EXACT_TRIANGLE, Z.EXACT_WEDGE, Z.EXACT_THREE_PATH, Z.EXACT_FIVE_STAR):
            assert g.exact_count(kind) == og.exact_naive(kind), kind
    # a graph built without the neighbour-ordered adjacency sorts its own lists
    gs = Z.Graph.gen_rmat(10, 8, seed=3, sampling_only=True) if gname == "rmat10" else None
    if gs is not None:
        for kind in (Z.EXACT_FIVE_HOUSE, Z.EXACT_FIVE_CHAIN, Z.EXACT_TRIANGLE):
            assert gs.exact_count(kind) == og.exact_fast(kind), kind


def test_weighted_exact_counts_match_oracle(graphs):
    e, nv = graphs["chunglu3k"]
    w = Z.gen_weights(len(e), 100, seed=4)
    g = Z.Graph.from_edges(e, nv, weights=w)
    og = O.OracleGraph(e, nv, w)
    for t in (0, 10, 50, 90, 100):
        assert g.exact_count_weighted(Z.EXACT_WEIGHTED_TRIANGLE, t) == og.exact_weighted_triangle(t, False), t
        assert g.exact_count_weighted(Z.EXACT_AT_LEAST_ONE_TRIANGLE, t) == og.exact_weighted_triangle(t, True), t
    assert g.exact_count_weighted(Z.EXACT_WEIGHTED_TRIANGLE, 0) == g.exact_count(Z.EXACT_TRIANGLE)
    with pytest.raises(Z.ZgError):
        Z.Graph.from_edges(e, nv).exact_count_weighted(Z.EXACT_WEIGHTED_TRIANGLE, 50)  # no edge data
    with pytest.raises(Z.ZgError):
        g.exact_count(Z.EXACT_WEIGHTED_TRIANGLE)  # takes a threshold: zg_exact_count_weighted


def test_edge_cases(graphs):
    Z.init(0)
    # empty graph: every sample fails (sample_edge returns p < 0, src/ZGraphInstance.cpp:322-324)
    g = Z.Graph.from_edges(np.zeros((0, 2), np.uint32), 4)
    c = Z.Program(Z.PROG_TRIANGLE).run(g, 1000, 1)
    assert (c.samples, c.hits, c.fails) == (1000, 0, 1000)
    assert g.exact_count(Z.EXACT_TRIANGLE) == 0
    # single edge: the conditional step finds nothing after it
    g = Z.Graph.from_edges(np.array([[0, 1]], np.uint32), 2)
    for kind in (Z.PROG_TRIANGLE, Z.PROG_THREE_CHAIN, Z.PROG_FOUR_CLIQUE):
        c = Z.Program(kind).run(g, 500, 1)
        assert c.fails == 500 and c.hits == 0
    # a triangle with isolated vertices around it, every program against the oracle
    e = np.array([[5, 2], [2, 9], [9, 5]], np.uint32)
    g = Z.Graph.from_edges(e, 12)
    og = O.OracleGraph(e, 12)
    for name, kind, param, pat in PROGRAMS:
        gt = Z.Program(kind, param, pat).run_debug(g, 3000, 8)
        ot, _ = O.traces(og, O.OracleProgram(kind, param, pat), 3000, 8)
        _assert_traces(gt, ot, "tiny/" + name)
    # invalid inputs are rejected with INVALID_GRAPH, not sampled
    for bad, nv in (([[0, 0]], 2), ([[0, 1], [1, 0]], 2), ([[0, 5]], 3)):
        with pytest.raises(Z.ZgError) as ex:
            Z.Graph.from_edges(np.array(bad, np.uint32), nv)
        assert ex.value.code == 4
    with pytest.raises(Z.ZgError):
        Z.Program(Z.PROG_CHAIN, 2)
    with pytest.raises(Z.ZgError):
        Z.Program(Z.PROG_PATTERN, pattern=(9, [(i, i + 1) for i in range(8)]))


def test_determinism_and_additivity(graphs):
    """Philox counters make runs reproducible and splittable by sample range (the multi-GPU shard)."""
    e, nv = graphs["rmat12"]
    g = Z.Graph.from_edges(e, nv)
    p = Z.Program(Z.PROG_FOUR_CLIQUE)
    a = p.run(g, 1 << 18, 5)
    b = p.run(g, 1 << 18, 5)
    assert _sums(a) == _sums(b) and a.sum_w == b.sum_w
    h1 = p.run(g, 100000, 5, first_sample=0)
    h2 = p.run(g, (1 << 18) - 100000, 5, first_sample=100000)
    assert h1.exact_sum() + h2.exact_sum() == a.exact_sum()
    assert h1.hits + h2.hits == a.hits


@pytest.mark.parametrize("name,kind,param,pattern", PROGRAMS[:9], ids=[p[0] for p in PROGRAMS[:9]])
def test_launch_variants_agree(graphs, name, kind, param, pattern):
    """Every launch shape (register cap / grid) gives the same exact sums; zg_tune keeps one."""
    L = Z.lib()
    e, nv = graphs["rmat12"]
    g = Z.Graph.from_edges(e, nv)
    p = Z.Program(kind, param, pattern)
    base = None
    for v in range(Z.VARIANTS):
        Z.check(L.zg_set_variant(kind, v))
        c = p.run(g, 1 << 19, 123)
        got = (c.samples, c.hits, c.fails, _sums(c))
        assert base is None or got == base, (name, v)
        base = got
    best, ms = p.tune(g, 1 << 18)
    assert 0 <= best < Z.VARIANTS and len(ms) == Z.VARIANTS and all(t > 0 for t in ms)
    assert p.variant()["variant"] == best


def test_unbiased_four_clique_counters_and_accuracy():
    """The canonical-path 4-clique program: exact sums equal the oracle's, and its estimate lands
    within 4 standard errors of the exact count where the reference's program is biased low."""
    import math
    e = Z.gen_rmat(11, 16, seed=12)
    g = Z.Graph.from_edges(e, 1 << 11)
    og = O.OracleGraph(e, 1 << 11)
    n = 1 << 20
    c = Z.Program(Z.PROG_FOUR_CLIQUE_UNBIASED).run(g, n, 17)
    oc = O.run(og, O.OracleProgram(Z.PROG_FOUR_CLIQUE_UNBIASED), n, 17)
    assert (c.hits, c.fails) == (oc.hits, oc.fails)
    assert [int(x) for x in c.sum_num] == [int(x) for x in oc.sum_num]
    ex = g.exact_count(Z.EXACT_FOUR_CLIQUE)
    big = Z.Program(Z.PROG_FOUR_CLIQUE_UNBIASED).run(g, 1 << 28, 3)
    se = math.sqrt(max(big.sum_w2 / big.samples - big.estimate ** 2, 0) / big.samples)
    assert abs(big.estimate - ex) < 4 * se, (big.estimate, ex, se)
    assert se < 0.01 * ex
    ref = Z.Program(Z.PROG_FOUR_CLIQUE).run(g, 1 << 28, 3)
    assert ref.estimate < 0.8 * ex  # the reference's estimator misses the non-canonical cliques
