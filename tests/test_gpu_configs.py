"""Device generators and the two largest configurations at full size.

* The device generators equal the host generators edge for edge (and weight for weight).
* Batched mixed queries on the Chung-Lu power-law graph with 4.8 M vertices, exponent 2.3, ~43 M
  edges and edge data uniform in [0, 100): 512 queries over {triangle, 3-motif, all-predicate
  triangle w >= T, at-least-one-predicate triangle (all triangles minus those whose edges all have
  w < T)}, T uniform in [10, 90], budgets 2^U(12, 24), in one submit.  Checked through properties
  that hold at any size: determinism, equality with single runs, additivity over sample ranges,
  and agreement with exact counts within the estimates' own confidence bounds.
* R-MAT scale 26, edge factor 24 (~1.4 G edges) built on the device; 4-clique, 5-star and 5-house
  estimators at 2^30 samples each in one batch, the 5-star checked against its exact count.
"""
import math

import numpy as np
import pytest

import zgraph as Z

pytestmark = pytest.mark.gpu


def _same(a, b, what=""):
    assert (a.samples, a.hits, a.fails) == (b.samples, b.hits, b.fails), what
    assert [int(x) for x in a.sum_num] == [int(x) for x in b.sum_num], what
    assert a.estimate == b.estimate, what


def _half_width(c, z=3.29):
    """z * sqrt(Var(1/p) / n) from the counters (z = 3.29: 99.9 % two-sided)."""
    n = c.samples
    mean = float(c.exact_sum()) / n
    var = max(c.sum_w2 / n - mean * mean, 0.0)
    return z * math.sqrt(var / n)


@pytest.fixture(scope="module", autouse=True)
def _init():
    Z.init(0)


@pytest.mark.parametrize("scale,ef,seed,wmax", [(11, 8, 3, 0), (12, 5, 9, 100), (9, 30, 1, 79)])
def test_device_rmat_equals_host(scale, ef, seed, wmax):
    e = Z.gen_rmat(scale, ef, seed=seed)
    g = Z.Graph.gen_rmat(scale, ef, seed=seed, max_weight=wmax, weight_seed=seed + 1)
    d = g.download()
    assert np.array_equal(d["edges"], e)
    if wmax:
        assert np.array_equal(d["weights"], Z.gen_weights(len(e), wmax, seed=seed + 1))
    ref = Z.Graph.from_edges(e, 1 << scale)
    assert np.array_equal(ref.download()["adj_n"], d["adj_n"])


def test_device_chung_lu_equals_host():
    e = Z.gen_chung_lu(50000, 2.3, 12.0, seed=5)
    g = Z.Graph.gen_chung_lu(50000, 2.3, 12.0, seed=5, sampling_only=True)
    d = g.download(neighbour_order=False)
    assert np.array_equal(d["edges"], e)
    with pytest.raises(Z.ZgError):
        g.download()  # the sampling-only build has no neighbour-ordered adjacency
    # sampling-only and full builds sample identically
    full = Z.Graph.from_edges(e, 50000)
    p = Z.Program(Z.PROG_FOUR_CLIQUE)
    _same(p.run(g, 1 << 20, 3), p.run(full, 1 << 20, 3))


def c3_queries(rng, nq=512):
    """The batched workload: kinds drawn uniformly from {triangle, 3-motif, all-predicate triangle,
    at-least-one-predicate triangle}; the last is two queries (all triangles, and the triangle on the
    w < T graph) whose estimates are subtracted."""
    qs, groups = [], []
    for i in range(nq):
        kind = int(rng.integers(4))
        n = int(2 ** rng.uniform(12, 24))
        t = int(rng.integers(10, 91))
        seed = int(rng.integers(1, 1 << 40))
        if kind == 0:
            groups.append(("triangle", [len(qs)], None))
            qs.append({"kind": Z.PROG_TRIANGLE, "n": n, "seed": seed, "stream_id": i})
        elif kind == 1:
            groups.append(("three_motif", [len(qs)], None))
            qs.append({"kind": Z.QUERY_THREE_MOTIF, "n": n, "seed": seed, "stream_id": 2 * i})
        elif kind == 2:
            groups.append(("all_pred", [len(qs)], t))
            qs.append({"kind": Z.PROG_TRIANGLE, "n": n, "seed": seed, "pred_op": Z.PRED_GE, "t0": t, "stream_id": i})
        else:
            groups.append(("at_least_one", [len(qs), len(qs) + 1], t))
            qs.append({"kind": Z.PROG_TRIANGLE, "n": n, "seed": seed, "stream_id": i})
            qs.append({"kind": Z.PROG_TRIANGLE, "n": n, "seed": seed + 1, "pred_op": Z.PRED_LT, "t0": t,
                       "stream_id": i})
    return qs, groups


@pytest.fixture(scope="module")
def c3_graph():
    return Z.Graph.gen_chung_lu(4800000, 2.3, 18.0, seed=2024, max_weight=100, weight_seed=7)


def test_c3_batched_mixed_queries_full_size(c3_graph):
    g = c3_graph
    m = g.num_local_edges
    assert 35e6 < m < 50e6, m
    rng = np.random.default_rng(3)
    qs, groups = c3_queries(rng)
    assert len(qs) <= 1024
    b = Z.Batch(g, max_queries=1024, cache_bytes=200 << 30)
    r1 = b.run(qs)
    r2 = b.run(qs)
    for (a, a2), (c, c2) in zip(r1, r2):
        assert a.as_dict() == c.as_dict() and a2.as_dict() == c2.as_dict()
    # equality with single runs on a sample of the queries
    for i in rng.choice(len(qs), size=24, replace=False):
        q = qs[int(i)]
        gg = b.filtered_graph(q["pred_op"], q["t0"]) if q.get("pred_op") else g
        if q["kind"] == Z.QUERY_THREE_MOTIF:
            ch, tr = Z.run_three_motif(gg, q["n"], q["n"], q["seed"], q["stream_id"], q["stream_id"] + 1)
            _same(r1[i][0], ch, q)
            _same(r1[i][1], tr, q)
        else:
            _same(r1[i][0], Z.Program(q["kind"]).run(gg, q["n"], q["seed"], stream_id=q["stream_id"]), q)
    # estimates against exact counts, within their own 99.9 % bounds (plus the unit of one triangle)
    tri = g.exact_count(Z.EXACT_TRIANGLE)
    checked = 0
    for name, idx, t in groups:
        if name == "triangle" and r1[idx[0]][0].samples >= 1 << 22:
            c = r1[idx[0]][0]
            assert abs(c.estimate - tri) <= _half_width(c) + 1, (name, c.estimate, tri)
            checked += 1
        elif name == "all_pred" and r1[idx[0]][0].samples >= 1 << 22 and checked < 8:
            c = r1[idx[0]][0]
            ex = b.filtered_graph(Z.PRED_GE, t).exact_count(Z.EXACT_TRIANGLE)
            assert abs(c.estimate - ex) <= _half_width(c) + 1, (name, t, c.estimate, ex)
            checked += 1
    assert checked >= 3


def test_c3_additivity_over_sample_ranges(c3_graph):
    b = Z.Batch(c3_graph, max_queries=8)
    n = 1 << 22
    q = {"kind": Z.PROG_TRIANGLE, "pred_op": Z.PRED_GE, "t0": 35, "seed": 99, "stream_id": 4}
    whole, lo, hi = b.run([dict(q, n=2 * n), dict(q, n=n), dict(q, n=n, first_sample=n)])
    assert whole[0].samples == lo[0].samples + hi[0].samples
    assert whole[0].hits == lo[0].hits + hi[0].hits
    assert whole[0].exact_sum() == lo[0].exact_sum() + hi[0].exact_sum()


def test_c5_large_rmat_patterns():
    g = Z.Graph.gen_rmat(26, 24, seed=26, sampling_only=True)
    m = g.num_local_edges
    assert 1.2e9 < m < 1.7e9, m
    star = Z.Program(Z.PROG_PATTERN, pattern=(5, [(0, 1), (0, 2), (0, 3), (0, 4)]))
    house = Z.Program(Z.PROG_PATTERN, pattern=(5, [(0, 1), (0, 2), (1, 2), (1, 3), (2, 4), (3, 4)]))
    n = 1 << 30
    b = Z.Batch(g, max_queries=8)
    qs = [{"kind": Z.PROG_FOUR_CLIQUE, "n": n, "seed": 1},
          {"kind": Z.PROG_PATTERN, "program": star, "n": n, "seed": 2},
          {"kind": Z.PROG_PATTERN, "program": house, "n": n, "seed": 3},
          {"kind": Z.PROG_PATTERN, "program": star, "n": n // 2, "seed": 2},
          {"kind": Z.PROG_PATTERN, "program": star, "n": n // 2, "seed": 2, "first_sample": n // 2}]
    res = b.run(qs)
    for c, _ in res:
        assert c.overflow == 0
    assert res[0][0].hits > 0
    # The 5-house estimator of SamplerGenerator (six edges drawn conditionally, canonical order
    # enforced) almost never completes on a sparse power-law graph: its hits at 2^30 samples are
    # recorded, not required (on dense graphs it does complete: test_cpp_host, zgh_replay_check).
    print("5-house on R-MAT 26/24: %d hits in %d samples" % (res[2][0].hits, res[2][0].samples))
    # additivity of the 5-star halves, exactly
    assert res[1][0].exact_sum() == res[3][0].exact_sum() + res[4][0].exact_sum()
    assert res[1][0].hits == res[3][0].hits + res[4][0].hits
    # the 5-star estimate against the exact count sum C(d, 4)
    ex = g.exact_count(Z.EXACT_FIVE_STAR)
    c = res[1][0]
    assert abs(c.estimate - ex) <= _half_width(c) + 1, (c.estimate, ex)
