"""Batched mixed queries (zg_batch_*): every query of a mixed batch equals its single run on the
same draws — zg_run on the base graph or on the batch's cached filtered graph, zg_run_three_motif
for 3-motif queries — exactly (samples, hits, fails, 320-bit sums, estimate); batches are
deterministic, survive cache eviction, replay through their CUDA graph with changing sizes, and
refuse what they cannot run."""
import numpy as np
import pytest

import zgraph as Z

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wgraph():
    Z.init(0)
    e = Z.gen_rmat(12, 12, seed=31)
    w = Z.gen_weights(len(e), 100, seed=5)
    return Z.Graph.from_edges(e, 1 << 12, weights=w, shuffle_seed=77)


def _same(a, b, what):
    assert (a.samples, a.hits, a.fails) == (b.samples, b.hits, b.fails), what
    assert [int(x) for x in a.sum_num] == [int(x) for x in b.sum_num], what
    assert a.den_log2 == b.den_log2 and a.estimate == b.estimate, what
    assert a.sum_w == b.sum_w, what
    assert abs(a.sum_w2 - b.sum_w2) <= 1e-12 * max(1.0, abs(b.sum_w2)), what


def _mixed(rng, nq):
    kinds = [(Z.PROG_TRIANGLE, 0), (Z.PROG_FOUR_CLIQUE, 0), (Z.PROG_THREE_CHAIN, 0), (Z.PROG_FOUR_CHAIN, 0),
             (Z.PROG_CHAIN, 5), (Z.QUERY_THREE_MOTIF, 0)]
    qs = []
    for i in range(nq):
        k, prm = kinds[int(rng.integers(len(kinds)))]
        q = {"kind": k, "param": prm, "n": int(2 ** rng.uniform(0, 17)) + 1, "seed": int(rng.integers(1, 1 << 40)),
             "stream_id": int(rng.integers(0, 1 << 20))}
        if k in (Z.PROG_TRIANGLE, Z.QUERY_THREE_MOTIF) and rng.random() < 0.6:
            q["pred_op"] = [Z.PRED_GE, Z.PRED_LT][int(rng.integers(2))] if k == Z.PROG_TRIANGLE else 0
            q["t0"] = int(rng.integers(10, 91))
        qs.append(q)
    return qs


def _check_against_single(b, g, qs, res):
    for q, (c, c2) in zip(qs, res):
        gg = b.filtered_graph(q["pred_op"], q["t0"]) if q.get("pred_op") else g
        if q["kind"] == Z.QUERY_THREE_MOTIF:
            ch, tr = Z.run_three_motif(gg, q["n"], q["n"], q["seed"], q["stream_id"], q["stream_id"] + 1)
            _same(c, ch, q)
            _same(c2, tr, q)
        else:
            p = Z.Program(q["kind"], q.get("param", 0))
            _same(c, p.run(gg, q["n"], q["seed"], stream_id=q["stream_id"]), q)


def test_mixed_batch_equals_single_runs(wgraph):
    rng = np.random.default_rng(7)
    qs = _mixed(rng, 60)
    b = Z.Batch(wgraph, max_queries=128)
    res = b.run(qs)
    _check_against_single(b, wgraph, qs, res)


def test_batch_is_deterministic_and_shape_independent(wgraph):
    rng = np.random.default_rng(8)
    qs = _mixed(rng, 40)
    b = Z.Batch(wgraph, max_queries=64)
    r1 = b.run(qs)
    r2 = b.run(qs)
    for (a, a2), (c, c2) in zip(r1, r2):
        assert a.as_dict() == c.as_dict() and a2.as_dict() == c2.as_dict()
    best, ms = b.tune(qs)
    assert 0 <= best < 3 and all(m > 0 for m in ms)
    r3 = b.run(qs)
    for q, (a, a2), (c, c2) in zip(qs, r1, r3):
        _same(a, c, q)
        _same(a2, c2, q)


def test_filtered_graph_matches_zg_graph_filter_semantics(wgraph):
    b = Z.Batch(wgraph, max_queries=8)
    fg = b.filtered_graph(Z.PRED_GE, 50)
    d = wgraph.download()
    assert fg.num_local_edges == int((d["weights"] >= 50).sum())
    fd = fg.download(neighbour_order=False)
    assert (fd["weights"] >= 50).all()
    # same edge multiset as the base graph's kept edges
    keep = d["edges"][d["weights"] >= 50]
    a = np.sort(np.sort(keep, axis=1).view(np.uint64).ravel())
    c = np.sort(np.sort(fd["edges"], axis=1).view(np.uint64).ravel())
    assert np.array_equal(a, c)
    # exact triangle count of the filtered graph: all-predicate triangles w >= 50
    ex = fg.exact_count(Z.EXACT_TRIANGLE)
    est = b.run([{"kind": Z.PROG_TRIANGLE, "pred_op": Z.PRED_GE, "t0": 50, "n": 1 << 24, "seed": 3}])[0][0]
    assert abs(est.estimate / ex - 1) < 0.05


def test_cache_eviction_keeps_results_exact(wgraph):
    b = Z.Batch(wgraph, max_queries=32, cache_bytes=1)  # every new predicate evicts the others
    qs = [{"kind": Z.PROG_TRIANGLE, "pred_op": Z.PRED_GE, "t0": t, "n": 5000, "seed": 11 + t} for t in (20, 40, 60, 80)]
    res = b.run(qs)
    for q, (c, _) in zip(qs, res):
        fg = b.filtered_graph(q["pred_op"], q["t0"])
        _same(c, Z.Program(Z.PROG_TRIANGLE).run(fg, q["n"], q["seed"]), q)


def test_graph_replay_with_changing_sizes(wgraph):
    b = Z.Batch(wgraph, max_queries=16)
    rng = np.random.default_rng(9)
    for nq in (1, 16, 3, 9):
        qs = [{"kind": Z.PROG_THREE_CHAIN, "n": int(rng.integers(1, 300000)), "seed": int(rng.integers(1, 99999)),
               "stream_id": 5} for _ in range(nq)]
        res = b.run(qs)
        assert len(res) == nq
        for q, (c, _) in zip(qs, res):
            _same(c, Z.Program(Z.PROG_THREE_CHAIN).run(wgraph, q["n"], q["seed"], stream_id=5), q)


def test_refusals(wgraph):
    b = Z.Batch(wgraph, max_queries=4)
    with pytest.raises(Z.ZgError) as e:
        b.run([{"kind": Z.PROG_TRIANGLE, "n": 0, "seed": 1}])
    assert e.value.code == Z.ZG_ERR_INVALID_ARG
    with pytest.raises(Z.ZgError) as e:
        b.run([{"kind": Z.PROG_PATTERN, "n": 10, "seed": 1}])
    assert e.value.code == Z.ZG_ERR_UNSUPPORTED_ESTIMATOR
    with pytest.raises(Z.ZgError) as e:
        b.run([{"kind": Z.PROG_TRIANGLE, "n": 10, "seed": 1}] * 5)
    assert e.value.code == Z.ZG_ERR_TOO_LARGE
    # the batch still works after refusals
    c = b.run([{"kind": Z.PROG_TRIANGLE, "n": 1000, "seed": 2}])[0][0]
    _same(c, Z.Program(Z.PROG_TRIANGLE).run(wgraph, 1000, 2), "after refusal")


def test_pattern_queries_and_first_sample(wgraph):
    star = Z.Program(Z.PROG_PATTERN, pattern=(5, [(0, 1), (0, 2), (0, 3), (0, 4)]))
    house = Z.Program(Z.PROG_PATTERN, pattern=(5, [(0, 1), (0, 2), (1, 2), (1, 3), (2, 4), (3, 4)]))
    tri = Z.Program(Z.PROG_PATTERN, pattern=(3, [(0, 1), (0, 2), (1, 2)]))
    qs = [{"kind": Z.PROG_PATTERN, "program": star, "n": 300000, "seed": 4, "stream_id": 2},
          {"kind": Z.PROG_TRIANGLE, "n": 50000, "seed": 9, "first_sample": 12345},
          {"kind": Z.PROG_PATTERN, "program": house, "n": 200000, "seed": 5, "first_sample": 777},
          {"kind": Z.PROG_PATTERN, "program": tri, "pred_op": Z.PRED_GE, "t0": 30, "n": 100000, "seed": 6},
          {"kind": Z.PROG_FOUR_CHAIN, "n": 70000, "seed": 8, "first_sample": 1 << 40}]
    b = Z.Batch(wgraph, max_queries=8)
    res = b.run(qs)
    for q, (c, _) in zip(qs, res):
        gg = b.filtered_graph(q["pred_op"], q["t0"]) if q.get("pred_op") else wgraph
        p = q.get("program") or Z.Program(q["kind"])
        _same(c, p.run(gg, q["n"], q["seed"], stream_id=q.get("stream_id", 0),
                       first_sample=q.get("first_sample", 0)), q)


def test_learned_sizing_of_a_batch(wgraph):
    """zg_batch_size_learned fills the n of every query without one, from pilot batches and one
    prediction, equal (to the last bit of the pilot's variance term) to zg_elp_learned per query."""
    rng = np.random.default_rng(12)
    net = Z.Mlp(3)
    net.train(rng.normal(size=(64, 16)).astype(np.float32), (rng.normal(size=(64, 2)) + 8).astype(np.float32),
              epochs=2, batch=32, lr=1e-3)
    star = Z.Program(Z.PROG_PATTERN, pattern=(5, [(0, 1), (0, 2), (0, 3), (0, 4)]))
    qs = [{"kind": Z.PROG_TRIANGLE, "seed": 5},
          {"kind": Z.PROG_TRIANGLE, "seed": 6, "pred_op": Z.PRED_GE, "t0": 40},
          {"kind": Z.PROG_FOUR_CHAIN, "seed": 7, "n": 12345},
          {"kind": Z.PROG_PATTERN, "program": star, "seed": 8},
          {"kind": Z.PROG_THREE_CHAIN, "seed": 9, "stream_id": 3}]
    b = Z.Batch(wgraph, max_queries=16)
    sized = b.size_learned(net, qs, 0.02, 0.95)
    assert sized[2]["n"] == 12345
    for q, s in zip(qs, sized):
        if "n" in q:
            continue
        gg = b.filtered_graph(q["pred_op"], q["t0"]) if q.get("pred_op") else wgraph
        p = q.get("program") or Z.Program(q["kind"])
        n, _, _ = Z.learned_budget(net, gg, p, 0.02, 0.95, seed=q["seed"])
        assert abs(s["n"] - n) <= 1e-6 * n + 1, (q, s["n"], n)
    res = b.run(sized)
    assert all(c.samples == q["n"] for (c, _), q in zip(res, sized))
    with pytest.raises(Z.ZgError):
        b.size_learned(net, [{"kind": Z.QUERY_THREE_MOTIF, "seed": 1}], 0.02, 0.95)


def test_bounded_batch_tops_up_until_the_bound_holds(wgraph):
    """Batch.bounded: learned sizing, one batch, top-up batches on fresh sample indices for the
    answers still outside the bound; each merged answer equals one run over all its samples."""
    rng = np.random.default_rng(13)
    net = Z.Mlp(4)
    net.train(rng.normal(size=(64, 16)).astype(np.float32), (rng.normal(size=(64, 2)) + 2).astype(np.float32),
              epochs=2, batch=32, lr=1e-3)  # predicts small variances: the top-ups do the work
    qs = [{"kind": Z.PROG_TRIANGLE, "seed": 21, "stream_id": 2},
          {"kind": Z.PROG_TRIANGLE, "seed": 22, "pred_op": Z.PRED_LT, "t0": 70},
          {"kind": Z.PROG_THREE_CHAIN, "seed": 23, "first_sample": 1000},
          {"kind": Z.PROG_FOUR_CHAIN, "seed": 24}]
    b = Z.Batch(wgraph, max_queries=8)
    total, met, rounds = b.bounded(net, qs, 0.05, 0.95, max_rounds=6)
    assert all(met) and rounds >= 1
    z = Z.lib().zg_normal_quantile(0.975)
    for q, c in zip(qs, total):
        var = max(c.sum_w2 / c.samples - c.estimate ** 2, 0.0)
        assert z * (var / c.samples) ** 0.5 <= 0.05 * c.estimate
        gg = b.filtered_graph(q["pred_op"], q["t0"]) if q.get("pred_op") else wgraph
        one = Z.Program(q["kind"]).run(gg, c.samples, q["seed"], stream_id=q.get("stream_id", 0),
                                       first_sample=q.get("first_sample", 0))
        assert (one.samples, one.hits, one.fails) == (c.samples, c.hits, c.fails)
        assert [int(x) for x in one.sum_num] == [int(x) for x in c.sum_num] and one.estimate == c.estimate
