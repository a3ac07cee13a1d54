"""GPU parity on the benchmark configurations themselves, bit-exact against the CPU oracle.

* R-MAT scale 13, edge factor 12, seed 1 (the reference's CPU-path configuration): triangle,
  4-clique, 3-chain and 4-chain, per-sample traces on a prefix and the exact sums of 2^20 samples;
  exact counts (all seven kinds) against the oracle's naive and fast counters.
* R-MAT scale 20, edge factor 3, seed 1 (the four-program bench graph, generated on the device as
  the bench does): the same four programs at 2^22 samples from a first sample index above 2^32,
  exact counts of all five kinds.
* The Chung-Lu batch's base graph (4.8 M vertices, exponent 2.3, edge data in [0, 100)), in the wide
  record layout the build picks for it: triangle at 2^20 and 3-motif at 2^18 samples.
* R-MAT scale 26, edge factor 24, seed 26 (the headline graph, 1.57 G edges): the 4-clique, 5-star
  and 5-house programs on sample prefixes, and the device generator against the host one.
The oracle restates the reference path (linear-scan closure as conditional_close,
src/ZGraphInstance.cpp:372-407); its own pinning is in tests/test_oracle_golden.py.
"""
import numpy as np
import pytest

import oracle as O
import zgraph as Z

pytestmark = pytest.mark.gpu

FIELDS = ("ndraws", "hit", "fail", "shift", "sectors", "closures", "num", "lo", "hi", "val")
FOUR = [("triangle", Z.PROG_TRIANGLE), ("four_clique", Z.PROG_FOUR_CLIQUE), ("three_chain", Z.PROG_THREE_CHAIN),
        ("four_chain", Z.PROG_FOUR_CHAIN)]
STAR = (5, [(0, 1), (0, 2), (0, 3), (0, 4)])
HOUSE = (5, [(0, 1), (0, 2), (1, 2), (1, 3), (2, 4), (3, 4)])


def _assert_traces(gt, ot, label):
    for f in FIELDS:
        if not np.array_equal(gt[f], ot[f]):
            bad = np.nonzero(np.any((gt[f] != ot[f]).reshape(len(gt), -1), axis=1))[0]
            raise AssertionError("%s: field %s differs at %d samples, first %d" % (label, f, len(bad), bad[0]))
    assert np.array_equal(gt["w"].view(np.uint64), ot["w"].view(np.uint64)), label + ": reference doubles differ"


def _same_counters(c, oc, label):
    assert (c.samples, c.hits, c.fails, c.den_log2) == (oc.samples, oc.hits, oc.fails, oc.den_log2), label
    assert [int(x) for x in c.sum_num] == [int(x) for x in oc.sum_num], label


@pytest.fixture(scope="module")
def c1():
    Z.init(0)
    e = O.gen_rmat(13, 12, seed=1)
    return e, Z.Graph.from_edges(e, 1 << 13), O.OracleGraph(e, 1 << 13)


@pytest.mark.parametrize("name,kind", FOUR, ids=[f[0] for f in FOUR])
def test_rmat13_programs_match_oracle(c1, name, kind):
    e, g, og = c1
    n, seed, stream = 1 << 20, 1, 3
    p, op = Z.Program(kind), O.OracleProgram(kind)
    gt = p.run_debug(g, 1 << 14, seed, stream_id=stream)
    ot, _ = O.traces(og, op, 1 << 14, seed, stream=stream)
    _assert_traces(gt, ot, "rmat13/" + name)
    _same_counters(p.run(g, n, seed, stream_id=stream), O.run(og, op, n, seed, stream), "rmat13/" + name)


def test_rmat13_exact_counts(c1):
    e, g, og = c1
    assert len(e) == 79403
    for kind in (Z.EXACT_TRIANGLE, Z.EXACT_WEDGE, Z.EXACT_THREE_PATH, Z.EXACT_FIVE_STAR):
        assert g.exact_count(kind) == og.exact_naive(kind) == og.exact_fast(kind), kind
    for kind in (Z.EXACT_FOUR_CLIQUE, Z.EXACT_FIVE_HOUSE, Z.EXACT_FIVE_CHAIN):
        assert g.exact_count(kind) == og.exact_fast(kind), kind
    assert g.exact_count(Z.EXACT_TRIANGLE) == 701151


@pytest.fixture(scope="module")
def c2():
    Z.init(0)
    g = Z.Graph.gen_rmat(20, 3, seed=1)  # as bench.py builds it
    e = O.gen_rmat(20, 3, seed=1)
    return e, g, O.OracleGraph(e, 1 << 20)


def test_rmat20_device_generator_matches_host(c2):
    e, g, _ = c2
    assert len(e) == 3081197
    assert np.array_equal(g.download_edges(), e)


@pytest.mark.parametrize("name,kind", FOUR, ids=[f[0] for f in FOUR])
def test_rmat20_programs_match_oracle(c2, name, kind):
    e, g, og = c2
    first, seed, stream = (1 << 32) + 12345, 20250101, 2
    p, op = Z.Program(kind), O.OracleProgram(kind)
    gt = p.run_debug(g, 4096, seed, stream_id=stream, first_sample=first)
    ot, _ = O.traces(og, op, 4096, seed, stream=stream, first=first)
    _assert_traces(gt, ot, "rmat20/" + name)
    n = 1 << 22
    _same_counters(p.run(g, n, seed, stream_id=stream, first_sample=first),
                   O.run(og, op, n, seed, stream, first), "rmat20/" + name)


def test_rmat20_exact_counts(c2):
    e, g, og = c2
    for kind in (Z.EXACT_TRIANGLE, Z.EXACT_WEDGE, Z.EXACT_THREE_PATH, Z.EXACT_FIVE_STAR, Z.EXACT_FOUR_CLIQUE):
        assert g.exact_count(kind) == og.exact_fast(kind), kind


def test_chunglu_base_graph_wide_layout_matches_oracle():
    Z.init(0)
    g = Z.Graph.gen_chung_lu(4800000, 2.3, 18.0, seed=2024, max_weight=100, weight_seed=7)
    assert g.meta().record_layout == Z.RECORDS_WIDE
    e = g.download_edges()
    og = O.OracleGraph(e, 4800000)
    n, seed = 1 << 20, 77
    p, op = Z.Program(Z.PROG_TRIANGLE), O.OracleProgram(Z.PROG_TRIANGLE)
    gt = p.run_debug(g, 1 << 13, seed, stream_id=5)
    ot, _ = O.traces(og, op, 1 << 13, seed, stream=5)
    _assert_traces(gt, ot, "chunglu/triangle")
    _same_counters(p.run(g, n, seed, stream_id=5), O.run(og, op, n, seed, 5), "chunglu/triangle")
    nm = 1 << 18  # the oracle's 3-motif runs on one thread
    ca, cb = Z.run_three_motif(g, nm, nm, seed, 4, 5)
    oa, ob = O.three_motif(og, nm, nm, seed, 4, 5)[2:]
    _same_counters(ca, oa, "chunglu/motif chain")
    _same_counters(cb, ob, "chunglu/motif triangle")


def test_rmat26_headline_graph_and_programs_match_oracle():
    """The headline graph (1.57 G edges): the device generator's edge list equals the host one the
    CPU arm samples, and the 4-clique, 5-star and 5-house programs' traces and exact sums on sample
    prefixes equal the oracle's (which scans the hubs' adjacency linearly, as conditional_close does)."""
    import gc
    Z.init(0)
    g = Z.Graph.gen_rmat(26, 24, seed=26, sampling_only=True)  # as bench.py builds it
    e = O.gen_rmat(26, 24, seed=26)
    assert np.array_equal(g.download_edges(), e)
    og = O.OracleGraph(e, 1 << 26)
    del e
    gc.collect()
    for kind, pat, n in ((Z.PROG_FOUR_CLIQUE, None, 1 << 13), (Z.PROG_PATTERN, STAR, 1 << 12),
                         (Z.PROG_PATTERN, HOUSE, 1 << 12)):
        p, op = Z.Program(kind, 0, pat), O.OracleProgram(kind, 0, pat)
        first = 123456789
        gt = p.run_debug(g, n, 9, stream_id=1, first_sample=first)
        ot, oc = O.traces(og, op, n, 9, stream=1, first=first)
        _assert_traces(gt, ot, "rmat26/%d" % kind)
        _same_counters(p.run(g, n, 9, stream_id=1, first_sample=first), oc, "rmat26/%d" % kind)
