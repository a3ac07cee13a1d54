"""The three per-edge record layouts (zg_set_record_layout): compact (16 bytes, steps read vertex
offsets), wide (32 bytes: each edge's slot and predecessor count in both endpoint lists) and
packed (16 bytes of bit fields: the vertices, suffix sizes and slots).  Every program, the fused
3-motif, batches, derived graphs and exports give identical results under each, sample for
sample; the parity tests against the oracle run on the layout the automatic choice picks for
their (small) graphs, packed, so equality here carries them to the others."""
import numpy as np
import pytest

import zgraph as Z

pytestmark = pytest.mark.gpu

STAR = (5, [(0, 1), (0, 2), (0, 3), (0, 4)])
HOUSE = (5, [(0, 1), (0, 2), (1, 2), (1, 3), (2, 4), (3, 4)])
TRI = (3, [(0, 1), (0, 2), (1, 2)])


def _same(a, b, what):
    assert (a.samples, a.hits, a.fails, a.overflow) == (b.samples, b.hits, b.fails, b.overflow), what
    assert [int(x) for x in a.sum_num] == [int(x) for x in b.sum_num], what
    assert a.estimate == b.estimate and a.sum_w == b.sum_w, what
    assert abs(a.sum_w2 - b.sum_w2) <= 1e-12 * max(1.0, abs(b.sum_w2)), what


def _build(layout, fn):
    Z.set_record_layout(layout)
    try:
        return fn()
    finally:
        Z.set_record_layout(Z.RECORDS_AUTO)


@pytest.fixture(scope="module")
def pair():
    Z.init(0)
    e = Z.gen_rmat(12, 10, seed=17)
    w = Z.gen_weights(len(e), 100, seed=4)
    mk = lambda: Z.Graph.from_edges(e, 1 << 12, weights=w, shuffle_seed=5)  # noqa: E731
    return _build(Z.RECORDS_COMPACT, mk), _build(Z.RECORDS_WIDE, mk), _build(Z.RECORDS_PACKED, mk)


def test_meta_and_exports(pair):
    c, wd, pk = pair
    assert (c.meta().record_bytes, wd.meta().record_bytes, pk.meta().record_bytes) == (16, 32, 16)
    assert (c.meta().record_layout, wd.meta().record_layout, pk.meta().record_layout) == (
        Z.RECORDS_COMPACT, Z.RECORDS_WIDE, Z.RECORDS_PACKED)
    assert wd.meta().device_bytes - c.meta().device_bytes == 16 * c.num_local_edges
    assert pk.meta().device_bytes == c.meta().device_bytes
    dc = c.download()
    for other in (wd, pk):
        do = other.download()
        for k in ("edges", "weights", "offsets", "adj_e", "adj_n", "suffix"):
            assert np.array_equal(dc[k], do[k]), k


PROGRAMS = [("triangle", Z.PROG_TRIANGLE, 0, None), ("four_clique", Z.PROG_FOUR_CLIQUE, 0, None),
            ("four_clique_unbiased", Z.PROG_FOUR_CLIQUE_UNBIASED, 0, None),
            ("three_chain", Z.PROG_THREE_CHAIN, 0, None), ("four_chain", Z.PROG_FOUR_CHAIN, 0, None),
            ("chain5", Z.PROG_CHAIN, 5, None), ("chain7", Z.PROG_CHAIN, 7, None),
            ("star5", Z.PROG_PATTERN, 0, STAR), ("house5", Z.PROG_PATTERN, 0, HOUSE),
            ("triangle_pattern", Z.PROG_PATTERN, 0, TRI)]


@pytest.mark.parametrize("name,kind,param,pat", PROGRAMS, ids=[p[0] for p in PROGRAMS])
def test_programs_identical(pair, name, kind, param, pat):
    c, wd, pk = pair
    p = Z.Program(kind, param, pat)
    for other in (wd, pk):
        for n, seed, first in ((1 << 20, 3, 0), (77777, 9, 1 << 33)):
            _same(p.run(c, n, seed, stream_id=4, first_sample=first),
                  p.run(other, n, seed, stream_id=4, first_sample=first), (name, n))
        tc, tw = p.run_debug(c, 4096, 11), p.run_debug(other, 4096, 11)
        for k in ("ndraws", "hit", "fail", "shift", "sectors", "closures", "w", "num", "lo", "hi", "val"):
            assert np.array_equal(tc[k], tw[k]), (name, k)


def test_three_motif_and_batch_identical(pair):
    c, wd, pk = pair
    for other in (wd, pk):
        for a, b in zip(Z.run_three_motif(c, 1 << 20, 1 << 19, 7, 1, 2),
                        Z.run_three_motif(other, 1 << 20, 1 << 19, 7, 1, 2)):
            _same(a, b, "three_motif")
    qs = [{"kind": Z.PROG_TRIANGLE, "n": 300000, "seed": 1, "pred_op": Z.PRED_GE, "t0": 40},
          {"kind": Z.QUERY_THREE_MOTIF, "n": 200000, "seed": 2},
          {"kind": Z.PROG_FOUR_CHAIN, "n": 250000, "seed": 3, "first_sample": 99},
          {"kind": Z.PROG_PATTERN, "program": Z.Program(Z.PROG_PATTERN, pattern=STAR), "n": 100000, "seed": 4}]
    rc = _build(Z.RECORDS_COMPACT, lambda: Z.Batch(c, max_queries=8).run(qs))
    rw = _build(Z.RECORDS_WIDE, lambda: Z.Batch(wd, max_queries=8).run(qs))
    rp = _build(Z.RECORDS_PACKED, lambda: Z.Batch(pk, max_queries=8).run(qs))
    for q, (a, a2), (b, b2), (d, d2) in zip(qs, rc, rw, rp):
        _same(a, b, q)
        _same(a2, b2, q)
        _same(a, d, q)
        _same(a2, d2, q)


def test_derived_graphs_and_exact_counts(pair):
    c, wd, pk = pair
    fc = _build(Z.RECORDS_COMPACT, lambda: c.filter(Z.PRED_LT, 50, shuffle_seed=8))
    fw = _build(Z.RECORDS_WIDE, lambda: wd.filter(Z.PRED_LT, 50, shuffle_seed=8))
    fp = _build(Z.RECORDS_PACKED, lambda: pk.filter(Z.PRED_LT, 50, shuffle_seed=8))
    assert fc.meta().record_bytes == 16 and fw.meta().record_bytes == 32
    assert fp.meta().record_layout == Z.RECORDS_PACKED
    assert np.array_equal(fc.download()["edges"], fw.download()["edges"])
    assert np.array_equal(fc.download()["edges"], fp.download()["edges"])
    p = Z.Program(Z.PROG_FOUR_CLIQUE)
    _same(p.run(fc, 1 << 19, 5), p.run(fw, 1 << 19, 5), "filtered")
    _same(p.run(fc, 1 << 19, 5), p.run(fp, 1 << 19, 5), "filtered")
    for kind in (Z.EXACT_TRIANGLE, Z.EXACT_WEDGE, Z.EXACT_FOUR_CLIQUE):
        assert c.exact_count(kind) == wd.exact_count(kind) == pk.exact_count(kind), kind
    e_c = _build(Z.RECORDS_COMPACT, lambda: Z.elp_plain(c, Z.Program(Z.PROG_TRIANGLE), 0.05, 0.95, 3))
    e_w = _build(Z.RECORDS_WIDE, lambda: Z.elp_plain(wd, Z.Program(Z.PROG_TRIANGLE), 0.05, 0.95, 3))
    assert e_c.n_required == e_w.n_required


def test_device_generator_layouts():
    Z.init(0)
    gc = _build(Z.RECORDS_COMPACT, lambda: Z.Graph.gen_chung_lu(30000, 2.4, 10.0, seed=3, sampling_only=True))
    gw = _build(Z.RECORDS_WIDE, lambda: Z.Graph.gen_chung_lu(30000, 2.4, 10.0, seed=3, sampling_only=True))
    gp = _build(Z.RECORDS_PACKED, lambda: Z.Graph.gen_chung_lu(30000, 2.4, 10.0, seed=3, sampling_only=True))
    assert gp.meta().record_layout == Z.RECORDS_PACKED
    p = Z.Program(Z.PROG_FOUR_CHAIN)
    _same(p.run(gc, 1 << 20, 2), p.run(gw, 1 << 20, 2), "chung-lu")
    _same(p.run(gc, 1 << 20, 2), p.run(gp, 1 << 20, 2), "chung-lu")
    with pytest.raises(Z.ZgError):
        Z.set_record_layout(4)


def test_tiny_graphs_and_sample_counts():
    """Empty, single-edge and isolated-vertex graphs, and sample counts that leave warps partly
    filled (the 4-chain's grouped queues drain their leftovers): both layouts agree exactly."""
    Z.init(0)
    cases = [(np.zeros((0, 2), np.uint32), 4), (np.array([[0, 1]], np.uint32), 2),
             (np.array([[5, 2], [2, 9], [9, 5]], np.uint32), 12),
             (np.array([[0, 1], [1, 2], [2, 3], [3, 0], [0, 2], [4, 0]], np.uint32), 6)]
    for e, nv in cases:
        gc = _build(Z.RECORDS_COMPACT, lambda: Z.Graph.from_edges(e, nv))
        gw = _build(Z.RECORDS_WIDE, lambda: Z.Graph.from_edges(e, nv))
        gp = _build(Z.RECORDS_PACKED, lambda: Z.Graph.from_edges(e, nv))
        for name, kind, param, pat in PROGRAMS:
            p = Z.Program(kind, param, pat)
            for n in (1, 31, 33, 1000):
                a = p.run(gc, n, 3, first_sample=n)
                _same(a, p.run(gw, n, 3, first_sample=n), (len(e), name, n))
                _same(a, p.run(gp, n, 3, first_sample=n), (len(e), name, n))


def test_packed_wide_vertex_fields():
    """Packed records whose vertex fields are 24 bits wide (the same edges on ids spread over 2^24)
    and 8 bits wide (ids packed below 256) give identical counters sample for sample: the map is
    monotone, so every order is kept."""
    Z.init(0)
    e = Z.gen_rmat(8, 4, seed=3)
    small = Z.Graph.from_edges(e, 1 << 8)
    spread = Z.Graph.from_edges((e.astype(np.uint64) * 65536 + 7).astype(np.uint32), 1 << 24)
    assert small.meta().record_layout == spread.meta().record_layout == Z.RECORDS_PACKED
    assert np.array_equal(small.download()["suffix"], spread.download()["suffix"])
    for name, kind, param, pat in PROGRAMS:
        p = Z.Program(kind, param, pat)
        _same(p.run(small, 1 << 18, 5), p.run(spread, 1 << 18, 5), name)
    for kind in (Z.EXACT_TRIANGLE, Z.EXACT_FOUR_CLIQUE):
        assert small.exact_count(kind) == spread.exact_count(kind), kind
