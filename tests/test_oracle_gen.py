"""The oracle's host-side inputs (CPU, no GPU): the R-MAT generator of oracle/zgo_gen.c against the
library's zg_gen_rmat (the device generator equals the latter, tests/test_gpu_bench_configs.py), and
the oracle's multi-threaded graph build against a plain restatement of
CSRConstructor::construct_bitmap_assisted_csr (src/Graph.cpp:255-311): half-edges appended in
edge-id order, so each list is sorted by edge id."""
import numpy as np
import pytest

import oracle as O
import zgraph as Z


@pytest.mark.parametrize("scale,ef,abc,seed", [(1, 4, (0.57, 0.19, 0.19), 1), (6, 8, (0.25, 0.25, 0.25), 3),
                                               (10, 8, (0.57, 0.19, 0.19), 1), (13, 12, (0.57, 0.19, 0.19), 1),
                                               (16, 5, (0.45, 0.25, 0.25), 77), (18, 3, (1.0, 0.0, 0.0), 2)])
def test_oracle_rmat_equals_library_generator(scale, ef, abc, seed):
    a, b, c = abc
    mine = O.gen_rmat(scale, ef, a, b, c, seed)
    lib = np.asarray(Z.gen_rmat(scale, ef, a, b, c, seed)).reshape(-1, 2)
    assert mine.shape == lib.shape
    assert np.array_equal(mine, lib)
    if len(mine):
        assert np.all(mine[:, 0] != mine[:, 1])
        lo, hi = mine.min(axis=1).astype(np.uint64), mine.max(axis=1).astype(np.uint64)
        assert len(np.unique(lo << np.uint64(32) | hi)) == len(mine)


def test_rmat13_edge_count():
    assert len(O.gen_rmat(13, 12, seed=1)) == 79403


def test_parallel_graph_build_matches_plain_csr():
    e = O.gen_rmat(17, 12, seed=5)  # over 2^20 edges: the multi-threaded build
    assert len(e) > (1 << 20)
    nv = 1 << 17
    og = O.OracleGraph(e, nv)
    a = og.arrays()
    m = len(e)
    ends = np.concatenate([e[:, 0], e[:, 1]]).astype(np.int64)
    nbrs = np.concatenate([e[:, 1], e[:, 0]])
    eids = np.concatenate([np.arange(m), np.arange(m)]).astype(np.uint64)
    order = np.lexsort((eids, ends))  # by vertex, then edge id
    off = np.zeros(nv + 1, np.uint64)
    np.add.at(off, ends + 1, 1)
    off = np.cumsum(off).astype(np.uint64)
    assert np.array_equal(a["off"], off)
    assert np.array_equal(a["adj_nbr"], nbrs[order])
    assert np.array_equal(a["adj_eid"], eids[order])
    assert og.max_degree == int(np.diff(off).max())
