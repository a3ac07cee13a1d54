"""zg_conditional_close (the closure primitive with its found edge ids written back,
src/ZGraphInstance.cpp:410-441) against the oracle's linear scan, bit-exact: closed flag, edges
found before the first miss and their edge ids."""
import numpy as np
import pytest

import oracle as O
import zgraph as Z

pytestmark = pytest.mark.gpu


def _queries(e, nv, rng, count):
    m = len(e)
    qs = []
    for _ in range(count):
        k = int(rng.integers(1, 6))
        picks = e[rng.integers(0, m, size=k)]
        verts = list(dict.fromkeys(int(x) for x in picks.reshape(-1)))[:16]
        if rng.random() < 0.3:  # a vertex that touches none of the edges
            verts.append(int(rng.integers(0, nv)))
        edges = []
        for _ in range(int(rng.integers(0, 6))):
            r = rng.random()
            if r < 0.5:  # an edge of the graph
                a, b = (int(x) for x in e[int(rng.integers(0, m))])
                if rng.random() < 0.5:
                    a, b = b, a
            elif r < 0.8:  # a pair of sampled vertices (an edge or not)
                a, b = int(rng.choice(verts)), int(rng.choice(verts))
            else:  # anything, out-of-range ids and self-pairs included
                a, b = int(rng.integers(0, nv + 3)), int(rng.integers(0, nv + 3))
            edges.append((a, b))
        mv = int(rng.integers(0, m + 1)) if rng.random() < 0.7 else 0
        qs.append((mv, verts[:16], edges))
    return qs


@pytest.mark.parametrize("gname", ["rmat10", "chunglu3k"])
def test_conditional_close_matches_oracle(gname):
    Z.init(0)
    rng = np.random.default_rng(7)
    if gname == "rmat10":
        e, nv = Z.gen_rmat(10, 8, seed=3), 1 << 10
    else:
        e, nv = Z.gen_chung_lu(3000, 2.3, 12.0, seed=9), 3000
    e = np.asarray(e).reshape(-1, 2)
    g = Z.Graph.from_edges(e, nv)
    og = O.OracleGraph(e, nv)
    qs = _queries(e, nv, rng, 4000)
    # exact boundaries: an edge's own id is valid, one more is not
    a, b = (int(x) for x in e[17])
    qs += [(17, [a], [(a, b)]), (18, [b], [(b, a)]), (0, [], [(a, b)]), (5, [a, b], [])]
    got = Z.conditional_close(g, qs)
    closed_any = 0
    for q, r in zip(qs, got):
        want = og.conditional_close(*q)
        assert r[0] == want[0] and r[1] == want[1], (q, r, want)
        assert [int(x) for x in want[2]] == r[2], (q, r, want)
        closed_any += r[0]
    assert got[-4] == (True, 1, [17]) and got[-3][0] is False and got[-2][0] is False and got[-1] == (True, 0, [])
    assert 0 < closed_any < len(qs)


def test_conditional_close_rejects_oversized_queries():
    Z.init(0)
    g = Z.Graph.from_edges(np.array([[0, 1]], np.uint32), 2)
    with pytest.raises(Z.ZgError):
        Z.conditional_close(g, [(0, list(range(17)), [])])
