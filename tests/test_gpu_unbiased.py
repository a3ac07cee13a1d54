"""The estimators behind the headline are unbiased: on graphs small enough to count exactly, the
mean of many samples lies within 4.5 of its own standard errors of the exact count (two-sided,
about 7e-6 per case for a normal mean).  The unbiased 4-clique (every clique counted once through
its canonical path), the 5-star and 5-house pattern programs (src/SamplerGenerator.cpp:461-546,
applications/FiveStar.cpp:18-26, FiveHouse.cpp:18-27) and the triangle, against
zg_exact_count (itself equal to naive_implementation/'s counters on the goldens and to the
oracle's counts).  Sample counts run in several launches over consecutive sample ranges and are
combined by their sums, as a caller splitting a query would."""
import math

import pytest

import zgraph as Z

pytestmark = pytest.mark.gpu

STAR = (5, [(0, 1), (0, 2), (0, 3), (0, 4)])
HOUSE = (5, [(0, 1), (0, 2), (1, 2), (1, 3), (2, 4), (3, 4)])

CASES = [("triangle", Z.PROG_TRIANGLE, None, Z.EXACT_TRIANGLE, 1 << 26, 1),
         ("four_clique_unbiased", Z.PROG_FOUR_CLIQUE_UNBIASED, None, Z.EXACT_FOUR_CLIQUE, 1 << 30, 2),
         ("five_star", Z.PROG_PATTERN, STAR, Z.EXACT_FIVE_STAR, 1 << 28, 1),
         ("five_house", Z.PROG_PATTERN, HOUSE, Z.EXACT_FIVE_HOUSE, 1 << 30, 32)]


@pytest.fixture(scope="module")
def graphs():
    Z.init(0)
    return {"rmat13": Z.Graph.gen_rmat(13, 12, seed=1),
            "chunglu2k": Z.Graph.from_edges(Z.gen_chung_lu(2000, 2.2, 24.0, seed=5), 2000)}


@pytest.mark.parametrize("gname", ["rmat13", "chunglu2k"])
@pytest.mark.parametrize("name,kind,pat,exact_kind,n,launches", CASES, ids=[c[0] for c in CASES])
def test_estimate_matches_exact_count(graphs, gname, name, kind, pat, exact_kind, n, launches):
    g = graphs[gname]
    exact = g.exact_count(exact_kind)
    p = Z.Program(kind, 0, pat)
    total = hits = 0
    sw = sw2 = 0.0
    for i in range(launches):
        c = p.run(g, n, 20 + i, stream_id=3, first_sample=i * n)
        assert c.samples == n and c.overflow == 0
        total += c.samples
        hits += c.hits
        sw += c.estimate * c.samples
        sw2 += c.sum_w2
    mean = sw / total
    se = math.sqrt(max(sw2 / total - mean * mean, 0.0) / total)
    assert hits >= 50, (gname, name, hits)
    assert abs(mean - exact) <= 4.5 * se, (gname, name, mean, exact, se, hits)
