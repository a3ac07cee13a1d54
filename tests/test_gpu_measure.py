"""The measurement entry points bench.py builds its roofline from: the touched-sector counter
(zg_touch_sectors: the production sampling kernel compiled again with every load counting its
32-byte sectors), the read-bandwidth probe (zg_read_bandwidth) and the random-sector rate over a
graph's arrays (zg_random_sector_rate)."""
import ctypes as C
import math

import pytest

import zgraph as Z

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graph():
    Z.init(0)
    return Z.Graph.gen_rmat(14, 8, seed=3)


def test_touched_sectors_are_deterministic_and_plausible(graph):
    for kind in (Z.PROG_TRIANGLE, Z.PROG_FOUR_CLIQUE, Z.PROG_FOUR_CHAIN):
        p = Z.Program(kind)
        a = p.touch_bytes_per_sample(graph, 1 << 16, 5)
        b = p.touch_bytes_per_sample(graph, 1 << 16, 5)
        assert a == b  # the same samples touch the same sectors
        # every sample reads at least its first edge's record (one sector); none reads 100 sectors
        assert 32.0 <= a <= 3200.0, (kind, a)


def test_read_bandwidth_probe():
    l2 = Z.read_bandwidth(48 << 20, 20)
    assert math.isfinite(l2) and l2 > 0


def test_random_sector_rate(graph):
    r = Z.random_sector_rate(graph, 16)
    assert math.isfinite(r) and r > 1e8  # sectors per second
    L = Z.lib()
    out = C.c_double(0)
    assert L.zg_random_sector_rate(None, 16, None, C.byref(out)) == Z.ZG_ERR_INVALID_ARG
    assert L.zg_random_sector_rate(graph.handle, 0, None, C.byref(out)) == Z.ZG_ERR_INVALID_ARG
