"""bench.py's host-side pieces (CPU): the Wilson score interval it prints beside each covered
fraction, against values worked out by hand; the committed ncu captures it reads; its CPU leg."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


@pytest.mark.parametrize("k,n,lo,hi", [(36, 40, 0.7695, 0.9604), (40, 40, 0.9124, 1.0), (0, 10, 0.0, 0.2775),
                                       (191, 200, 0.9166, 0.9762)])
def test_wilson_interval(k, n, lo, hi):
    a, b = bench.wilson(k, n)
    assert a == pytest.approx(lo, abs=2e-4) and b == pytest.approx(hi, abs=2e-4)
    assert 0.0 <= a <= k / n <= b <= 1.0


def test_random_sector_bytes_from_the_committed_capture():
    """The DRAM bytes one random 32-byte sector read moves, from profiles/dram_traffic.txt: between
    one sector and a 256-byte line while the capture matches the kernel sources, else a reason."""
    bps, src = bench.random_sector_bytes()
    if bps is None:
        assert src
    else:
        assert 32.0 <= bps <= 256.0 and "ncu capture" in src


def test_headline_traffic_is_current():
    """The committed ncu DRAM traffic of the headline's batch kernels (profiles/dram_traffic.txt)
    was captured at the current kernel sources and record layout, so the bench reports it; an edit
    of the sampling sources without a new capture fails here rather than silently dropping
    `roofline.traffic` from the headline line."""
    for workload in ("rmat26", "rmat21_batch"):
        dps, src = bench.profile_traffic("k_batch", workload, "wide")
        assert dps is not None, src
        assert 100.0 < dps < 2000.0
    bps, src = bench.random_sector_bytes()
    assert bps is not None, src


def test_cpu_baseline_leg_on_a_small_graph():
    """The GPU arm's CPU leg (bench.cpu_baseline: the oracle on the graph's edge list, a bounded sample
    of every program of the workload, the headline's patterns included, and the reference's plain-ELP
    time to a 1 %/95 % triangle answer) returns the fields the bench line carries."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    edges = O.gen_rmat(10, 8, seed=3)
    out = bench.cpu_baseline(edges, 1 << 10, ["four_clique", "five_star", "five_house", "triangle"], 2,
                             target_s=0.4)
    assert out["value"] > 0 and out["unit"] == "samples/s" and out["cores"] == 2 and out["kind"] == "port"
    assert "five_house" in out["sample"]
    ttb = out["time_to_bound"]  # the reference's host time to a 1 %/95 % triangle answer
    assert "error" not in ttb, ttb
    assert ttb["n_required"] > 0 and ttb["seconds"] > ttb["profile_s"] > 0
