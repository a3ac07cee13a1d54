"""bench.py's coverage report (CPU): the Wilson score interval it prints beside each covered
fraction, against values worked out by hand."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


@pytest.mark.parametrize("k,n,lo,hi", [(36, 40, 0.7695, 0.9604), (40, 40, 0.9124, 1.0), (0, 10, 0.0, 0.2775),
                                       (191, 200, 0.9166, 0.9762)])
def test_wilson_interval(k, n, lo, hi):
    a, b = bench.wilson(k, n)
    assert a == pytest.approx(lo, abs=2e-4) and b == pytest.approx(hi, abs=2e-4)
    assert 0.0 <= a <= k / n <= b <= 1.0
