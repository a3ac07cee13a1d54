"""The bound check every bounded answer goes through (zg_bound_half_width, host arithmetic only):
the empirical CLT half-width from 30 hits on, the empirical Bernstein half-width (Audibert, Munos,
Szepesvari 2009: values in [0, R], with probability >= 1 - delta, |mean - mu| <=
sqrt(2 var ln(3/delta) / n) + 3 R ln(3/delta) / n) at any n, the smaller one where both apply.
The reference's sampling/IEStop.cpp:27-56 stops on a CLT interval alone."""
import math

import pytest

import zgraph as Z

Z95 = 1.959963984540054


def clt(var, n):
    return Z95 * math.sqrt(var / n)


def bern(var, n, r, conf=0.95):
    x = math.log(3.0 / (1.0 - conf))
    return math.sqrt(2.0 * var * x / n) + 3.0 * r * x / n


@pytest.mark.parametrize("mean,var,n,hits,r", [(10.0, 400.0, 1 << 20, 5000, 1e4), (1e7, 1e16, 1 << 30, 10 ** 6, 1e11),
                                               (3.0, 2.0, 1000, 29, 5.0), (3.0, 2.0, 1000, 30, 5.0),
                                               (50.0, 10.0, 10 ** 6, 10 ** 6, 60.0)])
def test_half_width_is_the_smaller_valid_bound(mean, var, n, hits, r):
    h, method, met = Z.bound_half_width(mean, var, n, hits, 0.01, 0.95, r)
    c, b = clt(var, n), bern(var, n, r)
    if hits < 30:
        assert method == Z.BOUND_BERNSTEIN and h == pytest.approx(b, rel=1e-12)
    else:
        assert h == pytest.approx(min(c, b), rel=1e-12)
        assert method == (Z.BOUND_CLT if c <= b else Z.BOUND_BERNSTEIN)
    assert met == (h <= 0.01 * mean)


def test_bernstein_answers_below_thirty_hits():
    # few hits but a narrow range: Bernstein alone can certify the answer
    h, method, met = Z.bound_half_width(1.0, 0.5, 10 ** 7, 12, 0.05, 0.95, 2.0)
    assert method == Z.BOUND_BERNSTEIN and met
    # a wide range with few hits cannot
    h, method, met = Z.bound_half_width(1.0, 0.5, 10 ** 4, 12, 0.05, 0.95, 1e6)
    assert method == Z.BOUND_BERNSTEIN and not met
    # no estimator yet: never met
    assert not Z.bound_half_width(0.0, 0.0, 0, 0, 0.05, 0.95, 1.0)[2]


def test_invalid_arguments_rejected():
    for args in ((1.0, 1.0, 10, 10, 0.0, 0.95, 1.0), (1.0, 1.0, 10, 10, 0.1, 1.0, 1.0),
                 (1.0, -1.0, 10, 10, 0.1, 0.95, 1.0)):
        with pytest.raises(Z.ZgError):
            Z.bound_half_width(*args)
