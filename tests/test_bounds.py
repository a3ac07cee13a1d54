"""The bound check every bounded answer goes through (zg_bound_half_width, host arithmetic only):
the empirical CLT half-width from 30 hits on, the empirical Bernstein half-width (Audibert, Munos,
Szepesvari 2009: values in [0, R], with probability >= 1 - delta, |mean - mu| <=
sqrt(2 var ln(3/delta) / n) + 3 R ln(3/delta) / n) at any n, the smaller one where both apply.
Given the empirical mean of w^4, the CLT half-width takes an upper confidence bound on the variance,
var + z sqrt((m4 - var^2) / n) with m4 = E w^4 + 2 mean^2 var.
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


def var_ub(mean, var, ew4, n):
    if ew4 <= 0:  # unknown fourth moment: no inflation
        return var
    spread = ew4 + 2.0 * mean * mean * var - var * var
    return var + Z95 * math.sqrt(spread / n) if spread > 0 else var


@pytest.mark.parametrize("mean,var,ew4,n,hits,r", [(10.0, 400.0, 5e6, 1 << 20, 5000, 1e4),
                                                   (1e3, 1e8, 1e22, 1 << 24, 10 ** 5, 1e7),
                                                   (2.0, 1.0, 0.0, 1 << 20, 10 ** 4, 10.0)])
def test_fourth_moment_widens_the_clt_half_width(mean, var, ew4, n, hits, r):
    h, method, met = Z.bound_half_width(mean, var, n, hits, 0.01, 0.95, r, fourth_moment=ew4)
    c, b = clt(var_ub(mean, var, ew4, n), n), bern(var, n, r)
    assert h == pytest.approx(min(c, b), rel=1e-12)
    assert method == (Z.BOUND_CLT if c <= b else Z.BOUND_BERNSTEIN)
    if ew4 > 0 and method == Z.BOUND_CLT:
        assert h > clt(var, n)
    # heavier tails (larger E w^4 at the same variance) never narrow the interval
    assert Z.bound_half_width(mean, var, n, hits, 0.01, 0.95, r, fourth_moment=10 * ew4 + 1)[0] >= h


def test_invalid_arguments_rejected():
    for args in ((1.0, 1.0, 10, 10, 0.0, 0.95, 1.0), (1.0, 1.0, 10, 10, 0.1, 1.0, 1.0),
                 (1.0, -1.0, 10, 10, 0.1, 0.95, 1.0)):
        with pytest.raises(Z.ZgError):
            Z.bound_half_width(*args)
    with pytest.raises(Z.ZgError):
        Z.bound_half_width(1.0, 1.0, 10, 10, 0.1, 0.95, 1.0, fourth_moment=-1.0)


def test_overflowed_fourth_moment_counts_as_unknown():
    a = Z.bound_half_width(5.0, 4.0, 1 << 20, 10 ** 4, 0.01, 0.95, 1e3, fourth_moment=math.inf)
    assert a == Z.bound_half_width(5.0, 4.0, 1 << 20, 10 ** 4, 0.01, 0.95, 1e3)
