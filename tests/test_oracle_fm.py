"""Oracle Boys function against the reference's known-answer test
(src/tests/test_fm.f90:1-82): downward recursion from m = 1000 with a zero
start below t = 510, the asymptotic form above it; abs 1e-15, rel 1e-12."""
import math

import numpy as np
import pytest

XLIST = [0.0, 1e-9, 1e-6, 0.1, 0.5, 2.0, 10.0, 15.0, 19.0, 20.0, 21.0, 25.0, 30.0, 50.0, 100.0,
         150.0, 200.0, 500.0, 2000.0, 20000.0, 2e5, 2e6, 2e8]


def _downwards(maxm, t):
    F = np.zeros(maxm + 1)
    for m in range(maxm - 1, -1, -1):
        F[m] = (2 * t * F[m + 1] + math.exp(-t)) / (2 * m + 1)
    return F


def _asympt(maxm, t):
    m = np.arange(maxm + 1)
    return np.array([math.exp(math.lgamma(k + 0.5) - (k + 0.5) * math.log(t)) / 2 for k in m])


def _rel(a, b):
    d = np.abs(a - b)
    m = np.maximum(np.abs(a), np.abs(b))
    return np.where(d < np.finfo(float).tiny, 0.0, d / np.where(m == 0, 1, m))


@pytest.mark.parametrize("x", XLIST)
def test_fm_known_answers(oracle, x):
    F = _downwards(1000, x) if x < 510 else _asympt(1000, x)
    F0 = 1.0 if x < np.finfo(float).eps else 0.5 * math.sqrt(math.pi / x) * math.erf(math.sqrt(x))
    assert abs(F[0] - F0) < 1e-15
    assert abs(F[0] - F0) / F[0] < 1e-14
    for m in range(0, 501):
        G = oracle.boys(m, x)
        assert np.all(np.abs(G - F[:m + 1]) < 1e-15)
        assert np.all(_rel(F[:m + 1], G) < 1e-12)


def test_fm_rejects_bad_arguments(oracle):
    with pytest.raises(ValueError):
        oracle.boys(501, 1.0)
    with pytest.raises(ValueError):
        oracle.boys(2, -1.0)
