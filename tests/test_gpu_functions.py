"""Registered device functions against the oracle's independent definitions.

The device evaluates f from row/column partial sums, the oracle from the full
multi-index; both use the same deterministic exp/cos, so values are identical.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pts(rng, dims, n):
    return np.stack([rng.integers(1, d + 1, size=n) for d in dims], axis=1)


def test_lorentz(T, oracle):
    rng = np.random.default_rng(0)
    dims = [10] * 8
    P = _pts(rng, dims, 5000)
    g = T.feval(T.DeviceFunction("lorentz"), dims, P)
    r = oracle.feval(oracle.F_LORENTZ, [], P)
    assert np.array_equal(g, r)


def test_served(T, oracle):
    rng = np.random.default_rng(1)
    for _ in range(5):
        L = int(rng.integers(4, 17))
        d = int(rng.integers(2, 17))
        a, b, g = 10 ** rng.uniform(-2, 1, size=3)
        c = rng.integers(1, d + 1, size=L)
        prm = [a, b, g] + list(c)
        P = _pts(rng, [d] * L, 3000)
        assert np.array_equal(T.feval(T.DeviceFunction("served", prm), [d] * L, P),
                              oracle.feval(oracle.F_SERVED, prm, P))


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_qtt1d(T, oracle, kind):
    rng = np.random.default_rng(2 + kind)
    P = _pts(rng, [2] * 40, 5000)
    assert np.array_equal(T.feval(T.DeviceFunction("qtt1d", [kind]), [2] * 40, P),
                          oracle.feval(oracle.F_QTT1D, [kind], P))


def test_qtt2d(T, oracle):
    rng = np.random.default_rng(9)
    P = _pts(rng, [4] * 30, 5000)
    assert np.array_equal(T.feval(T.DeviceFunction("qtt2d"), [4] * 30, P), oracle.feval(oracle.F_QTT2D, [], P))


def test_dense(T, oracle):
    rng = np.random.default_rng(4)
    tab = rng.standard_normal((3, 4, 5))
    f = T.DeviceFunction.dense(tab)
    P = _pts(rng, [3, 4, 5], 200)
    assert np.array_equal(T.feval(f, [3, 4, 5], P), tab[P[:, 0] - 1, P[:, 1] - 1, P[:, 2] - 1])
