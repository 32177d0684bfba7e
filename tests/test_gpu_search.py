"""optfirstpivot (util.jl:78-108) and estimatetrueerror (globalsearch.jl:1-96) on
the device against the oracle: both evaluate f bit-identically and the train
with the same summation order, so pivots and errors must match exactly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _table_f(T, golden):
    g = golden["util"]["optfirstpivot"]
    table = np.zeros(g["localdims"])
    for idx in np.ndindex(*table.shape):
        table[idx] = 4 * idx[2] + 2 * idx[1] + idx[0]
    return g, table


def test_optfirstpivot_known_answer(T, golden):
    g, table = _table_f(T, golden)
    assert list(T.optfirstpivot(T.DeviceFunction.dense(table), g["localdims"], g["firstpivot"])) == g["expect"]

    def f(p):
        return 4.0 * (p[:, 2] - 1) + 2.0 * (p[:, 1] - 1) + (p[:, 0] - 1)

    assert list(T.optfirstpivot(T.BatchFunction(f), g["localdims"], g["firstpivot"])) == g["expect"]


def test_optfirstpivot_parity(T, oracle):
    rng = np.random.default_rng(31)
    L, d = 6, 7
    c = rng.integers(1, d + 1, size=L).astype(float)
    params = np.concatenate([[0.3, 2.0, 0.05], c])
    f = T.DeviceFunction("served", params)
    for _ in range(5):
        start = rng.integers(1, d + 1, size=L)
        got = T.optfirstpivot(f, [d] * L, start)
        want = oracle.optfirstpivot(oracle.F_SERVED, params, [d] * L, start)
        assert np.array_equal(got, want)


def test_estimatetrueerror_parity(T, oracle):
    R = 20
    f = T.DeviceFunction("qtt1d", [0])
    first = [np.ones(R, dtype=int), np.r_[1, np.full(R - 1, 2)]]
    tci, _, _ = T.crossinterpolate2(float, f, [2] * R, first, tolerance=1e-4, maxbonddim=1, normalizeerror=False)
    starts = np.random.default_rng(1240).integers(1, 3, size=(40, R))
    got = tci.estimatetrueerror(initialpoints=starts)
    want = oracle.estimatetrueerror(oracle.F_QTT1D, [0], tci.sitetensors, starts)
    assert len(got) == len(want)
    for (gp, ge), (wp, we) in zip(got, want):
        assert np.array_equal(gp, wp) and ge == we
    errs = [e for _, e in got]
    assert all(errs[k] >= errs[k + 1] for k in range(len(errs) - 1))
    pts = np.array([p for p, _ in got])
    assert np.allclose(np.abs(T.feval(f, [2] * R, pts) - tci.evaluate(pts)), errs, rtol=1e-12, atol=0)
    rnd = tci.estimatetrueerror(nsearch=20, seed=3)
    assert 1 <= len(rnd) <= 20 and all(rnd[k][1] >= rnd[k + 1][1] for k in range(len(rnd) - 1))


def test_estimatetrueerror_caller_f(T):
    def f(p):
        return 1.0 / (1.0 + (p.astype(np.int64) ** 2).sum(1))

    bf = T.BatchFunction(f)
    tci, _, _ = T.crossinterpolate2(float, bf, [6] * 5, tolerance=1e-3, maxbonddim=2)
    res = tci.estimatetrueerror(nsearch=10, seed=1)
    pts = np.array([p for p, _ in res])
    assert np.allclose(np.abs(f(pts) - tci.evaluate(pts)), [e for _, e in res], rtol=1e-12, atol=1e-300)
