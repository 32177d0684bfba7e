"""TensorCI2.addglobalpivots2sitesweep (tensorci2.jl:243-288) on the device
against the oracle, on the reference's own two cases
(test/test_tensorci2.jl:343-431) with f supplied by the caller: the same number
of pivots left, the same link dimensions, and the train within abstol of f at
every inserted pivot."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

R = 20


def _x(bits):
    return ((np.asarray(bits, np.int64) - 1) * (0.5 ** np.arange(1, bits.shape[1] + 1))).sum(1)


def _both(T, oracle, f, pivots, **kw):
    opts = dict(tolerance=kw["tolerance"], maxbonddim=1000, maxiter=20, normalizeerror=False, strictlynested=False)
    fid = oracle.register_fn(f)
    ref, _, _ = oracle.crossinterpolate2([2] * R, fid, (), None, **opts)
    nref = ref.addglobalpivots2sitesweep((fid, ()), pivots, **kw)
    bf = T.BatchFunction(f)
    try:
        tci, _, _ = T.crossinterpolate2(float, bf, [2] * R, **opts)
        n = tci.addglobalpivots2sitesweep(pivots, **kw)
        assert n == nref
        assert list(tci.linkdims()) == list(ref.linkdims())
        return tci, ref
    finally:
        bf.close()


def test_insert_single_missed_pivot(T, oracle):
    def f(p):
        return (np.all(p == 1, axis=1) | np.all(p == 2, axis=1)).astype(np.float64)

    r = np.full((1, R), 2, np.int64)
    tci, ref = _both(T, oracle, f, r, tolerance=1e-4, normalizeerror=False, maxbonddim=1000)
    assert tci.evaluate(r)[0] == pytest.approx(1.0)
    assert tci.evaluate(r)[0] == pytest.approx(ref.evaluate(r)[0], rel=1e-12, abs=1e-14)


def test_insert_narrow_peaks(T, oracle):
    rng = np.random.default_rng(1)
    abstol = 1e-4
    delta = 10.0 / 2**R
    rindex = rng.integers(1, 3, size=(100, R))
    rpoint = _x(rindex)

    def f(p):
        x = _x(p)
        return np.exp(-10 * x) + 2 * abstol * (np.abs(x[:, None] - rpoint[None, :]) < delta).sum(1)

    tci, ref = _both(T, oracle, f, rindex, tolerance=abstol, normalizeerror=False, maxbonddim=1000, ntry=1)
    assert np.sum(np.abs(tci.evaluate(rindex) - f(rindex)) > abstol) == 0
    assert np.allclose(tci.evaluate(rindex), ref.evaluate(rindex), rtol=1e-10, atol=1e-12)


def test_pivot_length_mismatch(T):
    tci, _, _ = T.crossinterpolate2(float, T.DeviceFunction("lorentz"), [3] * 4, tolerance=1e-6, maxiter=3)
    with pytest.raises(T.DimensionMismatch):
        tci.addglobalpivots2sitesweep([[1, 1, 1]])
    with pytest.raises(T.ArgumentError):
        tci.addglobalpivots2sitesweep([[1, 1, 1, 1]], pivotsearch="rook")
    assert tci.addglobalpivots2sitesweep([]) == 0


def test_globalsearch_nasty_function(T, oracle):
    """test_tensorci2.jl:433-459 on the device: from optfirstpivot of a random
    start, with 10 global-pivot searches per iteration, the same first pivot,
    ranks and errors as the oracle, and the last error below 1e-10."""
    n = 10

    def f(p):
        x = _x(p)
        return np.exp(-10 * x) * np.sin(2 * np.pi * 100 * x**1.1)

    start = np.random.default_rng(1234).integers(1, 3, size=n)
    ofid = oracle.register_fn(f)
    ofirst = oracle.optfirstpivot(ofid, (), [2] * n, start.copy())
    kw = dict(tolerance=1e-12, maxbonddim=100, maxiter=100, nsearchglobalpivot=10, strictlynested=False)
    _, rranks, rerrors = oracle.crossinterpolate2([2] * n, ofid, (), [ofirst], **kw)
    bf = T.BatchFunction(f)
    try:
        first = T.optfirstpivot(bf, [2] * n, start)
        assert list(first) == list(ofirst)
        _, ranks, errors = T.crossinterpolate2(float, bf, [2] * n, [first], **kw)
    finally:
        bf.close()
    assert list(ranks) == list(rranks)
    assert np.array_equal(errors, rerrors)
    assert errors[-1] < 1e-10
