"""addglobalpivots2sitesweep! (tensorci2.jl:243-288) on the oracle, as the
reference's own tests use it (test/test_tensorci2.jl:343-431): pivots that the
interpolation missed are inserted, and afterwards the train reproduces f there.
The reference draws its peak positions with Julia's rand and maps bit lists to
x through QuanticsGrids (DiscretizedGrid{1}(R, 0, 1): x = sum_i (b_i - 1) 2^-i);
here a seeded numpy generator and the same mapping stand in."""
import numpy as np
import pytest

R = 20


def _x(bits):
    return ((np.asarray(bits, np.int64) - 1) * (0.5 ** np.arange(1, bits.shape[1] + 1))).sum(1)


def test_insert_single_missed_pivot(oracle):
    """test_tensorci2.jl:395-431: f is 1 on all-ones and all-twos and 0 elsewhere;
    from the all-ones pivot the sweep never sees all-twos, inserting it fixes that."""

    def f(p):
        return (np.all(p == 1, axis=1) | np.all(p == 2, axis=1)).astype(np.float64)

    fid = oracle.register_fn(f)
    kw = dict(tolerance=1e-4, maxbonddim=1000, maxiter=20, normalizeerror=False, strictlynested=False)
    tci, _, _ = oracle.crossinterpolate2([2] * R, fid, (), None, **kw)
    r = np.full((1, R), 2, np.int64)
    assert abs(tci.evaluate(r)[0] - 1.0) > 0.5  # missed before
    left = tci.addglobalpivots2sitesweep((fid, ()), r, tolerance=1e-4, normalizeerror=False, maxbonddim=1000)
    assert left == 0
    assert tci.evaluate(r)[0] == pytest.approx(1.0)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_insert_narrow_peaks(oracle, seed):
    """test_tensorci2.jl:343-393: exp(-10x) plus 100 peaks of height 2e-4 and
    half-width 10 / 2^R at random lattice points; after crossinterpolate2 and
    addglobalpivots2sitesweep! with those points (ntry 1, pivotsearch full) the
    train is within abstol of f at every one of them."""
    rng = np.random.default_rng(seed)
    abstol = 1e-4
    delta = 10.0 / 2**R
    rindex = rng.integers(1, 3, size=(100, R))
    rpoint = _x(rindex)

    def f(p):
        x = _x(p)
        return np.exp(-10 * x) + 2 * abstol * (np.abs(x[:, None] - rpoint[None, :]) < delta).sum(1)

    fid = oracle.register_fn(f)
    kw = dict(tolerance=abstol, maxbonddim=1000, maxiter=20, normalizeerror=False, strictlynested=False)
    tci, _, _ = oracle.crossinterpolate2([2] * R, fid, (), None, **kw)
    tci.addglobalpivots2sitesweep((fid, ()), rindex, tolerance=abstol, normalizeerror=False, maxbonddim=1000,
                                  ntry=1)
    assert np.sum(np.abs(tci.evaluate(rindex) - f(rindex)) > abstol) == 0


def test_pivot_length_mismatch(oracle):
    """A pivot with the wrong number of legs: the reference's DimensionMismatch
    (tensorci2.jl:255-257), reported by the oracle's addglobalpivots!."""
    tci, _, _ = oracle.crossinterpolate2([3] * 4, oracle.F_LORENTZ, (), None, tolerance=1e-6, maxiter=3)
    with pytest.raises(oracle.OracleError, match="one index per leg") as e:
        tci.addglobalpivots2sitesweep((oracle.F_LORENTZ, ()), np.ones((1, 3), np.int64))
    assert e.value.code == 2
    assert tci.addglobalpivots2sitesweep((oracle.F_LORENTZ, ()), np.zeros((0, 4), np.int64)) == 0


def _nasty(p):
    x = _x(p)
    return np.exp(-10 * x) * np.sin(2 * np.pi * 100 * x**1.1)


def test_globalsearch_nasty_function(oracle):
    """test_tensorci2.jl:433-459: a 10-bit quantics function that oscillates
    100 times, from optfirstpivot of a random start, with 10 global-pivot
    searches per iteration: the last error is below 1e-10."""
    n = 10
    fid = oracle.register_fn(_nasty)
    start = np.random.default_rng(1234).integers(1, 3, size=n)
    first = oracle.optfirstpivot(fid, (), [2] * n, start)
    _, ranks, errors = oracle.crossinterpolate2([2] * n, fid, (), [first], tolerance=1e-12, maxbonddim=100,
                                                maxiter=100, nsearchglobalpivot=10, strictlynested=False)
    assert errors[-1] < 1e-10
