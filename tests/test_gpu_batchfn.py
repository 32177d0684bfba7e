"""Caller-supplied f (BatchFunction: the BatchEvaluator plugin point,
batcheval.jl:67-83, with CachedFunction's value cache, cachedfunction.jl:8-184,
held in device memory) against the CPU oracle calling the same Python f.

Both sides read identical function values, so pivots, ranks and bond errors
must match exactly, as for the registered device functions.  The f's below use
only + - * / and sum over sites in a fixed order (elementwise, one site at a
time), so that numpy gives the same bits whatever the batch it is called with.
"""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def lorentz(p):
    return 1.0 / (1.0 + (p.astype(np.int64) ** 2).sum(1))


def coupled(p):
    """Non-separable rational f of 1-based multi-indices."""
    v = p.astype(np.float64)
    s = np.zeros(v.shape[0])
    q = np.zeros(v.shape[0])
    for k in range(v.shape[1]):
        s = s + v[:, k] * (1.0 + k / 4.0)
        q = q + (v[:, k] - (1.0 + k % 3)) ** 2
    return 1.0 / (1.0 + s * s / 50.0) + 0.5 / (1.0 + q)


def quantics(p):
    """f(x) = 1/(1 + 100 (x - 0.37)^2) on x = sum_i b_i 2^-i, b_i = v_i - 1."""
    x = np.zeros(p.shape[0])
    for k in range(p.shape[1]):
        x = x + (p[:, k] - 1) * 0.5 ** (k + 1)
    return 1.0 / (1.0 + 100.0 * (x - 0.37) ** 2)


def _same_sets(tci, ref):
    for b in range(1, len(tci) + 1):
        gi, gj = tci.sets(b)
        ri, rj = ref.sets(b)
        assert np.array_equal(gi, ri), f"Iset[{b}] differs"
        assert np.array_equal(gj, rj), f"Jset[{b}] differs"


class Recorder:
    """Wraps f and keeps every point it was asked for."""

    def __init__(self, f):
        self.f = f
        self.seen = []

    def __call__(self, p):
        self.seen.append(p.copy())
        return self.f(p)


def test_batch_lorentz_equals_registered(T, oracle):
    """The Lorentzian as a caller-supplied f gives the registered function's
    solve bit for bit (pivots, errors, site tensors)."""
    kw = dict(tolerance=1e-10, maxiter=30)
    bf = T.BatchFunction(lorentz)
    a, ra, ea = T.crossinterpolate2(float, bf, [10] * 6, **kw)
    b, rb, eb = T.crossinterpolate2(float, T.DeviceFunction("lorentz"), [10] * 6, **kw)
    assert list(ra) == list(rb)
    assert np.array_equal(ea, eb)
    _same_sets(a, b)
    for s in range(1, 7):
        assert np.array_equal(a.sitetensor(s), b.sitetensor(s))
    assert a.sum() == b.sum()
    ofid = oracle.register_fn(lorentz)
    ref, rr, _ = oracle.crossinterpolate2([10] * 6, ofid, (), None, **kw)
    assert list(ra) == list(rr)
    _same_sets(a, ref)


@pytest.mark.parametrize("L,d,tol", [(7, 6, 1e-10), (5, 12, 1e-8), (9, 3, 1e-12)])
def test_batch_coupled_parity(T, oracle, L, d, tol):
    kw = dict(tolerance=tol, maxiter=40, maxbonddim=64)
    bf = T.BatchFunction(coupled)
    tci, ranks, errors = T.crossinterpolate2(float, bf, [d] * L, **kw)
    ofid = oracle.register_fn(coupled)
    ref, rranks, rerrors = oracle.crossinterpolate2([d] * L, ofid, (), None, **kw)
    assert list(ranks) == list(rranks)
    _same_sets(tci, ref)
    assert np.array_equal(tci.bonderrors, ref.errors()[1])
    for s in range(1, L + 1):
        assert np.allclose(tci.sitetensor(s), ref.core(s), rtol=1e-9, atol=1e-12)
    pts = np.random.default_rng(L).integers(1, d + 1, size=(2000, L))
    assert np.max(np.abs(tci.evaluate(pts) - coupled(pts))) <= 10 * max(tol, 1e-12) * np.abs(coupled(pts)).max()


def test_batch_cache_counts(T, oracle):
    """Every distinct point reaches f once: the device cache serves repeats
    across bonds, sweeps and the final sweep1site!, and f is called once per
    device step that needs new values."""
    rec = Recorder(coupled)
    bf = T.BatchFunction(rec)
    tci, ranks, _ = T.crossinterpolate2(float, bf, [6] * 7, tolerance=1e-10, maxiter=40)
    pts = np.concatenate(rec.seen)
    keys = {tuple(x) for x in pts.tolist()}
    assert len(keys) == pts.shape[0], "a point reached f twice"
    entries, evaluated, calls = tci.fcache_stats()
    assert entries == evaluated == pts.shape[0] == bf.npoints
    assert calls == bf.ncalls == len(rec.seen)
    ofid = oracle.register_fn(coupled)
    ref, _, _ = oracle.crossinterpolate2([6] * 7, ofid, (), None, tolerance=1e-10, maxiter=40)
    assert evaluated < ref.nfeval
    # more sweeps on the same solve revisit known points
    n0 = bf.npoints
    tci.optimize(tolerance=1e-10, maxiter=3)
    assert bf.npoints - n0 < n0


def test_batch_split_keys(T, oracle):
    """60 quantics sites: the cache keys span two words (2^60 > 2^52)."""
    kw = dict(tolerance=1e-9, maxiter=20, maxbonddim=32)
    bf = T.BatchFunction(quantics)
    tci, ranks, _ = T.crossinterpolate2(float, bf, [2] * 60, **kw)
    ofid = oracle.register_fn(quantics)
    ref, rranks, _ = oracle.crossinterpolate2([2] * 60, ofid, (), None, **kw)
    assert list(ranks) == list(rranks)
    _same_sets(tci, ref)
    pts = np.random.default_rng(5).integers(1, 3, size=(1000, 60))
    assert np.max(np.abs(tci.evaluate(pts) - quantics(pts))) < 1e-7


def test_batch_errors(T):
    """An exception in f and a NaN value map to the reference's failures; the
    context stays usable."""
    def boom(p):
        raise RuntimeError("no values")

    bf = T.BatchFunction(boom)
    with pytest.raises(RuntimeError, match="no values") as ei:
        T.crossinterpolate2(float, bf, [4] * 4, tolerance=1e-8)
    assert isinstance(ei.value.__cause__, T.TCIError)
    assert isinstance(bf.error, RuntimeError)

    def nan_at(p):
        v = lorentz(p)
        v[(p[:, 0] == 2) & (p[:, 1] == 3)] = np.nan
        return v

    with pytest.raises(T.TCIError, match="NaN"):
        T.crossinterpolate2(float, T.BatchFunction(nan_at), [4] * 4, tolerance=1e-8)
    tci, _, _ = T.crossinterpolate2(float, T.BatchFunction(lorentz), [4] * 4, tolerance=1e-8)
    assert tci.rank() >= 1


def test_batch_evaluate_feval_and_updatepivots(T, oracle):
    """evaluate() of the train does not call f; feval() calls it directly;
    the step-by-step entry points (updatepivots!, sweep1site!) agree with the
    oracle."""
    bf = T.BatchFunction(coupled)
    tci, _, _ = T.crossinterpolate2(float, bf, [5] * 5, tolerance=1e-10)
    n = bf.ncalls
    pts = np.array(list(itertools.product(*[range(1, 4)] * 5)))
    tci.evaluate(pts)
    assert bf.ncalls == n
    assert np.array_equal(T.feval(bf, [5] * 5, pts), coupled(pts))
    step = T.TensorCI2(bf, [5] * 5)
    ofid = oracle.register_fn(coupled)
    ref = oracle.OracleTCI.new([5] * 5, ofid)
    for p in range(1, 5):
        step.updatepivots(p, True, reltol=1e-10, maxbonddim=4)
        ref.updatepivots(p, True, reltol=1e-10, maxbonddim=4)
    _same_sets(step, ref)
    step.sweep1site("forward", reltol=1e-12)
    ref.sweep1site(True, reltol=1e-12)
    _same_sets(step, ref)
