"""Caller-supplied f (the BatchEvaluator plugin point, batcheval.jl:67-83) on
the CPU: the oracle's callback path against its registered-function path, and
the library's evaluator registry (host only, no device work)."""
import numpy as np
import pytest


def lorentz(p):
    return 1.0 / (1.0 + (p.astype(np.int64) ** 2).sum(1))


def test_oracle_callback_equals_registered(oracle):
    """The same f through the oracle's callback path and its registered Lorentzian:
    identical pivots, errors and site tensors, bit for bit."""
    fid = oracle.register_fn(lorentz)
    a, ra, ea = oracle.crossinterpolate2([10] * 5, oracle.F_LORENTZ, (), None, tolerance=1e-10, maxiter=50)
    b, rb, eb = oracle.crossinterpolate2([10] * 5, fid, (), None, tolerance=1e-10, maxiter=50)
    assert list(ra) == list(rb)
    assert np.array_equal(ea, eb)
    for s in range(1, 6):
        assert np.array_equal(a.core(s), b.core(s))
        for x, y in zip(a.sets(s), b.sets(s)):
            assert np.array_equal(x, y)
    pts = np.random.default_rng(3).integers(1, 11, size=(50, 5))
    assert np.array_equal(oracle.feval(fid, (), pts), lorentz(pts))


def test_library_registry(T):
    """tci_f_register hands out ids from TCI_F_USER on, reuses freed ids and
    rejects unknown ones (pure host logic of libtci_gpu.so)."""
    f1 = T.BatchFunction(lorentz)
    f2 = T.BatchFunction(lorentz)
    assert f1.fid >= 1024 and f2.fid >= 1024 and f1.fid != f2.fid
    old = f1.fid
    f1.close()
    f3 = T.BatchFunction(lorentz)
    assert f3.fid == old
    with pytest.raises(T.ArgumentError):
        T._check(T.load_library().tci_f_unregister(old + 1000))
    f2.close()
    f3.close()
