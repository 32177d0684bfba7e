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


def test_oracle_reconstructs_a_tensor_train(oracle):
    """test/test_tensorci2.jl:477-502: crossinterpolate2 of a function that is itself
    a tensor train (bonds 1, 2, 3, 2, 1; local dims 2, 3, 3, 2), tolerance 1e-10,
    maxbonddim 10, reproduces it at every point."""
    rng = np.random.default_rng(5)
    bonds, dims = [1, 2, 3, 2, 1], [2, 3, 3, 2]
    cores = [rng.random((bonds[n], dims[n], bonds[n + 1])) for n in range(4)]

    def tt(p):
        out = np.empty(p.shape[0])
        for k, q in enumerate(p):
            v = np.ones(1)
            for n, c in enumerate(cores):
                v = v @ c[:, q[n] - 1, :]
            out[k] = v[0]
        return out

    fid = oracle.register_fn(tt)
    ref, _, _ = oracle.crossinterpolate2(dims, fid, (), None, tolerance=1e-10, maxbonddim=10)
    pts = np.array(list(np.ndindex(*dims))) + 1
    assert np.allclose(ref.evaluate(pts), tt(pts), rtol=1e-9, atol=1e-12)
