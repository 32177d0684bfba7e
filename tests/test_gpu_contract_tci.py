"""contract(A, B; algorithm=:TCI) on the device (contraction.jl:399-434): the
Contraction evaluator's environments (contraction.jl:103-176) and batch
evaluation (:236-335) run as fixed-order FP64 kernels behind the solve's value
cache, so every value equals the oracle's bit for bit and the pivots, ranks and
bond errors match exactly; site tensors come from the SITE solve and match to
a tolerance.  Against dense products the results agree to rounding, as the
reference's tests check (test/test_contraction.jl:68-99, 148-183)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rand_tt(rng, bonds, s1, s2):
    return [rng.standard_normal((bonds[n], s1[n], s2[n], bonds[n + 1])) for n in range(len(s1))]


def _close_cores(got, ref):
    assert [c.shape for c in got] == [c.shape for c in ref]
    for g, r in zip(got, ref):
        assert np.allclose(g, r, rtol=1e-8, atol=1e-10 * max(1.0, np.abs(r).max()))


@pytest.mark.parametrize("f", [None, lambda x: 2 * x])
def test_mpo_mpo_tci(T, oracle, f):
    rng = np.random.default_rng(21)
    a = _rand_tt(rng, [1, 2, 3, 2, 1], [2] * 4, [3] * 4)
    b = _rand_tt(rng, [1, 2, 3, 2, 1], [3] * 4, [2] * 4)
    ab = T.contract(a, b, tolerance=1e-12, f=f)  # algorithm=:TCI is the default
    assert [c.shape[1:3] for c in ab.sitetensors] == [(2, 2)] * 4
    ref = oracle.tt4_full(a) @ oracle.tt4_full(b)
    if f is not None:
        ref = f(ref)
    assert np.allclose(oracle.tt4_full(ab.sitetensors), ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())
    _close_cores(ab.sitetensors, oracle.tt4_contract_tci(a, b, tolerance=1e-12, f=f))


def test_mpo_mps_tci_both_orders(T, oracle):
    rng = np.random.default_rng(22)
    a = _rand_tt(rng, [1, 2, 3, 2, 1], [3] * 4, [3] * 4)
    v = [rng.standard_normal((r0, 3, r1)) for r0, r1 in zip([1, 2, 3, 2], [2, 3, 2, 1])]
    av = T.contract(a, T.TensorTrain(v), tolerance=1e-12)
    va = T.contract(T.TensorTrain(v), a, tolerance=1e-12)
    assert all(c.ndim == 3 for c in av.sitetensors + va.sitetensors)
    A = oracle.tt4_full(a)
    x = oracle.tt4_full([c.reshape(c.shape[0], 3, 1, c.shape[2], order="F") for c in v])[:, 0]
    got_av = oracle.tt4_full([c.reshape(c.shape[0], c.shape[1], 1, c.shape[2], order="F") for c in av.sitetensors])
    got_va = oracle.tt4_full([c.reshape(c.shape[0], 1, c.shape[1], c.shape[2], order="F") for c in va.sitetensors])
    assert np.allclose(got_av[:, 0], A @ x, rtol=1e-10, atol=1e-12 * np.abs(A @ x).max())
    assert np.allclose(got_va[0, :], x @ A, rtol=1e-10, atol=1e-12 * np.abs(x @ A).max())


def test_tci_parity_larger(T, oracle):
    """A 10-site operator (bond 6, 3 x 3 sites) on a random train (bond 5):
    ranks and bond errors equal the oracle's; the result reproduces the exact
    (naive, uncompressed) product at random points."""
    rng = np.random.default_rng(23)
    L = 10
    a = _rand_tt(rng, [1] + [6] * (L - 1) + [1], [3] * L, [3] * L)
    b = _rand_tt(rng, [1] + [5] * (L - 1) + [1], [3] * L, [1] * L)
    kw = dict(tolerance=1e-10, maxbonddim=40, maxiter=10)
    ab = T.contract(a, b, **kw)
    _close_cores(ab.sitetensors, oracle.tt4_contract_tci(a, b, **kw))
    exact = oracle.tt4_contract(a, b, "naive", tolerance=0.0)

    def val(cores, p):
        v = np.ones((1,))
        for n, c in enumerate(cores):
            v = v @ c[:, p[n], 0, :]
        return v[0]

    scale = max(abs(val(exact, p)) for p in rng.integers(0, 3, size=(50, L)))
    for p in rng.integers(0, 3, size=(100, L)):
        assert abs(val(ab.sitetensors, p) - val(exact, p)) <= 1e-8 * scale


def test_tci_initialpivots_and_errors(T, oracle):
    rng = np.random.default_rng(24)
    a = _rand_tt(rng, [1, 2, 2, 1], [2] * 3, [2] * 3)
    b = _rand_tt(rng, [1, 2, 2, 1], [2] * 3, [2] * 3)
    ab = T.contract(a, b, tolerance=1e-12, initialpivots=[[1, 2, 3]])
    ref = oracle.tt4_full(a) @ oracle.tt4_full(b)
    assert np.allclose(oracle.tt4_full(ab.sitetensors), ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())
    _close_cores(ab.sitetensors, oracle.tt4_contract_tci(a, b, initialpivots=[[1, 2, 3]], tolerance=1e-12))
    c = _rand_tt(rng, [1, 2, 1], [2] * 2, [2] * 2)
    with pytest.raises(T.ArgumentError, match="different length"):
        T.contract(a, c)
    d = _rand_tt(rng, [1, 2, 2, 1], [3] * 3, [2] * 3)
    with pytest.raises(T.ArgumentError, match="non-matching site dimensions"):
        T.contract(a, d)
