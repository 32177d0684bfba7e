"""The oracle's tensor-train contraction against dense products, as the
reference's own tests check it (test/test_contraction.jl:68-99, 148-195):
_tomat(contract(a, b)) ≈ _tomat(a) * _tomat(b) for :naive and :zipup, and the
MPO-MPS case through unit legs."""
import numpy as np
import pytest


def _rand_tt(rng, bonds, s1, s2):
    return [rng.standard_normal((bonds[n], s1[n], s2[n], bonds[n + 1])) for n in range(len(s1))]


def _testdata(rng):
    # the reference's shapes (test_contraction.jl:5-30): N = 4, bonds [1,2,3,2,1],
    # local dims 2 / 3 / 2
    N = 4
    a = _rand_tt(rng, [1, 2, 3, 2, 1], [2] * N, [3] * N)
    b = _rand_tt(rng, [1, 2, 3, 2, 1], [3] * N, [2] * N)
    return a, b


@pytest.mark.parametrize("algorithm", ["naive", "zipup"])
def test_mpo_mpo(oracle, algorithm):
    a, b = _testdata(np.random.default_rng(1))
    ab = oracle.tt4_contract(a, b, algorithm, tolerance=1e-12)
    assert [c.shape[1:3] for c in ab] == [(2, 2)] * 4
    ref = oracle.tt4_full(a) @ oracle.tt4_full(b)
    assert np.allclose(oracle.tt4_full(ab), ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("algorithm", ["naive", "zipup"])
def test_mpo_mps(oracle, algorithm):
    rng = np.random.default_rng(2)
    a = _rand_tt(rng, [1, 2, 3, 2, 1], [3] * 4, [3] * 4)
    v = [rng.standard_normal((r0, 3, r1)) for r0, r1 in zip([1, 2, 3, 2], [2, 3, 2, 1])]
    v4 = [c.reshape(c.shape[0], 3, 1, c.shape[2], order="F") for c in v]
    ab = oracle.tt4_contract(a, v4, algorithm, tolerance=1e-12)
    ref = oracle.tt4_full(a) @ oracle.tt4_full(v4)
    assert np.allclose(oracle.tt4_full(ab), ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())


def test_zipup_truncation_and_compress(oracle):
    rng = np.random.default_rng(3)
    a = _rand_tt(rng, [1, 4, 6, 6, 4, 1], [2] * 5, [2] * 5)
    b = _rand_tt(rng, [1, 3, 5, 5, 3, 1], [2] * 5, [2] * 5)
    ref = oracle.tt4_full(a) @ oracle.tt4_full(b)
    ab = oracle.tt4_contract(a, b, "zipup", tolerance=1e-12, maxbonddim=7)
    assert max(c.shape[3] for c in ab) <= 7
    naive = oracle.tt4_contract(a, b, "naive", tolerance=0.0)
    assert [c.shape[3] for c in naive[:-1]] == [12, 30, 30, 12]
    comp = oracle.tt4_compress(naive, tolerance=1e-10)
    assert [c.shape[3] for c in comp[:-1]] == [4, 16, 16, 4]  # the exact ranks of the 2-by-2 product
    assert np.allclose(oracle.tt4_full(comp), ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max())


@pytest.mark.parametrize("method", ["LU", "CI"])
def test_factorization_methods(oracle, method):
    """compress!(:LU / :CI) and contract_zipup(method) reproduce the dense product
    (tensortrain.jl:94-110: _factorize with rrlu or MatrixLUCI)."""
    rng = np.random.default_rng(4)
    a = _rand_tt(rng, [1, 4, 6, 6, 4, 1], [2] * 5, [2] * 5)
    b = _rand_tt(rng, [1, 3, 5, 5, 3, 1], [2] * 5, [2] * 5)
    ref = oracle.tt4_full(a) @ oracle.tt4_full(b)
    naive = oracle.tt4_contract(a, b, "naive", tolerance=0.0)
    comp = oracle.tt4_compress(naive, method, tolerance=1e-10)
    assert [c.shape[3] for c in comp[:-1]] == [4, 16, 16, 4]
    assert np.allclose(oracle.tt4_full(comp), ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max())
    zu = oracle.tt4_contract(a, b, "zipup", tolerance=1e-12, method=method)
    assert np.allclose(oracle.tt4_full(zu), ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max())



@pytest.mark.parametrize("f", [None, lambda x: 2 * x])
def test_contract_tci(oracle, f):
    """contract(a, b; algorithm=:TCI, f) (contraction.jl:399-434) reproduces the
    dense product, as test/test_contraction.jl:68-99, 148-183 check it."""
    a, b = _testdata(np.random.default_rng(6))
    ab = oracle.tt4_contract_tci(a, b, tolerance=1e-12, f=f)
    assert [c.shape[1:3] for c in ab] == [(2, 2)] * 4
    ref = oracle.tt4_full(a) @ oracle.tt4_full(b)
    if f is not None:
        ref = f(ref)
    assert np.allclose(oracle.tt4_full(ab), ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())
    rng = np.random.default_rng(7)
    a = _rand_tt(rng, [1, 2, 3, 2, 1], [3] * 4, [3] * 4)
    v4 = [rng.standard_normal((r0, 3, 1, r1)) for r0, r1 in zip([1, 2, 3, 2], [2, 3, 2, 1])]
    av = oracle.tt4_contract_tci(a, v4, tolerance=1e-12, f=f)
    ref = oracle.tt4_full(a) @ oracle.tt4_full(v4)
    if f is not None:
        ref = f(ref)
    assert np.allclose(oracle.tt4_full(av), ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())
