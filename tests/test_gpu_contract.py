"""GPU tensor-train contraction (contract :naive / :zipup, compress! with :LU and :CI)
against the CPU oracle.  Both sum every contracted element in the same fixed
order with separate multiply and add and factor with the same bit-exact rrLU,
so the cores must be equal bit for bit; against dense products the results
agree to rounding, as the reference's tests check them
(test/test_contraction.jl:68-99, 148-195)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rand_tt(rng, bonds, s1, s2):
    return [rng.standard_normal((bonds[n], s1[n], s2[n], bonds[n + 1])) for n in range(len(s1))]


def _same(gpu_tt, ref_cores):
    assert len(gpu_tt) == len(ref_cores)
    for g, r in zip(gpu_tt.sitetensors, ref_cores):
        assert g.shape == r.shape
        assert np.array_equal(g, r)


@pytest.mark.parametrize("algorithm", ["naive", "zipup"])
def test_mpo_mpo_bitwise(T, oracle, algorithm):
    rng = np.random.default_rng(11)
    a = _rand_tt(rng, [1, 2, 3, 2, 1], [2] * 4, [3] * 4)
    b = _rand_tt(rng, [1, 2, 3, 2, 1], [3] * 4, [2] * 4)
    ab = T.contract(a, b, algorithm=algorithm, tolerance=1e-12, method="LU")
    _same(ab, oracle.tt4_contract(a, b, algorithm, tolerance=1e-12))
    ref = oracle.tt4_full(a) @ oracle.tt4_full(b)
    assert np.allclose(oracle.tt4_full(ab.sitetensors), ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("tol,maxbond", [(1e-12, None), (1e-6, None), (1e-12, 5), (0.0, 3)])
def test_zipup_truncation_bitwise(T, oracle, tol, maxbond):
    rng = np.random.default_rng(12)
    a = _rand_tt(rng, [1, 4, 6, 6, 4, 1], [2] * 5, [3] * 5)
    b = _rand_tt(rng, [1, 3, 5, 5, 3, 1], [3] * 5, [2] * 5)
    ab = T.contract(a, b, algorithm="zipup", tolerance=tol, maxbonddim=maxbond, method="LU")
    _same(ab, oracle.tt4_contract(a, b, "zipup", tolerance=tol, maxbonddim=maxbond))
    if maxbond:
        assert max(c.shape[3] for c in ab.sitetensors) <= maxbond


def test_naive_with_compression_bitwise(T, oracle):
    rng = np.random.default_rng(13)
    a = _rand_tt(rng, [1, 4, 6, 6, 4, 1], [2] * 5, [2] * 5)
    b = _rand_tt(rng, [1, 3, 5, 5, 3, 1], [2] * 5, [2] * 5)
    ab = T.contract(a, b, algorithm="naive", tolerance=1e-10, method="LU")
    _same(ab, oracle.tt4_contract(a, b, "naive", tolerance=1e-10))
    assert [c.shape[3] for c in ab.sitetensors[:-1]] == [4, 16, 16, 4]


def test_compress_bitwise(T, oracle):
    rng = np.random.default_rng(14)
    tt = _rand_tt(rng, [1, 6, 9, 9, 6, 1], [2] * 5, [2] * 5)
    for tol, mb, ne in [(1e-12, None, True), (1e-3, None, True), (1e-12, 4, True), (1e-8, None, False)]:
        got = T.compress(tt, tolerance=tol, maxbonddim=mb, normalizeerror=ne)
        _same(got, oracle.tt4_compress(tt, tolerance=tol, maxbonddim=mb, normalizeerror=ne))


@pytest.mark.parametrize("algorithm", ["naive", "zipup"])
def test_mpo_mps(T, oracle, algorithm):
    """contract(TT4, TT3) -> TT3 (contraction.jl:548-560)."""
    rng = np.random.default_rng(15)
    a = _rand_tt(rng, [1, 2, 3, 2, 1], [3] * 4, [3] * 4)
    v = [rng.standard_normal((r0, 3, r1)) for r0, r1 in zip([1, 2, 3, 2], [2, 3, 2, 1])]
    ab = T.contract(a, T.TensorTrain(v), algorithm=algorithm, tolerance=1e-12, method="LU")
    assert all(c.ndim == 3 for c in ab.sitetensors)
    v4 = [c.reshape(c.shape[0], 3, 1, c.shape[2], order="F") for c in v]
    ref = (oracle.tt4_full(a) @ oracle.tt4_full(v4))[:, 0]
    got = oracle.tt4_full([c.reshape(c.shape[0], c.shape[1], 1, c.shape[2], order="F") for c in ab.sitetensors])
    assert np.allclose(got[:, 0], ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())


def test_contract_with_tci_result(T, oracle):
    """contract(TT4 operator, TensorCI2) -> TT3, the MPO-MPS case of the 2-D
    quantics configuration at a small size."""
    rng = np.random.default_rng(17)
    tci, _, _ = T.crossinterpolate2(float, T.DeviceFunction("qtt2d"), [4] * 6, tolerance=1e-9, maxbonddim=64)
    bonds = [1, 3, 3, 3, 3, 3, 1]
    op = [rng.standard_normal((bonds[i], 4, 4, bonds[i + 1])) / 2.0 for i in range(6)]
    ab = T.contract(op, tci, algorithm="zipup", tolerance=1e-12, method="LU")
    v4 = [c.reshape(c.shape[0], 4, 1, c.shape[2], order="F") for c in tci.sitetensors]
    ref = (oracle.tt4_full(op) @ oracle.tt4_full(v4))[:, 0]
    got = oracle.tt4_full([c.reshape(c.shape[0], c.shape[1], 1, c.shape[2], order="F") for c in ab.sitetensors])
    assert np.allclose(got[:, 0], ref, rtol=1e-9, atol=1e-11 * np.abs(ref).max())


def test_contract_errors_like_reference(T):
    rng = np.random.default_rng(16)
    a = _rand_tt(rng, [1, 2, 2, 1], [2] * 3, [3] * 3)
    b = _rand_tt(rng, [1, 2, 1], [3] * 2, [2] * 2)
    with pytest.raises(T.ArgumentError):  # contraction.jl:452-454 / :40-42
        T.contract(a, b, algorithm="zipup")
    c = _rand_tt(rng, [1, 2, 2, 1], [4] * 3, [2] * 3)
    with pytest.raises(T.TCIError, match="identical index"):  # contraction.jl:43-46
        T.contract(a, c, algorithm="naive")
    with pytest.raises(T.TCIError, match="cannot contract matrix product with a function"):
        T.contract(a, a, algorithm="naive", f=lambda x: 2 * x)
    with pytest.raises(T.ArgumentError, match="Unknown algorithm"):
        T.contract(a, a, algorithm="bogus")


def test_ci_factorization_bitwise(T, oracle):
    """compress!(:CI) and contract(:zipup / :naive, method=:CI): MatrixLUCI's
    left/right (matrixluci.jl:40-84) on the device equal the oracle's bit for bit."""
    rng = np.random.default_rng(18)
    tt = _rand_tt(rng, [1, 6, 9, 9, 6, 1], [2] * 5, [2] * 5)
    for tol, mb, ne in [(1e-12, None, True), (1e-3, None, True), (1e-12, 4, True), (1e-8, None, False)]:
        got = T.compress(tt, method="CI", tolerance=tol, maxbonddim=mb, normalizeerror=ne)
        _same(got, oracle.tt4_compress(tt, "CI", tolerance=tol, maxbonddim=mb, normalizeerror=ne))
    a = _rand_tt(rng, [1, 4, 6, 6, 4, 1], [2] * 5, [3] * 5)
    b = _rand_tt(rng, [1, 3, 5, 5, 3, 1], [3] * 5, [2] * 5)
    for algorithm in ["zipup", "naive"]:
        ab = T.contract(a, b, algorithm=algorithm, tolerance=1e-10, method="CI")
        _same(ab, oracle.tt4_contract(a, b, algorithm, tolerance=1e-10, method="CI"))
        ref = oracle.tt4_full(a) @ oracle.tt4_full(b)
        assert np.allclose(oracle.tt4_full(ab.sitetensors), ref, rtol=1e-7, atol=1e-9 * np.abs(ref).max())
    with pytest.raises(T.TCIError, match="not available"):
        T.compress(tt, method="SVD")
