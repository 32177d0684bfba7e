"""GPU rank-revealing LU (step kernel, via the C ABI) against the CPU oracle.

Pivots, pivot count and error are bit-exact; L and U are bitwise equal as well,
since both sides do the same IEEE operations in the same order.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same(gpu, ref):
    K = ref["npivot"]
    assert gpu.npivot == K
    assert np.array_equal(gpu.rowpermutation - 1, ref["rowpermutation"])
    assert np.array_equal(gpu.colpermutation - 1, ref["colpermutation"])
    assert gpu.error == ref["error"] or (np.isnan(gpu.error) and np.isnan(ref["error"]))
    assert np.array_equal(gpu.L, ref["L"])
    assert np.array_equal(gpu.U, ref["U"])


def test_reference_known_answers(T, oracle, golden):
    for case in golden["rrlu"]:
        A = np.array(case["A"])
        g = T.rrlu(A, **case["kwargs"])
        r = oracle.rrlu(A, **case["kwargs"])
        _same(g, r)
        ex = case["expect"]
        if "npivot" in ex:
            assert g.npivot == ex["npivot"]
        if "pivoterrors" in ex:
            assert list(g.pivoterrors()) == ex["pivoterrors"]
        if "lastpivoterror" in ex:
            assert g.lastpivoterror() == ex["lastpivoterror"]
        if ex.get("left_right_approx_A"):
            assert np.allclose(g.left() @ g.right(), A, rtol=1e-12, atol=1e-14)


def test_exact_lowrank(T, oracle, golden):
    gl = golden["rrlu_lowrank"]
    A = np.array(gl["p"]) @ np.array(gl["q"])
    g = T.rrlu(A)
    assert g.npivot == 3
    _same(g, oracle.rrlu(A))


@pytest.mark.parametrize("shape", [(1, 1), (1, 7), (7, 1), (5, 9), (33, 17), (64, 64), (150, 130), (200, 60),
                                   (60, 300), (300, 300)])
@pytest.mark.parametrize("leftorth", [True, False])
def test_random_shapes(T, oracle, shape, leftorth):
    rng = np.random.default_rng(shape[0] * 1000 + shape[1])
    A = rng.standard_normal(shape)
    for kw in [{}, {"maxrank": 3}, {"reltol": 1e-3}, {"abstol": 0.5}]:
        _same(T.rrlu(A, leftorthogonal=leftorth, **kw), oracle.rrlu(A, leftorthogonal=leftorth, **kw))


def test_ties_follow_column_major_order(T, oracle):
    """Integer-valued matrices have many equal |a|: the first maximum in
    column-major order of the permuted matrix must win on both sides."""
    rng = np.random.default_rng(7)
    for trial in range(20):
        A = rng.integers(-3, 4, size=(24, 19)).astype(float)
        _same(T.rrlu(A), oracle.rrlu(A))
    A = np.ones((8, 8))
    _same(T.rrlu(A), oracle.rrlu(A))


def test_squares_that_round_equal(T, oracle):
    """Distinct |a| whose squares round to the same double (underflow to zero,
    overflow to Inf): the first in column-major order wins, not the larger one."""
    tiny = np.full((6, 6), 1e-170)
    tiny[4, 3] = 2e-170
    _same(T.rrlu(tiny), oracle.rrlu(tiny))
    huge = np.full((5, 5), 1e160)
    huge[3, 2] = 2e160
    _same(T.rrlu(huge, maxrank=2), oracle.rrlu(huge, maxrank=2))


def test_lowrank_with_noise(T, oracle):
    rng = np.random.default_rng(11)
    for r in [8, 20, 50]:
        m = n = 2 * r
        U, _ = np.linalg.qr(rng.standard_normal((m, m)))
        V, _ = np.linalg.qr(rng.standard_normal((n, n)))
        s = 10.0 ** (-np.arange(min(m, n)) / 4)
        A = (U[:, : len(s)] * s) @ V[:, : len(s)].T + 1e-12 * rng.standard_normal((m, n))
        _same(T.rrlu(A, reltol=1e-10, maxrank=256), oracle.rrlu(A, reltol=1e-10, maxrank=256))


def test_zero_and_empty(T, oracle):
    for A in [np.zeros((0, 3)), np.zeros((3, 0))]:
        _same(T.rrlu(A), oracle.rrlu(A))
    # The first pivot of an all-zero matrix is 0 and is accepted (npivot == 0,
    # matrixlu.jl:155), so the column scaling divides 0/0 and the reference
    # throws "lu.L contains NaNs"; both sides must do the same.
    A = np.zeros((4, 5))
    with pytest.raises(T.TCIError, match="NaN"):
        T.rrlu(A)
    with pytest.raises(oracle.OracleError, match="NaN"):
        oracle.rrlu(A)


def test_nan_raises_like_reference(T, oracle):
    # NaN that ends up in L (first pivot column): "lu.L contains NaNs"
    A = np.ones((4, 4))
    A[2, 0] = np.nan
    with pytest.raises(T.TCIError) as e:
        T.rrlu(A)
    assert e.value.code == T.TCI_ERR_NAN and "NaN" in str(e.value)
    with pytest.raises(oracle.OracleError):
        oracle.rrlu(A)
    # NaN never wins the argmax (v > m is false) and may stay in the unfactored
    # Schur complement, which is not part of L or U: no error on either side.
    A = np.ones((4, 4))
    A[2, 2] = np.nan
    _same(T.rrlu(A), oracle.rrlu(A))


def test_large_matrix_global_memory_path(T, oracle):
    """A matrix too large for shared memory runs from global memory."""
    rng = np.random.default_rng(5)
    r = 40
    A = rng.standard_normal((400, r)) @ rng.standard_normal((r, 380))
    _same(T.rrlu(A, maxrank=60), oracle.rrlu(A, maxrank=60))


def test_batched_matches_oracle(T, oracle):
    """rrlu over a batch of uneven low-rank matrices (the batched-microbench
    generator at a small count): pivot rows/cols bit-exact per matrix."""
    rng = np.random.default_rng(0)
    mats = []
    for _ in range(48):
        r = int(rng.integers(8, 41))
        m = n = 2 * r
        U, _ = np.linalg.qr(rng.standard_normal((m, m)))
        V, _ = np.linalg.qr(rng.standard_normal((n, n)))
        s = 10.0 ** (-np.arange(m) / 4)
        mats.append((U * s) @ V.T + 1e-12 * rng.standard_normal((m, n)))
    got = T.rrlu_batched(mats, maxrank=256, reltol=1e-10)
    for A, (rows, cols, K, err) in zip(mats, got):
        r = oracle.rrlu(A, maxrank=256, reltol=1e-10)
        assert K == r["npivot"]
        assert np.array_equal(rows - 1, r["rowpermutation"][:K])
        assert np.array_equal(cols - 1, r["colpermutation"][:K])
        assert err == r["error"]


@pytest.mark.parametrize("leftorth", [True, False])
def test_multi_cta_path(T, oracle, leftorth):
    """Matrices of 2^18 elements and more run on the multi-CTA kernel (column
    permutation kept as a map, pivot search over every SM): still bit-exact."""
    rng = np.random.default_rng(7)
    m, n, r = 600, 520, 40
    A = rng.standard_normal((m, r)) @ rng.standard_normal((r, n)) + 1e-9 * rng.standard_normal((m, n))
    _same(T.rrlu(A, maxrank=60, leftorthogonal=leftorth), oracle.rrlu(A, maxrank=60, leftorthogonal=leftorth))
    s = 10.0 ** (-np.arange(n) / 40)
    U, _ = np.linalg.qr(rng.standard_normal((m, n)))
    V, _ = np.linalg.qr(rng.standard_normal((n, n)))
    B = (U * s) @ V.T
    _same(T.rrlu(B, reltol=1e-10, leftorthogonal=leftorth), oracle.rrlu(B, reltol=1e-10, leftorthogonal=leftorth))


def test_multi_cta_ties_and_tiny_magnitudes(T, oracle):
    rng = np.random.default_rng(8)
    # many exactly equal |values|: first key in column-major order must win
    A = rng.integers(-2, 3, size=(530, 500)).astype(np.float64)
    _same(T.rrlu(A, maxrank=40), oracle.rrlu(A, maxrank=40))
    # magnitudes where squares underflow: the exact pass decides every pivot
    B = 1e-170 * rng.standard_normal((520, 520))
    _same(T.rrlu(B, maxrank=20), oracle.rrlu(B, maxrank=20))
    # wide and tall shapes
    C = rng.standard_normal((300, 1200)) @ np.diag(10.0 ** (-np.arange(1200) / 100))
    _same(T.rrlu(C, reltol=1e-8), oracle.rrlu(C, reltol=1e-8))
    D = C.T.copy()
    _same(T.rrlu(D, reltol=1e-8, leftorthogonal=False), oracle.rrlu(D, reltol=1e-8, leftorthogonal=False))


def test_multi_cta_nan(T, oracle):
    A = np.ones((520, 520))
    A[3, 0] = np.nan
    with pytest.raises(T.TCIError) as e:
        T.rrlu(A)
    assert e.value.code == T.TCI_ERR_NAN
    with pytest.raises(oracle.OracleError):
        oracle.rrlu(A)


@pytest.mark.parametrize("seed", [99, 100, 101])
def test_nan_inf_planted(T, oracle, seed):
    """NaN and +-Inf planted at random positions: the GPU raises "lu.L contains
    NaNs" exactly when the oracle does (the check is gathered pivot by pivot as
    the entries join L and U), and otherwise matches it bit for bit."""
    rng = np.random.default_rng(seed)
    raised = 0
    for trial in range(40):
        m = int(rng.integers(2, 160))
        n = int(rng.integers(2, 160))
        A = rng.standard_normal((m, n))
        for _ in range(int(rng.integers(1, 5))):
            A[rng.integers(m), rng.integers(n)] = rng.choice([np.nan, np.inf, -np.inf])
        kw = dict(leftorthogonal=bool(trial % 2), maxrank=int(rng.integers(1, min(m, n) + 1)))
        try:
            ref = oracle.rrlu(A, **kw)
        except oracle.OracleError:
            raised += 1
            with pytest.raises(T.TCIError) as e:
                T.rrlu(A, **kw)
            assert e.value.code == T.TCI_ERR_NAN
            continue
        _same(T.rrlu(A, **kw), ref)
    assert 0 < raised < 40  # both outcomes occur


def test_multi_cta_long_maps(T, oracle):
    """A tall matrix whose permutation maps take tens of KB of shared memory per
    CTA (two CTAs share an SM): the launch sizes its shared-memory carveout for
    them, and the result stays bit-exact."""
    rng = np.random.default_rng(12)
    m, n, r = 4000, 600, 30
    A = rng.standard_normal((m, r)) @ rng.standard_normal((r, n)) + 1e-10 * rng.standard_normal((m, n))
    _same(T.rrlu(A, maxrank=40), oracle.rrlu(A, maxrank=40))
    _same(T.rrlu(A.T.copy(), maxrank=40, leftorthogonal=False), oracle.rrlu(A.T.copy(), maxrank=40, leftorthogonal=False))
