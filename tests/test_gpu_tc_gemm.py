"""Split-precision tensor-core products (tcgen05 kind::tf32, TF32 hi/lo split,
FP32 accumulation) through the C ABI: tci_matmul and the zipup contraction with
precision = TF32x3.

  - Small-integer operands are represented exactly by the hi part, every product
    and partial sum is exact in FP32, so the tensor-core result must equal the
    FP64 product bit for bit: this pins the operand layouts (TMA swizzle, shared
    memory descriptors, tensor-memory read-back) on ragged shapes.
  - Gaussian operands: every entry within the split's error bound
    |C - AB| <= (3 * 2^-22 + K * 2^-23) (|A| |B|), and the sampled relative
    error the library reports (err_est) stays small.
  - zipup (contraction.jl:442-486) with TF32x3 site contractions against the
    FP64 dense product, within 1e-5 relative, err_est stated.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1, 1), (128, 64, 32), (129, 65, 33), (300, 200, 100), (1000, 257, 77), (64, 300, 500),
          (5000, 81, 324), (2, 3, 1000)]


@pytest.mark.parametrize("M,N,K", SHAPES)
def test_split_exact_on_small_integers(T, M, N, K):
    rng = np.random.default_rng(M * 7 + N * 3 + K)
    A = rng.integers(-8, 9, size=(M, K)).astype(np.float64)
    B = rng.integers(-8, 9, size=(K, N)).astype(np.float64)
    C, err = T.matmul(A, B, precision="tf32x3")
    assert np.array_equal(C, A @ B)
    assert err == 0.0


@pytest.mark.parametrize("M,N,K", SHAPES)
def test_split_within_bound(T, M, N, K):
    rng = np.random.default_rng(M + 11 * N + 13 * K)
    A = rng.standard_normal((M, K))
    B = rng.standard_normal((K, N))
    C, err = T.matmul(A, B, precision="tf32x3")
    exact = A @ B
    bound = (3 * 2.0 ** -22 + K * 2.0 ** -23) * (np.abs(A) @ np.abs(B)) + 1e-300
    assert np.all(np.abs(C - exact) <= bound)
    # relative to sum_k |a b| (the scale of the FP32 accumulation error); against
    # max |C| it is larger by ~sqrt(K) for Gaussian operands
    rel = (np.abs(C - exact) / (np.abs(A) @ np.abs(B))).max()
    assert rel < 2e-6
    assert 0.0 <= err < 1e-4
    C64, err64 = T.matmul(A, B, precision="fp64")
    assert err64 == 0.0
    assert np.allclose(C64, exact, rtol=1e-13, atol=1e-13 * np.abs(exact).max())


def test_split_rejects_unknown_precision(T):
    with pytest.raises(T.ArgumentError):
        T.matmul(np.ones((2, 2)), np.ones((2, 2)), precision="bf16")


def _rand_tt(rng, bonds, s1, s2):
    return [rng.standard_normal((bonds[n], s1[n], s2[n], bonds[n + 1])) for n in range(len(s1))]


@pytest.mark.parametrize("method", ["LU", "CI"])
def test_zipup_split_precision(T, oracle, method):
    rng = np.random.default_rng(21)
    a = _rand_tt(rng, [1, 4, 6, 6, 4, 1], [2] * 5, [3] * 5)
    b = _rand_tt(rng, [1, 3, 5, 5, 3, 1], [3] * 5, [2] * 5)
    ab = T.contract(a, b, algorithm="zipup", tolerance=1e-12, method=method, precision="tf32x3")
    ref = oracle.tt4_full(a) @ oracle.tt4_full(b)
    got = oracle.tt4_full(ab.sitetensors)
    rel = np.abs(got - ref).max() / np.abs(ref).max()
    assert rel < 1e-5, rel
    assert 0.0 < ab.err_est < 1e-5
    # the FP64 path stays bit-exact with the oracle
    ab64 = T.contract(a, b, algorithm="zipup", tolerance=1e-12, method=method)
    assert ab64.err_est == 0.0
    r64 = oracle.tt4_contract(a, b, "zipup", tolerance=1e-12, method=method)
    for g, r in zip(ab64.sitetensors, r64):
        assert np.array_equal(g, r)


def test_zipup_split_mpo_mps_wide_bonds(T, oracle):
    """Operator bond 16 and train bond 12 (products up to 12288 x 256 and
    2304 x 256, several tensor-core tiles in each dimension), no truncation:
    split and FP64 contractions represent the same product."""
    rng = np.random.default_rng(22)
    L = 6
    op = [rng.standard_normal((r0, 4, 4, r1)) / 4.0 for r0, r1 in zip([1] + [16] * (L - 1), [16] * (L - 1) + [1])]
    v = [rng.standard_normal((r0, 4, r1)) / 3.5 for r0, r1 in zip([1] + [12] * (L - 1), [12] * (L - 1) + [1])]
    tt_s = T.contract(op, T.TensorTrain(v), algorithm="zipup", tolerance=1e-14, maxbonddim=4096, precision="tf32x3",
                      method="LU")
    tt_d = T.contract(op, T.TensorTrain(v), algorithm="zipup", tolerance=1e-14, maxbonddim=4096, method="LU")
    pts = rng.integers(1, 5, size=(2000, L))
    ys = tt_s.evaluate(pts)
    yd = tt_d.evaluate(pts)
    rel = np.abs(ys - yd).max() / np.abs(yd).max()
    assert rel < 1e-4, rel
    assert 0.0 < tt_s.err_est < 1e-5


def _rand_tt3(rng, L, d, r, scale=None):
    bonds = [1] + [r] * (L - 1) + [1]
    return [rng.standard_normal((bonds[n], d, bonds[n + 1])) / np.sqrt(scale or bonds[n] * d) for n in range(L)]


@pytest.mark.parametrize("L,d,r", [(1, 3, 1), (2, 2, 5), (6, 2, 32), (8, 4, 64), (5, 3, 100), (12, 2, 128),
                                   (4, 32, 16)])
def test_split_evaluate_random_train(T, oracle, L, d, r):
    """Tensor-core evaluation against the oracle's FP64 evaluate: small-integer
    cores (exact in the split) agree bit for bit; Gaussian cores within the
    FP32-accumulation error, and err_est reports it."""
    rng = np.random.default_rng(100 * L + r)
    pts = np.stack([rng.integers(1, d + 1, size=3000) for _ in range(L)], 1)
    bonds = [1] + [r] * (L - 1) + [1]
    ints = [rng.integers(-2, 3, size=(bonds[n], d, bonds[n + 1])).astype(np.float64) for n in range(L)]
    if L <= 3:  # the exact partial sums stay below 2^24
        got = T.TensorTrain(ints).evaluate(pts, precision="tf32x3")
        assert np.array_equal(got, oracle.tt_evaluate(ints, pts))
    cores = _rand_tt3(rng, L, d, r)
    tt = T.TensorTrain(cores)
    got = tt.evaluate(pts, precision="tf32x3")
    ref = oracle.tt_evaluate(cores, pts)
    rel = np.abs(got - ref).max() / np.abs(ref).max()
    assert rel < 1e-5 * L, rel
    assert 0.0 <= tt.eval_err_est < 1e-5 * L
    assert np.allclose(tt.evaluate(pts), ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max())


def test_split_evaluate_quantics_config(T, oracle):
    """The R = 40 quantics function (tolerance 1e-10, maxbonddim 128): 1e5
    points evaluated on the tensor cores, error against FP64 stated."""
    f = T.DeviceFunction("qtt1d", [0])
    tci, _, _ = T.crossinterpolate2(float, f, [2] * 40, tolerance=1e-10, maxbonddim=128, maxiter=20)
    pts = np.random.default_rng(4).integers(1, 3, size=(100000, 40))
    y64 = tci.evaluate(pts)
    y = tci.evaluate(pts, precision="tf32x3")
    rel = np.abs(y - y64).max() / np.abs(y64).max()
    assert rel < 1e-4, rel
    assert 0.0 < tci.eval_err_est < 1e-4


def test_split_evaluate_rejects_wide_bonds(T):
    rng = np.random.default_rng(1)
    cores = _rand_tt3(rng, 3, 2, 200)
    with pytest.raises(T.ArgumentError):
        T.TensorTrain(cores).evaluate(np.ones((4, 3), np.int64), precision="tf32x3")
