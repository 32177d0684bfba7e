"""The CPU oracle against the reference's own known answers (no GPU).

Each case restates an assertion of TensorCrossInterpolation.jl's test suite
(file:line in the fixture) and checks that the oracle satisfies it.
"""
import itertools

import numpy as np
import pytest


def _check_rrlu_case(O, case):
    A = np.array(case["A"])
    res = O.rrlu(A, **case["kwargs"])
    ex = case["expect"]
    K = res["npivot"]
    L, U = res["L"], res["U"]
    if "npivot" in ex:
        assert K == ex["npivot"]
    if ex.get("left_right_approx_A"):
        assert np.allclose(O.left(res) @ O.right(res), A, rtol=1e-12, atol=1e-14)
    if ex.get("L_unit_lower"):
        assert np.all(L == np.tril(L)) and np.all(np.diag(L[:K, :K]) == 1.0)
    if ex.get("L_lower"):
        assert np.all(L == np.tril(L))
    if ex.get("U_upper"):
        assert np.all(U == np.triu(U))
    if "pivoterrors" in ex:
        assert list(O.pivoterrors(res)) == ex["pivoterrors"]
    if "n_pivoterrors" in ex:
        assert len(O.pivoterrors(res)) == ex["n_pivoterrors"]
    if "lastpivoterror" in ex:
        assert res["error"] == ex["lastpivoterror"]
    if ex.get("lastpivoterror_positive"):
        assert res["error"] > 0
    if "lastpivoterror_below" in ex:
        assert res["error"] < ex["lastpivoterror_below"]
    if "max_abs_residual_below" in ex:
        assert np.max(np.abs(O.left(res) @ O.right(res) - A)) < ex["max_abs_residual_below"]


def test_rrlu_known_answers(oracle, golden):
    for case in golden["rrlu"]:
        _check_rrlu_case(oracle, case)


def test_rrlu_exact_lowrank(oracle, golden):
    g = golden["rrlu_lowrank"]
    A = np.array(g["p"]) @ np.array(g["q"])
    res = oracle.rrlu(A)
    assert res["npivot"] == 3
    assert np.allclose(oracle.left(res) @ oracle.right(res), A, rtol=1e-10, atol=1e-12)


def test_luci_colstimespivotinv(oracle, golden):
    """test_matrixluci.jl:6-37: colstimespivotinv == A[:, J] * inv(A[I, J])."""
    A = np.array(golden["luci"]["A"])
    res = oracle.rrlu(A, maxrank=4)
    left, right = oracle.luci(A, maxrank=4)
    I = res["rowpermutation"][:4]
    J = res["colpermutation"][:4]
    P = A[np.ix_(I, J)]
    assert np.allclose(left, A[:, J] @ np.linalg.inv(P), rtol=1e-9, atol=1e-12)
    assert np.allclose(left @ right, A[:, J] @ np.linalg.inv(P) @ A[I, :], rtol=1e-9, atol=1e-12)


def test_luci_exact_lowrank(oracle, golden):
    """test_matrixluci.jl:48-74: MatrixLUCI of an exact rank-3 product has 3
    pivots, left * right reproduces it, and the first npivots rows of colmatrix
    (left when leftorthogonal is false, matrixluci.jl:40-42) are well conditioned."""
    g = golden["rrlu_lowrank"]
    A = np.array(g["p"]) @ np.array(g["q"])
    for leftorth in (True, False):
        left, right = oracle.luci(A, leftorthogonal=leftorth)
        assert left.shape == (A.shape[0], 3) and right.shape == (3, A.shape[1])
        assert np.allclose(left @ right, A, rtol=1e-10, atol=1e-12)
    colmatrix, _ = oracle.luci(A, leftorthogonal=False)
    res = oracle.rrlu(A)
    assert np.allclose(colmatrix, A[:, res["colpermutation"][:3]], rtol=1e-10, atol=1e-12)
    assert np.linalg.cond(colmatrix[:3, :]) < 1e12


def test_luci_near_duplicate_columns(oracle, golden):
    """test_matrixluci.jl:39-45: the 8 x 6 matrix beside a copy perturbed by
    1e-3 (seeded here in place of rand): at reltol 1e-2 fewer pivots than rows
    and columns, and left * right within 1e-2 of the matrix everywhere."""
    A = np.array(golden["luci"]["A"])
    A = np.hstack([A, A + 1e-3 * np.random.default_rng(7).random(A.shape)])
    left, right = oracle.luci(A, reltol=1e-2)
    res = oracle.rrlu(A, reltol=1e-2)
    assert res["npivot"] < A.shape[0] and res["npivot"] < A.shape[1]
    assert left.shape == (A.shape[0], res["npivot"])
    assert np.max(np.abs(left @ right - A)) < 1e-2


def test_argmax_first_in_column_major(oracle):
    """submatrixargmax keeps the first maximum of abs2 in column-major order
    (matrixlu.jl:16-31): with ties the earliest column, then the earliest row."""
    A = np.zeros((4, 4))
    A[2, 1] = -3.0
    A[1, 2] = 3.0
    A[3, 1] = 3.0
    res = oracle.rrlu(A, maxrank=1)
    assert res["rowpermutation"][0] == 2 and res["colpermutation"][0] == 1


def test_tci2_pivoterrors(oracle, golden):
    g = golden["tci2"]["pivoterrors"]
    T = np.diag(g["diags"])
    t, _, _ = oracle.crossinterpolate2(g["localdims"], oracle.F_DENSE, oracle.dense_params(T), [[1, 1]],
                                       tolerance=g["tolerance"])
    assert list(t.errors()[0]) == g["expect_pivoterrors"]


def test_tci2_lorentz_updatepivots_and_global_pivot(oracle, golden):
    g = golden["tci2"]["lorentz"]
    n, d = g["n"], g["localdim"]
    t = oracle.OracleTCI.new([d] * n, oracle.F_LORENTZ)
    assert list(t.linkdims()) == [1] * (n - 1)
    for p in range(1, n):
        t.updatepivots(p, True, reltol=1e-8, maxbonddim=2)
    assert list(t.linkdims()) == g["maxbonddim2_linkdims"]
    t.addglobalpivots1sitesweep([g["globalpivot"]], reltol=1e-12)
    assert list(t.linkdims()) == g["after_globalpivot_linkdims"]
    for _ in range(4, 21):
        for p in range(1, n):
            t.updatepivots(p, True, reltol=1e-8)
    t2, _, _ = oracle.crossinterpolate2([d] * n, oracle.F_LORENTZ, (), None, tolerance=1e-8, maxiter=8,
                                        sweepstrategy="forward")
    assert t.rank() == t2.rank()


@pytest.mark.parametrize("pivots", [None, "initialpivots4"])
def test_tci2_lorentz_tight_tolerance(oracle, golden, pivots):
    g = golden["tci2"]["lorentz"]
    n, d = g["n"], g["localdim"]
    piv = g[pivots] if pivots else None
    t, _, _ = oracle.crossinterpolate2([d] * n, oracle.F_LORENTZ, (), piv, tolerance=1e-12, maxiter=200)
    assert max(t.errors()[1]) <= g["tol3_pivoterror_max"]
    assert all(x <= 200 for x in t.linkdims())
    pts = np.array(list(itertools.product(*[range(1, 4)] * n)))
    vals = t.evaluate(pts)
    assert np.allclose(vals, 1.0 / (1.0 + (pts ** 2).sum(1)), rtol=1e-10)


def test_convergencecriterion_truth_table(oracle, golden):
    for c in golden["tci2"]["convergencecriterion"]["cases"]:
        got = oracle.convergencecriterion(c["ranks"], c["errors"], c["ngp"], c["tol"], c["maxbonddim"],
                                          c["ncheck"])
        assert got == c["expect"], c


def test_trivial_mps_exp(oracle):
    """test_tensorci2.jl:55-101: exp(-x) on R=8 quantics bits has bond dimension 1."""
    R = 8
    for nsearch, strict in [(0, False), (0, True), (10, False)]:
        t, _, _ = oracle.crossinterpolate2([2] * R, oracle.F_QTT1D, [1.0], [[1] * R, [1] + [2] * (R - 1)],
                                           tolerance=1e-4, maxbonddim=1, maxiter=2, normalizeerror=False,
                                           nsearchglobalpivot=nsearch, strictlynested=strict)
        assert all(x == 1 for x in t.linkdims())
        for x in [0.1, 0.3, 0.6, 0.9]:
            k = int(np.floor(x * 2 ** R))
            bits = [((k >> (R - 1 - i)) & 1) + 1 for i in range(R)]
            fx = np.exp(-sum((b - 1) * 2.0 ** -(i + 1) for i, b in enumerate(bits)))
            assert abs(t.evaluate([bits])[0] - fx) < 1e-4


def test_sum_matches_bruteforce(oracle):
    t, _, _ = oracle.crossinterpolate2([6] * 4, oracle.F_LORENTZ, (), None, tolerance=1e-12, maxiter=50)
    pts = np.array(list(itertools.product(*[range(1, 7)] * 4)))
    brute = (1.0 / (1.0 + (pts ** 2).sum(1))).sum()
    assert abs(t.sum() - brute) <= 1e-10 * brute


def test_function_library_against_numpy(oracle):
    """The oracle's f values (own exp/cos) agree with numpy's libm to a few ulps."""
    rng = np.random.default_rng(3)
    R = 40
    bits = rng.integers(1, 3, size=(2000, R))
    x = ((bits - 1) * 2.0 ** -np.arange(1, R + 1)).sum(1)
    got = oracle.feval(oracle.F_QTT1D, [0.0], bits)
    ref = np.exp(-x) * np.cos(2 * np.pi * 1000 * x) + 0.5 * np.exp(-(x - 0.3) ** 2 / 1e-4)
    assert np.max(np.abs(got - ref)) < 1e-12
    L = 8
    v = rng.integers(1, 11, size=(2000, L))
    c = rng.integers(1, 11, size=L)
    a, b, g = 0.3, 2.0, 0.05
    got = oracle.feval(oracle.F_SERVED, [a, b, g] + list(c), v)
    ref = 1 / (1 + a * (v ** 2).sum(1)) + b * np.exp(-g * ((v - c) ** 2).sum(1))
    assert np.allclose(got, ref, rtol=4e-16 * 8, atol=0)
