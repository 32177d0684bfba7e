"""Argument checks of the Python mirror that run before any device work, with the
reference's exception types (no GPU): optimize!'s tolerance / pivottolerance rules
(tensorci2.jl:724-741, test/test_tensorci2.jl:234-245), contract's algorithm and
f rules (contraction.jl:515-545) and its SVD default, compress!/_factorize methods
(tensortrain.jl:94-137), sweep directions (tensorci2.jl:402-411) and pivot shapes
(tensorci2.jl:197-199)."""
import numpy as np
import pytest


def test_optimize_keyword_rules(T):
    with pytest.raises(T.ArgumentError, match="pivottolerance"):
        T.make_opts(tolerance=1e-9, pivottolerance=1e-2)
    o = T.make_opts(pivottolerance=1e-3)  # the deprecated name alone sets tolerance
    assert o.tolerance == 1e-3
    with pytest.raises(T.ArgumentError, match="pivotsearch"):
        T.make_opts(pivotsearch="rook")
    with pytest.raises(T.ArgumentError, match="global pivot finder"):
        T.make_opts(globalpivotfinder=object())
    d = T.make_opts()
    assert d.tolerance == 1e-8 and d.maxiter == 20 and d.nsearchglobalpivot == 5 and d.maxnglobalpivot == 5


def test_contract_rules(T):
    rng = np.random.default_rng(0)
    a = [rng.standard_normal((1, 2, 2, 1)), rng.standard_normal((1, 2, 2, 1))]
    with pytest.raises(T.TCIError, match="cannot contract matrix product with a function"):
        T.contract(a, a, algorithm="naive", f=lambda x: x)
    with pytest.raises(T.TCIError, match="cannot contract matrix product with a function"):
        T.contract(a, a, algorithm="zipup", f=lambda x: x)
    with pytest.raises(T.ArgumentError, match="Unknown algorithm"):
        T.contract(a, a, algorithm="bogus")
    with pytest.raises(T.TCIError, match="not available"):
        T.contract(a, a, algorithm="zipup", method="SVD")
    with pytest.raises(T.TCIError, match="not available"):
        T.compress(a, method="SVD")
    with pytest.raises(T.ArgumentError, match="different length"):
        T.contract(a, a[:1], algorithm="zipup")
    with pytest.raises(T.ArgumentError, match="different length"):
        T.contract(a, a[:1])  # algorithm=:TCI, contraction.jl:406-408
    with pytest.raises(T.ArgumentError, match="3 or all have 4 legs"):
        T.compress([np.zeros((1, 2, 1)), np.zeros((1, 2, 2, 1))])
    # the reference factorizes zipup and truncated naive contractions with SVD
    # (contraction.jl:369, :446): without an explicit method the call says so
    with pytest.raises(T.TCIError, match="SVD"):
        T.contract(a, a, algorithm="zipup")
    with pytest.raises(T.TCIError, match="SVD"):
        T.contract(a, a, algorithm="naive", tolerance=1e-10)
    b = [rng.standard_normal((1, 3, 2, 1)), rng.standard_normal((1, 3, 2, 1))]
    with pytest.raises(T.TCIError, match="identical index"):
        T.contract(a, b, algorithm="zipup")


def test_pivot_shapes(T):
    with pytest.raises(T.DimensionMismatch, match="one index per leg"):
        T._pivots_array([[1, 2, 3]], 4)
    p = T._pivots_array([[1, 2, 3, 4], np.array([4, 3, 2, 1])], 4)
    assert p.shape == (2, 4) and p.dtype == np.int64


def test_integrate_rules(T):
    f = T.ProductIntegrand(lambda x: x)
    with pytest.raises(T.TCIError, match="must be odd"):
        T.integrate(float, f, [0.0], [1.0], GKorder=14)
    with pytest.raises(T.ArgumentError, match="Float64"):
        T.integrate(complex, f, [0.0], [1.0])
