"""integrate() (integration.jl:20-58) on the reference's own known answers
(test/test_integration.jl:6-28): the integral of f(x) = prod_n p(x_n) for the
reference's 15-coefficient polynomial p over [0,1]^5 and over a random box
equals prod_n (P(b_n) - P(a_n)), P' = p, to the reference's `≈` (sqrt(eps)).
The CPU tests run the oracle's crossinterpolate2 on the same device-function
parameters; the GPU test runs the library's integrate().  A general integrand
(a caller-supplied f) is checked on the reference's 10-D integral
(test/test_integration.jl:61-70), within its 1e-3."""
import numpy as np
import pytest


def _poly(c):
    p = lambda x: sum(ci * x ** i for i, ci in enumerate(c))  # noqa: E731
    P = lambda x: sum(ci * x ** (i + 1) / (i + 1) for i, ci in enumerate(c))  # noqa: E731
    return p, P


def test_kronrod_rule(T):
    from tci_gb300.quadrature import kronrod

    x, w, gw = kronrod(7)
    assert x.size == 15 and np.all(np.diff(x) > 0) and np.all(w > 0)
    assert np.allclose(x, -x[::-1], atol=0) and abs(x[7]) == 0.0
    for k in range(23):  # exact to degree 3n+1 = 22
        exact = 0.0 if k % 2 else 2.0 / (k + 1)
        assert abs((w * x ** k).sum() - exact) < 1e-14
    for k in range(14):  # the embedded 7-point Gauss rule, exact to degree 13
        exact = 0.0 if k % 2 else 2.0 / (k + 1)
        assert abs((gw * x ** k).sum() - exact) < 1e-14


def _oracle_integrate(T, oracle, p, a, b, GKorder=15, **kw):
    from tci_gb300.quadrature import kronrod

    x1, w1, _ = kronrod(GKorder // 2)
    N = len(a)
    nodes = (b - a)[:, None] * (x1[None, :] + 1) / 2 + a[:, None]
    weights = (b - a)[:, None] * w1[None, :] / 2
    norm = float(GKorder) ** N
    tables = weights * p(nodes)
    f = T.product_function(tables, norm)
    kw.setdefault("nsearchglobalpivot", 10)
    ref, _, _ = oracle.crossinterpolate2([x1.size] * N, oracle.F_PRODUCT, f.params, None, **kw)
    return ref.sum() / norm


def test_oracle_integrates_reference_polynomials(T, oracle, golden):
    g = golden["integration"]
    p, P = _poly(g["coefficients"])
    N = g["N"]
    a, b = np.zeros(N), np.ones(N)
    exact = P(1.0) ** N
    assert _oracle_integrate(T, oracle, p, a, b) == pytest.approx(exact, rel=1.5e-8)
    rng = np.random.default_rng(1234)
    b, a = rng.random(N), rng.random(N)
    exact = np.prod(P(b) - P(a))
    assert _oracle_integrate(T, oracle, p, a, b) == pytest.approx(exact, rel=1.5e-8)


def test_integrate_errors_like_reference(T):
    f = T.ProductIntegrand(lambda x: x)
    with pytest.raises(T.TCIError, match="must be odd"):
        T.integrate(float, f, [0.0, 0.0], [1.0, 1.0], GKorder=14)
    with pytest.raises(T.TCIError, match="same dimensionality"):
        T.integrate(float, f, [0.0, 0.0], [1.0, 1.0, 1.0])


@pytest.mark.gpu
def test_gpu_integrates_reference_polynomials(T, oracle, golden):
    g = golden["integration"]
    p, P = _poly(g["coefficients"])
    N = g["N"]
    f = T.ProductIntegrand(p)
    got = T.integrate(float, f, np.zeros(N), np.ones(N))
    assert got == pytest.approx(P(1.0) ** N, rel=1.5e-8)
    rng = np.random.default_rng(1234)
    b, a = rng.random(N), rng.random(N)
    got = T.integrate(float, f, a, b)
    assert got == pytest.approx(np.prod(P(b) - P(a)), rel=1.5e-8)
    assert got == pytest.approx(_oracle_integrate(T, oracle, p, a, b), rel=1e-12)


def _tend_f(x):
    """test/test_integration.jl:64-66, vectorized over rows of x."""
    return 1000.0 * np.cos(10.0 * (x ** 2).sum(1)) * np.exp(-x.sum(1) ** 4 / 1000.0)


def test_oracle_integrates_reference_10d_function(T, oracle, golden):
    """The reference's 10-D integral (test/test_integration.jl:61-70) through the
    oracle with the same quadrature integrand the library builds."""
    from tci_gb300.quadrature import kronrod

    g = golden["integration"]["tenD"]
    N, GK = g["N"], g["GKorder"]
    x1, w1, _ = kronrod(GK // 2)
    a, b = np.full(N, g["a"]), np.full(N, g["b"])
    nodes = (b - a)[:, None] * (x1[None, :] + 1.0) / 2.0 + a[:, None]
    weights = (b - a)[:, None] * w1[None, :] / 2.0
    norm = float(GK) ** N
    fid = oracle.register_fn(T.quadrature_integrand(_tend_f, nodes, weights, norm))
    ref, _, _ = oracle.crossinterpolate2([x1.size] * N, fid, (), None, tolerance=g["tolerance"],
                                         nsearchglobalpivot=10)
    assert abs(ref.sum() / norm - g["Iref"]) < g["abs_tol"]


@pytest.mark.gpu
def test_gpu_integrates_reference_10d_function(T, golden):
    """integrate(Float64, f, -ones(10), ones(10); GKorder=15, tolerance=1e-8) of a
    general integrand (a caller-supplied f) within 1e-3 of the reference's value."""
    g = golden["integration"]["tenD"]
    N = g["N"]
    got = T.integrate(float, _tend_f, np.full(N, g["a"]), np.full(N, g["b"]), GKorder=g["GKorder"],
                      tolerance=g["tolerance"])
    assert abs(got - g["Iref"]) < g["abs_tol"]
