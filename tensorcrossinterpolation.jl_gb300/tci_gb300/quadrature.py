"""Gauss--Kronrod rules on [-1, 1] (the nodes integrate() runs on).

The (2n+1)-point Kronrod extension of the n-point Gauss--Legendre rule adds the
n+1 roots of the Stieltjes polynomial E_{n+1}, the monic polynomial of degree
n+1 orthogonal to every polynomial of degree <= n under the weight P_n(x) on
[-1, 1]; the 2n+1 weights then make the rule exact for polynomials of degree
<= 3n+1 (Kronrod 1965, Patterson 1968).  Computed here from that definition:
the orthogonality conditions are a linear system for the coefficients of E_{n+1}
(integrals done exactly with a high-order Gauss rule, in the Legendre basis),
and the weights solve the exactness conditions for P_0 .. P_{2n}.
"""
import numpy as np
from numpy.polynomial import legendre as L


def kronrod(n):
    """Nodes (ascending), Kronrod weights and the weights of the embedded Gauss
    rule (zero at the Kronrod-only nodes) of the (2n+1)-point rule on [-1, 1]."""
    if n < 1:
        raise ValueError("kronrod needs n >= 1")
    xg, wg = L.leggauss(n)
    xq, wq = L.leggauss(3 * n + 4)  # exact for the degree <= 4n+1 integrands below
    pn = L.legval(xq, np.eye(n + 1)[n])
    # E(x) = sum_{j<=n+1} c_j P_j(x), c_{n+1} = 1; conditions: int E P_n P_k = 0, k = 0..n
    basis = np.array([L.legval(xq, np.eye(n + 2)[j]) for j in range(n + 2)])  # (n+2) x q
    A = np.empty((n + 1, n + 1))
    rhs = np.empty(n + 1)
    for k in range(n + 1):
        pk = L.legval(xq, np.eye(n + 1)[k])
        row = (basis * (pn * pk * wq)).sum(axis=1)
        A[k] = row[: n + 1]
        rhs[k] = -row[n + 1]
    c = np.append(np.linalg.solve(A, rhs), 1.0)
    xk = np.sort(np.real(L.legroots(c)))
    x = np.sort(np.concatenate([xg, xk]))
    x = 0.5 * (x - x[::-1])  # exact symmetry about 0
    # weights: sum_i w_i P_k(x_i) = int P_k = 2 [k == 0], k = 0..2n
    V = np.array([L.legval(x, np.eye(2 * n + 1)[k]) for k in range(2 * n + 1)])
    b = np.zeros(2 * n + 1)
    b[0] = 2.0
    w = np.linalg.solve(V, b)
    w = 0.5 * (w + w[::-1])
    gw = np.zeros_like(w)
    for xi, wi in zip(xg, wg):
        gw[np.argmin(np.abs(x - xi))] = wi
    return x, w, gw
