"""Seeded synthetic workloads of the benchmark configurations.

No dataset is involved anywhere: every input is generated here from a seed.
"""
import numpy as np


def served_requests(n, seed, tol_range=(-10.0, -6.0)):
    """Requests of the served-stream family: f(v) = 1/(1 + a v.v) + b exp(-g |v - c|^2)
    with a, b, g log-uniform in [1e-2, 1e1], c uniform on the lattice; L uniform in
    4..16, d uniform in 2..16, tolerance log-uniform in [1e-10, 1e-6] (log10 bounds
    `tol_range`), maxbonddim uniform in {32, 64, 128, 256}.  Returns (L, d, params,
    tolerance, maxbonddim)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        L = int(rng.integers(4, 17))
        d = int(rng.integers(2, 17))
        a, b, g = 10 ** rng.uniform(-2, 1, size=3)
        c = rng.integers(1, d + 1, size=L)
        tol = float(10 ** rng.uniform(*tol_range))
        mbd = int(rng.choice([32, 64, 128, 256]))
        out.append((L, d, [a, b, g] + [float(x) for x in c], tol, mbd))
    return out


def rrlu_batch(count=4096, seed=0, rmin=8, rmax=128, noise=1e-12):
    """The batched-rrLU microbenchmark: `count` matrices of shape (2r) x (2r), r
    uniform in [rmin, rmax]; each is U diag(s) V^T with Haar-random U, V (QR of a
    Gaussian matrix with the signs of R's diagonal fixed), s_k = 10^(-k/4), plus
    i.i.d. normal noise of standard deviation `noise`.  Column-major float64."""
    rng = np.random.default_rng(seed)
    mats = []
    for _ in range(count):
        r = int(rng.integers(rmin, rmax + 1))
        m = 2 * r
        U = _haar(rng, m)
        V = _haar(rng, m)
        s = 10.0 ** (-np.arange(m) / 4.0)
        A = (U * s) @ V.T + noise * rng.standard_normal((m, m))
        mats.append(np.asfortranarray(A))
    return mats


def _haar(rng, n):
    q, r = np.linalg.qr(rng.standard_normal((n, n)))
    return q * np.sign(np.diag(r))
