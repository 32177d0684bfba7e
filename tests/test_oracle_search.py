"""The oracle's greedy point searches pinned on the reference's own tests:
optfirstpivot's known answer (test/test_util.jl:29-37) and estimatetrueerror's
properties (test/test_globalsearch.jl:7-36: each reported error is |f(p) - tt(p)|
at its pivot, and the list is sorted in descending order)."""
import numpy as np


def _dense_params(table):
    dims = table.shape
    strides = np.cumprod((1,) + dims[:-1])
    return np.concatenate([[len(dims)], strides, table.reshape(-1, order="F")])


def test_optfirstpivot_known_answer(oracle, golden):
    g = golden["util"]["optfirstpivot"]
    table = np.zeros(g["localdims"])
    for idx in np.ndindex(*table.shape):  # f(v) = 4 (v3 - 1) + 2 (v2 - 1) + (v1 - 1), 0-based idx
        table[idx] = 4 * idx[2] + 2 * idx[1] + idx[0]
    got = oracle.optfirstpivot(oracle.F_DENSE, _dense_params(table), g["localdims"], g["firstpivot"])
    assert list(got) == g["expect"]


def test_estimatetrueerror_properties(oracle):
    L = 12

    def f(p):  # quantics: x = sum_i b_i 2^-i, f = exp(-x) + 1e-3 sin-like ripple (rational here)
        x = np.zeros(p.shape[0])
        for k in range(L):
            x = x + (p[:, k] - 1) * 0.5 ** (k + 1)
        return 1.0 / (1.0 + x) + 1e-3 / (1.0 + 1e4 * (x - 0.3) ** 2)

    fid = oracle.register_fn(f)
    ref, _, _ = oracle.crossinterpolate2([2] * L, fid, (), [np.ones(L), np.r_[1, np.full(L - 1, 2)]],
                                         tolerance=1e-4, maxbonddim=1, normalizeerror=False)
    cores = [ref.core(b) for b in range(1, L + 1)]
    starts = np.random.default_rng(1240).integers(1, 3, size=(30, L))
    res = oracle.estimatetrueerror(fid, (), cores, starts)
    assert len(res) >= 1
    errs = [e for _, e in res]
    assert all(errs[k] >= errs[k + 1] for k in range(len(errs) - 1))
    pts = np.array([p for p, _ in res])
    tt = oracle.tt_evaluate(cores, pts)
    assert np.allclose(np.abs(f(pts) - tt), errs, rtol=1e-12, atol=0)
