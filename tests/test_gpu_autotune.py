"""The rrLU autotuner: per (rows, cols) bucket, the trailing-block size at which
a factorization continues on one warp is chosen by timing candidates on seeded
matrices.  The choice changes the schedule only: pivots, errors and factors stay
bit-identical to the oracle with any table."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CANDIDATES = {1, 96, 192, 384, 768, 1536}


def test_autotune_table_and_identical_results(T, oracle):
    ctx = T.Context(0)
    sp, ms_def, ms_tuned = ctx.autotune_rrlu(reps=1)
    table = ctx.tune_table()
    assert len(table) == 12 and set(table) <= CANDIDATES
    assert sp >= 1.0 and ms_tuned <= ms_def  # the default (192) is one of the candidates
    rng = np.random.default_rng(31)
    mats = []
    for _ in range(40):
        m = int(rng.integers(8, 200))
        n = int(rng.integers(8, 200))
        k = min(m, n)
        mats.append(rng.standard_normal((m, k)) @ np.diag(10.0 ** (-np.arange(k) / 4)) @ rng.standard_normal((k, n)))
    tuned = T.rrlu_batched(mats, reltol=1e-10, ctx=ctx)
    ctx.tune_table([1] * 12)  # every factorization tail on one warp as early as possible
    one = T.rrlu_batched(mats, reltol=1e-10, ctx=ctx)
    ctx.tune_table([0] * 12)  # the kernel's default
    dflt = T.rrlu_batched(mats, reltol=1e-10, ctx=ctx)
    for A, a, b, c in zip(mats, tuned, one, dflt):
        r = oracle.rrlu(A, reltol=1e-10)
        for x in (a, b, c):
            assert x[2] == r["npivot"] and x[3] == r["error"]
            assert np.array_equal(x[0] - 1, r["rowpermutation"][:x[2]])
            assert np.array_equal(x[1] - 1, r["colpermutation"][:x[2]])


def test_autotune_table_set_rejects_negative(T):
    ctx = T.Context(0)
    with pytest.raises(T.ArgumentError):
        ctx.tune_table([-1] * 12)
    assert ctx.tune_table([0] * 11 + [512]) == [0] * 11 + [512]
