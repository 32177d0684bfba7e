"""Failure handling without a GPU fault.

  - The resident kernel's waits are bounded: a worker CTA waits for its task
    ticket at most wait_us, and a wait that runs out makes every CTA leave and
    the call in progress return TCI_ERR_TIMEOUT (the kernel returns on its own;
    nothing is left running).  The test sets the limit to 20 us while the host
    cannot publish tasks for every waiting worker that fast.
  - HBM-budget admission: a context whose budget is below every solve's
    estimate (L d^2 maxbonddim^2 doubles) runs one solve at a time, and the
    results equal those of an unlimited context bit for bit.
"""
import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _specs(T, n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        L = int(rng.integers(4, 9))
        d = int(rng.integers(2, 9))
        a, b, g = 10 ** rng.uniform(-2, 1, size=3)
        c = rng.integers(1, d + 1, size=L)
        out.append((T.DeviceFunction("served", [a, b, g] + [float(x) for x in c]), [d] * L,
                    dict(tolerance=10 ** rng.uniform(-10, -6), maxbonddim=32)))
    return out


def test_worker_wait_limit_reports_timeout(T):
    ctx = T.Context(0)
    ctx.set_resident_limits(idle_us=500000, wait_us=20)
    with pytest.raises(T.TCIError) as ei:
        T.crossinterpolate2_batched(_specs(T, 8, 1), ctx=ctx)
    assert ei.value.code == T.TCI_ERR_TIMEOUT
    assert "limit" in str(ei.value)
    del ei, ctx  # a context that timed out is discarded
    gc.collect()
    # a fresh context with the default limits solves the same requests
    ctx2 = T.Context(0)
    res = T.crossinterpolate2_batched(_specs(T, 8, 1), ctx=ctx2)
    assert all(r is not None and r.rank() >= 1 for r in res)


def test_hbm_budget_admission_queues_without_changing_results(T):
    specs = _specs(T, 12, 2)
    big = T.Context(0)
    big.stats(reset=True)
    ref = T.crossinterpolate2_batched(specs, ctx=big)
    assert big.stats()["peak_live"] > 1
    tiny = T.Context(0, hbm_budget=1)
    tiny.stats(reset=True)
    got = T.crossinterpolate2_batched(specs, ctx=tiny)
    assert tiny.stats()["peak_live"] == 1
    for (f, dims, _), a, b in zip(specs, ref, got):
        assert list(a.linkdims()) == list(b.linkdims())
        for s in range(1, len(dims) + 1):
            assert np.array_equal(a.sets(s)[0], b.sets(s)[0])
            assert np.array_equal(a.sets(s)[1], b.sets(s)[1])
            assert np.array_equal(a.sitetensor(s), b.sitetensor(s))
