"""Tasks planned against a small shared-memory budget (TCI_PLAN_SMEM) run with
their Π in global scratch, and with the row/column f states there as well: the
pivots, site tensors and batched results stay bit-identical to the oracle's and
to the default layout's."""
import os

import numpy as np
import pytest

from test_gpu_tci import _same_sets, _served

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_plan_ctx(T):
    old = os.environ.get("TCI_PLAN_SMEM")
    os.environ["TCI_PLAN_SMEM"] = "6144"  # Π of more than ~25 x 25 leaves shared memory
    try:
        ctx = T.Context(0)
    finally:
        if old is None:
            del os.environ["TCI_PLAN_SMEM"]
        else:
            os.environ["TCI_PLAN_SMEM"] = old
    return ctx


def test_global_layouts_match_oracle(T, oracle, small_plan_ctx):
    rng = np.random.default_rng(77)
    for _ in range(4):
        L = int(rng.integers(4, 8))
        d = int(rng.integers(6, 14))
        prm = _served(rng, L, d)
        kw = dict(tolerance=10 ** rng.uniform(-10, -7), maxbonddim=int(rng.choice([32, 64])))
        tci, ranks, _ = T.crossinterpolate2(float, T.DeviceFunction("served", prm), [d] * L, ctx=small_plan_ctx, **kw)
        ref, rranks, _ = oracle.crossinterpolate2([d] * L, oracle.F_SERVED, prm, None, **kw)
        assert list(ranks) == list(rranks)
        _same_sets(tci, ref)
        for b in range(1, L + 1):
            assert np.array_equal(tci.sitetensor(b), ref.core(b)), f"site tensor {b} differs"


def test_global_layouts_batched_equal_default(T, small_plan_ctx):
    """The batched path (resident kernel, per-task scratch) under the small plan
    gives the same solves as the default context."""
    rng = np.random.default_rng(78)
    specs = []
    for _ in range(10):
        L = int(rng.integers(4, 8))
        d = int(rng.integers(4, 12))
        specs.append((T.DeviceFunction("served", _served(rng, L, d)), [d] * L,
                      dict(tolerance=10 ** rng.uniform(-10, -6), maxbonddim=64)))
    small = T.crossinterpolate2_batched(specs, max_live=4, ctx=small_plan_ctx)
    dflt = T.crossinterpolate2_batched(specs, max_live=4)
    for (f, dims, kw), a, b in zip(specs, small, dflt):
        assert list(a.linkdims()) == list(b.linkdims())
        for s in range(1, len(dims) + 1):
            assert np.array_equal(a.sets(s)[0], b.sets(s)[0])
            assert np.array_equal(a.sets(s)[1], b.sets(s)[1])
            assert np.array_equal(a.sitetensor(s), b.sitetensor(s))


def test_task_beyond_the_plan_fails_cleanly(T):
    """A Π whose permutations alone exceed the (here artificially small) budget:
    the solve fails with the plan error, and the context keeps working."""
    old = os.environ.get("TCI_PLAN_SMEM")
    os.environ["TCI_PLAN_SMEM"] = "1024"
    try:
        ctx = T.Context(0)
    finally:
        if old is None:
            del os.environ["TCI_PLAN_SMEM"]
        else:
            os.environ["TCI_PLAN_SMEM"] = old
    rng = np.random.default_rng(79)
    prm = _served(rng, 6, 12)
    with pytest.raises(T.TCIError, match="on-chip plan"):
        T.crossinterpolate2(float, T.DeviceFunction("served", prm), [12] * 6, tolerance=1e-10, maxbonddim=64, ctx=ctx)
    tci, ranks, _ = T.crossinterpolate2(float, T.DeviceFunction("lorentz"), [4] * 4, tolerance=1e-8, ctx=ctx)
    assert max(ranks) >= 1


def test_throughput_variant_matches_oracle(T, oracle):
    """Enough live solves that the resident kernel runs two 256-thread task CTAs
    per SM (the throughput variant) for most of the batch: pivots and site
    tensors still equal the oracle's."""
    rng = np.random.default_rng(80)
    specs, raw = [], []
    for _ in range(400):
        L = int(rng.integers(4, 8))
        d = int(rng.integers(2, 9))
        prm = _served(rng, L, d)
        kw = dict(tolerance=10 ** rng.uniform(-10, -6), maxbonddim=32)
        specs.append((T.DeviceFunction("served", prm), [d] * L, kw))
        raw.append((L, d, prm, kw))
    res = T.crossinterpolate2_batched(specs, max_live=400)
    for i in range(0, 400, 20):
        L, d, prm, kw = raw[i]
        ref, _, _ = oracle.crossinterpolate2([d] * L, oracle.F_SERVED, prm, None, **kw)
        _same_sets(res[i], ref)
        for b in range(1, L + 1):
            assert np.array_equal(res[i].sitetensor(b), ref.core(b)), f"solve {i} site tensor {b} differs"
