"""GPU crossinterpolate2 / TensorCI2 against the CPU oracle.

The registered functions evaluate bit-identically on both sides and the rrLU is
bit-exact, so pivot index sets and ranks must match exactly.  The final site
tensors (left(MatrixLUCI) of sweep1site!, tensorci2.jl:402-461, and the last
Pi1) follow the oracle's operation order, so they are compared bit for bit, and
sum() to 1e-12 relative.  The sampled error on 1e5 seeded lattice points must
be within the requested tolerance (relative to maxsamplevalue, the reference's
normalizeerror) and at most 2x the oracle's.
"""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same_sets(tci, ref):
    L = len(tci)
    for b in range(1, L + 1):
        gi, gj = tci.sets(b)
        ri, rj = ref.sets(b)
        assert np.array_equal(gi, ri), f"Iset[{b}] differs"
        assert np.array_equal(gj, rj), f"Jset[{b}] differs"


def test_pivoterrors_known_answer(T, golden):
    g = golden["tci2"]["pivoterrors"]
    f = T.DeviceFunction.dense(np.diag(g["diags"]))
    tci, _, _ = T.crossinterpolate2(float, f, g["localdims"], [[1, 1]], tolerance=g["tolerance"])
    assert list(tci.pivoterrors) == g["expect_pivoterrors"]


def test_lorentz_updatepivots_known_answers(T, oracle, golden):
    g = golden["tci2"]["lorentz"]
    n, d = g["n"], g["localdim"]
    f = T.DeviceFunction("lorentz")
    tci = T.TensorCI2(f, [d] * n)
    ref = oracle.OracleTCI.new([d] * n, oracle.F_LORENTZ)
    assert list(tci.linkdims()) == [1] * (n - 1)
    for p in range(1, n):
        tci.updatepivots(p, True, reltol=1e-8, maxbonddim=2)
        ref.updatepivots(p, True, reltol=1e-8, maxbonddim=2)
    assert list(tci.linkdims()) == g["maxbonddim2_linkdims"]
    _same_sets(tci, ref)
    tci.addglobalpivots1sitesweep([g["globalpivot"]], reltol=1e-12)
    ref.addglobalpivots1sitesweep([g["globalpivot"]], reltol=1e-12)
    assert list(tci.linkdims()) == g["after_globalpivot_linkdims"]
    _same_sets(tci, ref)
    for _ in range(4, 21):
        for p in range(1, n):
            tci.updatepivots(p, True, reltol=1e-8)
            ref.updatepivots(p, True, reltol=1e-8)
    _same_sets(tci, ref)
    tci2, _, _ = T.crossinterpolate2(float, f, [d] * n, tolerance=1e-8, maxiter=8, sweepstrategy="forward")
    assert tci.rank() == tci2.rank()


@pytest.mark.parametrize("tol", [1e-6, 1e-8, 1e-12])
def test_lorentz5_parity(T, oracle, tol):
    f = T.DeviceFunction("lorentz")
    tci, ranks, errors = T.crossinterpolate2(float, f, [10] * 5, tolerance=tol, maxiter=200)
    ref, rranks, rerrors = oracle.crossinterpolate2([10] * 5, oracle.F_LORENTZ, (), None, tolerance=tol,
                                                    maxiter=200)
    assert list(ranks) == list(rranks)
    _same_sets(tci, ref)
    assert np.array_equal(tci.bonderrors, ref.errors()[1])
    pts = np.array(list(itertools.product(*[range(1, 4)] * 5)))
    assert np.allclose(tci.evaluate(pts), 1.0 / (1.0 + (pts ** 2).sum(1)), rtol=max(tol, 1e-12) * 10)
    for b in range(1, 6):
        assert np.array_equal(tci.sitetensor(b), ref.core(b)), f"site tensor {b} differs"
    assert tci.sum() == ref.sum()


def test_config1_lorentz8(T, oracle):
    """8-site Lorentzian, tolerance 1e-8, maxbonddim 200, all-ones pivot: pivots
    and ranks bit-exact, max error on 1e5 seeded lattice points within tolerance
    and at most 2x the oracle's, sum to 1e-12 relative."""
    f = T.DeviceFunction("lorentz")
    kw = dict(tolerance=1e-8, maxbonddim=200, maxiter=20)
    tci, ranks, errors = T.crossinterpolate2(float, f, [10] * 8, **kw)
    ref, rranks, rerrors = oracle.crossinterpolate2([10] * 8, oracle.F_LORENTZ, (), None, **kw)
    assert list(ranks) == list(rranks)
    _same_sets(tci, ref)
    pts = np.random.default_rng(1234).integers(1, 11, size=(100000, 8))
    fx = 1.0 / (1.0 + (pts ** 2).sum(1))
    _check_sampled_error(tci, ref, pts, fx, 1e-8)
    for b in range(1, 9):
        assert np.array_equal(tci.sitetensor(b), ref.core(b)), f"site tensor {b} differs"
    s, sr = tci.sum(), ref.sum()
    assert abs(s - sr) <= 1e-12 * abs(sr)


def _check_sampled_error(tci, ref, pts, fx, tol, margin=1.0):
    """Max |f - tt| on the sampled points: at most 2x the oracle's and within
    margin x the requested tolerance, relative to maxsamplevalue (optimize!
    normalises its errors, tensorci2.jl:711, :843-845).  margin = 1 where the
    reference's algorithm itself meets the tolerance on the sample; the quantics
    configurations use the reference's own guarantee instead: its global pivot
    search only adds points whose error exceeds tolmarginglobalsearch (10) x
    tol (globalpivotfinder.jl:179-182), and the oracle's sampled error there is
    1.5x (R = 40, tol 1e-10) and 1.3x (2-D, tol 1e-9) the tolerance."""
    err_gpu = float(np.max(np.abs(tci.evaluate(pts) - fx)))
    err_ref = float(np.max(np.abs(ref.evaluate(pts) - fx)))
    assert err_gpu <= margin * tol * tci.maxsamplevalue, (err_gpu, tci.maxsamplevalue)
    assert err_gpu <= 2 * err_ref + 1e-300, (err_gpu, err_ref)
    return err_gpu, err_ref


def _served(rng, L, d):
    a, b, g = 10 ** rng.uniform(-2, 1, size=3)
    c = rng.integers(1, d + 1, size=L)
    return [a, b, g] + list(c)


def test_served_family_parity(T, oracle):
    rng = np.random.default_rng(42)
    for _ in range(6):
        L = int(rng.integers(4, 12))
        d = int(rng.integers(2, 12))
        prm = _served(rng, L, d)
        tol = 10 ** rng.uniform(-10, -6)
        mbd = int(rng.choice([32, 64, 128, 256]))
        tci, ranks, _ = T.crossinterpolate2(float, T.DeviceFunction("served", prm), [d] * L, tolerance=tol,
                                            maxbonddim=mbd)
        ref, rranks, _ = oracle.crossinterpolate2([d] * L, oracle.F_SERVED, prm, None, tolerance=tol,
                                                  maxbonddim=mbd)
        assert list(ranks) == list(rranks)
        _same_sets(tci, ref)
        pts = np.stack([rng.integers(1, d + 1, size=2000) for _ in range(L)], 1)
        assert np.allclose(tci.evaluate(pts), ref.evaluate(pts), rtol=1e-9, atol=1e-12 * ref.maxsamplevalue)


def test_quantics_1d(T, oracle):
    """Quantics R=40, tolerance 1e-10, maxbonddim 128 (the split-precision
    config's TCI part)."""
    f = T.DeviceFunction("qtt1d", [0])
    kw = dict(tolerance=1e-10, maxbonddim=128, maxiter=20)
    tci, ranks, _ = T.crossinterpolate2(float, f, [2] * 40, **kw)
    ref, rranks, _ = oracle.crossinterpolate2([2] * 40, oracle.F_QTT1D, [0], None, **kw)
    assert list(ranks) == list(rranks)
    _same_sets(tci, ref)
    for b in range(1, 41):
        assert np.array_equal(tci.sitetensor(b), ref.core(b)), f"site tensor {b} differs"
    assert abs(tci.sum() - ref.sum()) <= 1e-12 * abs(ref.sum())
    pts = np.random.default_rng(10).integers(1, 3, size=(100000, 40))
    fx = oracle.feval(oracle.F_QTT1D, [0], pts)
    _check_sampled_error(tci, ref, pts, fx, 1e-10, margin=10.0)


def test_quantics_2d_config(T, oracle):
    """The 30-site 2-D quantics function (d = 4, tol 1e-9, maxbonddim 512): ranks
    near 80, Pi up to 320 x 320 (global-memory rrLU)."""
    kw = dict(tolerance=1e-9, maxbonddim=512, maxiter=20)
    tci, ranks, _ = T.crossinterpolate2(float, T.DeviceFunction("qtt2d"), [4] * 30, **kw)
    ref, rranks, _ = oracle.crossinterpolate2([4] * 30, oracle.F_QTT2D, [], None, **kw)
    assert list(ranks) == list(rranks)
    _same_sets(tci, ref)
    for b in range(1, 31):
        assert np.array_equal(tci.sitetensor(b), ref.core(b)), f"site tensor {b} differs"
    assert abs(tci.sum() - ref.sum()) <= 1e-12 * abs(ref.sum())
    pts = np.random.default_rng(9).integers(1, 5, size=(100000, 30))
    fx = oracle.feval(oracle.F_QTT2D, [], pts)
    _check_sampled_error(tci, ref, pts, fx, 1e-9, margin=10.0)


def test_batched_equals_alone(T):
    """Each solve gives the same pivots alone and in a batch with others."""
    rng = np.random.default_rng(3)
    specs = []
    for _ in range(12):
        L = int(rng.integers(4, 10))
        d = int(rng.integers(2, 10))
        specs.append((T.DeviceFunction("served", _served(rng, L, d)), [d] * L,
                      dict(tolerance=10 ** rng.uniform(-10, -6), maxbonddim=64)))
    batch = T.crossinterpolate2_batched(specs, max_live=5)
    for (f, dims, kw), tb in zip(specs, batch):
        ta, _, _ = T.crossinterpolate2(float, f, dims, **kw)
        assert list(tb.linkdims()) == list(ta.linkdims())
        for b in range(1, len(dims) + 1):
            assert np.array_equal(tb.sets(b)[0], ta.sets(b)[0])
            assert np.array_equal(tb.sets(b)[1], ta.sets(b)[1])
        assert np.array_equal(tb.sitetensor(1), ta.sitetensor(1))


def test_serve_stream(T):
    rng = np.random.default_rng(5)
    specs = []
    for _ in range(30):
        L = int(rng.integers(4, 9))
        d = int(rng.integers(2, 9))
        specs.append((T.DeviceFunction("served", _served(rng, L, d)), [d] * L,
                      dict(tolerance=10 ** rng.uniform(-10, -6), maxbonddim=32)))
    arrival = np.cumsum(rng.exponential(1 / 500.0, size=len(specs)))
    lat, rank, wall = T.serve(specs, arrival, max_live=16)
    assert np.all(lat > 0) and np.all(rank >= 1)
    for i in [0, 7, 29]:
        f, dims, kw = specs[i]
        ta, _, _ = T.crossinterpolate2(float, f, dims, **kw)
        assert ta.rank() == rank[i]


def test_errors_like_reference(T):
    f = T.DeviceFunction("lorentz")
    with pytest.raises(T.ArgumentError):  # tensorci2.jl:750-754
        T.crossinterpolate2(float, f, [2] * 5, tolerance=0.0)
    with pytest.raises(T.DimensionMismatch):  # tensorci2.jl:197-199
        tci = T.TensorCI2(f, [3] * 4)
        tci.addglobalpivots([[1, 2, 3]])
    z = T.DeviceFunction.dense(np.zeros((3, 3)))
    with pytest.raises(T.TCIError, match="maxsamplevalue is zero"):  # tensorci2.jl:50
        T.TensorCI2(z, [3, 3])
    # NaN that reaches L in the first bond: "lu.L contains NaNs" (matrixlu.jl:164-166)
    bad = np.ones((3, 3))
    bad[1, 0] = np.nan
    with pytest.raises(T.TCIError, match="NaN"):
        T.crossinterpolate2(float, T.DeviceFunction.dense(bad), [3, 3])


def test_bulk_export_matches_per_core(T):
    rng = np.random.default_rng(8)
    specs = []
    for _ in range(6):
        L = int(rng.integers(4, 8))
        d = int(rng.integers(2, 6))
        specs.append((T.DeviceFunction("served", _served(rng, L, d)), [d] * L, dict(tolerance=1e-8, maxbonddim=32)))
    res = T.crossinterpolate2_batched(specs)
    tts = T.tensortrains(res)
    for tci, tt in zip(res, tts):
        for b in range(1, len(tci) + 1):
            assert np.array_equal(tt.sitetensors[b - 1], tci.sitetensor(b))


def _served_specs(T, seed, n, maxbonddim):
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(n):
        L = int(rng.integers(4, 10))
        d = int(rng.integers(2, 10))
        specs.append((T.DeviceFunction("served", _served(rng, L, d)), [d] * L,
                      dict(tolerance=10 ** rng.uniform(-10, -6), maxbonddim=maxbonddim)))
    return specs


def test_resident_equals_batched_launches(T, monkeypatch):
    """The resident kernel (ring in pinned memory) and one launch per engine step
    give identical solves."""
    specs = _served_specs(T, 21, 24, 64)
    monkeypatch.setenv("TCI_RESIDENT", "0")
    ctx_b = T.Context(0)
    monkeypatch.setenv("TCI_RESIDENT", "1")
    ctx_r = T.Context(0)
    a = T.crossinterpolate2_batched(specs, max_live=8, ctx=ctx_b)
    b = T.crossinterpolate2_batched(specs, max_live=8, ctx=ctx_r)
    assert ctx_r.stats()["tasks"] > 0
    for ta, tb, (_, dims, _) in zip(a, b, specs):
        assert list(ta.linkdims()) == list(tb.linkdims())
        for s in range(1, len(dims) + 1):
            assert np.array_equal(ta.sets(s)[0], tb.sets(s)[0])
            assert np.array_equal(ta.sets(s)[1], tb.sets(s)[1])
            assert np.array_equal(ta.sitetensor(s), tb.sitetensor(s))


def test_resident_relaunch_after_idle(T, monkeypatch):
    """With a short idle limit the resident kernel leaves between sparse
    arrivals and is launched again; every request is still served."""
    monkeypatch.setenv("TCI_RESIDENT", "1")
    monkeypatch.setenv("TCI_RESIDENT_IDLE_US", "300")
    ctx = T.Context(0)
    specs = _served_specs(T, 22, 8, 32)
    arrival = np.arange(len(specs)) * 0.02  # 20 ms apart: longer than the idle limit
    lat, rank, wall = T.serve(specs, arrival, max_live=4, ctx=ctx)
    assert np.all(lat > 0) and np.all(rank >= 1)
    assert ctx.stats()["launches"] >= 2
    for i in [0, 5]:
        f, dims, kw = specs[i]
        ta, _, _ = T.crossinterpolate2(float, f, dims, ctx=ctx, **kw)
        assert ta.rank() == rank[i]


OPTION_CASES = [
    dict(sweepstrategy="forward"),
    dict(sweepstrategy="backward"),
    dict(strictlynested=True),
    dict(normalizeerror=False, tolerance=1e-6),
    dict(maxnglobalpivot=0),
    dict(nsearchglobalpivot=0),
    dict(checkconvglobalpivot=False, ncheckhistory=1),
    dict(tolmarginglobalsearch=1.0, nsearchglobalpivot=8, maxnglobalpivot=2),
    dict(maxbonddim=5, maxiter=6),
    dict(seed=12345),
]


@pytest.mark.parametrize("opts", OPTION_CASES, ids=[",".join(f"{k}={v}" for k, v in o.items()) for o in OPTION_CASES])
def test_optimize_options_parity(T, oracle, opts):
    """The optimize! keyword arguments (tensorci2.jl:700-720) change the sweeps the
    same way on both sides: identical ranks history and pivot sets."""
    rng = np.random.default_rng(31)
    L, d = 6, 5
    prm = _served(rng, L, d)
    kw = dict(tolerance=1e-9, maxiter=12)
    kw.update(opts)
    tci, ranks, errs = T.crossinterpolate2(float, T.DeviceFunction("served", prm), [d] * L, **kw)
    ref, rranks, rerrs = oracle.crossinterpolate2([d] * L, oracle.F_SERVED, prm, None, **kw)
    assert list(ranks) == list(rranks)
    _same_sets(tci, ref)
    assert np.allclose(errs, rerrs, rtol=1e-12, atol=0)


def test_batch_with_a_failing_request(T):
    """A request whose f makes lu.L NaN fails with the reference's error; the other
    solves of the batch and later calls are unaffected (the resident kernel is
    stopped cleanly and the context stays usable)."""
    rng = np.random.default_rng(41)
    bad = np.ones((3, 3))
    bad[1, 0] = np.nan
    good = _served_specs(T, 42, 6, 32)
    specs = good[:3] + [(T.DeviceFunction.dense(bad), [3, 3], dict(tolerance=1e-8))] + good[3:]
    with pytest.raises(T.TCIError, match="NaN"):
        T.crossinterpolate2_batched(specs, max_live=4)
    again = T.crossinterpolate2_batched(good, max_live=4)
    for (f, dims, kw), tb in zip(good, again):
        ta, _, _ = T.crossinterpolate2(float, f, dims, **kw)
        assert list(tb.linkdims()) == list(ta.linkdims())
    del rng


def test_tt_evaluate_and_sum_of_given_trains(T, oracle):
    """evaluate / sum of a tensor train the caller gives (not from a solve)."""
    rng = np.random.default_rng(51)
    bonds = [1, 3, 4, 2, 1]
    cores = [rng.standard_normal((bonds[n], 3, bonds[n + 1])) for n in range(4)]
    tt = T.TensorTrain(cores)
    pts = rng.integers(1, 4, size=(500, 4))
    ref = oracle.tt_evaluate(cores, pts)
    assert np.allclose(tt.evaluate(pts), ref, rtol=1e-13, atol=1e-14)
    assert tt.sum() == pytest.approx(oracle.tt_sum(cores), rel=1e-13)


def test_set_sets_and_bonderrors(T, oracle):
    f = T.DeviceFunction("lorentz")
    tci, _, _ = T.crossinterpolate2(float, f, [6] * 4, tolerance=1e-10)
    I, J = tci.sets(2)
    be = np.zeros(3)
    T.load_library().tci_bonderrors(tci.h, be.ctypes.data_as(T.F64P))
    assert np.all(be >= 0)
    tci.set_sets(2, I, J)  # same sets back: nothing changes but the cores are rebuilt on demand
    I2, J2 = tci.sets(2)
    assert np.array_equal(I, I2) and np.array_equal(J, J2)
    with pytest.raises(T.ArgumentError):
        tci.set_sets(2, np.array([[7]]), J)


def test_incremental_server(T):
    """tci_serve_start / submit / poll / stop: requests submitted in bursts while
    earlier ones run; every one completes with the rank it has alone."""
    import time as _time

    specs = _served_specs(T, 61, 16, 32)
    srv = T.Server(max_live=8)
    done = {}
    ids = {}
    try:
        for k, (f, dims, kw) in enumerate(specs[:8]):
            ids[srv.submit(f, dims, **kw)] = k
        for rid, st, rank, lat in srv.poll(timeout_ms=50):
            done[rid] = (st, rank, lat)
        _time.sleep(0.05)
        for k, (f, dims, kw) in enumerate(specs[8:], start=8):
            ids[srv.submit(f, dims, **kw)] = k
        t0 = _time.time()
        while len(done) < len(specs) and _time.time() - t0 < 60:
            for rid, st, rank, lat in srv.poll(timeout_ms=100):
                done[rid] = (st, rank, lat)
    finally:
        srv.stop()
    assert sorted(done) == list(range(len(specs)))
    for rid, (st, rank, lat) in done.items():
        f, dims, kw = specs[ids[rid]]
        assert st == 0 and lat > 0
        ta, _, _ = T.crossinterpolate2(float, f, dims, **kw)
        assert ta.rank() == rank


def _quantics_index(x, R):
    """1-based bits of floor(x 2^R), most significant first (a 1-D quantics grid on [0, 1))."""
    k = int(np.floor(x * 2 ** R))
    return [((k >> (R - 1 - i)) & 1) + 1 for i in range(R)]


@pytest.mark.parametrize("strictlynested,nsearch", [(False, 0), (True, 0), (False, 10)])
def test_trivial_mps_exp(T, oracle, strictlynested, nsearch):
    """test/test_tensorci2.jl:55-104: f(x) = exp(-x) on an 8-bit quantics grid,
    maxbonddim 1, two first pivots: all link dimensions 1 and |tci(x) - f(x)| < 1e-4
    at x = 0.1, 0.3, 0.6, 0.9; pivots equal the oracle's."""
    R = 8
    f = T.DeviceFunction("qtt1d", [1])
    first = [[1] * R, [1] + [2] * (R - 1)]
    kw = dict(tolerance=1e-4, maxbonddim=1, maxiter=2, normalizeerror=False, nsearchglobalpivot=nsearch,
              strictlynested=strictlynested)
    tci, ranks, _ = T.crossinterpolate2(float, f, [2] * R, first, **kw)
    assert list(tci.linkdims()) == [1] * (R - 1)
    ref, rranks, _ = oracle.crossinterpolate2([2] * R, oracle.F_QTT1D, [1], first, **kw)
    assert list(ranks) == list(rranks)
    _same_sets(tci, ref)
    tt = tci.tensortrain()
    for x in [0.1, 0.3, 0.6, 0.9]:
        v = _quantics_index(x, R)
        fx = np.exp(-np.floor(x * 2 ** R) / 2 ** R)
        assert abs(tci.evaluate(v) - fx) < 1e-4
        assert abs(tt.evaluate(v) - fx) < 1e-4


def test_trivial_mps_exp_small_maxbonddim(T, oracle):
    """test/test_tensorci2.jl:168-213: exp(-x) + 1e-4 exp(-2x), tolerance 1e-10 but
    maxbonddim 1, nsearchglobalpivot 10: link dimensions 1, error below 1e-4."""
    R = 8
    f = T.DeviceFunction("qtt1d", [2])
    first = [[1] * R, [1] + [2] * (R - 1)]
    kw = dict(tolerance=1e-10, maxbonddim=1, maxiter=10, normalizeerror=False, nsearchglobalpivot=10)
    tci, ranks, _ = T.crossinterpolate2(float, f, [2] * R, first, **kw)
    assert list(tci.linkdims()) == [1] * (R - 1)
    ref, rranks, _ = oracle.crossinterpolate2([2] * R, oracle.F_QTT1D, [2], first, **kw)
    assert list(ranks) == list(rranks)
    _same_sets(tci, ref)
    for x in [0.1, 0.3, 0.6, 0.9]:
        v = _quantics_index(x, R)
        t = np.floor(x * 2 ** R) / 2 ** R
        assert abs(tci.evaluate(v) - (np.exp(-t) + 1e-4 * np.exp(-2 * t))) < 1e-4


def test_trivial_mps_one_pivot(T):
    """test/test_tensorci2.jl:215-232: TensorCI2(f, fill(2, n), [fill(1, n)]) has rank 1."""
    n = 5
    tci = T.TensorCI2(T.BatchFunction(lambda p: 0.5 * p.sum(1).astype(float)), [2] * n, [[1] * n])
    assert len(tci) == n
    assert tci.rank() == 1
    assert list(tci.linkdims()) == [1] * (n - 1)
