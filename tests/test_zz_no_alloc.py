"""tci_rrlu_noalloc: the rrLU entry point that allocates nothing.

Some callers cannot let a library allocate device memory: a host whose every
device buffer comes from its own allocator (a Julia GPU array pool, a
framework's arena), where an allocation behind its back breaks its accounting
or fails against its reservation, and latency-critical loops where a
cudaMalloc/cudaFree would synchronise the device.  This entry point takes
device buffers from the caller and works in one fixed device array of the
library.  The tests call it through the C ABI and check it

  - against the allocating entry point tci_rrlu, bit for bit, on two calls in a
    row (the second larger than shared memory, so the fixed array holds the
    working matrix), at the two limit shapes (16384 x 32 and m*n = 2^19) and
    when captured into a CUDA graph and replayed on new inputs;
  - against the CPU oracle directly on the reference's own rrLU test matrices
    (test/test_matrixlu.jl), and on a matrix whose L holds a NaN, where the
    status output must carry TCI_ERR_NAN (the reference's "lu.L contains NaNs",
    matrixlu.jl:164-169).

This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _buffers(torch, m, n):
    dev = torch.device("cuda:0")
    return dict(a=torch.empty(m * n, dtype=torch.float64, device=dev),
                rowp=torch.full((m,), -1, dtype=torch.int32, device=dev),
                colp=torch.full((n,), -1, dtype=torch.int32, device=dev),
                npiv=torch.full((1,), -1, dtype=torch.int32, device=dev),
                err=torch.full((1,), -1.0, dtype=torch.float64, device=dev),
                status=torch.full((1,), -1, dtype=torch.int32, device=dev),
                fac=torch.empty(m * n, dtype=torch.float64, device=dev))


def _load(torch, b, A):
    b["a"].copy_(torch.from_numpy(np.asfortranarray(A).reshape(-1, order="F").copy()))


def _enqueue(T, b, m, n, stream, **kw):
    """Only enqueues (no synchronisation), so it can run inside a stream capture."""
    rc = T.load_library().tci_rrlu_noalloc(
        ctypes.c_void_p(b["a"].data_ptr()), m, n, int(kw.get("maxrank") or 0), kw.get("reltol", 1e-14),
        kw.get("abstol", 0.0), int(kw.get("leftorthogonal", True)), ctypes.c_void_p(b["rowp"].data_ptr()),
        ctypes.c_void_p(b["colp"].data_ptr()), ctypes.c_void_p(b["npiv"].data_ptr()),
        ctypes.c_void_p(b["err"].data_ptr()), ctypes.c_void_p(b["status"].data_ptr()),
        ctypes.c_void_p(b["fac"].data_ptr()), stream)
    assert rc == 0, T.load_library().tci_last_error()


def _collect(b, m, n):
    F = b["fac"].cpu().numpy().reshape((m, n), order="F")
    return dict(rowperm=b["rowp"].cpu().numpy(), colperm=b["colp"].cpu().numpy(), npivot=int(b["npiv"].item()),
                error=float(b["err"].item()), status=int(b["status"].item()), F=F)


def _noalloc(T, torch, A, **kw):
    m, n = A.shape
    dev = torch.device("cuda:0")
    b = _buffers(torch, m, n)
    _load(torch, b, A)
    _enqueue(T, b, m, n, torch.cuda.current_stream(dev).cuda_stream, **kw)
    torch.cuda.synchronize(dev)
    return _collect(b, m, n)


def _factors(r, leftorthogonal):
    K = r["npivot"]
    F = r["F"]
    L = np.tril(F[:, :K])
    U = np.triu(F[:K, :])
    if leftorthogonal:
        np.fill_diagonal(L, 1.0)
    else:
        np.fill_diagonal(U, 1.0)
    return L, U


def _check_against_allocating(T, torch, A, r=None, **kw):
    if r is None:
        r = _noalloc(T, torch, A, **kw)
    ref = T.rrlu(A, **kw)
    assert r["status"] == 0
    assert r["npivot"] == ref.npivot
    assert np.array_equal(r["rowperm"] + 1, ref.rowpermutation)
    assert np.array_equal(r["colperm"] + 1, ref.colpermutation)
    assert r["error"] == ref.error
    L, U = _factors(r, kw.get("leftorthogonal", True))
    assert np.array_equal(L, ref.L)
    assert np.array_equal(U, ref.U)


def _check_against_oracle(T, torch, oracle, A, **kw):
    r = _noalloc(T, torch, A, **kw)
    ref = oracle.rrlu(A, **kw)
    assert r["status"] == 0
    assert r["npivot"] == ref["npivot"]
    assert np.array_equal(r["rowperm"], ref["rowpermutation"])
    assert np.array_equal(r["colperm"], ref["colpermutation"])
    assert r["error"] == ref["error"]
    L, U = _factors(r, kw.get("leftorthogonal", True))
    assert np.array_equal(L, ref["L"])
    assert np.array_equal(U, ref["U"])
    return r


def test_noalloc_matches_allocating_entry_point(T):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(2024)
    # call 1: fits in shared memory
    A1 = rng.standard_normal((40, 30)) @ rng.standard_normal((30, 50))
    _check_against_allocating(T, torch, A1, reltol=1e-12)
    # call 2, right after: larger than shared memory, works in the fixed array
    r = 25
    A2 = rng.standard_normal((300, r)) @ rng.standard_normal((r, 280)) + 1e-13 * rng.standard_normal((300, 280))
    _check_against_allocating(T, torch, A2, reltol=1e-10, maxrank=64, leftorthogonal=False)


@pytest.mark.parametrize("shape", [(16384, 32), (512, 1024)])
def test_noalloc_limit_shapes(T, shape):
    """The largest accepted shapes: 16384 rows (64 KB of permutations beside the
    matrix) and m*n = 2^19 exactly."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(shape[0])
    m, n = shape
    k = 20
    A = rng.standard_normal((m, k)) @ rng.standard_normal((k, n)) + 1e-12 * rng.standard_normal((m, n))
    _check_against_allocating(T, torch, A, reltol=1e-10, maxrank=24)


def test_noalloc_in_cuda_graph(T):
    """The call captured into a CUDA graph after a warm-up call (which does the
    per-device set-up outside the capture), then replayed on new contents of the
    same input buffer: every replay matches tci_rrlu bit for bit.  The matrix is
    larger than shared memory, so the replays also reuse the fixed array."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(77)
    m, n, k = 200, 150, 18
    kw = dict(reltol=1e-10, maxrank=32)

    def matrix():
        return rng.standard_normal((m, k)) @ rng.standard_normal((k, n)) + 1e-12 * rng.standard_normal((m, n))

    dev = torch.device("cuda:0")
    b = _buffers(torch, m, n)
    A = matrix()
    _load(torch, b, A)
    _enqueue(T, b, m, n, torch.cuda.current_stream(dev).cuda_stream, **kw)
    torch.cuda.synchronize(dev)
    _check_against_allocating(T, torch, A, r=_collect(b, m, n), **kw)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, capture_error_mode="thread_local"):
        _enqueue(T, b, m, n, torch.cuda.current_stream(dev).cuda_stream, **kw)
    for _ in range(3):
        A = matrix()
        _load(torch, b, A)
        for key in ("rowp", "colp", "npiv", "status"):
            b[key].fill_(-1)
        g.replay()
        torch.cuda.synchronize(dev)
        _check_against_allocating(T, torch, A, r=_collect(b, m, n), **kw)


def test_noalloc_reference_matrices_against_oracle(T, oracle, golden):
    """The reference's own rrLU test matrices (test/test_matrixlu.jl), through the
    entry point and through the oracle: identical permutations, pivots, errors
    and factors."""
    torch = pytest.importorskip("torch")
    for case in golden["rrlu"]:
        A = np.array(case["A"], dtype=np.float64)
        kw = dict(case["kwargs"])
        _check_against_oracle(T, torch, oracle, A, **kw)
        _check_against_oracle(T, torch, oracle, A, leftorthogonal=False, **kw)


def test_noalloc_reports_nan(T, oracle):
    """A NaN that reaches L: the oracle raises the reference's "lu.L contains
    NaNs" and the entry point's status output holds TCI_ERR_NAN."""
    torch = pytest.importorskip("torch")
    A = np.ones((3, 3))
    A[1, 0] = np.nan
    with pytest.raises(oracle.OracleError):
        oracle.rrlu(A)
    r = _noalloc(T, torch, A)
    assert r["status"] == T.TCI_ERR_NAN
    with pytest.raises(T.TCIError, match="NaN"):
        T.rrlu(A)
    # the next call on a clean matrix reports success again
    _check_against_allocating(T, torch, np.arange(1.0, 13.0).reshape(3, 4) ** 2)


def test_noalloc_rejects_oversize(T):
    L = T.load_library()
    rc = L.tci_rrlu_noalloc(None, 20000, 10, 0, 1e-14, 0.0, 1, None, None, None, None, None, None, 0)
    assert rc == T.TCI_ERR_ARG
    assert b"16384" in L.tci_last_error()
    rc = L.tci_rrlu_noalloc(None, 1024, 1024, 0, 1e-14, 0.0, 1, None, None, None, None, None, None, 0)
    assert rc == T.TCI_ERR_ARG
