"""tci_rrlu_noalloc: the rrLU entry point that allocates nothing.

It exists for callers that cannot let the library allocate device memory (a
stream being captured into a CUDA graph, allocation-free serving loops, hosts
that own every device buffer).  The caller passes device buffers; the library
works in its own fixed device array.  This test calls it through the C ABI on
two matrices in a row -- the second larger than shared memory, so the fixed
array is used as the working matrix -- and checks each result against the
allocating entry point tci_rrlu on the same matrix.  This file is collected
last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(T, torch, A, **kw):
    m, n = A.shape
    dev = torch.device("cuda:0")
    a = torch.from_numpy(np.asfortranarray(A).reshape(-1, order="F").copy()).to(dev)
    rowp = torch.empty(m, dtype=torch.int32, device=dev)
    colp = torch.empty(n, dtype=torch.int32, device=dev)
    npiv = torch.empty(1, dtype=torch.int32, device=dev)
    err = torch.empty(1, dtype=torch.float64, device=dev)
    fac = torch.empty(m * n, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = T.load_library().tci_rrlu_noalloc(
        ctypes.c_void_p(a.data_ptr()), m, n, int(kw.get("maxrank") or 0), kw.get("reltol", 1e-14),
        kw.get("abstol", 0.0), int(kw.get("leftorthogonal", True)), ctypes.c_void_p(rowp.data_ptr()),
        ctypes.c_void_p(colp.data_ptr()), ctypes.c_void_p(npiv.data_ptr()), ctypes.c_void_p(err.data_ptr()),
        ctypes.c_void_p(fac.data_ptr()), stream)
    assert rc == 0, T.load_library().tci_last_error()
    torch.cuda.synchronize(dev)
    F = fac.cpu().numpy().reshape((m, n), order="F")
    return rowp.cpu().numpy(), colp.cpu().numpy(), int(npiv.item()), float(err.item()), F


def _check_against_allocating(T, torch, A, **kw):
    rp, cp, K, err, F = _noalloc(T, torch, A, **kw)
    ref = T.rrlu(A, **kw)
    assert K == ref.npivot
    assert np.array_equal(rp + 1, ref.rowpermutation)
    assert np.array_equal(cp + 1, ref.colpermutation)
    assert err == ref.error
    L = np.tril(F[:, :K])
    U = np.triu(F[:K, :])
    if kw.get("leftorthogonal", True):
        np.fill_diagonal(L, 1.0)
    else:
        np.fill_diagonal(U, 1.0)
    assert np.allclose(L, ref.L, rtol=0, atol=0)
    assert np.allclose(U, ref.U, rtol=0, atol=0)


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


def test_noalloc_rejects_oversize(T):
    L = T.load_library()
    rc = L.tci_rrlu_noalloc(None, 20000, 10, 0, 1e-14, 0.0, 1, None, None, None, None, None, 0)
    assert rc == T.TCI_ERR_ARG
    assert b"16384" in L.tci_last_error()
