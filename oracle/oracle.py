"""ctypes bindings of the CPU oracle (test infrastructure only).

The oracle is a C++ restatement of TensorCrossInterpolation.jl's TCI2 path
(oracle/tci_oracle.cpp).  Only the tests, the smoke check and the CPU-baseline
legs of bench.py use this module, as the checker or the timed CPU baseline.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

F_LORENTZ, F_SERVED, F_QTT1D, F_QTT2D, F_DENSE, F_PRODUCT = 1, 2, 3, 4, 5, 6
FUNCTION_IDS = {"lorentz": 1, "served": 2, "qtt1d": 3, "qtt2d": 4, "dense": 5, "product": 6}

I64P = ctypes.POINTER(ctypes.c_int64)
F64P = ctypes.POINTER(ctypes.c_double)
I32P = ctypes.POINTER(ctypes.c_int32)


class Opts(ctypes.Structure):
    """optimize! keyword arguments (tensorci2.jl:700-720)."""
    _fields_ = [
        ("tolerance", ctypes.c_double),
        ("maxbonddim", ctypes.c_int64),
        ("maxiter", ctypes.c_int64),
        ("sweepstrategy", ctypes.c_int32),
        ("normalizeerror", ctypes.c_int32),
        ("ncheckhistory", ctypes.c_int32),
        ("maxnglobalpivot", ctypes.c_int32),
        ("nsearchglobalpivot", ctypes.c_int32),
        ("strictlynested", ctypes.c_int32),
        ("checkconvglobalpivot", ctypes.c_int32),
        ("pad_", ctypes.c_int32),
        ("tolmarginglobalsearch", ctypes.c_double),
        ("seed", ctypes.c_uint64),
    ]


SWEEP = {"backandforth": 0, "forward": 1, "backward": 2}


def make_opts(tolerance=1e-8, maxbonddim=None, maxiter=20, sweepstrategy="backandforth",
              normalizeerror=True, ncheckhistory=3, maxnglobalpivot=5, nsearchglobalpivot=5,
              tolmarginglobalsearch=10.0, strictlynested=False, checkconvglobalpivot=True, seed=0):
    o = Opts()
    o.tolerance = tolerance
    o.maxbonddim = 0 if maxbonddim is None else int(maxbonddim)
    o.maxiter = int(maxiter)
    o.sweepstrategy = SWEEP[sweepstrategy]
    o.normalizeerror = int(bool(normalizeerror))
    o.ncheckhistory = int(ncheckhistory)
    o.maxnglobalpivot = int(maxnglobalpivot)
    o.nsearchglobalpivot = int(nsearchglobalpivot)
    o.strictlynested = int(bool(strictlynested))
    o.checkconvglobalpivot = int(bool(checkconvglobalpivot))
    o.tolmarginglobalsearch = float(tolmarginglobalsearch)
    o.seed = int(seed)
    return o


def build():
    src = os.path.join(HERE, "tci_oracle.cpp")
    if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE])
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_rrlu.argtypes = [F64P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_double,
                               ctypes.c_double, ctypes.c_int, I64P, I64P, F64P, F64P, I64P, F64P]
        L.orc_luci.argtypes = [F64P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_double,
                               ctypes.c_double, ctypes.c_int, F64P, F64P, I64P]
        L.orc_rrlu_batched.argtypes = [ctypes.c_int64, F64P, I64P, I64P, I64P, ctypes.c_int64,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_int, I64P, I64P,
                                       I64P, F64P, ctypes.c_int]
        L.orc_feval.argtypes = [ctypes.c_int, F64P, ctypes.c_int64, ctypes.c_int, I64P, ctypes.c_int64,
                                F64P]
        L.orc_tci_new.restype = ctypes.c_void_p
        L.orc_tci_new.argtypes = [ctypes.c_int, I64P, ctypes.c_int, F64P, ctypes.c_int64, I64P,
                                  ctypes.c_int64, ctypes.POINTER(ctypes.c_int)]
        L.orc_crossinterpolate2.restype = ctypes.c_void_p
        L.orc_crossinterpolate2.argtypes = [ctypes.c_int, I64P, ctypes.c_int, F64P, ctypes.c_int64, I64P,
                                            ctypes.c_int64, ctypes.POINTER(Opts),
                                            ctypes.POINTER(ctypes.c_int)]
        L.orc_tci_free.argtypes = [ctypes.c_void_p]
        L.orc_register_fn.argtypes = [BATCH_FN, ctypes.c_void_p]
        L.orc_register_fn.restype = ctypes.c_int
        L.orc_tci_optimize.argtypes = [ctypes.c_void_p, ctypes.POINTER(Opts)]
        L.orc_tci_updatepivots.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_int64]
        L.orc_tci_sweep2site.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_tci_sweep1site.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_int64, ctypes.c_int]
        L.orc_tci_fillsitetensors.argtypes = [ctypes.c_void_p]
        L.orc_tci_addglobalpivots.argtypes = [ctypes.c_void_p, I64P, ctypes.c_int64]
        L.orc_tci_addglobalpivots1sitesweep.argtypes = [ctypes.c_void_p, I64P, ctypes.c_int64,
                                                        ctypes.c_double, ctypes.c_double,
                                                        ctypes.c_int64]
        L.orc_tci_L.argtypes = [ctypes.c_void_p]
        L.orc_tci_maxsample.argtypes = [ctypes.c_void_p]
        L.orc_tci_maxsample.restype = ctypes.c_double
        L.orc_tci_nfeval.argtypes = [ctypes.c_void_p]
        L.orc_tci_nfeval.restype = ctypes.c_int64
        L.orc_tci_linkdims.argtypes = [ctypes.c_void_p, I64P]
        L.orc_tci_sets.argtypes = [ctypes.c_void_p, ctypes.c_int, I64P, I64P, I64P, I64P]
        L.orc_tci_core.argtypes = [ctypes.c_void_p, ctypes.c_int, F64P, I64P]
        L.orc_tci_errors.argtypes = [ctypes.c_void_p, F64P, I64P, F64P]
        L.orc_tci_history.argtypes = [ctypes.c_void_p, I64P, F64P, I64P, I64P]
        L.orc_tci_evaluate.argtypes = [ctypes.c_void_p, I64P, ctypes.c_int64, F64P]
        L.orc_tci_sum.argtypes = [ctypes.c_void_p]
        L.orc_tci_sum.restype = ctypes.c_double
        L.orc_tt_evaluate.argtypes = [ctypes.c_int, I64P, I64P, F64P, I64P, ctypes.c_int64, F64P]
        L.orc_tt_sum.argtypes = [ctypes.c_int, I64P, I64P, F64P]
        L.orc_tt_sum.restype = ctypes.c_double
        L.orc_convergencecriterion.argtypes = [I64P, F64P, I64P, ctypes.c_int64, ctypes.c_double,
                                               ctypes.c_int64, ctypes.c_int64, ctypes.c_int]
        L.orc_solve_batch.argtypes = [ctypes.c_int64, I32P, I64P, I64P, I32P, F64P, I64P, I64P, F64P,
                                      I64P, ctypes.POINTER(Opts), I64P, F64P, ctypes.c_int]
        L.orc_tt4_contract.restype = ctypes.c_void_p
        L.orc_tt4_contract.argtypes = [ctypes.c_int, I64P, F64P, I64P, F64P, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_double, ctypes.c_int64, ctypes.POINTER(ctypes.c_int)]
        L.orc_tt4_compress.restype = ctypes.c_void_p
        L.orc_tt4_compress.argtypes = [ctypes.c_int, I64P, F64P, ctypes.c_int, ctypes.c_double, ctypes.c_int64,
                                       ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        L.orc_tt4_contract_tci.restype = ctypes.c_void_p
        L.orc_tt4_contract_tci.argtypes = [ctypes.c_int, I64P, F64P, I64P, F64P, I64P, ctypes.c_int64, ctypes.c_int,
                                           VALUE_FN, ctypes.c_void_p, ctypes.POINTER(Opts),
                                           ctypes.POINTER(ctypes.c_int)]
        L.orc_optfirstpivot.argtypes = [ctypes.c_int, F64P, ctypes.c_int64, ctypes.c_int, I64P, I64P, ctypes.c_int]
        L.orc_estimatetrueerror.argtypes = [ctypes.c_int, F64P, ctypes.c_int64, ctypes.c_int, I64P, I64P, F64P, I64P,
                                            ctypes.c_int64, I64P, F64P, ctypes.POINTER(ctypes.c_int64)]
        L.orc_tt4_length.argtypes = [ctypes.c_void_p]
        L.orc_tt4_dims.argtypes = [ctypes.c_void_p, I64P]
        L.orc_tt4_core.argtypes = [ctypes.c_void_p, ctypes.c_int, F64P]
        L.orc_tt4_free.argtypes = [ctypes.c_void_p]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"oracle error {code}: {msg}")
        self.code = code


def _check(rc):
    if rc:
        raise OracleError(rc, lib().orc_last_error().decode())


def rrlu(A, maxrank=None, reltol=1e-14, abstol=0.0, leftorthogonal=True):
    """rrlu (matrixlu.jl:217-225).  Returns dict with 0-based permutations."""
    A = np.asfortranarray(A, dtype=np.float64)
    m, n = A.shape
    k = min(m, n)
    rp = np.zeros(m, np.int64)
    cp = np.zeros(n, np.int64)
    Lb = np.zeros(max(m * k, 1))
    Ub = np.zeros(max(k * n, 1))
    npiv = ctypes.c_int64()
    err = ctypes.c_double()
    flat = np.ascontiguousarray(A.reshape(-1, order="F"))
    rc = lib().orc_rrlu(_p(flat, F64P), m, n, 0 if maxrank is None else int(maxrank), reltol, abstol,
                        int(leftorthogonal), _p(rp, I64P), _p(cp, I64P), _p(Lb, F64P), _p(Ub, F64P),
                        ctypes.byref(npiv), ctypes.byref(err))
    K = npiv.value
    res = dict(rowpermutation=rp, colpermutation=cp, npivot=K, error=err.value,
               L=Lb[: m * K].reshape((m, K), order="F").copy(),
               U=Ub[: K * n].reshape((K, n), order="F").copy(), leftorthogonal=leftorthogonal, rc=rc)
    _check(rc)
    return res


def rrlu_batched(mats, maxrank=None, reltol=1e-14, abstol=0.0, leftorthogonal=True, nthreads=None):
    """Many rrLUs on host threads -> list of (rows, cols, npivot, error), 0-based."""
    import os
    ms = np.array([a.shape[0] for a in mats], np.int64)
    ns = np.array([a.shape[1] for a in mats], np.int64)
    offs = np.concatenate([[0], np.cumsum(ms * ns)[:-1]]).astype(np.int64)
    flat = np.ascontiguousarray(np.concatenate([np.asarray(a, np.float64).reshape(-1, order="F") for a in mats]))
    kcap = np.minimum(ms, ns)
    poffs = np.concatenate([[0], np.cumsum(2 * kcap)[:-1]]).astype(np.int64)
    piv = np.zeros(int(2 * kcap.sum()) + 1, np.int64)
    npiv = np.zeros(len(mats), np.int64)
    errs = np.zeros(len(mats))
    _check(lib().orc_rrlu_batched(len(mats), _p(flat, F64P), _p(offs, I64P), _p(ms, I64P), _p(ns, I64P),
                                  0 if maxrank is None else int(maxrank), reltol, abstol, int(leftorthogonal),
                                  _p(piv, I64P), _p(poffs, I64P), _p(npiv, I64P), _p(errs, F64P),
                                  int(nthreads or os.cpu_count() or 1)))
    out = []
    for i in range(len(mats)):
        K = int(npiv[i])
        o = poffs[i]
        out.append((piv[o:o + 2 * K:2].copy(), piv[o + 1:o + 2 * K:2].copy(), K, float(errs[i])))
    return out


def luci(A, maxrank=None, reltol=1e-14, abstol=0.0, leftorthogonal=True):
    """MatrixLUCI left/right (matrixluci.jl:70-84)."""
    A = np.asfortranarray(A, dtype=np.float64)
    m, n = A.shape
    k = min(m, n)
    left = np.zeros(max(m * k, 1))
    right = np.zeros(max(k * n, 1))
    npiv = ctypes.c_int64()
    flat = np.ascontiguousarray(A.reshape(-1, order="F"))
    _check(lib().orc_luci(_p(flat, F64P), m, n, 0 if maxrank is None else int(maxrank), reltol, abstol,
                          int(leftorthogonal), _p(left, F64P), _p(right, F64P), ctypes.byref(npiv)))
    K = npiv.value
    return (left[: m * K].reshape((m, K), order="F"), right[: K * n].reshape((K, n), order="F"))


def pivoterrors(res):
    """pivoterrors(lu) (matrixlu.jl:409-411)."""
    K = res["npivot"]
    if res["leftorthogonal"]:
        d = np.abs(np.diag(res["U"][:K, :K]))
    else:
        d = np.abs(np.diag(res["L"][:K, :K]))
    return np.concatenate([d, [res["error"]]])


def left(res):
    """left(lu; permute=true) (matrixlu.jl:374-382)."""
    out = np.empty_like(res["L"])
    out[res["rowpermutation"], :] = res["L"]
    return out


def right(res):
    """right(lu; permute=true) (matrixlu.jl:384-392)."""
    out = np.empty_like(res["U"])
    out[:, res["colpermutation"]] = res["U"]
    return out


# orc_batch_fn: (user, L, npoints, points[npoints x L], values[npoints]) -> status
BATCH_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, I64P, F64P)
_registered = []


def register_fn(f):
    """Register a caller-supplied f (the BatchEvaluator plugin point): f gets an
    (npoints, L) int64 array of 1-based multi-indices and returns npoints values.
    Returns the oracle's function id."""

    def _call(user, L, n, pts, vals):
        try:
            a = np.ctypeslib.as_array(pts, shape=(n, L)).copy()
            np.ctypeslib.as_array(vals, shape=(n,))[:] = np.asarray(f(a), dtype=np.float64).reshape(-1)
            return 0
        except BaseException:
            return 1

    cb = BATCH_FN(_call)
    _registered.append(cb)
    return lib().orc_register_fn(cb, None)


def feval(fid, params, points):
    pts = np.ascontiguousarray(points, dtype=np.int64)
    prm = np.ascontiguousarray(params if params is not None else [], dtype=np.float64)
    out = np.zeros(pts.shape[0])
    lib().orc_feval(int(fid), _p(prm, F64P) if prm.size else None, prm.size, pts.shape[1], _p(pts, I64P),
                    pts.shape[0], _p(out, F64P))
    return out


class OracleTCI:
    """TensorCI2 state held by the oracle (tensorci2.jl:6-40)."""

    def __init__(self, handle, L):
        self.h = ctypes.c_void_p(handle)
        self.L = L

    def __del__(self):
        try:
            lib().orc_tci_free(self.h)
        except Exception:
            pass

    @classmethod
    def new(cls, localdims, fid, params=(), initialpivots=None):
        L = len(localdims)
        d = np.ascontiguousarray(localdims, dtype=np.int64)
        prm = np.ascontiguousarray(params, dtype=np.float64)
        piv = np.ascontiguousarray(initialpivots if initialpivots is not None else [np.ones(L)],
                                   dtype=np.int64)
        rc = ctypes.c_int()
        h = lib().orc_tci_new(L, _p(d, I64P), int(fid), _p(prm, F64P) if prm.size else None, prm.size,
                              _p(piv, I64P), piv.shape[0], ctypes.byref(rc))
        obj = cls(h, L)
        _check(rc.value)
        return obj

    def optimize(self, **kw):
        o = make_opts(**kw)
        _check(lib().orc_tci_optimize(self.h, ctypes.byref(o)))

    def updatepivots(self, b, leftorthogonal=True, reltol=1e-14, abstol=0.0, maxbonddim=None):
        _check(lib().orc_tci_updatepivots(self.h, b, int(leftorthogonal), reltol, abstol,
                                          0 if maxbonddim is None else int(maxbonddim)))

    def sweep2site(self, niter=2, iter1=1, abstol=1e-8, maxbonddim=None, sweepstrategy="backandforth",
                   strictlynested=False, fillsitetensors=True):
        _check(lib().orc_tci_sweep2site(self.h, niter, iter1, abstol, 0 if maxbonddim is None else maxbonddim,
                                        SWEEP[sweepstrategy], int(strictlynested), int(fillsitetensors)))

    def sweep1site(self, forward=True, reltol=1e-14, abstol=0.0, maxbonddim=None, updatetensors=True):
        _check(lib().orc_tci_sweep1site(self.h, int(forward), reltol, abstol,
                                        0 if maxbonddim is None else maxbonddim, int(updatetensors)))

    def fillsitetensors(self):
        _check(lib().orc_tci_fillsitetensors(self.h))

    def addglobalpivots(self, pivots):
        piv = np.ascontiguousarray(pivots, dtype=np.int64).reshape(-1, self.L)
        _check(lib().orc_tci_addglobalpivots(self.h, _p(piv, I64P), piv.shape[0]))

    def addglobalpivots1sitesweep(self, pivots, reltol=1e-14, abstol=0.0, maxbonddim=None):
        piv = np.ascontiguousarray(pivots, dtype=np.int64).reshape(-1, self.L)
        _check(lib().orc_tci_addglobalpivots1sitesweep(self.h, _p(piv, I64P), piv.shape[0], reltol, abstol,
                                                       0 if maxbonddim is None else maxbonddim))

    def addglobalpivots2sitesweep(self, f, pivots, tolerance=1e-8, normalizeerror=True, maxbonddim=None,
                                  ntry=10, strictlynested=False):
        """addglobalpivots2sitesweep! (tensorci2.jl:243-288), f = (fid, params):
        add the pivots, run two 2-site sweeps at abstol = tolerance (times
        maxsamplevalue when normalizeerror), then keep the requested pivots whose
        |tt - f| is still above abstol and try again with those, at most ntry
        times; returns how many remain."""
        rows = [np.asarray(p, dtype=np.int64).ravel() for p in pivots]
        if any(r.size != self.L for r in rows):  # tensorci2.jl:255-257
            raise OracleError(2, "Please specify a pivot as one index per leg of the MPS.")
        piv = np.ascontiguousarray(np.array(rows, dtype=np.int64).reshape(-1, self.L))
        fvals = feval(f[0], f[1], piv) if piv.shape[0] else np.zeros(0)
        cur = piv
        for _ in range(ntry):
            abstol = tolerance * (self.maxsamplevalue if normalizeerror else 1.0)
            self.addglobalpivots(cur)
            self.sweep2site(2, abstol=abstol, maxbonddim=maxbonddim, strictlynested=strictlynested)
            new = piv[np.abs(self.evaluate(piv) - fvals) > abstol] if piv.shape[0] else piv
            if new.shape[0] == 0 or {tuple(p) for p in new} == {tuple(p) for p in cur}:
                return int(new.shape[0])
            cur = new
        return int(cur.shape[0])

    @property
    def maxsamplevalue(self):
        return lib().orc_tci_maxsample(self.h)

    @property
    def nfeval(self):
        return lib().orc_tci_nfeval(self.h)

    def linkdims(self):
        out = np.zeros(self.L - 1, np.int64)
        lib().orc_tci_linkdims(self.h, _p(out, I64P))
        return out

    def rank(self):
        return int(self.linkdims().max())

    def sets(self, b):
        """(Iset[b], Jset[b]) for 1-based site b, as int arrays of 1-based indices."""
        nI, nJ = ctypes.c_int64(), ctypes.c_int64()
        lib().orc_tci_sets(self.h, b, None, ctypes.byref(nI), None, ctypes.byref(nJ))
        I = np.zeros((nI.value, b - 1), np.int64)
        J = np.zeros((nJ.value, self.L - b), np.int64)
        lib().orc_tci_sets(self.h, b, _p(I, I64P), ctypes.byref(nI), _p(J, I64P), ctypes.byref(nJ))
        return I, J

    def core(self, b):
        dims = np.zeros(3, np.int64)
        lib().orc_tci_core(self.h, b, None, _p(dims, I64P))
        out = np.zeros(int(np.prod(dims)))
        lib().orc_tci_core(self.h, b, _p(out, F64P) if out.size else None, _p(dims, I64P))
        return out.reshape(tuple(dims), order="F")

    def cores(self):
        return [self.core(b) for b in range(1, self.L + 1)]

    def errors(self):
        n = ctypes.c_int64()
        lib().orc_tci_errors(self.h, None, ctypes.byref(n), None)
        pe = np.zeros(n.value)
        be = np.zeros(self.L - 1)
        lib().orc_tci_errors(self.h, _p(pe, F64P) if pe.size else None, ctypes.byref(n), _p(be, F64P))
        return pe, be

    def history(self):
        n = ctypes.c_int64()
        lib().orc_tci_history(self.h, None, None, None, ctypes.byref(n))
        r = np.zeros(n.value, np.int64)
        e = np.zeros(n.value)
        g = np.zeros(n.value, np.int64)
        if n.value:
            lib().orc_tci_history(self.h, _p(r, I64P), _p(e, F64P), _p(g, I64P), ctypes.byref(n))
        return r, e, g

    def evaluate(self, points):
        pts = np.ascontiguousarray(points, dtype=np.int64).reshape(-1, self.L)
        out = np.zeros(pts.shape[0])
        lib().orc_tci_evaluate(self.h, _p(pts, I64P), pts.shape[0], _p(out, F64P))
        return out

    def sum(self):
        return lib().orc_tci_sum(self.h)


def crossinterpolate2(localdims, fid, params=(), initialpivots=None, **kw):
    """crossinterpolate2 (tensorci2.jl:943-953) -> (OracleTCI, ranks, errors)."""
    L = len(localdims)
    d = np.ascontiguousarray(localdims, dtype=np.int64)
    prm = np.ascontiguousarray(params, dtype=np.float64)
    piv = np.ascontiguousarray(initialpivots if initialpivots is not None else [np.ones(L)], dtype=np.int64)
    o = make_opts(**kw)
    rc = ctypes.c_int()
    h = lib().orc_crossinterpolate2(L, _p(d, I64P), int(fid), _p(prm, F64P) if prm.size else None,
                                    prm.size, _p(piv, I64P), piv.shape[0], ctypes.byref(o),
                                    ctypes.byref(rc))
    t = OracleTCI(h, L)
    _check(rc.value)
    r, e, _ = t.history()
    return t, r, e


def convergencecriterion(ranks, errors, nglobalpivots, tolerance, maxbonddim, ncheckhistory,
                         checkconvglobalpivot=True):
    r = np.ascontiguousarray(ranks, np.int64)
    e = np.ascontiguousarray(errors, np.float64)
    g = np.ascontiguousarray(nglobalpivots, np.int64)
    return bool(lib().orc_convergencecriterion(_p(r, I64P), _p(e, F64P), _p(g, I64P), r.size, tolerance,
                                               maxbonddim, ncheckhistory, int(checkconvglobalpivot)))


def tt_evaluate(cores, points):
    L = len(cores)
    link = np.array([c.shape[0] for c in cores] + [cores[-1].shape[2]], np.int64)
    d = np.array([c.shape[1] for c in cores], np.int64)
    flat = np.ascontiguousarray(np.concatenate([c.reshape(-1, order="F") for c in cores]))
    pts = np.ascontiguousarray(points, np.int64).reshape(-1, L)
    out = np.zeros(pts.shape[0])
    lib().orc_tt_evaluate(L, _p(link, I64P), _p(d, I64P), _p(flat, F64P), _p(pts, I64P), pts.shape[0],
                          _p(out, F64P))
    return out


def tt_sum(cores):
    L = len(cores)
    link = np.array([c.shape[0] for c in cores] + [cores[-1].shape[2]], np.int64)
    d = np.array([c.shape[1] for c in cores], np.int64)
    flat = np.ascontiguousarray(np.concatenate([c.reshape(-1, order="F") for c in cores]))
    return lib().orc_tt_sum(L, _p(link, I64P), _p(d, I64P), _p(flat, F64P))


def dense_params(table):
    """Parameter block of the DENSE function for a column-major table."""
    table = np.asarray(table, dtype=np.float64)
    dims = table.shape
    strides = np.cumprod((1,) + dims[:-1])
    return np.concatenate([[len(dims)], strides.astype(np.float64), table.reshape(-1, order="F")])


def _tt4_pack(cores):
    cores = [np.asarray(c, dtype=np.float64) for c in cores]
    dims = np.ascontiguousarray([list(c.shape) for c in cores], dtype=np.int64).reshape(-1)
    vals = np.ascontiguousarray(np.concatenate([c.reshape(-1, order="F") for c in cores]))
    return dims, vals


def _tt4_unpack(h, rc):
    L = lib()
    try:
        if rc.value:
            raise OracleError(rc.value, L.orc_last_error().decode())
        n = L.orc_tt4_length(h)
        dims = np.zeros(4 * n, np.int64)
        L.orc_tt4_dims(h, _p(dims, I64P))
        out = []
        for b in range(n):
            shape = tuple(int(x) for x in dims[4 * b:4 * b + 4])
            buf = np.zeros(int(np.prod(shape)), np.float64)
            L.orc_tt4_core(h, b, _p(buf, F64P))
            out.append(buf.reshape(shape, order="F"))
        return out
    finally:
        L.orc_tt4_free(h)


METHODS = {"LU": 0, "CI": 1}


def tt4_contract(a, b, algorithm="zipup", tolerance=1e-12, maxbonddim=None, method="LU"):
    """contract_naive / contract_zipup(:LU or :CI) (contraction.jl:351-372, 442-486)
    of two trains of 4-leg cores; returns the list of cores."""
    ad, av = _tt4_pack(a)
    bd, bv = _tt4_pack(b)
    rc = ctypes.c_int()
    h = lib().orc_tt4_contract(len(a), _p(ad, I64P), _p(av, F64P), _p(bd, I64P), _p(bv, F64P),
                               1 if algorithm == "naive" else 2, METHODS[method], float(tolerance),
                               int(maxbonddim or 0), ctypes.byref(rc))
    return _tt4_unpack(h, rc)


def tt4_compress(cores, method="LU", tolerance=1e-12, maxbonddim=None, normalizeerror=True):
    """compress!(tt, method) with :LU or :CI (tensortrain.jl:149-183); returns the
    list of cores."""
    d, v = _tt4_pack(cores)
    rc = ctypes.c_int()
    h = lib().orc_tt4_compress(len(cores), _p(d, I64P), _p(v, F64P), METHODS[method], float(tolerance),
                               int(maxbonddim or 0), int(bool(normalizeerror)), ctypes.byref(rc))
    return _tt4_unpack(h, rc)


VALUE_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, F64P)


def tt4_contract_tci(a, b, initialpivots=10, f=None, **kw):
    """contract(a, b; algorithm=:TCI, f, initialpivots, kwargs...) (contraction.jl:399-434);
    returns the list of cores (legs split)."""
    ad, av = _tt4_pack(a)
    bd, bv = _tt4_pack(b)
    L = len(a)
    if isinstance(initialpivots, (int, np.integer)):
        piv, ninit = np.zeros((0, L), np.int64), int(initialpivots)
    else:
        piv, ninit = np.ascontiguousarray(initialpivots, dtype=np.int64).reshape(-1, L), 0
    cb = None
    if f is not None:
        def _call(user, n, vals):
            v = np.ctypeslib.as_array(vals, shape=(n,))
            v[:] = np.asarray(f(v.copy()), dtype=np.float64).reshape(-1)
            return 0
        cb = VALUE_FN(_call)
        _registered.append(cb)
    o = make_opts(**kw)
    rc = ctypes.c_int()
    h = lib().orc_tt4_contract_tci(L, _p(ad, I64P), _p(av, F64P), _p(bd, I64P), _p(bv, F64P),
                                   _p(piv, I64P) if piv.size else None, piv.shape[0], ninit,
                                   cb if cb is not None else VALUE_FN(), None,
                                   ctypes.byref(o), ctypes.byref(rc))
    return _tt4_unpack(h, rc)


def optfirstpivot(fid, params, localdims, firstpivot=None, maxsweep=1000):
    """optfirstpivot (util.jl:78-108) -> the improved pivot (1-based)."""
    L = len(localdims)
    d = np.ascontiguousarray(localdims, dtype=np.int64)
    p = np.ascontiguousarray(firstpivot if firstpivot is not None else np.ones(L), dtype=np.int64)
    prm = np.ascontiguousarray(params if params is not None else [], dtype=np.float64)
    lib().orc_optfirstpivot(int(fid), _p(prm, F64P) if prm.size else None, prm.size, L, _p(d, I64P), _p(p, I64P),
                            int(maxsweep))
    return p


def estimatetrueerror(fid, params, cores, starts):
    """estimatetrueerror(tt, f; initialpoints) (globalsearch.jl:19-96) for a train of
    3-leg cores -> list of (pivot, error), error descending."""
    L = len(cores)
    links = np.ascontiguousarray([c.shape[0] for c in cores] + [1], dtype=np.int64)
    dims = np.ascontiguousarray([c.shape[1] for c in cores], dtype=np.int64)
    vals = np.ascontiguousarray(np.concatenate([np.asarray(c, np.float64).reshape(-1, order="F") for c in cores]))
    st = np.ascontiguousarray(starts, dtype=np.int64).reshape(-1, L)
    prm = np.ascontiguousarray(params if params is not None else [], dtype=np.float64)
    piv = np.zeros((st.shape[0], L), np.int64)
    err = np.zeros(st.shape[0])
    n = ctypes.c_int64()
    lib().orc_estimatetrueerror(int(fid), _p(prm, F64P) if prm.size else None, prm.size, L, _p(links, I64P),
                                _p(dims, I64P), _p(vals, F64P), _p(st, I64P), st.shape[0], _p(piv, I64P),
                                _p(err, F64P), ctypes.byref(n))
    return [(piv[k], float(err[k])) for k in range(n.value)]


def tt4_full(cores):
    """The operator of a train of 4-leg cores as a dense (prod s_in) x (prod s_out)
    matrix, first site fastest (the reference tests' _tomat)."""
    t = np.ones((1, 1, 1))  # (rows, cols, bond)
    for c in cores:
        r0, s1, s2, r1 = c.shape
        x = np.einsum("abr,rstq->asbtq", t, c)  # (rows, s1, cols, s2, r1)
        t = x.reshape(t.shape[0] * s1, t.shape[1] * s2, r1, order="F")
    return t[:, :, 0]
