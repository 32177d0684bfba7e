"""GB300-native TCI2 two-site sweep, with the reference's Python-facing API.

Mirrors TensorCrossInterpolation.jl's interface for this path:
``crossinterpolate2``, ``TensorCI2`` (``updatepivots!``, ``sweep2site!``,
``sweep1site!``, ``optimize!``, ``addglobalpivots!``, ...), ``TensorTrain``
(``evaluate``, ``sum``) and ``rrlu`` / ``rrLU``.  Everything that computes runs
in libtci_gpu.so (CUDA kernels for sm_103a behind a C ABI, include/tci_gb300.h).
There is no CPU fallback: without the library or a GPU every call raises.

Indices are 1-based, as in Julia.  Matrices are numpy arrays; site tensors are
returned as (r_{b-1}, d_b, r_b) arrays.
"""
import ctypes
import threading
import weakref
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtci_gpu.so")

I64P = ctypes.POINTER(ctypes.c_int64)
F64P = ctypes.POINTER(ctypes.c_double)
# tci_batch_fn: (user, L, npoints, points[npoints x L], values[npoints]) -> status
BATCH_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, I64P, F64P)
# tci_value_fn: (user, n, values[n]) -> status, values mapped in place
VALUE_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, F64P)

TCI_OK, TCI_ERR_ARG, TCI_ERR_DIM, TCI_ERR_NAN, TCI_ERR_SINGULAR, TCI_ERR_GENERIC = 0, 1, 2, 3, 4, 5
TCI_ERR_CUDA, TCI_ERR_OOM, TCI_ERR_TIMEOUT, TCI_ERR_TOO_LARGE = 6, 7, 8, 9
TCI_CONTRACT_NAIVE, TCI_CONTRACT_ZIPUP = 1, 2
# precision of contractions and matrix products: FP64, or TF32 hi/lo split products on the tensor cores
PRECISION = {"fp64": 0, "tf32x3": 1}
FACTORIZE = {"LU": 0, "CI": 1}  # _factorize methods on the device (tensortrain.jl:94-137)
SWEEP = {"backandforth": 0, "forward": 1, "backward": 2}
FUNCTIONS = {"lorentz": 1, "served": 2, "qtt1d": 3, "qtt2d": 4, "dense": 5, "product": 6}


class TCIError(RuntimeError):
    """A failure reported by the library (code + the reference's message)."""

    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


class ArgumentError(TCIError, ValueError):
    pass


class DimensionMismatch(TCIError, ValueError):
    pass


_EXC = {TCI_ERR_ARG: ArgumentError, TCI_ERR_DIM: DimensionMismatch}


class Opts(ctypes.Structure):
    """tci_opts: keyword arguments of optimize! (tensorci2.jl:700-720)."""
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


class Request(ctypes.Structure):
    _fields_ = [
        ("L", ctypes.c_int32),
        ("fid", ctypes.c_int32),
        ("localdims", I64P),
        ("fparams", F64P),
        ("nparams", ctypes.c_int64),
        ("opts", Opts),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("steps", ctypes.c_int64),
        ("launches", ctypes.c_int64),
        ("tasks", ctypes.c_int64),
        ("kernel_ms", ctypes.c_double),
        ("feval", ctypes.c_int64),
        ("lu_updates", ctypes.c_int64),
        ("h2d_bytes", ctypes.c_int64),
        ("d2h_bytes", ctypes.c_int64),
        ("host_launch_ms", ctypes.c_double),
        ("host_wait_ms", ctypes.c_double),
        ("host_resume_ms", ctypes.c_double),
        ("task_cycles", ctypes.c_int64),
        ("feval_tabulated", ctypes.c_int64),
        ("tc_ms", ctypes.c_double),
        ("tc_flops", ctypes.c_double),
        ("peak_live", ctypes.c_int64),
        ("dense_macs", ctypes.c_int64),
    ]


# Every exported symbol of include/tci_gb300.h with its ctypes signature.
_SIGNATURES = {
    "tci_opts_default": (None, [ctypes.POINTER(Opts)]),
    "tci_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_size_t, ctypes.POINTER(ctypes.c_void_p)]),
    "tci_ctx_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "tci_last_error": (ctypes.c_char_p, []),
    "tci_f_lookup": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]),
    "tci_f_register": (ctypes.c_int, [BATCH_FN, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]),
    "tci_f_unregister": (ctypes.c_int, [ctypes.c_int32]),
    "tci_fcache_stats": (ctypes.c_int, [ctypes.c_void_p, I64P, I64P, I64P]),
    "tci_solve_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, I64P, ctypes.c_int32, F64P,
                                        ctypes.c_int64, I64P, ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)]),
    "tci_solve_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "tci_crossinterpolate2": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, I64P, ctypes.c_int32, F64P,
                                             ctypes.c_int64, I64P, ctypes.c_int64, ctypes.POINTER(Opts),
                                             ctypes.POINTER(ctypes.c_void_p)]),
    "tci_optimize": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Opts)]),
    "tci_updatepivots": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_int64]),
    "tci_sweep2site": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                      ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "tci_sweep1site": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_int64, ctypes.c_int32]),
    "tci_fillsitetensors": (ctypes.c_int, [ctypes.c_void_p]),
    "tci_addglobalpivots": (ctypes.c_int, [ctypes.c_void_p, I64P, ctypes.c_int64]),
    "tci_addglobalpivots1sitesweep": (ctypes.c_int, [ctypes.c_void_p, I64P, ctypes.c_int64, ctypes.c_double,
                                                     ctypes.c_double, ctypes.c_int64]),
    "tci_solve_length": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32)]),
    "tci_linkdims": (ctypes.c_int, [ctypes.c_void_p, I64P]),
    "tci_maxsamplevalue": (ctypes.c_double, [ctypes.c_void_p]),
    "tci_get_sets": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, I64P, I64P, I64P, I64P]),
    "tci_get_core": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, F64P, I64P]),
    "tci_get_errors": (ctypes.c_int, [ctypes.c_void_p, F64P, I64P, F64P]),
    "tci_get_history": (ctypes.c_int, [ctypes.c_void_p, I64P, F64P, I64P, I64P]),
    "tci_solve_nfeval": (ctypes.c_int64, [ctypes.c_void_p]),
    "tci_evaluate": (ctypes.c_int, [ctypes.c_void_p, I64P, ctypes.c_int64, F64P]),
    "tci_evaluate_prec": (ctypes.c_int, [ctypes.c_void_p, I64P, ctypes.c_int64, F64P, ctypes.c_int32, F64P]),
    "tci_sum": (ctypes.c_int, [ctypes.c_void_p, F64P]),
    "tci_crossinterpolate2_batched": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(Request),
                                                     ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)]),
    "tci_serve_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(Request), F64P,
                                     ctypes.c_int64, F64P, I64P, F64P]),
    "tci_rrlu": (ctypes.c_int, [ctypes.c_void_p, F64P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                ctypes.c_double, ctypes.c_double, ctypes.c_int32, I64P, I64P, F64P, F64P, I64P,
                                F64P]),
    "tci_rrlu_batched": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, F64P, I64P, I64P, I64P, ctypes.c_int64,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_int32, I64P, I64P, I64P,
                                        F64P]),
    "tci_ctx_stream": (ctypes.c_size_t, [ctypes.c_void_p]),
    "tci_ctx_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "tci_ctx_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Stats), ctypes.c_int32]),
    "tci_feval": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, F64P, ctypes.c_int64, ctypes.c_int32, I64P, I64P,
                                 ctypes.c_int64, F64P]),
    "tci_convergencecriterion": (ctypes.c_int, [I64P, F64P, I64P, ctypes.c_int64, ctypes.c_double,
                                                ctypes.c_int64, ctypes.c_int64, ctypes.c_int32]),
    "tci_fp64_peak": (ctypes.c_int, [ctypes.c_size_t, F64P, F64P]),
    "tci_tt4_contract": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, I64P, ctypes.c_void_p, I64P,
                                        ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                        ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)]),
    "tci_tt4_contract_prec": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, I64P, ctypes.c_void_p, I64P,
                                             ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                             ctypes.c_int64, ctypes.c_int32, F64P, ctypes.POINTER(ctypes.c_void_p)]),
    "tci_matmul": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, F64P, F64P, F64P,
                                  ctypes.c_int32, F64P]),
    "tci_tt4_compress": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, I64P, ctypes.c_void_p, ctypes.c_int32,
                                        ctypes.c_double, ctypes.c_int64, ctypes.c_int32,
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "tci_tt4_contract_tci": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, I64P, ctypes.c_void_p, I64P,
                                            ctypes.c_void_p, I64P, ctypes.c_int64, ctypes.c_int32, VALUE_FN,
                                            ctypes.c_void_p, ctypes.POINTER(Opts), ctypes.POINTER(ctypes.c_void_p)]),
    "tci_optfirstpivot": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, F64P, ctypes.c_int64, ctypes.c_int32,
                                         I64P, I64P, ctypes.c_int32]),
    "tci_estimatetrueerror": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, I64P, ctypes.c_int64, ctypes.c_uint64,
                                             ctypes.c_int64, I64P, F64P, ctypes.POINTER(ctypes.c_int64)]),
    "tci_tt4_length": (ctypes.c_int32, [ctypes.c_void_p]),
    "tci_tt4_dims": (ctypes.c_int, [ctypes.c_void_p, I64P]),
    "tci_tt4_get_core": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, F64P]),
    "tci_tt4_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "tci_get_core_dims_batched": (ctypes.c_int, [ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p), I64P]),
    "tci_get_cores_pinned": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p),
                                            ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_int64)]),
    "tci_host_free": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "tci_serve_start": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)]),
    "tci_serve_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64)]),
    "tci_serve_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, I64P, ctypes.POINTER(ctypes.c_int32), I64P,
                                      F64P, ctypes.POINTER(ctypes.c_int64), ctypes.c_int32]),
    "tci_serve_stop": (ctypes.c_int, [ctypes.c_void_p]),
    "tci_set_sets": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, I64P, ctypes.c_int64, I64P, ctypes.c_int64]),
    "tci_bonderrors": (ctypes.c_int, [ctypes.c_void_p, F64P]),
    "tci_tt_evaluate": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, I64P, ctypes.c_void_p, I64P, ctypes.c_int64,
                                       F64P]),
    "tci_tt_sum": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, I64P, ctypes.c_void_p, F64P]),
    "tci_tt_evaluate_prec": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, I64P, ctypes.c_void_p, I64P,
                                            ctypes.c_int64, F64P, ctypes.c_int32, F64P]),
    "tci_get_cores_batched": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p), F64P,
                                             I64P]),
    "tci_ctx_set_resident_limits": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64]),
    "tci_autotune_rrlu": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, F64P, F64P, F64P]),
    "tci_autotune_table": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32),
                                          ctypes.POINTER(ctypes.c_int32), ctypes.c_int32]),
    "tci_rrlu_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_int32, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_size_t]),
}

_lib = None


def load_library(path=None):
    """Load libtci_gpu.so; raises OSError if it has not been built."""
    global _lib
    if _lib is None:
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise OSError(f"{p} not found: build it with tensorcrossinterpolation.jl_gb300/build.py")
        L = ctypes.CDLL(p)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGNATURES)


_cb_state = threading.local()  # the exception a BatchFunction's f raised on this thread


def _check(rc):
    if rc:
        msg = load_library().tci_last_error()
        msg = msg.decode() if msg else ""
        err = _EXC.get(rc, TCIError)(rc, msg or f"error code {rc}")
        pending = getattr(_cb_state, "error", None)
        _cb_state.error = None
        if pending is not None and rc == TCI_ERR_GENERIC:
            raise pending from err  # the caller's own exception, not the library's code
        raise err
    _cb_state.error = None


def _p(a, t):
    return a.ctypes.data_as(t)


class Context:
    """A device context: one CUDA stream, the batched step engine, its buffers."""

    def __init__(self, device=0, hbm_budget=0):
        lib = load_library()
        h = ctypes.c_void_p()
        _check(lib.tci_ctx_create(int(device), int(hbm_budget), ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            load_library().tci_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        return load_library().tci_ctx_stream(self.h)

    def synchronize(self):
        _check(load_library().tci_ctx_synchronize(self.h))

    def set_resident_limits(self, idle_us=20000, wait_us=60_000_000):
        """Bounds of the resident kernel's waits: it leaves after idle_us with
        nothing to do, and a worker waits at most wait_us for its task."""
        _check(load_library().tci_ctx_set_resident_limits(self.h, int(idle_us), int(wait_us)))

    def autotune_rrlu(self, reps=2):
        """Time the rrLU tail-size candidates per (rows, cols) bucket on seeded
        matrices and keep, for this context's later tasks, the fastest one where
        it beats the default by 2 % on the calibration set and on a fresh
        validation set.  Returns (speedup over the default, default ms, tuned ms)."""
        out = np.zeros(3)
        _check(load_library().tci_autotune_rrlu(self.h, int(reps), _p(out[0:], F64P), _p(out[1:], F64P),
                                                _p(out[2:], F64P)))
        return float(out[0]), float(out[1]), float(out[2])

    def tune_table(self, table=None):
        """The tuned tail sizes per bucket; with `table`, set them (0 = default)."""
        lib = load_library()
        nb = ctypes.c_int32()
        _check(lib.tci_autotune_table(self.h, None, ctypes.byref(nb), 0))
        if table is not None:
            arr = (ctypes.c_int32 * nb.value)(*[int(x) for x in table])
            _check(lib.tci_autotune_table(self.h, arr, ctypes.byref(nb), 1))
        arr = (ctypes.c_int32 * nb.value)()
        _check(lib.tci_autotune_table(self.h, arr, ctypes.byref(nb), 0))
        return list(arr)

    def stats(self, reset=False):
        s = Stats()
        load_library().tci_ctx_stats(self.h, ctypes.byref(s), int(bool(reset)))
        return {k: getattr(s, k) for k, _ in Stats._fields_}


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class DeviceFunction:
    """A registered device function f (the BatchEvaluator plugin point,
    cachedtensortrain.jl:1 / batcheval.jl:67-83), selected by name."""

    def __init__(self, name, params=()):
        if name not in FUNCTIONS:
            raise ArgumentError(TCI_ERR_ARG, f"unknown function {name}")
        self.name = name
        self.fid = FUNCTIONS[name]
        self.params = np.ascontiguousarray(params, dtype=np.float64)

    @staticmethod
    def dense(table):
        """f(v) = table[v] for a small dense tensor (column-major)."""
        table = np.asarray(table, dtype=np.float64)
        dims = table.shape
        strides = np.cumprod((1,) + dims[:-1])
        return DeviceFunction("dense", np.concatenate([[len(dims)], strides, table.reshape(-1, order="F")]))


class BatchFunction:
    """A caller-supplied f: the BatchEvaluator plugin point (cachedtensortrain.jl:1,
    batcheval.jl:67-83) for functions with no device implementation.

    ``f(points)`` gets an (npoints, L) int64 array of 1-based multi-indices and
    returns npoints float64 values; it must be a pure function of the
    multi-index.  Each solve keeps the values it has asked for in a device hash
    table (CachedFunction, cachedfunction.jl:8-184) and calls f only for points
    it has not seen, once per device step that needs new values.  An exception
    raised by f ends the library call and is re-raised to its caller (and kept
    in ``self.error``)."""

    def __init__(self, f):
        self.f = f
        self.ncalls = 0
        self.npoints = 0
        self.error = None
        self.params = np.zeros(0)
        self.name = "batch"

        def _call(user, L, n, pts, vals):
            try:
                a = np.ctypeslib.as_array(pts, shape=(n, L)).copy()
                v = np.ascontiguousarray(self.f(a), dtype=np.float64).reshape(-1)
                if v.size != n:
                    raise ValueError(f"f returned {v.size} values for {n} points")
                np.ctypeslib.as_array(vals, shape=(n,))[:] = v
                self.ncalls += 1
                self.npoints += n
                return 0
            except BaseException as e:  # reported through the library's error code
                self.error = e
                _cb_state.error = e
                return 1

        self._cb = BATCH_FN(_call)
        fid = ctypes.c_int32()
        _check(load_library().tci_f_register(self._cb, None, ctypes.byref(fid)))
        self.fid = fid.value

    def close(self):
        if self.fid:
            load_library().tci_f_unregister(self.fid)
            self.fid = 0

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_opts(tolerance=None, maxbonddim=None, maxiter=20, sweepstrategy="backandforth", normalizeerror=True,
              ncheckhistory=3, maxnglobalpivot=5, nsearchglobalpivot=5, tolmarginglobalsearch=10.0,
              strictlynested=False, checkconvglobalpivot=True, seed=0, pivottolerance=None, verbosity=0,
              loginterval=10, pivotsearch="full", globalpivotfinder=None):
    """Map the reference's optimize! keyword arguments to tci_opts."""
    if pivotsearch != "full":
        raise ArgumentError(TCI_ERR_ARG, "only pivotsearch=:full is implemented on the device")
    if globalpivotfinder is not None:
        raise ArgumentError(TCI_ERR_ARG, "custom global pivot finders are not supported on the device")
    if pivottolerance is not None:
        if tolerance is not None and tolerance != pivottolerance:
            raise ArgumentError(TCI_ERR_ARG, "Got different values for pivottolerance and tolerance in "
                                "optimize!(TCI2). For TCI2, both of these options have the same meaning. "
                                "Please assign only `tolerance`.")
        tolerance = pivottolerance
    o = Opts()
    o.tolerance = 1e-8 if tolerance is None else float(tolerance)
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


def _pivots_array(pivots, L):
    rows = [np.asarray(p, dtype=np.int64).ravel() for p in pivots] if len(pivots) else []
    if any(r.size != L for r in rows):
        # addglobalpivots! (tensorci2.jl:197-199)
        raise DimensionMismatch(TCI_ERR_DIM, "Please specify a pivot as one index per leg of the MPS.")
    return np.ascontiguousarray(np.array(rows, dtype=np.int64).reshape(-1, L))


class TensorCI2:
    """TensorCI2{Float64} (tensorci2.jl:6-40) held on the device."""

    def __init__(self, f, localdims, initialpivots=None, ctx=None, _handle=None):
        self.ctx = ctx or default_context()
        self.f = f
        self.localdims = [int(d) for d in localdims]
        L = len(self.localdims)
        if _handle is not None:
            self.h = _handle
            return
        lib = load_library()
        d = np.ascontiguousarray(self.localdims, dtype=np.int64)
        piv = _pivots_array(initialpivots if initialpivots is not None else [np.ones(L)], L)
        h = ctypes.c_void_p()
        _check(lib.tci_solve_create(self.ctx.h, L, _p(d, I64P), f.fid,
                                    _p(f.params, F64P) if f.params.size else None, f.params.size,
                                    _p(piv, I64P), piv.shape[0], ctypes.byref(h)))
        self.h = h

    @classmethod
    def _wrap(cls, f, localdims, ctx, handle):
        """A solve the library created (batched entry points)."""
        t = cls.__new__(cls)
        t.ctx, t.f, t.h = ctx, f, handle
        t.localdims = [int(d) for d in localdims]
        return t

    def __del__(self):
        try:
            if self.h:
                load_library().tci_solve_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def __len__(self):
        return len(self.localdims)

    # ---- algorithm steps
    def updatepivots(self, b, leftorthogonal=True, reltol=1e-14, abstol=0.0, maxbonddim=None):
        """updatepivots! (tensorci2.jl:510-607), b 1-based."""
        _check(load_library().tci_updatepivots(self.h, int(b), int(bool(leftorthogonal)), reltol, abstol,
                                               0 if maxbonddim is None else int(maxbonddim)))

    def sweep2site(self, niter=2, iter1=1, abstol=1e-8, maxbonddim=None, sweepstrategy="backandforth",
                   strictlynested=False, fillsitetensors=True):
        """sweep2site! (tensorci2.jl:855-916)."""
        _check(load_library().tci_sweep2site(self.h, niter, iter1, abstol,
                                             0 if maxbonddim is None else int(maxbonddim), SWEEP[sweepstrategy],
                                             int(strictlynested), int(fillsitetensors)))

    def sweep1site(self, sweepdirection="forward", reltol=1e-14, abstol=0.0, maxbonddim=None, updatetensors=True):
        """sweep1site! (tensorci2.jl:402-461)."""
        if sweepdirection not in ("forward", "backward"):
            raise ArgumentError(TCI_ERR_ARG, f"Unknown sweep direction {sweepdirection}: choose between "
                                ":forward, :backward.")
        _check(load_library().tci_sweep1site(self.h, int(sweepdirection == "forward"), reltol, abstol,
                                             0 if maxbonddim is None else int(maxbonddim), int(updatetensors)))

    def fillsitetensors(self):
        _check(load_library().tci_fillsitetensors(self.h))

    def optimize(self, **kw):
        """optimize! (tensorci2.jl:700-850) -> (ranks, errors)."""
        o = make_opts(**kw)
        _check(load_library().tci_optimize(self.h, ctypes.byref(o)))
        return self.history()[:2]

    def addglobalpivots(self, pivots):
        piv = _pivots_array(pivots, len(self))
        _check(load_library().tci_addglobalpivots(self.h, _p(piv, I64P), piv.shape[0]))

    def addglobalpivots1sitesweep(self, pivots, reltol=1e-14, abstol=0.0, maxbonddim=None):
        piv = _pivots_array(pivots, len(self))
        _check(load_library().tci_addglobalpivots1sitesweep(self.h, _p(piv, I64P), piv.shape[0], reltol, abstol,
                                                            0 if maxbonddim is None else int(maxbonddim)))

    def addglobalpivots2sitesweep(self, pivots, tolerance=1e-8, normalizeerror=True, maxbonddim=None,
                                  pivotsearch="full", verbosity=0, ntry=10, strictlynested=False):
        """addglobalpivots2sitesweep! (tensorci2.jl:243-288): add the pivots, run
        two 2-site sweeps at abstol = tolerance (times maxsamplevalue when
        normalizeerror), then keep the requested pivots whose |tt - f| is still
        above abstol and try again with those, at most ntry times, stopping early
        when the remaining set repeats.  Returns how many pivots remain."""
        if pivotsearch != "full":
            raise ArgumentError(TCI_ERR_ARG, "only pivotsearch=:full is implemented on the device")
        piv = _pivots_array(pivots, len(self))
        fvals = self._fvalues(piv)
        cur = piv
        for _ in range(ntry):
            abstol = tolerance * (self.maxsamplevalue if normalizeerror else 1.0)
            self.addglobalpivots(cur)
            self.sweep2site(2, abstol=abstol, maxbonddim=maxbonddim, strictlynested=strictlynested)
            new = piv[np.abs(self.evaluate(piv) - fvals) > abstol] if piv.shape[0] else piv
            if verbosity > 0:
                print(f"Trying to add {cur.shape[0]} global pivots, {new.shape[0]} still remain.")
            if new.shape[0] == 0 or {tuple(p) for p in new} == {tuple(p) for p in cur}:
                return int(new.shape[0])
            cur = new
        return int(cur.shape[0])

    def _fvalues(self, points):
        """f at points (n x L, 1-based): the device function, or the caller's f."""
        if points.shape[0] == 0:
            return np.zeros(0)
        if isinstance(self.f, BatchFunction):
            return np.ascontiguousarray(self.f.f(points.copy()), dtype=np.float64).reshape(-1)
        return feval(self.f, self.localdims, points, ctx=self.ctx)

    # ---- state
    def linkdims(self):
        out = np.zeros(len(self) - 1, np.int64)
        load_library().tci_linkdims(self.h, _p(out, I64P))
        return out

    def rank(self):
        return int(self.linkdims().max())

    @property
    def maxsamplevalue(self):
        return load_library().tci_maxsamplevalue(self.h)

    @property
    def nfeval(self):
        return load_library().tci_solve_nfeval(self.h)

    def sets(self, b):
        """(Iset[b], Jset[b]) for 1-based site b as int arrays of 1-based indices."""
        lib = load_library()
        nI, nJ = ctypes.c_int64(), ctypes.c_int64()
        _check(lib.tci_get_sets(self.h, b, None, ctypes.byref(nI), None, ctypes.byref(nJ)))
        I = np.zeros((nI.value, b - 1), np.int64)
        J = np.zeros((nJ.value, len(self) - b), np.int64)
        _check(lib.tci_get_sets(self.h, b, _p(I, I64P), ctypes.byref(nI), _p(J, I64P), ctypes.byref(nJ)))
        return I, J

    @property
    def Iset(self):
        return [self.sets(b)[0] for b in range(1, len(self) + 1)]

    @property
    def Jset(self):
        return [self.sets(b)[1] for b in range(1, len(self) + 1)]

    def sitetensor(self, b):
        lib = load_library()
        dims = np.zeros(3, np.int64)
        _check(lib.tci_get_core(self.h, b, None, _p(dims, I64P)))
        out = np.zeros(int(np.prod(dims)))
        _check(lib.tci_get_core(self.h, b, _p(out, F64P) if out.size else None, _p(dims, I64P)))
        return out.reshape(tuple(dims), order="F")

    @property
    def sitetensors(self):
        return [self.sitetensor(b) for b in range(1, len(self) + 1)]

    def set_sets(self, b, I, J):
        """Replace Iset[b] and Jset[b] (1-based multi-indices); invalidates the site tensors."""
        L = len(self)
        I = np.ascontiguousarray(np.asarray(I, dtype=np.int64).reshape(-1, b - 1) if b > 1
                                 else np.zeros((len(I), 0), np.int64))
        J = np.ascontiguousarray(np.asarray(J, dtype=np.int64).reshape(-1, L - b) if b < L
                                 else np.zeros((len(J), 0), np.int64))
        _check(load_library().tci_set_sets(self.h, b, _p(I, I64P), I.shape[0], _p(J, I64P), J.shape[0]))

    def errors(self):
        lib = load_library()
        n = ctypes.c_int64()
        lib.tci_get_errors(self.h, None, ctypes.byref(n), None)
        pe = np.zeros(n.value)
        be = np.zeros(len(self) - 1)
        lib.tci_get_errors(self.h, _p(pe, F64P) if pe.size else None, ctypes.byref(n), _p(be, F64P))
        return pe, be

    @property
    def pivoterrors(self):
        return self.errors()[0]

    @property
    def bonderrors(self):
        return self.errors()[1]

    def pivoterror(self):
        """pivoterror(tci) = maximum(bonderrors) (tensorci2.jl:157-159)."""
        return float(self.bonderrors.max())

    def estimatetrueerror(self, nsearch=100, initialpoints=None, seed=0):
        """estimatetrueerror(TensorTrain(tci), f; nsearch, initialpoints)
        (globalsearch.jl:1-96) -> [(pivot, error)], error descending.  Random
        starts come from `seed`."""
        L = len(self)
        if initialpoints is not None:
            st = _pivots_array(initialpoints, L)
        else:
            if nsearch <= 0:
                raise TCIError(TCI_ERR_GENERIC, "No search is performed")
            st = np.zeros((0, L), np.int64)
        cap = max(st.shape[0], int(nsearch), 1)
        piv = np.zeros((cap, L), np.int64)
        err = np.zeros(cap)
        n = ctypes.c_int64()
        _check(load_library().tci_estimatetrueerror(self.h, int(nsearch), _p(st, I64P) if st.size else None,
                                                    st.shape[0], int(seed), cap, _p(piv, I64P), _p(err, F64P),
                                                    ctypes.byref(n)))
        return [(piv[k].copy(), float(err[k])) for k in range(min(n.value, cap))]

    def fcache_stats(self):
        """(distinct points stored, points passed to f, calls of f) of a solve
        whose f is a BatchFunction; zeros otherwise."""
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _check(load_library().tci_fcache_stats(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def history(self):
        lib = load_library()
        n = ctypes.c_int64()
        lib.tci_get_history(self.h, None, None, None, ctypes.byref(n))
        r = np.zeros(n.value, np.int64)
        e = np.zeros(n.value)
        g = np.zeros(n.value, np.int64)
        if n.value:
            lib.tci_get_history(self.h, _p(r, I64P), _p(e, F64P), _p(g, I64P), ctypes.byref(n))
        return r, e, g

    # ---- tensor train
    def evaluate(self, points, precision="fp64"):
        """evaluate(tci, indexset) for one point or an array of points (1-based).
        precision "tf32x3": split-precision tensor-core evaluation; its error
        against FP64 (sampled) is left in self.eval_err_est."""
        if precision not in PRECISION:
            raise ArgumentError(TCI_ERR_ARG, f"Unknown precision {precision}.")
        pts = np.asarray(points, dtype=np.int64)
        single = pts.ndim == 1
        pts = np.ascontiguousarray(pts.reshape(-1, len(self)))
        out = np.zeros(pts.shape[0])
        err = np.zeros(1)
        _check(load_library().tci_evaluate_prec(self.h, _p(pts, I64P), pts.shape[0], _p(out, F64P),
                                                PRECISION[precision], _p(err, F64P)))
        self.eval_err_est = float(err[0])
        return float(out[0]) if single else out

    __call__ = evaluate

    def sum(self):
        out = ctypes.c_double()
        _check(load_library().tci_sum(self.h, ctypes.byref(out)))
        return out.value

    def tensortrain(self):
        return TensorTrain(self.sitetensors)


class TensorTrain:
    """TensorTrain{Float64,3} (tensortrain.jl:17-31) with host-side cores."""

    def __init__(self, sitetensors):
        for i in range(len(sitetensors) - 1):
            if sitetensors[i].shape[-1] != sitetensors[i + 1].shape[0]:
                raise ArgumentError(TCI_ERR_ARG, f"The tensors at {i + 1} and {i + 2} must have consistent "
                                    "dimensions for a tensor train.")
        self._cores = [np.asarray(t, dtype=np.float64) for t in sitetensors]
        self._buf = None

    @classmethod
    def _from_buffer(cls, buf, dims, offsets):
        """Cores stored one after the other (column-major) in a host buffer; the
        array views are made on first access."""
        t = cls.__new__(cls)
        t._cores = None
        t._buf, t._dims, t._offs = buf, dims, offsets
        return t

    @property
    def sitetensors(self):
        if self._cores is None:
            self._cores = [self._buf[o:o + a * b * c].reshape((a, b, c), order="F")
                           for (a, b, c), o in zip(self._dims, self._offs)]
        return self._cores

    def __len__(self):
        return len(self._dims) if self._cores is None else len(self._cores)

    def linkdims(self):
        if self._cores is None:
            return [d[0] for d in self._dims[1:]]
        return [t.shape[0] for t in self._cores[1:]]

    def rank(self):
        return max(self.linkdims())

    def _args(self):
        cores = [np.asfortranarray(c, dtype=np.float64) for c in self.sitetensors]
        if not all(c.ndim == 3 for c in cores):
            raise ArgumentError(TCI_ERR_ARG, "evaluate/sum need 3-leg site tensors")
        dims = np.ascontiguousarray([list(c.shape) for c in cores], dtype=np.int64).reshape(-1)
        return cores, dims, (ctypes.c_void_p * len(cores))(*[c.ctypes.data for c in cores])

    def evaluate(self, points, ctx=None, precision="fp64"):
        """evaluate(tt, indexset) (abstracttensortrain.jl:124-162) on the device, 1-based.
        precision "tf32x3": split-precision tensor-core evaluation; its error
        against FP64 (sampled) is left in self.eval_err_est."""
        if precision not in PRECISION:
            raise ArgumentError(TCI_ERR_ARG, f"Unknown precision {precision}.")
        ctx = ctx or default_context()
        cores, dims, ptrs = self._args()
        pts = np.asarray(points, dtype=np.int64)
        single = pts.ndim == 1
        pts = np.ascontiguousarray(pts.reshape(-1, len(cores)))
        out = np.zeros(pts.shape[0])
        err = np.zeros(1)
        _check(load_library().tci_tt_evaluate_prec(ctx.h, len(cores), _p(dims, I64P), ptrs, _p(pts, I64P),
                                                   pts.shape[0], _p(out, F64P), PRECISION[precision],
                                                   _p(err, F64P)))
        self.eval_err_est = float(err[0])
        return float(out[0]) if single else out

    def sum(self, ctx=None):
        """sum(tt) (abstracttensortrain.jl:164-199) on the device."""
        ctx = ctx or default_context()
        cores, dims, ptrs = self._args()
        out = ctypes.c_double()
        _check(load_library().tci_tt_sum(ctx.h, len(cores), _p(dims, I64P), ptrs, ctypes.byref(out)))
        return out.value


def _tt4_args(cores):
    cores = [np.asfortranarray(c, dtype=np.float64) for c in cores]
    dims = np.ascontiguousarray([list(c.shape) for c in cores], dtype=np.int64).reshape(-1)
    ptrs = (ctypes.c_void_p * len(cores))(*[c.ctypes.data for c in cores])
    return cores, dims, ptrs


def _tt4_fetch(h):
    lib = load_library()
    try:
        L = lib.tci_tt4_length(h)
        dims = np.zeros(4 * L, np.int64)
        _check(lib.tci_tt4_dims(h, _p(dims, I64P)))
        out = []
        for b in range(L):
            shape = tuple(int(x) for x in dims[4 * b:4 * b + 4])
            buf = np.zeros(int(np.prod(shape)), np.float64)
            _check(lib.tci_tt4_get_core(h, b + 1, _p(buf, F64P)))
            out.append(buf.reshape(shape, order="F"))
        return out
    finally:
        lib.tci_tt4_destroy(h)


def _as_tt4(t, left_operand):
    """Cores of a tensor train as 4-leg tensors; 3-leg cores get a unit leg
    (TensorTrain{4}(A, [(1, s...)]) for the left operand, (s..., 1) for the
    right one, contraction.jl:548-560)."""
    cores = t.sitetensors if isinstance(t, (TensorTrain, TensorCI2)) else t
    cores = [np.asarray(c, dtype=np.float64) for c in cores]
    three = all(c.ndim == 3 for c in cores)
    if three:
        cores = [c.reshape((c.shape[0], 1, c.shape[1], c.shape[2]) if left_operand else
                           (c.shape[0], c.shape[1], 1, c.shape[2]), order="F") for c in cores]
    elif not all(c.ndim == 4 for c in cores):
        raise ArgumentError(TCI_ERR_ARG, "site tensors must all have 3 or all have 4 legs")
    return cores, three


def _value_callback(f):
    """tci_value_fn from an elementwise Python function (values mapped in place)."""
    def _call(user, n, vals):
        try:
            v = np.ctypeslib.as_array(vals, shape=(n,))
            v[:] = np.asarray(f(v.copy()), dtype=np.float64).reshape(-1)
            return 0
        except BaseException as e:  # reported through the library's error code
            _cb_state.error = e
            return 1
    return VALUE_FN(_call)


def contract(A, B, algorithm="TCI", tolerance=1e-12, maxbonddim=None, method=None, ctx=None, f=None,
             initialpivots=10, precision="fp64", **kwargs):
    """contract(A, B; algorithm, tolerance, maxbonddim) (contraction.jl:515-560) of
    tensor trains with 4-leg cores (A's third leg against B's second), or of a
    3-leg train with a 4-leg one.  algorithm "TCI" (the default: crossinterpolate2
    of the Contraction evaluator on the device, with f applied elementwise,
    `initialpivots` a count of random starts or a list of fused 1-based
    pivots, and crossinterpolate2 keywords in kwargs), "naive" or "zipup";
    factorizations use the rank-revealing LU (method "LU") or MatrixLUCI over it
    (method "CI").  The reference factorizes these two algorithms with
    LinearAlgebra.svd (contraction.jl:369, :446), which is not on the device:
    without an explicit method, an algorithm that factorizes (zipup, or naive
    with truncation) raises instead of silently giving different factors.  precision
    "tf32x3" (zipup) runs the site contractions as TF32 hi/lo split products on
    the tensor cores; the result's `err_est` is the largest relative error of
    those products against FP64 at sampled entries.  Returns a TensorTrain."""
    if precision not in PRECISION:
        raise ArgumentError(TCI_ERR_ARG, f"Unknown precision {precision}.")
    if f is not None and algorithm != "TCI":
        raise TCIError(TCI_ERR_GENERIC, f"{algorithm.capitalize()} contraction implementation cannot contract "
                       "matrix product with a function. Use algorithm=:TCI instead.")
    if algorithm == "TCI":
        return _contract_tci(A, B, tolerance, maxbonddim, f, initialpivots, ctx, kwargs)
    alg = {"naive": TCI_CONTRACT_NAIVE, "zipup": TCI_CONTRACT_ZIPUP}.get(algorithm)
    if alg is None:
        raise ArgumentError(TCI_ERR_ARG, f"Unknown algorithm {algorithm}.")
    if method not in FACTORIZE and method is not None:
        raise TCIError(TCI_ERR_GENERIC, f"method=:{method} is not available on the device (:LU, :CI)")
    a, a3 = _as_tt4(A, True)
    b, b3 = _as_tt4(B, False)
    if len(a) != len(b):
        raise ArgumentError(TCI_ERR_ARG, "Cannot contract tensor trains with different length.")
    for n, (x, y) in enumerate(zip(a, b)):  # contraction.jl:43-46
        if np.shape(x)[2] != np.shape(y)[1]:
            raise TCIError(TCI_ERR_GENERIC, f"Tensor trains must share the identical index at n={n + 1}!")
    if method is None:
        if alg == TCI_CONTRACT_ZIPUP or tolerance > 0 or maxbonddim:
            raise TCIError(TCI_ERR_GENERIC, f"contract(algorithm=:{algorithm}) factorizes with :SVD in the reference "
                           "(contraction.jl:369, :446), which is not on the device: pass method='LU' or "
                           "method='CI'")
        method = "LU"  # nothing is factorized
    ctx = ctx or default_context()
    a, ad, ap = _tt4_args(a)
    b, bd, bp = _tt4_args(b)
    h = ctypes.c_void_p()
    err = np.zeros(1)
    _check(load_library().tci_tt4_contract_prec(ctx.h, len(a), _p(ad, I64P), ap, _p(bd, I64P), bp, alg,
                                                FACTORIZE[method], float(tolerance), int(maxbonddim or 0),
                                                PRECISION[precision], _p(err, F64P), ctypes.byref(h)))
    cores = _tt4_fetch(h)
    if a3 or b3:  # TensorTrain{3}(tt, prod.(sitedims(tt)))
        cores = [c.reshape((c.shape[0], c.shape[1] * c.shape[2], c.shape[3]), order="F") for c in cores]
    tt = TensorTrain(cores)
    tt.err_est = float(err[0])
    return tt


def matmul(A, B, precision="fp64", ctx=None):
    """A * B of FP64 matrices on the device (the product of contraction.jl:92):
    "fp64" is the fixed-order FP64 kernel, "tf32x3" the TF32 hi/lo split product
    on the tensor cores.  Returns (C, err_est): err_est is the relative error of
    the split product against FP64 at sampled entries (0 for "fp64")."""
    if precision not in PRECISION:
        raise ArgumentError(TCI_ERR_ARG, f"Unknown precision {precision}.")
    A = np.asfortranarray(A, dtype=np.float64)
    B = np.asfortranarray(B, dtype=np.float64)
    if A.ndim != 2 or B.ndim != 2 or A.shape[1] != B.shape[0]:
        raise DimensionMismatch(TCI_ERR_DIM, f"matrix A has dimensions {A.shape}, matrix B has dimensions {B.shape}")
    ctx = ctx or default_context()
    M, K = A.shape
    N = B.shape[1]
    a = np.ascontiguousarray(A.reshape(-1, order="F"))
    b = np.ascontiguousarray(B.reshape(-1, order="F"))
    c = np.zeros(max(M * N, 1))
    err = np.zeros(1)
    _check(load_library().tci_matmul(ctx.h, M, N, K, _p(a, F64P) if a.size else None,
                                     _p(b, F64P) if b.size else None, _p(c, F64P), PRECISION[precision],
                                     _p(err, F64P)))
    return c[: M * N].reshape((M, N), order="F"), float(err[0])


def _contract_tci(A, B, tolerance, maxbonddim, f, initialpivots, ctx, kwargs):
    """contract_TCI (contraction.jl:399-434) through tci_tt4_contract_tci."""
    a, a3 = _as_tt4(A, True)
    b, b3 = _as_tt4(B, False)
    if len(a) != len(b):
        raise ArgumentError(TCI_ERR_ARG, "Cannot contract tensor trains with different length.")
    ctx = ctx or default_context()
    a, ad, ap = _tt4_args(a)
    b, bd, bp = _tt4_args(b)
    L = len(a)
    if isinstance(initialpivots, (int, np.integer)):
        piv, ninit = np.zeros((0, L), np.int64), int(initialpivots)
    else:
        piv, ninit = _pivots_array(initialpivots, L), 0
    o = make_opts(tolerance=tolerance, maxbonddim=maxbonddim, **kwargs)
    cb = _value_callback(f) if f is not None else VALUE_FN()  # a null pointer without f
    h = ctypes.c_void_p()
    _check(load_library().tci_tt4_contract_tci(ctx.h, L, _p(ad, I64P), ap, _p(bd, I64P), bp,
                                               _p(piv, I64P) if piv.size else None, piv.shape[0], ninit,
                                               cb, None, ctypes.byref(o), ctypes.byref(h)))
    cores = _tt4_fetch(h)
    if a3 or b3:  # TensorTrain{3}(tt, prod.(sitedims(tt)))
        cores = [c.reshape((c.shape[0], c.shape[1] * c.shape[2], c.shape[3]), order="F") for c in cores]
    return TensorTrain(cores)


def compress(tt, method="LU", tolerance=1e-12, maxbonddim=None, normalizeerror=True, ctx=None):
    """compress!(tt, method; tolerance, maxbonddim, normalizeerror) (tensortrain.jl:149-183)
    with method "LU" or "CI" on a train with 4-leg (or 3-leg) cores; returns a new
    TensorTrain."""
    if method not in FACTORIZE:
        raise TCIError(TCI_ERR_GENERIC, f"method=:{method} is not available on the device (:LU, :CI)")
    cores, three = _as_tt4(tt, True)
    ctx = ctx or default_context()
    cores, d, ptrs = _tt4_args(cores)
    h = ctypes.c_void_p()
    _check(load_library().tci_tt4_compress(ctx.h, len(cores), _p(d, I64P), ptrs, FACTORIZE[method],
                                           float(tolerance), int(maxbonddim or 0), int(bool(normalizeerror)),
                                           ctypes.byref(h)))
    out = _tt4_fetch(h)
    if three:
        out = [c.reshape((c.shape[0], c.shape[2], c.shape[3]), order="F") for c in out]
    return TensorTrain(out)


class ProductIntegrand:
    """An integrand f(x) = prod_n g_n(x_n) for integrate(): `g` is one callable
    used at every coordinate, or a list of one callable per coordinate.  It is
    evaluated on the host at the quadrature nodes only; the interpolation of the
    integrand runs on the device (registered function "product")."""

    def __init__(self, g):
        self.g = g

    def factor(self, n):
        return self.g[n] if isinstance(self.g, (list, tuple)) else self.g


def product_function(tables, C=1.0):
    """DeviceFunction f(v) = C * prod_n tables[n][v_n] (tables: L x D).  log|t| is
    rounded to a multiple of 2^-40 so that the device sums it exactly."""
    t = np.asarray(tables, dtype=np.float64)
    L, D = t.shape
    with np.errstate(divide="ignore"):
        q = np.log(np.abs(t))
    q = np.where(q < -745.0, -np.inf, np.round(q * 2.0 ** 40) / 2.0 ** 40)
    finite = np.abs(q[np.isfinite(q)])
    if finite.size and L * finite.max() >= 8192.0:
        raise ArgumentError(TCI_ERR_ARG, "product f: factors too far from 1 for exact log sums")
    neg = (t < 0).astype(np.float64)
    return DeviceFunction("product", np.concatenate([[L, D, C], q.reshape(-1), neg.reshape(-1)]))


def integrate(ValueType, f, a, b, GKorder=15, ctx=None, **kwargs):
    """integrate(ValueType, f, a, b; GKorder, kwargs...) (integration.jl:20-58):
    Gauss--Kronrod nodes per coordinate, crossinterpolate2 of
    F(i) = prod_n w[n, i_n] * f(x(i)) * GKorder^N with nsearchglobalpivot = 10,
    then sum(tci) / GKorder^N.  f is a ProductIntegrand (interpolated by the
    registered device function "product") or any vectorized callable taking an
    (npoints, N) array of coordinates and returning npoints values (a
    caller-supplied f behind the device value cache)."""
    from .quadrature import kronrod

    if ValueType not in (float, np.float64, "Float64"):
        raise ArgumentError(TCI_ERR_ARG, "only Float64 is supported")
    if GKorder % 2 == 0:
        raise TCIError(TCI_ERR_GENERIC, "Gauss--Kronrod order must be odd, e.g. 15 or 61.")
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.size != b.size:
        raise TCIError(TCI_ERR_GENERIC, "Integral bounds must have the same dimensionality, but got "
                       f"{a.size} lower bounds and {b.size} upper bounds.")
    x1, w1, _ = kronrod(GKorder // 2)
    N = a.size
    nodes = (b - a)[:, None] * (x1[None, :] + 1.0) / 2.0 + a[:, None]
    weights = (b - a)[:, None] * w1[None, :] / 2.0
    norm = float(GKorder) ** N
    kw = dict(nsearchglobalpivot=10)
    kw.update(kwargs)
    if isinstance(f, ProductIntegrand):
        tables = np.array([[weights[n, i] * f.factor(n)(nodes[n, i]) for i in range(x1.size)] for n in range(N)])
        F = product_function(tables, norm)
    else:
        F = BatchFunction(quadrature_integrand(f, nodes, weights, norm))
    tci, _, _ = crossinterpolate2(ValueType, F, [x1.size] * N, ctx=ctx, **kw)
    return tci.sum() / norm


def quadrature_integrand(f, nodes, weights, norm):
    """F(indices) = prod_n weights[n, i_n] * f(x) * norm, x_n = nodes[n, i_n]
    (integration.jl:41-45), for a batch of 1-based multi-indices."""
    cols = np.arange(nodes.shape[0])[None, :]

    def F(idx):
        i0 = idx - 1
        x = nodes[cols, i0]
        w = np.prod(weights[cols, i0], axis=1)
        return w * np.asarray(f(x), dtype=np.float64).reshape(-1) * norm
    return F


def crossinterpolate2(ValueType, f, localdims, initialpivots=None, ctx=None, **kwargs):
    """crossinterpolate2 (tensorci2.jl:943-953) -> (tci, ranks, errors)."""
    if ValueType not in (float, np.float64, "Float64"):
        raise ArgumentError(TCI_ERR_ARG, "only Float64 is supported")
    ctx = ctx or default_context()
    lib = load_library()
    localdims = [int(d) for d in localdims]
    L = len(localdims)
    d = np.ascontiguousarray(localdims, dtype=np.int64)
    piv = _pivots_array(initialpivots if initialpivots is not None else [np.ones(L)], L)
    o = make_opts(**kwargs)
    h = ctypes.c_void_p()
    _check(lib.tci_crossinterpolate2(ctx.h, L, _p(d, I64P), f.fid, _p(f.params, F64P) if f.params.size else None,
                                     f.params.size, _p(piv, I64P), piv.shape[0], ctypes.byref(o), ctypes.byref(h)))
    tci = TensorCI2(f, localdims, ctx=ctx, _handle=h)
    r, e, _ = tci.history()
    return tci, r, e


def make_requests(specs):
    """specs: list of (f: DeviceFunction, localdims, opts kwargs).  Keeps buffers alive."""
    keep = []
    arr = (Request * len(specs))()
    for i, (f, localdims, kw) in enumerate(specs):
        d = np.ascontiguousarray(localdims, dtype=np.int64)
        keep.append(d)
        keep.append(f.params)
        arr[i].L = len(localdims)
        arr[i].fid = f.fid
        arr[i].localdims = _p(d, I64P)
        arr[i].fparams = _p(f.params, F64P) if f.params.size else None
        arr[i].nparams = f.params.size
        arr[i].opts = make_opts(**kw)
    return arr, keep


_REQ_DTYPE = None


def _req_dtype():
    """numpy mirror of Request (pointers as uint64, opts flattened), built from the
    ctypes field offsets."""
    global _REQ_DTYPE
    if _REQ_DTYPE is None:
        def np_type(ct):
            if ct in (I64P, F64P):
                return np.uint64
            return {ctypes.c_int32: np.int32, ctypes.c_int64: np.int64, ctypes.c_double: np.float64,
                    ctypes.c_uint64: np.uint64}[ct]

        names, formats, offsets = [], [], []
        for nm, ct in Request._fields_:
            if ct is Opts:
                for onm, oct_ in Opts._fields_:
                    names.append("opts_" + onm)
                    formats.append(np_type(oct_))
                    offsets.append(Request.opts.offset + getattr(Opts, onm).offset)
            else:
                names.append(nm)
                formats.append(np_type(ct))
                offsets.append(getattr(Request, nm).offset)
        _REQ_DTYPE = np.dtype({"names": names, "formats": formats, "offsets": offsets,
                               "itemsize": ctypes.sizeof(Request)})
    return _REQ_DTYPE


def pack_requests(specs):
    """The same requests as make_requests, packed with whole-array operations: all
    local dims and f parameters in two arrays, the option structs from one
    make_opts per distinct set of keyword arguments besides tolerance and
    maxbonddim.  Returns (POINTER(Request), buffers to keep alive)."""
    n = len(specs)
    rec = np.zeros(max(n, 1), _req_dtype())
    if n == 0:
        return rec.ctypes.data_as(ctypes.POINTER(Request)), [rec]
    Ls = np.fromiter((len(ld) for _, ld, _ in specs), np.int64, n)
    dims = np.ascontiguousarray(np.concatenate([np.asarray(ld, dtype=np.int64).ravel() for _, ld, _ in specs]))
    plist = [f.params for f, _, _ in specs]
    npar = np.fromiter((p.size for p in plist), np.int64, n)
    prm = np.ascontiguousarray(np.concatenate(plist).astype(np.float64)) if npar.sum() else np.zeros(1)
    doff = np.concatenate([[0], np.cumsum(Ls)[:-1]]).astype(np.uint64)
    poff = np.concatenate([[0], np.cumsum(npar)[:-1]]).astype(np.uint64)
    rec["L"] = Ls
    rec["fid"] = np.fromiter((f.fid for f, _, _ in specs), np.int32, n)
    rec["localdims"] = np.uint64(dims.ctypes.data) + np.uint64(8) * doff
    rec["fparams"] = np.where(npar > 0, np.uint64(prm.ctypes.data) + np.uint64(8) * poff, np.uint64(0))
    rec["nparams"] = npar
    fields = [nm for nm, _ in Opts._fields_]
    groups, tol, mbd, single = {}, np.empty(n), np.empty(n, np.int64), []
    for i, (_, _, kw) in enumerate(specs):
        if "pivottolerance" in kw:  # its consistency check with tolerance is per request
            single.append(i)
            continue
        rest = tuple(sorted((k, v) for k, v in kw.items() if k not in ("tolerance", "maxbonddim")))
        groups.setdefault(rest, []).append(i)
        t = kw.get("tolerance")
        tol[i] = 1e-8 if t is None else float(t)
        b = kw.get("maxbonddim")
        mbd[i] = 0 if b is None else int(b)
    for rest, idx in groups.items():
        o = make_opts(**dict(rest))
        idx = np.asarray(idx, np.int64)
        for nm in fields:
            rec["opts_" + nm][idx] = getattr(o, nm)
        rec["opts_tolerance"][idx] = tol[idx]
        rec["opts_maxbonddim"][idx] = mbd[idx]
    for i in single:
        o = make_opts(**specs[i][2])
        for nm in fields:
            rec["opts_" + nm][i] = getattr(o, nm)
    return rec.ctypes.data_as(ctypes.POINTER(Request)), [rec, dims, prm, specs]


def crossinterpolate2_batched(specs, max_live=0, ctx=None):
    """Solve many crossinterpolate2 problems together (one launch per step for all)."""
    ctx = ctx or default_context()
    arr, keep = pack_requests(specs)
    out = (ctypes.c_void_p * len(specs))()
    rc = load_library().tci_crossinterpolate2_batched(ctx.h, len(specs), arr, int(max_live), out)
    wrap = TensorCI2._wrap
    res = [wrap(f, ld, ctx, ctypes.c_void_p(h)) if h else None for (f, ld, _), h in zip(specs, out)]
    _check(rc)
    return res


def core_dims(tci):
    lib = load_library()
    dims = []
    d = np.zeros(3, np.int64)
    for b in range(1, len(tci) + 1):
        _check(lib.tci_get_core(tci.h, b, None, _p(d, I64P)))
        dims.append(tuple(int(x) for x in d))
    return dims


class _PinnedBlock:
    """A pinned host buffer of the library seen as a float64 array; given back to
    the library's pool when the last array view of it is gone."""

    def __init__(self, ctx, addr, n):
        self.ctx = ctx  # the context owns the pool: keep it alive
        self.__array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (addr, False), "version": 3}
        fin = weakref.finalize(self, load_library().tci_host_free, ctx.h, ctypes.c_void_p(addr))
        fin.atexit = False  # at exit the process releases everything; the context may be gone


def tensortrains(tcis, ctx=None):
    """TensorTrain(tci) for many solves with one device-to-host copy."""
    ctx = ctx or default_context()
    handles = (ctypes.c_void_p * len(tcis))(*[t.h.value if isinstance(t.h, ctypes.c_void_p) else t.h for t in tcis])
    lens = [len(t) for t in tcis]
    dims = np.zeros(3 * max(sum(lens), 1), np.int64)
    lib = load_library()
    _check(lib.tci_get_core_dims_batched(len(tcis), handles, _p(dims, I64P)))
    d3 = dims[:3 * sum(lens)].reshape(-1, 3)
    elems = d3.prod(axis=1)
    core_off = np.concatenate([[0], np.cumsum(elems)]).astype(np.int64)
    solve_first = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    ptr = ctypes.c_void_p()
    total = ctypes.c_int64()
    _check(lib.tci_get_cores_pinned(ctx.h, len(tcis), handles, ctypes.byref(ptr), ctypes.byref(total)))
    out = np.asarray(_PinnedBlock(ctx, ptr.value, max(int(total.value), 1)))
    d3l = d3.tolist()
    col = core_off.tolist()
    sf = solve_first.tolist()
    return [TensorTrain._from_buffer(out, d3l[sf[i]:sf[i + 1]], col[sf[i]:sf[i + 1]]) for i in range(len(tcis))]


def serve(specs, arrival, max_live=0, ctx=None):
    """Continuous-batching server over a request stream -> (latency, rank, wall)."""
    ctx = ctx or default_context()
    arr, keep = pack_requests(specs)
    arrival = np.ascontiguousarray(arrival, dtype=np.float64)
    lat = np.zeros(len(specs))
    rank = np.zeros(len(specs), np.int64)
    wall = ctypes.c_double()
    _check(load_library().tci_serve_run(ctx.h, len(specs), arr, _p(arrival, F64P), int(max_live), _p(lat, F64P),
                                        _p(rank, I64P), ctypes.byref(wall)))
    return lat, rank, wall.value


class Server:
    """Incremental server (tci_serve_start/submit/poll/stop): requests go in one at
    a time while earlier ones are being solved with continuous batching; the
    context is reserved for the server until stop()."""

    def __init__(self, max_live=0, ctx=None):
        self.ctx = ctx or default_context()
        self.h = ctypes.c_void_p()
        _check(load_library().tci_serve_start(self.ctx.h, int(max_live), ctypes.byref(self.h)))

    def submit(self, f, localdims, **kwargs):
        arr, keep = make_requests([(f, localdims, kwargs)])
        rid = ctypes.c_int64()
        _check(load_library().tci_serve_submit(self.h, ctypes.byref(arr[0]), ctypes.byref(rid)))
        return rid.value

    def poll(self, cap=4096, timeout_ms=0):
        """[(id, status, rank, latency_s), ...] of the requests finished since the last poll."""
        ids = np.zeros(cap, np.int64)
        st = np.zeros(cap, np.int32)
        rk = np.zeros(cap, np.int64)
        lat = np.zeros(cap)
        n = ctypes.c_int64()
        _check(load_library().tci_serve_poll(self.h, cap, _p(ids, I64P), st.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                             _p(rk, I64P), _p(lat, F64P), ctypes.byref(n), int(timeout_ms)))
        return [(int(ids[i]), int(st[i]), int(rk[i]), float(lat[i])) for i in range(n.value)]

    def stop(self):
        if self.h:
            h, self.h = self.h, None
            _check(load_library().tci_serve_stop(h))


def feval(f, localdims, points, ctx=None):
    """Evaluate a registered device function at points (n x L, 1-based) on the GPU."""
    ctx = ctx or default_context()
    localdims = np.ascontiguousarray(localdims, dtype=np.int64)
    pts = np.ascontiguousarray(np.asarray(points, dtype=np.int64).reshape(-1, localdims.size))
    out = np.zeros(pts.shape[0])
    _check(load_library().tci_feval(ctx.h, f.fid, _p(f.params, F64P) if f.params.size else None, f.params.size,
                                    localdims.size, _p(localdims, I64P), _p(pts, I64P), pts.shape[0],
                                    _p(out, F64P)))
    return out


def optfirstpivot(f, localdims, firstpivot=None, maxsweep=1000, ctx=None):
    """optfirstpivot(f, localdims, firstpivot; maxsweep) (util.jl:78-108) on the
    device: coordinate ascent of |f| from firstpivot (1-based)."""
    ctx = ctx or default_context()
    d = np.ascontiguousarray(localdims, dtype=np.int64)
    p = np.ascontiguousarray(firstpivot if firstpivot is not None else np.ones(d.size), dtype=np.int64).copy()
    if p.size != d.size:
        raise DimensionMismatch(TCI_ERR_DIM, "firstpivot must have one index per leg")
    _check(load_library().tci_optfirstpivot(ctx.h, f.fid, _p(f.params, F64P) if f.params.size else None,
                                            f.params.size, d.size, _p(d, I64P), _p(p, I64P), int(maxsweep)))
    return p


def convergencecriterion(ranks, errors, nglobalpivots, tolerance, maxbonddim, ncheckhistory,
                         checkconvglobalpivot=True):
    """convergencecriterion (tensorci2.jl:609-628); host-side logic of the library."""
    r = np.ascontiguousarray(ranks, np.int64)
    e = np.ascontiguousarray(errors, np.float64)
    g = np.ascontiguousarray(nglobalpivots, np.int64)
    return bool(load_library().tci_convergencecriterion(_p(r, I64P), _p(e, F64P), _p(g, I64P), r.size, tolerance,
                                                        maxbonddim, ncheckhistory, int(bool(checkconvglobalpivot))))


def fp64_peak(ctx=None):
    """Measured FP64 operations per second: (separate mul+sub, fused)."""
    ctx = ctx or default_context()
    a, b = ctypes.c_double(), ctypes.c_double()
    _check(load_library().tci_fp64_peak(ctx.stream, ctypes.byref(a), ctypes.byref(b)))
    return a.value, b.value


# ---------------------------------------------------------------- rrLU
class rrLU:
    """Result of rrlu (matrixlu.jl:71-96): 1-based permutations, L, U."""

    def __init__(self, rowpermutation, colpermutation, L, U, leftorthogonal, npivot, error):
        self.rowpermutation = rowpermutation
        self.colpermutation = colpermutation
        self.L = L
        self.U = U
        self.leftorthogonal = leftorthogonal
        self.npivot = npivot
        self.error = error

    @property
    def shape(self):
        return (self.L.shape[0], self.U.shape[1])

    def rowindices(self):
        return self.rowpermutation[: self.npivot]

    def colindices(self):
        return self.colpermutation[: self.npivot]

    def npivots(self):
        return self.npivot

    def left(self, permute=True):
        if not permute:
            return self.L
        out = np.empty_like(self.L)
        out[self.rowpermutation - 1, :] = self.L
        return out

    def right(self, permute=True):
        if not permute:
            return self.U
        out = np.empty_like(self.U)
        out[:, self.colpermutation - 1] = self.U
        return out

    def diag(self):
        K = self.npivot
        return np.diag(self.U[:K, :K]) if self.leftorthogonal else np.diag(self.L[:K, :K])

    def pivoterrors(self):
        return np.concatenate([np.abs(self.diag()), [self.error]])

    def lastpivoterror(self):
        return self.error


def rrlu(A, maxrank=None, reltol=1e-14, abstol=0.0, leftorthogonal=True, ctx=None):
    """rrlu(A; maxrank, reltol, abstol, leftorthogonal) (matrixlu.jl:217-225) on the GPU."""
    ctx = ctx or default_context()
    A = np.asarray(A, dtype=np.float64)
    m, n = A.shape
    k = min(m, n)
    flat = np.ascontiguousarray(A.reshape(-1, order="F"))
    rp = np.zeros(m, np.int64)
    cp = np.zeros(n, np.int64)
    Lb = np.zeros(max(m * k, 1))
    Ub = np.zeros(max(k * n, 1))
    npiv = ctypes.c_int64()
    err = ctypes.c_double()
    _check(load_library().tci_rrlu(ctx.h, _p(flat, F64P), m, n, 0 if maxrank is None else int(maxrank), reltol,
                                   abstol, int(bool(leftorthogonal)), _p(rp, I64P), _p(cp, I64P), _p(Lb, F64P),
                                   _p(Ub, F64P), ctypes.byref(npiv), ctypes.byref(err)))
    K = npiv.value
    return rrLU(rp, cp, Lb[: m * K].reshape((m, K), order="F").copy(), Ub[: K * n].reshape((K, n), order="F").copy(),
                bool(leftorthogonal), K, err.value)


def rrlu_batched(mats, maxrank=None, reltol=1e-14, abstol=0.0, leftorthogonal=True, ctx=None):
    """Many independent rrLUs in one launch -> list of (rows, cols, npivot, error), 1-based."""
    ctx = ctx or default_context()
    ms = np.array([a.shape[0] for a in mats], np.int64)
    ns = np.array([a.shape[1] for a in mats], np.int64)
    offs = np.concatenate([[0], np.cumsum(ms * ns)[:-1]]).astype(np.int64)
    flat = np.ascontiguousarray(np.concatenate([np.asarray(a, np.float64).reshape(-1, order="F") for a in mats]))
    kcap = np.minimum(np.minimum(ms, ns), maxrank if maxrank else np.iinfo(np.int64).max)
    poffs = np.concatenate([[0], np.cumsum(2 * kcap)[:-1]]).astype(np.int64)
    piv = np.zeros(int(2 * kcap.sum()) + 1, np.int64)
    npiv = np.zeros(len(mats), np.int64)
    errs = np.zeros(len(mats))
    _check(load_library().tci_rrlu_batched(ctx.h, len(mats), _p(flat, F64P), _p(offs, I64P), _p(ms, I64P),
                                           _p(ns, I64P), 0 if maxrank is None else int(maxrank), reltol, abstol,
                                           int(bool(leftorthogonal)), _p(piv, I64P), _p(poffs, I64P),
                                           _p(npiv, I64P), _p(errs, F64P)))
    out = []
    for i in range(len(mats)):
        K = int(npiv[i])
        o = poffs[i]
        out.append((piv[o:o + K].copy(), piv[o + kcap[i]:o + kcap[i] + K].copy(), K, float(errs[i])))
    return out
