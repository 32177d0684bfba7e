"""The C ABI library loads and exports every symbol of include/tci_gb300.h (no GPU)."""
import ctypes
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "tci_gb300.h")
PKG = os.path.join(ROOT, "tensorcrossinterpolation.jl_gb300")


def _declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tci_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    sys.path.insert(0, PKG)
    import build as pkg_build

    pkg_build.build()
    import tci_gb300

    return tci_gb300


def test_every_declared_symbol_is_exported(lib):
    L = lib.load_library()
    declared = _declared_functions()
    assert len(declared) >= 30
    for name in declared:
        assert hasattr(L, name), f"{name} declared in tci_gb300.h but not exported"
        assert name in lib._SIGNATURES, f"{name} has no ctypes signature in tci_gb300"


def test_exported_symbols_are_declared(lib):
    so = lib.LIB_PATH
    out = subprocess.check_output(["nm", "-D", "--defined-only", so], text=True)
    exported = sorted({l.split()[-1] for l in out.splitlines() if re.search(r" T tci_", l)})
    declared = set(_declared_functions())
    for name in exported:
        assert name in declared, f"{name} exported but not declared in include/tci_gb300.h"


def test_opts_default_matches_reference(lib):
    o = lib.Opts()
    lib.load_library().tci_opts_default(ctypes.byref(o))
    # optimize! defaults, tensorci2.jl:700-720
    assert o.tolerance == 1e-8 and o.maxiter == 20 and o.sweepstrategy == 0
    assert o.normalizeerror == 1 and o.ncheckhistory == 3 and o.maxnglobalpivot == 5
    assert o.nsearchglobalpivot == 5 and o.tolmarginglobalsearch == 10.0 and o.strictlynested == 0
    assert o.checkconvglobalpivot == 1


def test_convergencecriterion_host_logic(lib, golden):
    for c in golden["tci2"]["convergencecriterion"]["cases"]:
        got = lib.convergencecriterion(c["ranks"], c["errors"], c["ngp"], c["tol"], c["maxbonddim"], c["ncheck"])
        assert got == c["expect"], c


def test_function_lookup(lib):
    L = lib.load_library()
    fid = ctypes.c_int()
    for name, want in lib.FUNCTIONS.items():
        assert L.tci_f_lookup(name.encode(), ctypes.byref(fid)) == 0 and fid.value == want
    assert L.tci_f_lookup(b"nope", ctypes.byref(fid)) == lib.TCI_ERR_ARG


def test_no_cpu_fallback_without_device(lib):
    """Without a CUDA device the library refuses to compute (no silent fallback)."""
    L = lib.load_library()
    h = ctypes.c_void_p()
    rc = L.tci_ctx_create(0, 0, ctypes.byref(h))
    if rc == 0:
        L.tci_ctx_destroy(h)
        pytest.skip("a CUDA device is present")
    assert rc == lib.TCI_ERR_CUDA
    assert L.tci_last_error()


def test_make_opts_rejects_conflicting_tolerances(lib):
    """optimize! throws ArgumentError for pivottolerance != tolerance (tensorci2.jl:735-737)."""
    with pytest.raises(lib.ArgumentError):
        lib.make_opts(tolerance=1e-9, pivottolerance=1e-2)
    assert lib.make_opts(pivottolerance=1e-3).tolerance == 1e-3
    with pytest.raises(lib.ArgumentError):
        lib.make_opts(pivotsearch="rook")


def test_dense_params_layout(lib):
    T = np.arange(12, dtype=float).reshape(3, 4)
    f = lib.DeviceFunction.dense(T)
    assert f.params[0] == 2 and list(f.params[1:3]) == [1, 3]
    assert np.array_equal(f.params[3:], T.reshape(-1, order="F"))
