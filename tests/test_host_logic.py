"""Host logic of the engine on the CPU through the library's own C++ symbols,
built into small checkers linked against libtci_gpu.so: the index-set
operations (kronecker, union, select, pushunique!; tests/host/indexset_check.cpp and,
on randomized inputs, tests/host/indexset_random_check.cpp) and the key layout of
the device value cache (tests/host/fcache_keys_check.cpp)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "tensorcrossinterpolation.jl_gb300")


def _run_checker(T, tmp_path, name):
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if cxx is None:
        pytest.skip("no C++ compiler")
    lib = os.path.dirname(T.load_library()._name)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    exe = str(tmp_path / name)
    cmd = [cxx, "-std=c++20", "-O1", "-I", os.path.join(PKG, "csrc"), "-I", os.path.join(cuda, "include"),
           os.path.join(HERE, "host", name + ".cpp"), "-o", exe, "-L", lib, "-ltci_gpu",
           f"-Wl,-rpath,{lib}", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr


def test_index_sets(T, tmp_path):
    _run_checker(T, tmp_path, "indexset_check")


def test_fcache_keys(T, tmp_path):
    _run_checker(T, tmp_path, "fcache_keys_check")


def test_index_sets_randomized(T, tmp_path):
    """kronecker / union / select against direct restatements on randomized
    inputs (both union paths, many duplicates), and the task layouts' global
    scratch sizes."""
    _run_checker(T, tmp_path, "indexset_random_check")
