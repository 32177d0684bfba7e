"""Build libtci_gpu.so (CUDA kernels for sm_103a + the C ABI) in-tree.

    python tensorcrossinterpolation.jl_gb300/build.py

Kernels are compiled by nvcc for sm_103a only; the host engine and C ABI by
g++ (C++20 coroutines).  Translation units compile in parallel.  The shared
library lands next to the Python package (tci_gb300/libtci_gpu.so).
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
OUT = os.path.join(HERE, "tci_gb300", "libtci_gpu.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# Kernels whose arithmetic must not be contracted into FMA (bit-exact pivots and
# function values) are built with -fmad=false.
# (source, object, flags): step_kernel.cu is built twice, as the throughput
# variant (two 256-thread task CTAs per SM) and the latency variant (one
# 512-thread CTA per SM), in separate namespaces (csrc/kernels.h).
CU_SOURCES = [
    ("step_kernel.cu", "step_kernel.cu.o", ["-fmad=false"]),
    ("step_kernel.cu", "step_kernel_k512.cu.o",
     ["-fmad=false", "-DTCI_KNS=tci_k512", "-DTCI_STEP_THREADS=512", "-DTCI_CTAS_PER_SM=1", "-DTCI_SECONDARY"]),
    ("contract.cu", "contract.cu.o", ["-fmad=false"]),
    ("peak.cu", "peak.cu.o", []),
    ("gather.cu", "gather.cu.o", []),
    ("fcache.cu", "fcache.cu.o", []),
    ("tc_gemm.cu", "tc_gemm.cu.o", []),
]
CXX_SOURCES = ["engine.cpp", "capi.cpp", "contract.cpp", "fcache.cpp", "contract_tci.cpp", "pivotsearch.cpp"]
HEADERS = ["kernels.h", "tci_tasks.h", "tci_functions.h", "tci_math.h", "tci_rng.h", "engine.h", "contract.h", "contract_tci.h", "fcache.h", "fc_slot.h", "tc_gemm.h"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "tci_gb300.h")]
    jobs = []
    objs = []
    for src, obj, extra in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, obj)
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            jobs.append([NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                                         "-Xptxas", "-v"] + extra + ["-c", s, "-o", o])
    cxx = os.environ.get("CXX", "g++")
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _newer(o, [s] + hdrs):
            jobs.append([cxx, "-std=c++20", "-O2", "-fPIC", "-Wall", "-Wno-unused-function",
                         "-I", os.path.join(CUDA_HOME, "include"), "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for l in logs:
            sys.stdout.write(l)
    if force or _newer(OUT, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", OUT] + objs + ["-Xcompiler", "-fPIC", "-lpthread"])
    return OUT


if __name__ == "__main__":
    if "--clean" in sys.argv:
        shutil.rmtree(BUILD, ignore_errors=True)
    print(build(verbose="-v" in sys.argv, force="--force" in sys.argv))
