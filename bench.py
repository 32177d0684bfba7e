"""Benchmark: TCI solves/sec of the served + batched GB300 path.

Workload (one "step"): a batch of B crossinterpolate2 requests drawn from the
served-stream family -- f(v) = 1/(1 + a v.v) + b exp(-g |v - c|^2) with a, b, g
log-uniform in [1e-2, 1e1] and c uniform on the lattice; L uniform in 4..16,
d uniform in 2..16, tolerance log-uniform in [1e-10, 1e-6], maxbonddim uniform
in {32, 64, 128, 256} -- seeded synthetic requests (no dataset is involved).
The batch is solved with continuous batching: host threads run the live solves
as coroutines and publish each GPU task the moment a solve needs it into a ring
in pinned memory; one resident kernel (a dispatcher warp plus one worker CTA
per SM) runs the tasks as they come and each solve resumes as soon as its own
task is done.

Reported (one JSON line):
  value  solves/s with everything on the device, CUDA events bracketing the
         whole batch;
  e2e    solves/s through the public C ABI (host request buffers in, every
         solve's site tensors and pivot sets copied back to host), wall clock;
  plain_solves_per_s   the one-solve-at-a-time GPU path on a subset;
  serve_p50_ms / serve_p99_ms   latency under Poisson arrivals at 80 % of the rate;
  serve_sweep  p50 / p99 at Poisson rates 50 ... 2000 requests/s;
  roofline  FP64 pipe of the step kernel vs the measured FP64 peak;
  cpu_baseline  the CPU oracle (C++ restatement of the reference) solving a
         bounded sample of the same requests on all host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--batch B] [--live M] [--impl reference]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "tensorcrossinterpolation.jl_gb300"))

METRIC = "TCI solves/sec and p50/p99 latency, served+batched vs plain GPU at error ≤1e-8"
UNIT = "solves/s"


def make_requests(n, seed, tol_range=(-10.0, -6.0)):
    """Served-stream family requests (L, d, params, tol, maxbonddim)."""
    from tci_gb300 import workloads

    return workloads.served_requests(n, seed, tol_range=tol_range)


def step_seed(step, rank):
    """Seed of the request list of bench step `step` on replica `rank`; both arms
    draw their requests from it."""
    return 1000 * step + rank


def oracle_solve(reqs, cores):
    """crossinterpolate2 of every request (initial pivot all ones) by the oracle
    on `cores` host threads; returns (wall seconds, ranks)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ctypes

    import oracle as O

    lib = O.lib()
    n = len(reqs)
    Ls = np.array([r[0] for r in reqs], np.int32)
    dims = np.concatenate([[r[1]] * r[0] for r in reqs]).astype(np.int64)
    doff = np.concatenate([[0], np.cumsum(Ls)[:-1]]).astype(np.int64)
    fids = np.full(n, O.F_SERVED, np.int32)
    prm = np.concatenate([r[2] for r in reqs]).astype(np.float64)
    np_ = np.array([len(r[2]) for r in reqs], np.int64)
    poff = np.concatenate([[0], np.cumsum(np_)[:-1]]).astype(np.int64)
    tol = np.array([r[3] for r in reqs])
    mbd = np.array([r[4] for r in reqs], np.int64)
    o = O.make_opts()
    rank = np.zeros(n, np.int64)
    secs = np.zeros(n)
    I32P = ctypes.POINTER(ctypes.c_int32)
    t0 = time.perf_counter()
    rc = lib.orc_solve_batch(n, Ls.ctypes.data_as(I32P), dims.ctypes.data_as(O.I64P),
                             doff.ctypes.data_as(O.I64P), fids.ctypes.data_as(I32P), prm.ctypes.data_as(O.F64P),
                             poff.ctypes.data_as(O.I64P), np_.ctypes.data_as(O.I64P), tol.ctypes.data_as(O.F64P),
                             mbd.ctypes.data_as(O.I64P), ctypes.byref(o), rank.ctypes.data_as(O.I64P),
                             secs.ctypes.data_as(O.F64P), int(cores))
    dt = time.perf_counter() - t0
    if rc:
        raise RuntimeError(f"oracle solve failed with code {rc}")
    return dt, rank


# FP64 operations per registered-function evaluation of the served family,
# counted from tci_functions.h/tci_math.h: 1/(1+a s1) (3), exp (2 reduction
# FMAs = 4, 13 Horner FMAs = 26, 2 more) and a + b*e (2), plus the two sums of
# the row/column states (2).
SERVED_F_OPS = 39


def served_ops(st):
    """FP64 operations of a served batch from the engine's counters: the rank-1
    updates of the factorizations (multiply + subtract), the triangular solves of
    setsitetensor! and the train contractions of the global pivot search
    (multiply + add or subtract), f from tables (one operation per element) and
    f evaluated directly."""
    return (2.0 * st["lu_updates"] + 2.0 * st.get("dense_macs", 0) + 1.0 * st["feval_tabulated"] +
            SERVED_F_OPS * (st["feval"] - st["feval_tabulated"]))


# DRAM bytes (read + write) per FP64 operation of the served task code: the sum of
# dram__bytes_read.sum + dram__bytes_write.sum over all 1181 tci_step_kernel
# launches of one 512-request served batch run as batched launches (TCI_RESIDENT=0):
# 843.7 MB read + 3.3 MB written for 6.896e9 served_ops.  The resident kernel runs
# the same task code.
SERVED_DRAM_BYTES_PER_OP = 847.04e6 / 6.8957e9


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 9 or p[0] != "0":
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(reqs, n=6000, what="the bench stream"):
    """The oracle solving the first n requests in one batch on all host cores
    (threads take the next request as they finish, so no thread idles on a
    chunk's slowest solve)."""
    cores = os.cpu_count() or 1
    sub = reqs[:n]
    dt, _ = oracle_solve(sub, cores)
    return {"value": len(sub) / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"the first {len(sub)} requests of {what}, crossinterpolate2 by the C++ "
                      f"oracle on {cores} threads in one batch, {dt:.1f} s"}


def parity_sample(T, res, reqs, nsample=200, npts=10000, seed=123):
    """Checks a sample of the timed solves against the oracle: `nsample` requests
    spread over the whole size range (every k-th by the HBM estimate
    L d^2 maxbonddim^2), each solved again by the oracle on the host threads.
    Per solve: pivot index sets identical, site tensors identical, and the max
    error |f - tt| on `npts` seeded lattice points against the request's
    tolerance (relative to maxsamplevalue)."""
    from concurrent.futures import ThreadPoolExecutor

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    order = sorted(range(len(reqs)), key=lambda i: reqs[i][0] * reqs[i][1] ** 2 * reqs[i][4] ** 2)
    pick = sorted({order[int(k)] for k in np.linspace(0, len(order) - 1, nsample)})

    def solve(i):
        L, d, prm, tol, mbd = reqs[i]
        ref, _, _ = O.crossinterpolate2([d] * L, O.F_SERVED, prm, None, tolerance=tol, maxbonddim=mbd)
        return ref

    t0 = time.perf_counter()
    with ThreadPoolExecutor(os.cpu_count() or 1) as ex:
        refs = list(ex.map(solve, pick))
    rng = np.random.default_rng(seed)
    same_piv = same_cores = within_tol = within_10tol = within_2x_oracle = 0
    uncapped = unc_tol = unc_10tol = 0
    worst = worst_unc = 0.0
    for i, ref in zip(pick, refs):
        L, d, prm, tol, mbd = reqs[i]
        tci = res[i]
        sp = all(np.array_equal(tci.sets(b)[0], ref.sets(b)[0]) and np.array_equal(tci.sets(b)[1], ref.sets(b)[1])
                 for b in range(1, L + 1))
        sc = sp and all(np.array_equal(tci.sitetensor(b), ref.core(b)) for b in range(1, L + 1))
        same_piv += sp
        same_cores += sc
        pts = rng.integers(1, d + 1, size=(npts, L))
        fx = O.feval(O.F_SERVED, prm, pts)
        err = float(np.max(np.abs(tci.evaluate(pts) - fx)))
        err_ref = err if sc else float(np.max(np.abs(ref.evaluate(pts) - fx)))
        ratio = err / (tol * tci.maxsamplevalue)
        worst = max(worst, ratio)
        within_tol += ratio <= 1.0
        within_10tol += ratio <= 10.0
        within_2x_oracle += err <= 2 * err_ref + 1e-300
        if tci.rank() < mbd:  # the rank cap did not bind: the tolerance decides the error
            uncapped += 1
            unc_tol += ratio <= 1.0
            unc_10tol += ratio <= 10.0
            worst_unc = max(worst_unc, ratio)
    return {"solves_checked": len(pick), "of_timed": len(reqs), "points_per_solve": npts,
            "pivots_identical": int(same_piv), "site_tensors_identical": int(same_cores),
            "mismatches": int(len(pick) - same_piv),
            "sampled_err_within_tol": int(within_tol), "sampled_err_within_10tol": int(within_10tol),
            "sampled_err_within_2x_oracle": int(within_2x_oracle), "max_err_over_tol": worst,
            "below_rank_cap": int(uncapped), "below_rank_cap_within_tol": int(unc_tol),
            "below_rank_cap_within_10tol": int(unc_10tol), "below_rank_cap_max_err_over_tol": worst_unc,
            "oracle_s": time.perf_counter() - t0,
            "selection": "every k-th of the last timed step's requests ordered by L d^2 maxbonddim^2"}


def dist_setup(world):
    """torch.distributed for N > 1 replicas (one process per GPU): NCCL when the
    ranks have GPUs, else gloo.  Returns None for a single process."""
    if world <= 1:
        return None
    import torch
    import torch.distributed as dist

    if not dist.is_initialized():
        dist.init_process_group(backend="nccl" if torch.cuda.is_available() else "gloo")
    return dist


def max_over_ranks(values, dist):
    """Elementwise maximum of a list of floats over all ranks (the slowest replica
    sets the whole-job time)."""
    if dist is None:
        return list(values)
    import torch

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor(list(values), dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.cpu()]


def barrier(dist):
    if dist is not None:
        import torch

        if dist.get_backend() == "nccl":
            torch.cuda.synchronize()
        dist.barrier()


def _best_of(fn, reps=3):
    best = None
    out = None
    for _ in range(reps):
        t0 = time.perf_counter()
        out = fn()
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return best, out


def large_rrlu_bench(T, ctx, peak_sep, with_cpu=True, n=2048, k=512):
    """One rank-revealing LU of a dense n x n Gaussian matrix (seed 3) to maxrank k
    on the multi-CTA kernel; FP64 rate of its rank-1 updates; the oracle on one
    host thread beside it."""
    import numpy as np

    A = np.random.default_rng(3).standard_normal((n, n))
    T.rrlu(A[:600, :600].copy(), maxrank=8, ctx=ctx)  # warm-up
    ctx.stats(reset=True)
    t, g = _best_of(lambda: T.rrlu(A, maxrank=k, ctx=ctx), reps=3)
    st = ctx.stats(reset=True)
    kern_s = st["kernel_ms"] / 3e3
    ops = 2.0 * sum((n - q) * (n - q) for q in range(1, k))
    out = {"workload": f"rrlu of a {n}x{n} N(0,1) matrix (seed 3), maxrank {k}, multi-CTA kernel",
           "e2e_s": t, "kernel_s": kern_s, "fp64_tflops": ops / kern_s / 1e12,
           "fp64_frac_of_measured": ops / kern_s / peak_sep}
    if with_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O

        tc, r = _best_of(lambda: O.rrlu(A, maxrank=k), reps=1)
        out.update(cpu_s=tc, cpu_threads=1,
                   same_pivots=bool(np.array_equal(g.rowpermutation - 1, r["rowpermutation"])))
    return out


def single_solve_configs(T, ctx, with_cpu=True):
    """The single-solve configurations, each on the GPU (plain path) and, as the
    baseline, by the oracle on one host thread: the 8-site Lorentzian, the R = 40
    quantics-1D function with a 1e6-point evaluation and its sum, the 30-site
    2-D quantics function and its zipup contraction with a seeded random
    operator (bond 64, 4 x 4 sites, N(0, 1/64) entries)."""
    import numpy as np

    O = None
    if with_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
    out = {}
    # 8-site Lorentzian, tol 1e-8, maxbonddim 200
    kw = dict(tolerance=1e-8, maxbonddim=200, maxiter=20)
    f = T.DeviceFunction("lorentz")
    t, (tci, ranks, _) = _best_of(lambda: T.crossinterpolate2(float, f, [10] * 8, ctx=ctx, **kw))
    c = {"gpu_s": t, "rank": int(tci.rank())}
    if O:
        tc, (ref, rr, _) = _best_of(lambda: O.crossinterpolate2([10] * 8, O.F_LORENTZ, [], None, **kw))
        c.update(cpu_s=tc, cpu_threads=1, same_ranks=list(rr) == list(ranks))
    out["lorentz8"] = c
    # the same solve with f supplied by the caller (numpy, evaluated on the host
    # for the points the device cache misses)
    def lorentz_np(p):
        return 1.0 / (1.0 + (p.astype(np.int64) ** 2).sum(1))

    counts = []

    def solve_batchfn():
        bf = T.BatchFunction(lorentz_np)
        res = T.crossinterpolate2(float, bf, [10] * 8, ctx=ctx, **kw)
        counts.append((bf.npoints, bf.ncalls))
        return res

    t, (tci_b, ranks_b, _) = _best_of(solve_batchfn)
    cb = {"gpu_s": t, "rank": int(tci_b.rank()), "same_ranks_as_device_f": list(ranks_b) == list(ranks),
          "f_points": counts[-1][0], "f_calls": counts[-1][1]}
    if O:
        cb["oracle_f_points"] = int(ref.nfeval)
    out["lorentz8_caller_f"] = cb
    # quantics 1-D, R = 40, tol 1e-10, maxbonddim 128; 1e6 seeded points
    kw = dict(tolerance=1e-10, maxbonddim=128, maxiter=20)
    f = T.DeviceFunction("qtt1d", [0])
    t, (tci, ranks, _) = _best_of(lambda: T.crossinterpolate2(float, f, [2] * 40, ctx=ctx, **kw))
    pts = np.random.default_rng(2024).integers(1, 3, size=(1000000, 40))
    te, vals = _best_of(lambda: tci.evaluate(pts), reps=2)
    ts, sm = _best_of(lambda: tci.sum(), reps=2)
    ctx.stats(reset=True)
    tse, vs = _best_of(lambda: tci.evaluate(pts, precision="tf32x3"), reps=2)
    st = ctx.stats(reset=True)
    c = {"gpu_s": t, "rank": int(tci.rank()), "eval_points": 1000000, "gpu_eval_s": te,
         "gpu_eval_points_per_s": 1e6 / te, "gpu_sum_s": ts,
         "split_eval": {"precision": "tf32x3 (TF32 hi/lo, 3 tensor-core products, FP32 accumulation)",
                        "e2e_s": tse, "points_per_s": 1e6 / tse, "kernel_ms": st["tc_ms"] / 2,
                        "max_rel_err_vs_fp64": float(np.abs(vs - vals).max() / np.abs(vals).max()),
                        "err_est_reported": tci.eval_err_est}}
    if O:
        tc, (ref, rr, _) = _best_of(lambda: O.crossinterpolate2([2] * 40, O.F_QTT1D, [0], None, **kw))
        sample = pts[:100000]
        tce, rv = _best_of(lambda: ref.evaluate(sample), reps=1)
        c.update(cpu_s=tc, cpu_threads=1, same_ranks=list(rr) == list(ranks), cpu_eval_points_per_s=1e5 / tce,
                 eval_max_abs_diff=float(np.abs(rv - vals[:100000]).max()))
    out["quantics1d_R40"] = c
    # 2-D quantics, 30 sites, d = 4, tol 1e-9, maxbonddim 512, then zipup contraction
    kw = dict(tolerance=1e-9, maxbonddim=512, maxiter=20)
    f = T.DeviceFunction("qtt2d")
    t, (tci, ranks, _) = _best_of(lambda: T.crossinterpolate2(float, f, [4] * 30, ctx=ctx, **kw))
    c = {"gpu_s": t, "rank": int(tci.rank())}
    if O:
        tc, (ref, rr, _) = _best_of(lambda: O.crossinterpolate2([4] * 30, O.F_QTT2D, [], None, **kw), reps=1)
        c.update(cpu_s=tc, cpu_threads=1, same_ranks=list(rr) == list(ranks))
    mps = T.tensortrains([tci], ctx=ctx)[0]
    rng = np.random.default_rng(55)
    bonds = [1] + [64] * 29 + [1]
    op = [rng.standard_normal((bonds[i], 4, 4, bonds[i + 1])) / 8.0 for i in range(30)]
    tz, res = _best_of(lambda: T.contract(op, mps, algorithm="zipup", tolerance=1e-9, maxbonddim=512, method="LU", ctx=ctx),
                       reps=1)
    ctx.stats(reset=True)
    tzs, res_s = _best_of(lambda: T.contract(op, mps, algorithm="zipup", tolerance=1e-9, maxbonddim=512, method="LU", ctx=ctx,
                                              precision="tf32x3"), reps=1)
    st = ctx.stats(reset=True)
    pts = rng.integers(1, 5, size=(20, 30))
    exact = np.array([_exact_mpo_mps(op, mps.sitetensors, p) for p in pts])
    scale = np.abs(exact).max()
    tc_tflops = st["tc_flops"] / (st["tc_ms"] * 1e-3) / 1e12 if st["tc_ms"] > 0 else None
    c.update(zipup_gpu_s=tz, zipup_rank=int(res.rank()),
             zipup_rel_err_20pts=float(np.abs(res.evaluate(pts, ctx=ctx) - exact).max() / scale),
             zipup_split={"precision": "tf32x3: both site contractions per site on the tensor cores, "
                                       "rrLU factorizations in FP64",
                          "gpu_s": tzs, "rank": int(res_s.rank()),
                          "rel_err_20pts": float(np.abs(res_s.evaluate(pts, ctx=ctx) - exact).max() / scale),
                          "products_err_est": res_s.err_est,
                          "tensor_kernel_ms": st["tc_ms"], "product_tflops": tc_tflops,
                          "tensor_pipe_tflops": 3 * tc_tflops if tc_tflops else None})
    out["quantics2d_30"] = c
    return out


def contract_tci_bench(T, ctx, maxbonddim=128):
    """contract(operator, mps; algorithm=:TCI) for the 2-D quantics configuration:
    the 30-site TCI result (tol 1e-9) under the seeded random operator (bond 64,
    4 x 4 sites, N(0, 1/64) entries), maxbonddim capped; the result checked
    against the zipup contraction at random points."""
    import numpy as np

    f = T.DeviceFunction("qtt2d")
    tci, _, _ = T.crossinterpolate2(float, f, [4] * 30, ctx=ctx, tolerance=1e-9, maxbonddim=512, maxiter=20)
    mps = T.tensortrains([tci], ctx=ctx)[0]
    rng = np.random.default_rng(55)
    bonds = [1] + [64] * 29 + [1]
    op = [rng.standard_normal((bonds[i], 4, 4, bonds[i + 1])) / 8.0 for i in range(30)]
    t0 = time.perf_counter()
    res = T.contract(op, mps, algorithm="TCI", tolerance=1e-9, maxbonddim=maxbonddim, ctx=ctx)
    t = time.perf_counter() - t0
    pts = rng.integers(1, 5, size=(20, 30))
    exact = np.array([_exact_mpo_mps(op, mps.sitetensors, p) for p in pts])
    got = res.evaluate(pts, ctx=ctx)
    return {"workload": f"contract(algorithm=:TCI) of the bond-64 operator with the 30-site 2-D quantics train "
                        f"(rank {int(tci.rank())}), tolerance 1e-9, maxbonddim {maxbonddim}",
            "gpu_s": t, "rank": int(res.rank()),
            "max_rel_err_20_points": float(np.abs(got - exact).max() / np.abs(exact).max())}


def tc_gemm_bench(T, ctx, M=16384, N=2048, K=1024, reps=3):
    """The split-precision tensor-core product alone on a large shape: C = A B
    with A (M x K), B (K x N) N(0, 1) (seed 5).  Device time of operand packing
    + tcgen05 GEMM from CUDA events (stats tc_ms), host copies excluded."""
    rng = np.random.default_rng(5)
    A = rng.standard_normal((M, K))
    B = rng.standard_normal((K, N))
    T.matmul(A[:256], B, precision="tf32x3", ctx=ctx)  # warm-up
    ctx.stats(reset=True)
    C = None
    for _ in range(reps):
        C, err = T.matmul(A, B, precision="tf32x3", ctx=ctx)
    st = ctx.stats(reset=True)
    ms = st["tc_ms"] / reps
    useful = 2.0 * M * N * K
    sub = slice(0, 512)
    rel = float((np.abs(C[sub] - A[sub] @ B) / (np.abs(A[sub]) @ np.abs(B))).max())
    meas = _measured_peaks()
    tf32_peak = meas.get("bf16_tflops", 1900.0) / 2 if meas else 950.0
    tensor = 3 * useful / (ms * 1e-3) / 1e12
    return {"workload": f"C = A B, A {M}x{K}, B {K}x{N}, FP64 in/out, TF32 hi/lo split (3 tensor-core products)",
            "kernel_ms": ms, "product_tflops": useful / (ms * 1e-3) / 1e12, "tensor_pipe_tflops": tensor,
            "tf32_peak_tflops": tf32_peak, "tensor_frac": tensor / tf32_peak,
            "tf32_peak_source": "half the measured bf16 dense peak (TF32 runs at half the BF16 rate)",
            "max_err_over_sum_abs": rel, "err_est": err}


def _measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _exact_mpo_mps(op, mps, p):
    """(op * mps)[p] by a left-to-right environment sweep on the host (1-based p)."""
    import numpy as np

    env = np.ones((1, 1))
    for n, (a, b) in enumerate(zip(op, mps)):
        env = np.einsum("ab,asc,bsd->cd", env, a[:, p[n] - 1, :, :], b, optimize=True)
    return float(env[0, 0])


def rrlu_batch_bench(T, ctx, peak_sep, with_cpu=True, reps=3):
    """The batched-rrLU configuration: 4096 matrices (2r)x(2r), r in [8, 128], seed 0,
    reltol 1e-10, maxrank 256, one launch.  Device time from CUDA events around the
    step kernel; e2e through tci_rrlu_batched with host buffers."""
    from tci_gb300 import workloads

    mats = workloads.rrlu_batch(4096, seed=0)
    nbytes = sum(a.size for a in mats) * 8
    T.rrlu_batched(mats[:64], maxrank=256, reltol=1e-10, ctx=ctx)  # warm-up

    def run():
        e2e, kern, ops, res = [], [], 0.0, None
        for _ in range(reps):
            ctx.stats(reset=True)
            t0 = time.perf_counter()
            res = T.rrlu_batched(mats, maxrank=256, reltol=1e-10, ctx=ctx)
            e2e.append(time.perf_counter() - t0)
            st = ctx.stats(reset=True)
            kern.append(st["kernel_ms"] * 1e-3)
            ops = 2.0 * st["lu_updates"]
        return res, float(np.median(kern)), e2e, ops

    tuned = ctx.tune_table()
    res, kt, e2e, ops = run()
    # the same launch with the kernel's fixed default for every bucket
    ctx.tune_table([0] * len(tuned))
    res_f, kt_f, _, _ = run()
    ctx.tune_table(tuned)
    same = all(np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[3] == b[3]
               for a, b in zip(res, res_f))
    out = {"workload": "4096 matrices (2r)x(2r), r uniform in [8,128] (seed 0), U diag(10^(-k/4)) V^T + 1e-12 "
                       "noise, reltol 1e-10, maxrank 256",
           "matrices_per_s_device": len(mats) / kt, "kernel_ms": kt * 1e3,
           "e2e_matrices_per_s": len(mats) / float(np.median(e2e)),
           "mean_npivot": float(np.mean([r[2] for r in res])),
           "fp64_tflops": ops / kt / 1e12, "fp64_frac_of_measured": ops / kt / peak_sep,
           "input_gb": nbytes / 1e9, "input_read_gbs": nbytes / kt / 1e9,
           "autotune": {"tuned_table": tuned, "fixed_kernel_ms": kt_f * 1e3, "tuned_over_fixed": kt_f / kt,
                        "same_pivots_and_errors": bool(same)}}
    if with_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O

        sub = mats[::16]
        t0 = time.perf_counter()
        O.rrlu_batched(sub, maxrank=256, reltol=1e-10)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": len(sub) / dt, "unit": "matrices/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": f"every 16th matrix ({len(sub)}), oracle rrlu on {os.cpu_count()} threads"}
    return out


def bench_config(args):
    """The `config` object of both arms' JSON lines."""
    return {"workload": f"served-stream family: {args.batch} crossinterpolate2 requests per step "
                        "(L 4..16, d 2..16, tol 1e-10..1e-6, maxbonddim 32..256), continuous batching "
                        f"with up to {args.live} live solves",
            "max_live": args.live, "global_batch": args.batch, "parallelism": f"replicas{args.gpus}",
            "requests": "step s draws its list from seed 1000*s + rank",
            "l2": "inputs are per-step index lists; Pi matrices stay on chip"}


def run_reference(args):
    """The reference's CPU path (the oracle port: Julia is absent) on the same
    seeded request lists as the GPU arm's steps: each step solves the first
    --ref-sample requests of that step's list on all host threads."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    sample = min(args.ref_sample, args.batch)
    step_s = []
    for s in range(args.warmup + args.steps):
        reqs = make_requests(args.batch, seed=step_seed(s, 0))
        n = 64 if s < args.warmup else sample  # warm-up steps: a short prefix
        dt, _ = oracle_solve(reqs[:n], cores)
        if s >= args.warmup:
            step_s.append(dt)
    total = sum(step_s)
    v = sample * args.steps / total
    desc = (f"the first {sample} of each timed step's {args.batch} requests (the GPU arm's seeded lists), "
            f"crossinterpolate2 by the C++ restatement of the reference on {cores} host threads")
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(args),
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=10000)
    ap.add_argument("--live", type=int, default=1024)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--ref-sample", type=int, default=2000,
                    help="requests of each step's list that the reference arm solves")
    ap.add_argument("--no-parity", action="store_true", help="skip the parity sample of the timed solves")
    ap.add_argument("--no-autotune", action="store_true", help="keep the kernel's fixed rrLU tail size")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-rrlu", action="store_true", help="skip the batched-rrLU sub-measurement")
    ap.add_argument("--no-single", action="store_true", help="skip the single-solve configurations")
    ap.add_argument("--no-sweep", action="store_true", help="skip the latency sweep over arrival rates")
    ap.add_argument("--only", default="", help="'rrlu': only the batched-rrLU configuration; 'big-rrlu': only the multi-CTA rrLU; "
                    "'contract-tci': only contract(algorithm=:TCI) of the 2-D quantics configuration; "
                    "'single': only the single-solve configurations; 'tc-gemm': only the tensor-core product")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import tci_gb300 as T

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    ctx = T.Context(int(os.environ.get("LOCAL_RANK", "0")))
    peak_sep, peak_fma = T.fp64_peak(ctx)
    if args.only == "rrlu":  # the batched-rrLU configuration alone (one warm-up launch, then --steps)
        if not args.no_autotune:
            ctx.autotune_rrlu()
        print(json.dumps(rrlu_batch_bench(T, ctx, peak_sep, with_cpu=False, reps=max(1, args.steps))))
        return
    if args.only == "big-rrlu":  # the multi-CTA rrLU alone
        print(json.dumps(large_rrlu_bench(T, ctx, peak_sep, with_cpu=not args.no_cpu)))
        return
    if args.only == "contract-tci":  # contract(algorithm=:TCI) of the 2-D quantics configuration alone
        print(json.dumps(contract_tci_bench(T, ctx)))
        return
    if args.only == "tc-gemm":  # the split-precision tensor-core product alone
        print(json.dumps(tc_gemm_bench(T, ctx)))
        return
    if args.only == "single":  # the single-solve configurations alone
        print(json.dumps(single_solve_configs(T, ctx, with_cpu=not args.no_cpu)))
        return
    if args.only == "served-step":  # one served batch (the first timed step's list), nothing else
        reqs = make_requests(args.batch, seed=step_seed(args.warmup, rank))
        specs = [(T.DeviceFunction("served", r[2]), [r[1]] * r[0], dict(tolerance=r[3], maxbonddim=r[4]))
                 for r in reqs]
        ctx.stats(reset=True)
        T.crossinterpolate2_batched(specs, max_live=args.live, ctx=ctx)
        st = ctx.stats(reset=True)
        print(json.dumps({"requests": len(specs), "fp64_ops": served_ops(st), "launches": st["launches"],
                          "kernel_ms": st["kernel_ms"]}))
        return

    def specs_for(step, tol_range=(-10.0, -6.0)):
        reqs = make_requests(args.batch, seed=step_seed(step, rank), tol_range=tol_range)
        return reqs, [(T.DeviceFunction("served", r[2]), [r[1]] * r[0],
                       dict(tolerance=r[3], maxbonddim=r[4])) for r in reqs]

    import ctypes

    lib = T.load_library()
    ev = None
    try:
        import torch  # only for CUDA events on the library's own stream

        ev = torch.cuda
        tstream = torch.cuda.ExternalStream(ctx.stream)
    except Exception:
        tstream = None

    # the autotuner: rrLU tail size per (rows, cols) bucket, calibrated on seeded
    # matrices before anything is timed; every later task of the context uses it
    tune = None
    if not args.no_autotune:
        t0 = time.perf_counter()
        sp, md, mt = ctx.autotune_rrlu()
        tune = {"calibration_speedup": sp, "calibration_ms_default": md, "calibration_ms_tuned": mt,
                "table": ctx.tune_table(), "calibration_s": time.perf_counter() - t0,
                "knob": "trailing-block size (elements) below which a factorization continues on one warp, "
                        "per (rows, cols) bucket"}

    # warm-up
    for s in range(args.warmup):
        _, specs = specs_for(s)
        T.crossinterpolate2_batched(specs, max_live=args.live, ctx=ctx)

    # timed: device throughput (events on the engine stream around each batch);
    # replicas: barrier + device sync on both sides, the slowest rank's time
    dist = dist_setup(world)
    barrier(dist)
    if tstream is not None:
        torch.cuda.synchronize()
    clocks = ClockSampler()
    clocks.start()
    ctx.stats(reset=True)
    dev_ms = []
    e2e_s = []
    h2d = d2h = 0
    nsolves = 0
    for s in range(args.steps):
        reqs, specs = specs_for(args.warmup + s)
        if tstream is not None:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(tstream)
        t0 = time.perf_counter()
        res = T.crossinterpolate2_batched(specs, max_live=args.live, ctx=ctx)
        if tstream is not None:
            e1.record(tstream)
            e1.synchronize()
            dev_ms.append(e0.elapsed_time(e1))
        # end to end: pull every result back to host memory
        st0 = ctx.stats()
        tts = T.tensortrains(res, ctx=ctx)
        ranks = [tt.rank() for tt in tts]
        e2e_s.append(time.perf_counter() - t0)
        nsolves += len(res)
        last_reqs, last_res = reqs, res
        del res
    if tstream is not None:
        torch.cuda.synchronize()
    barrier(dist)
    st = ctx.stats(reset=True)
    clk = clocks.stop()
    kernel_ms = st["kernel_ms"]
    total_dev_s = sum(dev_ms) / 1e3 if dev_ms else sum(e2e_s)
    total_dev_s, total_e2e_s = max_over_ranks([total_dev_s, sum(e2e_s)], dist)
    value = nsolves * world / total_dev_s
    e2e = nsolves * world / total_e2e_s
    ops = served_ops(st)
    # FP64 rate of the dominant kernel: the resident kernel's own lifetime
    # (CUDA events around each launch on its stream; one launch per batch)
    kern_s = kernel_ms / 1e3 if kernel_ms > 0 else total_dev_s
    achieved = ops / kern_s / 1e12 if kern_s > 0 else 0.0
    peak = peak_sep / 1e12

    # a seeded sample of the last timed step's solves against the oracle
    parity = None
    if rank == 0 and not args.no_parity:
        parity = parity_sample(T, last_res, last_reqs)
    del last_res

    # tuned over fixed on the served stream: one step's device time each
    if tune is not None and tstream is not None:
        def step_ms(table):
            ctx.tune_table(table)
            _, sp_ = specs_for(8888)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(tstream)
            T.crossinterpolate2_batched(sp_, max_live=args.live, ctx=ctx)
            e1.record(tstream)
            e1.synchronize()
            return e0.elapsed_time(e1)
        # interleaved (fixed, tuned) x 2, the faster of each
        fixed_ms, tuned_ms = 1e300, 1e300
        for _ in range(2):
            fixed_ms = min(fixed_ms, step_ms([0] * len(tune["table"])))
            tuned_ms = min(tuned_ms, step_ms(tune["table"]))
        ctx.tune_table(tune["table"])
        tune["served_step_ms_fixed"] = fixed_ms
        tune["served_step_ms_tuned"] = tuned_ms
        tune["served_tuned_over_fixed"] = fixed_ms / tuned_ms
        ctx.stats(reset=True)

    # the same family at tolerances 1e-10 .. 1e-8 only (the metric's error bar)
    _, specs_t = specs_for(7777, tol_range=(-10.0, -8.0))
    if tstream is not None:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(tstream)
    t0 = time.perf_counter()
    T.crossinterpolate2_batched(specs_t, max_live=args.live, ctx=ctx)
    tight_s = time.perf_counter() - t0
    if tstream is not None:
        e1.record(tstream)
        e1.synchronize()
        tight_s = e0.elapsed_time(e1) / 1e3
    tight = {"workload": f"{len(specs_t)} requests of the served family with tolerance log-uniform in "
                         "[1e-10, 1e-8]", "solves_per_s_device": len(specs_t) / tight_s}
    ctx.stats(reset=True)

    # plain one-at-a-time GPU path on a subset
    reqs, specs = specs_for(9999)
    nplain = min(64, len(specs))
    t0 = time.perf_counter()
    for f, dims, kw in specs[:nplain]:
        T.crossinterpolate2(float, f, dims, ctx=ctx, **kw)
    plain = nplain / (time.perf_counter() - t0)

    # latency under Poisson arrivals at 80% of the measured batched rate
    lam = 0.8 * e2e / world  # this replica's share
    rng = np.random.default_rng(77)
    nserve = min(2000, max(200, int(lam * 5)))
    reqs_s, specs_s = specs_for(5555)
    while len(specs_s) < nserve:
        specs_s = specs_s + specs_s
    specs_s = specs_s[:nserve]
    arrival = np.cumsum(rng.exponential(1.0 / lam, size=nserve))
    lat, rk, wall = T.serve(specs_s, arrival, ctx=ctx)
    # the served configuration's arrival rates: p50 / p99 latency at each
    sweep = []
    if not args.no_sweep:
        for rate in (50, 200, 500, 1000, 2000):
            n_r = int(min(2000, max(100, rate * 2.0)))
            arr_r = np.cumsum(np.random.default_rng(rate).exponential(1.0 / rate, size=n_r))
            sp = (specs_s * (n_r // len(specs_s) + 1))[:n_r]
            lat_r, _, wall_r = T.serve(sp, arr_r, ctx=ctx)
            sweep.append({"rate_per_s": rate, "requests": n_r, "p50_ms": float(np.percentile(lat_r, 50) * 1e3),
                          "p99_ms": float(np.percentile(lat_r, 99) * 1e3), "served_per_s": n_r / wall_r})

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(make_requests(args.batch, seed=step_seed(args.warmup, 0)),
                           what="the first timed step's list")
    rrlu_line = None if args.no_rrlu else rrlu_batch_bench(T, ctx, peak_sep, with_cpu=not args.no_cpu)
    single = None if args.no_single else single_solve_configs(T, ctx, with_cpu=not args.no_cpu)
    large = None if args.no_rrlu else large_rrlu_bench(T, ctx, peak_sep, with_cpu=not args.no_cpu)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": (total_dev_s * 1e3) / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(args),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": st["h2d_bytes"] // max(args.steps, 1),
                "d2h_bytes_per_step": st["d2h_bytes"] // max(args.steps, 1)},
        "gpu_launches": st["launches"],
        "plain_solves_per_s": plain,
        "batched_over_plain": e2e / world / plain,
        "serve_p50_ms": float(np.percentile(lat, 50) * 1e3), "serve_p99_ms": float(np.percentile(lat, 99) * 1e3),
        "serve_rate_per_s": lam,
        "serve_sweep": sweep,
        "tight_tolerance": tight,
        "autotune": tune,
        "parity_sample": parity,
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None,
                     "traffic": (SERVED_DRAM_BYTES_PER_OP * ops / args.steps
                                 if SERVED_DRAM_BYTES_PER_OP is not None else None),
                     "traffic_unit": "bytes per launch (one resident-kernel launch per step), scaled by FP64 "
                                     "operations from an ncu capture of the same task code as batched launches",
                     "peak_source": "measured FP64 mul+sub throughput (tci_fp64_peak), this run",
                     "fp64_fused_peak": peak_fma / 1e12},
        "kernel_ms_per_step": kernel_ms / args.steps,
        "clocks": clk,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    if rrlu_line:
        line["rrlu_batch"] = rrlu_line
    if single:
        line["single_solves"] = single
    if large:
        line["rrlu_large"] = large
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
