"""bench.py on the CPU: the replica timing across ranks (gloo, world size 2):
the whole-job time is the slowest rank's, every rank sees the same result; and
the reference arm's JSON line."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    bench.barrier(dist)
    got = bench.max_over_ranks([1.0 + rank, 10.0 - 3 * rank], dist)
    bench.barrier(dist)
    out.put((rank, got))
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 2000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0] == res[1] == [2.0, 10.0]


def test_single_process_passthrough():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.dist_setup(1) is None
    assert bench.max_over_ranks([3.0, 4.0], None) == [3.0, 4.0]


def _run_bench(extra_env, *argv):
    import json
    import subprocess

    env = dict(os.environ, **extra_env)
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *argv], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    return [json.loads(ln) for ln in lines]


def test_reference_arm_line():
    """The reference arm (the oracle on the host cores, no GPU) prints one JSON
    line with the GPU arm's metric, unit and config, and its own cpu_baseline and
    e2e; under torchrun only rank 0 runs."""
    sys.path.insert(0, ROOT)
    import bench

    argv = ["--impl", "reference", "--steps", "1", "--warmup", "0", "--ref-sample", "12", "--batch", "48"]
    (line,) = _run_bench({"RANK": "0"}, *argv)
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] == 0
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert abs(line["value"] - 12 * 1e3 / line["ms_per_step"]) <= 1e-6 * line["value"]
    args = type("A", (), dict(batch=48, live=1024, gpus=1))
    assert line["config"] == bench.bench_config(args)
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert "first 12" in cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": bench.UNIT, "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert _run_bench({"RANK": "1"}, *argv) == []
