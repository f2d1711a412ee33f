"""CPU: bench.py's reference arm (the oracle port timed on host cores).

It prints one JSON line with the contract's keys and no host<->device bytes.
Under torchrun with two ranks (gloo here) rank 0 alone runs and prints it, and
the other rank exits 0 without work.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = {"impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
        "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"}


def _json_lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def _check(line):
    assert KEYS <= set(line)
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["higher_is_better"] is False
    assert line["cpu_baseline"]["kind"] in ("port", "reference")
    assert line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"]["L"] == 14


def test_reference_arm_single_process():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--L", "14", "--steps", "1",
                        "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    _check(lines[0])


def test_reference_arm_two_ranks():
    env = dict(os.environ, BENCH_BACKEND="gloo", OMP_NUM_THREADS="2")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", "29533", "bench.py", "--impl", "reference",
                        "--gpus", "2", "--L", "14", "--steps", "1", "--warmup", "0"],
                       cwd=ROOT, capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1
    _check(lines[0])


def test_cpu_baseline_sample_of_the_gpu_arm():
    """The GPU arm's cpu_baseline leg: the oracle port's table at a small width
    and a share of the product two sites below the target width, scaled by
    the 2^L*L work ratio (here to L=16 so it runs in seconds)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    sys.path.insert(0, ROOT)
    try:
        spec.loader.exec_module(bench)
        cpu = bench.cpu_baseline_sample(12, 46, L=16)
    finally:
        sys.path.remove(ROOT)
    assert set(cpu) == {"value", "unit", "cores", "kind", "sample"}
    assert cpu["value"] > 0 and cpu["unit"] == "s" and cpu["kind"] == "port" and cpu["cores"] >= 1
    assert "L=12" in cpu["sample"] and "46 products" in cpu["sample"] and "L=14" in cpu["sample"]
