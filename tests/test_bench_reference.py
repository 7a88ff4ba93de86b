"""bench.py's reference arm (--impl reference): the oracle port timed on the
host cores prints one JSON line with the engine arm's metric, unit and config
keys, a cpu_baseline describing the run, and an e2e object with no copies.
It needs no GPU."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def run(*args, env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *args],
                         capture_output=True, text=True, cwd=ROOT, env=env, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    return [json.loads(line) for line in out.stdout.splitlines() if line.startswith("{")]


def test_reference_arm_line():
    (line,) = run("--workload", "laplacian2d_256_AA", "--steps", "2", "--warmup", "1")
    assert line["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["unit"] == "GFLOPS" and line["higher_is_better"] is True
    assert line["steps"] == 2 and line["warmup"] == 1 and line["value"] > 0
    cfg = line["config"]
    assert cfg["workload"] == "laplacian2d_256_AA"
    assert cfg["n"] == 65536 and cfg["products"] == 1629192 and cfg["nnz_C"] == 846852
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_print_nothing():
    assert run("--workload", "laplacian2d_256_AA", "--steps", "1", "--warmup", "0", env_extra={"RANK": "1"}) == []


def test_reference_arm_batched_workload_is_unavailable():
    (line,) = run("--workload", "amg512_galerkin", "--steps", "1", "--warmup", "0")
    assert line["impl"] == "reference" and "unavailable" in line
