"""bench.py's reference arm (CPU only): one JSON line with the GPU arm's
metric, unit and direction, the oracle timed solving the stream's own
requests with one worker process per host core (the excluded requests
listed), and no host<->device bytes."""

import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.timeout(300)
def test_reference_arm_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], capture_output=True, text=True, timeout=280, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["unit"] == "solves/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 0
    assert d["metric"].startswith("solves/s")
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port"
    assert cb["cores"] == (os.cpu_count() or 1)
    assert d["e2e"] == {"value": d["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("serving_stream_poisson")
    # measured, not extrapolated: the timed requests and the wall time that
    # gives the value are in the line, and the step time covers them
    assert cb["requests_in_sample"] > 0
    assert sum(cb["excluded"]["classes"].values()) == cb["excluded"]["requests"]
    assert cb["requests_in_sample"] + cb["excluded"]["requests"] == 60
    assert abs(d["ms_per_step"] * d["steps"] / 1000.0 - (os.cpu_count() or 1) / d["value"]) < 1e-6 * d["ms_per_step"]


def test_non_zero_rank_prints_nothing():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], capture_output=True, text=True, timeout=120, cwd=ROOT, env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    assert not [l for l in out.stdout.splitlines() if l.startswith("{")]
