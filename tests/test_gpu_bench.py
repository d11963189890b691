"""bench.py on the GPU: the JSON line of the default job and of a small batch
carry the keys and units the measurement contract names."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                       timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_default_line():
    line = run_bench("--no-cpu-baseline", "--steps", "3", "--warmup", "3")
    assert line["unit"] == "ms/job" and line["higher_is_better"] is False
    assert line["value"] > 0 and line["ms_per_step"] == line["value"]
    assert line["config"]["workload"] == "chung_lu_100k" and line["config"]["k"] == 3
    assert line["e2e"]["unit"] == "ms/job" and line["e2e"]["value"] >= line["value"] * 0.5
    assert line["e2e"]["h2d_bytes_per_step"] > 0 and line["e2e"]["d2h_bytes_per_step"] > 0
    roof = line["roofline"]
    assert roof["bound"] == "hbm" and roof["unit"] == "GB/s" and 0 < roof["frac"] < 2
    assert abs(roof["frac"] - roof["achieved"] / roof["peak"]) < 1e-9
    assert line["gpu_launches"] > 0 and line["patterns"] == 9
    assert line["extended_per_step"] == 19419741293
    assert "sm_mhz" in line["clocks"]


def test_batch_line():
    """The batch workload reports milliseconds per batched job, the plain
    engine's time beside it, and their ratio."""
    line = run_bench("--workload", "batch_16", "--steps", "1", "--warmup", "1")
    assert line["unit"] == "ms/job" and line["higher_is_better"] is False
    assert line["value"] == line["ms_per_step"] > 0
    assert line["plain"]["unit"] == "ms/job" and line["plain"]["value"] > 0
    assert abs(line["batched_over_plain"] - line["plain"]["value"] / line["value"]) < 1e-9
    assert line["embeddings_per_s"]["batched"] > 0 and line["patterns"] > 0
