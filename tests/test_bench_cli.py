"""bench.py on the CPU: the workload list, and the reference arm (the CPU
implementation of the path), which needs no GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_workloads_listed():
    sys.path.insert(0, ROOT)
    import bench
    names = set(bench.workloads())
    assert {"chung_lu_100k", "chung_lu_100k_s15k", "chung_lu_3_7m", "chung_lu_3_7m_k4", "chung_lu_100k_wide",
            "er_3300"} <= names


def test_reference_arm_line():
    """Same job, metric and unit as the GPU arm: milliseconds per job at 3 edges,
    the last level timed in slices that add up to the whole job."""
    line = run_bench("--impl", "reference", "--workload", "er_3300", "--steps", "3", "--warmup", "1")
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "ms/job"
    assert line["higher_is_better"] is False and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["config"]["k"] == 3 and line["config"]["workload"] == "er_3300"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["extended_per_job"] == 91207   # the whole k = 3 job (tests/test_oracle.py)


def test_reference_arm_loads_no_native_library():
    """The reference arm never maps this repository's libgspan_gb300.so."""
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'er_3300', "
            "'--steps', '1', '--warmup', '0']; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); assert 'libgspan_gb300' not in maps, 'library mapped'")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]


def test_reference_arm_unavailable_where_the_port_cannot_run():
    line = run_bench("--impl", "reference", "--workload", "chung_lu_3_7m")
    assert line["impl"] == "reference" and "unavailable" in line


def test_hbm_peak_fallback(tmp_path, monkeypatch):
    """The roofline denominator comes from MEASURED_PEAKS.json when it is
    there and falls back to the earlier GB300 measurement, labelled, when not."""
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    peak, source = bench.hbm_peak()
    assert peak == 6800.0 and source.startswith("fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 7000.5}))
    peak, source = bench.hbm_peak()
    assert peak == 7000.5 and "measured" in source
