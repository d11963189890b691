import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA path")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Builds the native library (sm_103a) and the CPU oracle port once per session."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("gspan_gb300_build", os.path.join(ROOT, "gspan_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    yield
