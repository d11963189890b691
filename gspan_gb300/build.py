"""In-tree build of the CUDA library and command-line tools.

Produces, under ``gspan_gb300/_lib/``:
  * ``libgspan_gb300.so`` - the C ABI of include/gspan_gb300.h plus the C++
    drop-in surface of include/graph.h and include/gspan.h; CUDA code compiled
    for sm_103a only, CUDA runtime linked statically;
  * ``fsm`` and ``convert`` - the reference's two command-line programs.

Translation units compile in parallel; an object is rebuilt when its source or
any header under ``csrc/`` or ``include/`` is newer.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(HERE, "_lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libgspan_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["kernels.cu", "table_support.cu", "miner.cc", "capi.cc", "canonical.cc", "host_graph.cc",
           "host_fsm.cc", "graph_store.cc", "server.cc", "autotune.cc", "results.cc", "text_loader.cu", "prune.cu"]
TOOLS = {"fsm": "tools/fsm_main.cc", "convert": "tools/convert_main.cc"}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gspan_gb300")


def _headers_mtime() -> float:
    t = 0.0
    for d in (CSRC, INCLUDE):
        for name in os.listdir(d):
            if name.endswith((".h", ".cuh")):
                t = max(t, os.path.getmtime(os.path.join(d, name)))
    return t


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile everything that is out of date; returns the library path."""
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    hdr = _headers_mtime()
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp",
              f"-I{INCLUDE}", f"-I{CSRC}"] + ARCH
    cmds = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OBJ, src + ".o")
        objs.append(obj)
        if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(path), hdr):
            continue
        cmds.append([nvcc, *common, "-c", path, "-o", obj])
    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 2)) as ex:
        list(ex.map(_run, cmds))
    if cmds or not os.path.exists(LIB):
        _run([nvcc, "-shared", "-cudart", "static", *ARCH, "-Xcompiler", "-fopenmp", "-o", LIB, *objs])
    tool_cmds = []
    for name, src in TOOLS.items():
        exe = os.path.join(OUT, name)
        path = os.path.join(CSRC, src)
        if os.path.exists(exe) and os.path.getmtime(exe) >= max(os.path.getmtime(path), os.path.getmtime(LIB), hdr):
            continue
        tool_cmds.append([nvcc, "-O2", "-std=c++17", f"-I{INCLUDE}", path, "-o", exe, "-L" + OUT,
                          "-lgspan_gb300", "-Xlinker", "-rpath,$ORIGIN"])
    with ThreadPoolExecutor(max_workers=2) as ex:
        list(ex.map(_run, tool_cmds))
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
