"""The C ABI and the C++ drop-in surface, without a GPU: exported symbols,
the loud no-GPU failure, and the host-side minimum-code test against the
oracle."""
import ctypes
import os
import random
import re
import subprocess

import pytest

from helpers import PORT, ROOT, golden_cases, golden_lines
import gspan_gb300 as gs

HEADER = os.path.join(ROOT, "include", "gspan_gb300.h")


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_every_declared_function_is_exported():
    decl = re.findall(r"^\s*(?:[\w\s\*]+?)\b(gspan_\w+)\s*\(", open(HEADER).read(), re.M)
    decl = sorted(set(d for d in decl if not d.endswith("_fn")))
    assert decl, "no declarations parsed"
    lib = ctypes.CDLL(gs.LIB_PATH)
    for name in decl:
        assert hasattr(lib, name), name
    assert sorted(gs.ABI_SYMBOLS) == decl


def test_cpp_dropin_symbols_are_exported():
    out = subprocess.run(["nm", "-D", "--defined-only", gs.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    for sym in ["_Z3fsmRK8CSRGraphii", "_ZN8CSRGraph4loadEPKc", "_ZN8CSRGraph4saveEPKc", "_ZN8CSRGraphC1ER5Graph",
                "_ZN5Graph8from_txtEPKc", "_Z11prune_graphR8CSRGraphRKS_i", "_ZNK9EmbVector8has_edgeERK4Edge"]:
        assert sym in out, sym


def test_status_strings_and_limits():
    assert gs._lib.gspan_status_string(0) == b"ok"
    assert gs._lib.gspan_status_string(7) == b"no CUDA device"
    assert gs.max_pattern_edges() == 15


@pytest.mark.skipif(_has_gpu(), reason="checks the behaviour without a GPU")
def test_no_gpu_fails_loudly(tmp_path):
    with pytest.raises(gs.GspanError) as e:
        gs.Miner()
    assert e.value.status == 7
    from gspan_gb300 import datagen
    path = tmp_path / "g.bin"
    datagen.er_3300(0).save(str(path))
    r = subprocess.run([os.path.join(ROOT, "gspan_gb300", "_lib", "fsm"), str(path), "50", "3"],
                       capture_output=True, text=True)
    assert r.returncode == 1
    assert "no CUDA device" in r.stderr
    assert r.stdout == ""          # nothing mined on the CPU


def _parse(line):
    body = line.rsplit(":", 1)[0]
    return [tuple(map(int, t.split())) for t in re.findall(r"\(([^)]*)\)", body)]


def test_reported_codes_are_canonical():
    for case in golden_cases():
        for line in golden_lines(case):
            assert gs.is_canonical(_parse(line)), line


def _random_code(rng, nedges, nlabels, nelabels):
    code = [(0, 1, rng.randrange(nlabels), rng.randrange(nelabels), rng.randrange(nlabels))]
    rm = [0, 1]           # rightmost path vertices, v0 .. v_n
    nv = 2
    for _ in range(nedges - 1):
        vn = rm[-1]
        back = [v for v in rm[:-2]]
        if back and rng.random() < 0.35:
            code.append((vn, rng.choice(back), -1, rng.randrange(nelabels), -1))
        else:
            src = rng.choice(rm)
            code.append((src, nv, -1, rng.randrange(nelabels), rng.randrange(nlabels)))
            rm = rm[:rm.index(src) + 1] + [nv]
            nv += 1
    return code


def test_canonical_matches_oracle():
    rng = random.Random(5)
    codes = []
    for _ in range(3000):
        codes.append(_random_code(rng, rng.randrange(1, 6), rng.randrange(1, 4), rng.randrange(1, 3)))
    inp = "".join(f"{len(c)} " + " ".join(" ".join(map(str, e)) for e in c) + "\n" for c in codes)
    out = subprocess.run([PORT, "--canonical"], input=inp, capture_output=True, text=True, check=True).stdout
    want = [x == "1" for x in out.split()]
    got = [gs.is_canonical(c) for c in codes]
    assert len(want) == len(codes)
    assert got == want
    assert 0 < sum(got) < len(got)


def test_is_canonical_rejects_malformed():
    with pytest.raises(gs.GspanError):
        gs.is_canonical([(0, 0, 1, 0, 1)])
