"""Test helpers: the CPU oracle port as a subprocess, golden fixtures, graphs."""
import hashlib
import json
import os
import subprocess
import tempfile

import numpy as np

from gspan_gb300 import datagen

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
PORT = os.path.join(ROOT, "oracle", "_port", "fsm_port")


def run_port(g, min_support, k, threads=None, with_stats=False, stream_last=False):
    """Pattern lines of the oracle port (timing line removed), optionally with
    its counts; stream_last counts the last level without materialising it."""
    env = dict(os.environ)
    if threads:
        env["OMP_NUM_THREADS"] = str(threads)
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "g.bin")
        g.save(path)
        args = ([PORT, path, str(min_support), str(k)] + (["--stats"] if with_stats else [])
                + (["--stream-last"] if stream_last else []))
        r = subprocess.run(args, capture_output=True, text=True, check=True, env=env)
    lines = r.stdout.splitlines()
    assert lines and lines[-1].startswith("load:")
    if with_stats:
        return lines[:-1], json.loads(r.stderr.strip().splitlines()[-1])
    return lines[:-1]


def golden_cases():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def large_golden_cases():
    """Full-size jobs pinned by the streaming oracle (tests/golden/make_golden.py --large)."""
    with open(os.path.join(GOLDEN, "large_manifest.json")) as f:
        return json.load(f)


def golden_graph(case):
    g = eval(case["graph"], {"datagen": datagen})
    assert hashlib.sha256(g.to_bytes()).hexdigest() == case["sha256"], "graph generator drifted"
    return g


def golden_lines(case):
    path = os.path.join(GOLDEN, case["expected"])
    if path.endswith(".gz"):
        import gzip
        with gzip.open(path, "rt") as f:
            return f.read().splitlines()
    with open(path) as f:
        return f.read().splitlines()


def lines_of(patterns):
    from gspan_gb300 import format_pattern
    return [format_pattern(c, s) for c, s in patterns]


def random_graphs():
    """Small seeded graphs over the corner cases the reference accepts."""
    out = []
    for seed in range(24):
        n = 6 + seed % 17
        m = 10 + (seed * 7) % 45
        out.append((f"mg{seed}", datagen.random_multigraph(n, m, 1 + seed % 4, 1 + seed % 3, 100 + seed,
                                                           self_loops=seed % 2 == 0), [(1, 3), (2, 4)]))
    for seed in range(8):
        out.append((f"er{seed}", datagen.erdos_renyi(80 + 9 * seed, 150 + 13 * seed, 2 + seed % 4, 200 + seed,
                                                     nelabels=1 + seed % 3), [(2, 4), (5, 3)]))
    for seed in range(4):
        out.append((f"cl{seed}", datagen.chung_lu(500, 1500, 2.1, 5, 1.0, 300 + seed, max_deg=60,
                                                  nelabels=1 + seed % 2), [(20, 3), (8, 4)]))
    return out


def numpy_prune(g, min_sup):
    """graph.cc:216-266: keep vertices whose label has >= min_sup vertices,
    renumber them in ascending order, keep entries between kept vertices in
    their original order."""
    labels, counts = np.unique(g.vlabels, return_counts=True)
    freq = dict(zip(labels.tolist(), counts.tolist()))
    keep = np.array([freq[int(x)] >= min_sup for x in g.vlabels], dtype=bool)
    new_id = np.cumsum(keep) - 1
    e = g.edges
    ek = keep[e[:, 0]] & keep[e[:, 1]] if len(e) else np.zeros(0, bool)
    edges = np.stack([new_id[e[ek, 0]], new_id[e[ek, 1]], e[ek, 2]], axis=1).astype(np.int32) \
        if ek.any() else np.zeros((0, 3), np.int32)
    deg = np.bincount(edges[:, 0], minlength=int(keep.sum())) if len(edges) else np.zeros(int(keep.sum()), int)
    offsets = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
    return datagen.CSR(offsets, g.vlabels[keep].astype(np.int32), edges)
