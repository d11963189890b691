"""The CPU oracle is pinned to the reference: its output must equal the golden
fixtures, which the reference itself produced (tests/golden/make_golden.py)."""
import os
import subprocess

import pytest

from helpers import ROOT, golden_cases, golden_graph, golden_lines, large_golden_cases, run_port
from gspan_gb300 import datagen

REF = os.path.join(ROOT, "oracle", "_ref", "fsm")


@pytest.mark.parametrize("case", golden_cases(), ids=lambda c: f"{c['name']}-s{c['min_support']}-k{c['k']}")
def test_port_matches_reference_golden(case):
    g = golden_graph(case)
    assert run_port(g, case["min_support"], case["k"], threads=4) == golden_lines(case)


@pytest.mark.parametrize("case", golden_cases(), ids=lambda c: f"{c['name']}-s{c['min_support']}-k{c['k']}")
def test_streamed_last_level_matches_reference_golden(case):
    """Counting the last level without storing it gives the reference's lines
    and the same extended-embedding count as materialising it."""
    g = golden_graph(case)
    lines, st = run_port(g, case["min_support"], case["k"], threads=4, with_stats=True, stream_last=True)
    assert lines == golden_lines(case)
    _, st_mat = run_port(g, case["min_support"], case["k"], threads=4, with_stats=True)
    assert (st["extended"], st["seeds"], st["support_calls"]) == \
        (st_mat["extended"], st_mat["seeds"], st_mat["support_calls"])


def test_streamed_last_level_at_headline_size():
    """The 100,000-vertex Chung-Lu graph at 2 edges (117M two-edge embeddings):
    streamed and materialised last levels agree on every line and count."""
    g = datagen.chung_lu_100k(1)
    a, sa = run_port(g, 10000, 2, with_stats=True)
    b, sb = run_port(g, 10000, 2, with_stats=True, stream_last=True)
    assert a == b and len(a) == 4
    assert sa["extended"] == sb["extended"] == 112_007_442


def test_shards_add_up():
    """Slices of a streamed last level add up to the whole level's count."""
    g = datagen.er_3300(0)
    _, whole = run_port(g, 20, 3, with_stats=True, stream_last=True)
    with __import__("tempfile").TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "g.bin")
        g.save(path)
        parts = []
        for i in range(3):
            r = subprocess.run([os.path.join(ROOT, "oracle", "_port", "fsm_port"), path, "20", "3", "--stats",
                                "--stream-last", "--shard", f"{i}/3"], capture_output=True, text=True, check=True)
            parts.append(__import__("json").loads(r.stderr.strip().splitlines()[-1]))
    _, upper = run_port(g, 20, 2, with_stats=True)
    last = whole["extended"] - upper["extended"]
    assert sum(p["extended"] - upper["extended"] for p in parts) == last


def test_large_fixtures_match_generator():
    """The full-size fixtures name the graph their generator still produces."""
    import hashlib
    for case in large_golden_cases():
        g = eval(case["graph"], {"datagen": datagen})
        assert hashlib.sha256(g.to_bytes()).hexdigest() == case["sha256"]
        assert len(golden_lines(case)) == case["patterns"]


@pytest.mark.parametrize("threads", [1, 3])
def test_port_is_thread_count_independent(threads):
    g = datagen.er_3300(0)
    case = [c for c in golden_cases() if c["name"] == "er3300" and c["min_support"] == 20][0]
    assert run_port(g, 20, 3, threads=threads) == golden_lines(case)


@pytest.mark.skipif(not os.path.exists(REF), reason="reference sources not present (oracle/_ref not built)")
@pytest.mark.parametrize("seed", range(6))
def test_port_matches_reference_binary(seed, tmp_path):
    """Where the reference compiled here, compare it with the port directly."""
    g = datagen.random_multigraph(12 + seed, 30 + 5 * seed, 3, 2, 900 + seed, self_loops=seed % 2 == 0)
    path = tmp_path / "g.bin"
    g.save(str(path))
    ref = subprocess.run([REF, str(path), "1", "4"], capture_output=True, text=True, check=True,
                         env={**os.environ, "OMP_NUM_THREADS": "2"}).stdout.splitlines()[:-1]
    assert run_port(g, 1, 4, threads=2) == ref
    assert run_port(g, 1, 4, threads=2, stream_last=True) == ref


def test_port_embedding_counts():
    """The port counts level-1 seeds and extension outputs like the reference's
    extend_omp (every directed edge with from-label <= to-label seeds)."""
    g = datagen.er_3300(0)
    _, st = run_port(g, 20, 3, threads=2, with_stats=True)
    fl = g.vlabels[g.edges[:, 0]]
    tl = g.vlabels[g.edges[:, 1]]
    assert st["seeds"] == int((fl <= tl).sum())
    assert st["extended"] > 0 and st["patterns"] == 966
