"""The CPU oracle is pinned to the reference: its output must equal the golden
fixtures, which the reference itself produced (tests/golden/make_golden.py)."""
import os
import subprocess

import pytest

from helpers import ROOT, golden_cases, golden_graph, golden_lines, run_port
from gspan_gb300 import datagen

REF = os.path.join(ROOT, "oracle", "_ref", "fsm")


@pytest.mark.parametrize("case", golden_cases(), ids=lambda c: f"{c['name']}-s{c['min_support']}-k{c['k']}")
def test_port_matches_reference_golden(case):
    g = golden_graph(case)
    assert run_port(g, case["min_support"], case["k"], threads=4) == golden_lines(case)


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


def test_port_embedding_counts():
    """The port counts level-1 seeds and extension outputs like the reference's
    extend_omp (every directed edge with from-label <= to-label seeds)."""
    g = datagen.er_3300(0)
    _, st = run_port(g, 20, 3, threads=2, with_stats=True)
    fl = g.vlabels[g.edges[:, 0]]
    tl = g.vlabels[g.edges[:, 1]]
    assert st["seeds"] == int((fl <= tl).sum())
    assert st["extended"] > 0 and st["patterns"] == 966
