"""Label-frequency pruning inside the miner (opts.prune; the reference's
prune_graph, graph.cc:216-266, run on the device before mining).  Patterns and
supports must equal the unpruned run's (and the reference's goldens); the
extended count must equal the oracle's on the pruned graph."""
import pytest

from helpers import golden_cases, golden_graph, golden_lines, large_golden_cases, lines_of, numpy_prune, run_port

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", [c for c in golden_cases() if c["min_support"] > 1],
                         ids=lambda c: f"{c['name']}-s{c['min_support']}-k{c['k']}")
def test_pruned_mining_matches_golden(case):
    from gspan_gb300 import Miner
    g = golden_graph(case)
    with Miner(prune=True) as m:
        patterns, st = m.fsm(g, case["k"], case["min_support"])
    assert lines_of(patterns) == golden_lines(case)
    pruned = numpy_prune(g, case["min_support"])
    assert st["pruned_vertices"] == g.n - pruned.n and st["pruned_entries"] == g.m - pruned.m
    _, want = run_port(pruned, case["min_support"], case["k"], with_stats=True)
    assert st["extended"] == want["extended"] and st["seeds"] == want["seeds"]


def test_pruned_headline_job():
    """The 100,000-vertex graph at min support 10,000 and 3 edges: same lines
    as the full-size fixture, fewer extended embeddings."""
    from gspan_gb300 import Miner, datagen
    case = [c for c in large_golden_cases() if c["name"] == "chung_lu_100k"][0]
    g = datagen.chung_lu_100k(1)
    with Miner(prune=True) as m:
        dg = m.upload(g)
        patterns, st = m.mine(dg, 3, 10000)
        again, st2 = m.mine(dg, 3, 10000)
    assert lines_of(patterns) == golden_lines(case) and again == patterns
    assert st["pruned_vertices"] == g.n - numpy_prune(g, 10000).n
    assert 0 < st["extended"] < case["extended"] and st2["extended"] == st["extended"]


def test_nothing_to_prune_is_the_plain_run():
    from gspan_gb300 import Miner, datagen
    g = datagen.er_3300(0)
    with Miner(prune=True) as m:
        a, sa = m.fsm(g, 3, 1)
    with Miner() as m:
        b, sb = m.fsm(g, 3, 1)
    assert a == b and sa["pruned_vertices"] == 0 and sa["extended"] == sb["extended"]
