"""Two-level last step (opts.fused_last): the next-to-last level's embeddings
are generated from their parents' rows inside the last level's row pass
(k_mask_gen) instead of being stored.  Every line, support and count must be
the same as with stored rows: against the reference's goldens, the oracle on
random graphs, and the streaming oracle's full-size fixtures (the 100,000-vertex
headline job at 3 edges, and the 3.7M-vertex configuration scaled to 20,000
vertices at 4 edges)."""
import pytest

from helpers import golden_cases, golden_graph, golden_lines, large_golden_cases, lines_of, random_graphs, run_port

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fused():
    from gspan_gb300 import Miner
    with Miner(fused_last=2, profile=True) as m:
        yield m


@pytest.mark.parametrize("case", [c for c in golden_cases() if c["k"] >= 2],
                         ids=lambda c: f"{c['name']}-s{c['min_support']}-k{c['k']}")
def test_golden(fused, case):
    g = golden_graph(case)
    patterns, st = fused.fsm(g, case["k"], case["min_support"])
    assert lines_of(patterns) == golden_lines(case)
    _, ref = run_port(g, case["min_support"], case["k"], with_stats=True, stream_last=True)
    assert st["extended"] == ref["extended"]


@pytest.mark.parametrize("name,g,runs", random_graphs(), ids=lambda x: x if isinstance(x, str) else "")
def test_random_vs_oracle(fused, name, g, runs):
    dg = fused.upload(g)
    try:
        for sup, k in runs + [(runs[0][0], 4)]:
            patterns, st = fused.mine(dg, k, sup)
            ref, ref_st = run_port(g, sup, k, threads=4, with_stats=True, stream_last=True)
            assert lines_of(patterns) == ref, (name, sup, k)
            assert st["extended"] == ref_st["extended"], (name, sup, k)
    finally:
        fused.free(dg)


def test_generated_rows_are_counted(fused):
    """The next-to-last level really is generated (not stored) in this mode."""
    from gspan_gb300 import datagen
    g = datagen.chung_lu(2000, 6000, 2.1, 6, 1.0, 11, max_deg=120)
    _, st = fused.fsm(g, 3, 60)
    assert st["fused_rows"] > 0 and st["rows_launches"] > 0


@pytest.mark.parametrize("name", ["chung_lu_100k", "chung_lu_3_7m_scaled_20k"])
def test_full_size_fixture(fused, name):
    from gspan_gb300 import datagen
    case = [c for c in large_golden_cases() if c["name"] == name][0]
    g = eval(case["graph"], {"datagen": datagen})
    dg = fused.upload(g)
    try:
        patterns, st = fused.mine(dg, case["k"], case["min_support"])
    finally:
        fused.free(dg)
    assert lines_of(patterns) == golden_lines(case)
    assert st["extended"] == case["extended"] and st["seeds"] == case["seeds"]
    assert st["fused_rows"] > 0


def test_stored_and_generated_agree_at_four_edges():
    """The same 4-edge job with the next-to-last level stored and generated."""
    from gspan_gb300 import Miner, datagen
    case = [c for c in large_golden_cases() if c["name"] == "chung_lu_3_7m_scaled_20k"][0]
    g = eval(case["graph"], {"datagen": datagen})
    with Miner(fused_last=1) as m:
        stored, s1 = m.fsm(g, 4, 108)
    assert lines_of(stored) == golden_lines(case)
    assert s1["extended"] == case["extended"] and s1["fused_rows"] == 0
