"""The headline job at full size (Chung-Lu 100,000 vertices / 1,080,000 edges,
min support 10,000, up to 3 edges).  The reference cannot run it: the
3-edge level has about 1.9e10 embeddings, which it materialises in host RAM.
Parity is pinned by the oracle port counting that level without storing it
(tests/golden/chung_lu_100k_s10000_k3.txt, made by make_golden.py --large; the
streaming mode equals the reference's own output on every small golden case):
  * every line, support included, and the extended-embedding count equal the
    fixture on each kernel path;
  * the patterns with at most 2 edges equal the oracle's run at k = 2, and the
    embedding counts of that run agree;
  * MNI support is anti-monotone: a child's support never exceeds its parent's;
  * repeated runs are identical."""
import pytest

from helpers import golden_lines, large_golden_cases, lines_of, run_port

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def graph():
    from gspan_gb300 import datagen
    return datagen.chung_lu_100k(1)


@pytest.fixture(scope="module")
def runs(graph):
    from gspan_gb300 import Miner
    out = {}
    for path in (0, 1, 2):
        with Miner(path=path) as m:
            dg = m.upload(graph)
            out[path] = [m.mine(dg, 3, 10000), m.mine(dg, 2, 10000)]
            m.free(dg)
    return out


def test_matches_streaming_oracle_fixture(runs):
    case = [c for c in large_golden_cases() if c["name"] == "chung_lu_100k" and c["k"] == 3][0]
    want = golden_lines(case)
    for path in (0, 1, 2):
        patterns, st = runs[path][0]
        assert lines_of(patterns) == want, f"path {path}"
        assert st["extended"] == case["extended"] and st["seeds"] == case["seeds"], f"path {path}"


def test_two_edge_prefix_matches_oracle(graph, runs):
    want, st = run_port(graph, 10000, 2, with_stats=True)
    (p3, _), (p2, s2) = runs[0]
    assert lines_of(p2) == want
    assert s2["extended"] == st["extended"] and s2["seeds"] == st["seeds"]
    assert [line for line in lines_of(p3) if line.count("(") <= 2] == want


def test_paths_agree(runs):
    for path in (1, 2):
        for j in (0, 1):
            assert runs[path][j][0] == runs[0][j][0]
            assert runs[path][j][1]["extended"] == runs[0][j][1]["extended"]
    assert runs[0][0][1]["extended"] == 19_419_741_293


def test_anti_monotone(runs):
    patterns, _ = runs[0][0]
    sup = {code: s for code, s in patterns}
    for code, s in patterns:
        if len(code) > 1:
            assert s <= sup[code[:-1]], code


def test_repeatable(graph, runs):
    from gspan_gb300 import Miner
    with Miner() as m:
        again, _ = m.fsm(graph, 3, 10000)
    assert again == runs[0][0][0]
