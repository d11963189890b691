"""Device-side text loader: the same graph (and mining results) as the host
reader (Graph::from_txt + CSRGraph, the convert tool) on the same text."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from helpers import ROOT, golden_cases, golden_graph, golden_lines, lines_of

pytestmark = pytest.mark.gpu

CONVERT = os.path.join(ROOT, "gspan_gb300", "_lib", "convert")

ODD = (
    "t # 0\r\n"
    "v 10 3\n"
    "v -5 2\n"
    "v 10 1\n"                 # the last 'v' record of a vertex names its label
    "e 10 -5 0\n"
    "e 7 10 1\n"               # 7 is never declared: label 0
    "e 7 7 0\n"                # self-loop
    "e 10 -5 0\n"              # parallel edge
    "x junk words 12\n"        # skipped (no token starts with t, v or e)
    "t # 1\n"
    "v 1000000 2\n"
    "e 1000000 7 0\n"
    "\te\t-5\t7\t2\n"
    "t v 5\n"                  # 't' takes "v" and 5: no vertex record here
    "v 3 3 e 3 10 1\n"
)


def host_graph(text: str):
    from gspan_gb300 import datagen
    with tempfile.TemporaryDirectory() as tmp:
        src, dst = os.path.join(tmp, "g.txt"), os.path.join(tmp, "g.bin")
        with open(src, "w", newline="") as f:
            f.write(text)
        subprocess.run([CONVERT, src, dst], check=True, capture_output=True)
        return datagen.load_bin(dst)


def both(m, text, k=3, sup=1):
    g = host_graph(text)
    want, _ = m.fsm(g, k, sup)
    dg = m.upload_text(text)
    got, _ = m.mine(dg, k, sup)
    return g, dg, want, got


@pytest.fixture(scope="module")
def miner():
    from gspan_gb300 import Miner
    with Miner() as m:
        yield m


def test_golden_fixtures_through_text(miner):
    from gspan_gb300 import datagen
    for case in golden_cases():
        g = golden_graph(case)
        dg = miner.upload_text(datagen.to_gspan_text(g))
        assert (dg.n, dg.m) == (g.n, g.m), case["name"]
        got, _ = miner.mine(dg, case["k"], case["min_support"])
        assert lines_of(got) == golden_lines(case), case["name"]


def test_odd_text(miner):
    g, dg, want, got = both(miner, ODD)
    assert (dg.n, dg.m) == (g.n, g.m)
    assert got == want and len(want) > 0


@pytest.mark.parametrize("text", ["", "   \n\t \n", "v 5 1\n", "t # 0\nt # 1\nv 2 3\n"])
def test_edge_cases_like_the_host_reader(miner, text):
    g, dg, want, got = both(miner, text)
    assert (dg.n, dg.m) == (g.n, g.m)
    assert got == want


# Records that the reference's reader completes with the previous record's
# values (the host reader reproduces that, tests/test_formats.py); the device
# loader refuses them rather than read them differently.
MALFORMED = [
    "v 1 2\nv 2 2\ne 1 2 0\nv abc 3\ne 1 3 0\nv 3 2\n",     # a field that is not an integer
    "v 1 2\nv 2 2\ne 1 2 0\ne 1\n",                        # cut off by the end of the text
    "v 1 2 v 2 2 e 1 2 0 e 2 - 0 e 1 1 0",                 # a lone sign fails
    "t # x\nv 1 2\n",                                      # a 't' record's integer fails
]


@pytest.mark.parametrize("text", MALFORMED + ["v 12ab 3\n", "v 1 2\ne 1 99999999999 0\n",
                                              "v " + "7" * 70 + " 1\n", "xx" * 40 + " v 1 2\n"])
def test_refuses_what_a_token_parser_cannot_read_like_scanf(miner, text):
    from gspan_gb300 import GspanError
    with pytest.raises(GspanError) as e:
        miner.upload_text(text)
    assert e.value.status == 1


@pytest.mark.parametrize("seed", range(6))
def test_random_graphs_with_sparse_ids(miner, seed):
    """Random multigraphs written with shuffled, sparse, negative ids."""
    from gspan_gb300 import datagen
    rng = np.random.default_rng(seed)
    g = datagen.random_multigraph(40 + 10 * seed, 120 + 30 * seed, 3, 1 + seed % 2, 900 + seed, self_loops=True)
    ids = rng.choice(np.arange(-500, 100000), size=g.n, replace=False)
    lines = ["t # 0"]
    for v in rng.permutation(g.n):
        lines.append(f"v {ids[v]} {g.vlabels[v]}")
    for v in range(g.n):
        for j in range(g.offsets[v], g.offsets[v + 1]):
            u, w, lab = g.edges[j]
            if u <= w:
                lines.append(f"e {ids[u]} {ids[w]} {lab}")
    text = "\n".join(lines) + "\n"
    hg, dg, want, got = both(miner, text, k=3, sup=2)
    assert (dg.n, dg.m) == (hg.n, hg.m)
    assert got == want


def test_large_text_matches_host_csr(miner):
    """A 100k-vertex graph: the device-built graph mines like the uploaded CSR."""
    from gspan_gb300 import datagen
    g = datagen.chung_lu(100_000, 600_000, 2.1, 12, 1.0, 77, max_deg=800)
    dg = miner.upload_text(datagen.to_gspan_text(g))
    assert (dg.n, dg.m) == (g.n, g.m)
    want, _ = miner.mine(miner.upload(g), 3, 3000)
    got, _ = miner.mine(dg, 3, 3000)
    assert got == want
