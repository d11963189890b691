"""Parity of the CUDA miner with the reference, through the C ABI.

Bit-exact: the pattern lines (codes, supports, order) must equal the
reference's (golden fixtures made by the reference itself) or the CPU oracle
port's, and the embedding counts must equal the oracle port's.
"""
import os
import subprocess
import tempfile

import pytest

from helpers import (ROOT, golden_cases, golden_graph, golden_lines, lines_of, random_graphs, run_port)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=[0, 1, 2], ids=["auto", "per-candidate", "mask"])
def miner(request):
    """One context per extension-kernel choice: automatic, per-candidate only,
    mask path wherever the label space allows.  All must agree bit for bit."""
    from gspan_gb300 import Miner
    m = Miner(path=request.param)
    yield m
    m.close()


@pytest.mark.parametrize("case", golden_cases(), ids=lambda c: f"{c['name']}-s{c['min_support']}-k{c['k']}")
def test_golden(miner, case):
    g = golden_graph(case)
    patterns, _ = miner.fsm(g, case["k"], case["min_support"])
    assert lines_of(patterns) == golden_lines(case)


@pytest.mark.parametrize("name,g,runs", random_graphs(), ids=lambda x: x if isinstance(x, str) else "")
def test_random_vs_oracle(miner, name, g, runs):
    dg = miner.upload(g)
    try:
        for sup, k in runs:
            patterns, st = miner.mine(dg, k, sup)
            ref, ref_st = run_port(g, sup, k, threads=4, with_stats=True)
            assert lines_of(patterns) == ref, (name, sup, k)
            assert st["seeds"] == ref_st["seeds"]
            assert st["extended"] == ref_st["extended"]
            assert st["patterns"] == ref_st["patterns"]
    finally:
        miner.free(dg)


@pytest.mark.parametrize("mode,thr", [(1, 1.0), (2, 1.0), (0, 1e9), (0, 1e-9)])
def test_domain_switch_same_supports(mode, thr):
    """Bitmap and hashset domains give identical supports on both sides of the switch."""
    from gspan_gb300 import Miner, datagen
    g = datagen.chung_lu(3000, 9000, 2.1, 5, 1.0, 77, max_deg=150)
    want = run_port(g, 40, 3, threads=4)
    with Miner(domain_mode=mode, hash_threshold=thr) as m:
        patterns, st = m.fsm(g, 3, 40)
    assert lines_of(patterns) == want
    if mode == 2 or thr > 1:
        assert st["hash_domains"] > 0
    if mode == 1 or thr < 1e-6:
        assert st["hash_domains"] == 0


def test_repeat_is_identical(miner):
    from gspan_gb300 import datagen
    g = datagen.er_3300(0)
    dg = miner.upload(g)
    try:
        a, sa = miner.mine(dg, 3, 20)
        b, sb = miner.mine(dg, 3, 20)
    finally:
        miner.free(dg)
    assert a == b
    assert sa["extended"] == sb["extended"]


def test_errors(miner):
    from gspan_gb300 import GspanError, datagen
    g = datagen.er_3300(0)
    dg = miner.upload(g)
    try:
        with pytest.raises(GspanError) as e:
            miner.mine(dg, 0, 10)
        assert e.value.status == 1
        with pytest.raises(GspanError) as e:
            miner.mine(dg, 16, 10)
        assert e.value.status == 4
    finally:
        miner.free(dg)
    bad = datagen.er_3300(0)
    bad.edges = bad.edges.copy()
    bad.edges[5, 0] += 1          # an entry whose `from` is not its vertex
    with pytest.raises(GspanError) as e:
        miner.upload(bad)
    assert e.value.status == 1
    bad2 = datagen.er_3300(0)
    bad2.edges = bad2.edges.copy()
    bad2.edges[7, 1] = 10 ** 6    # `to` out of range
    with pytest.raises(GspanError):
        miner.upload(bad2)


def test_fsm_cli_matches_golden():
    """The drop-in `fsm` program (graph.h loader + gspan.h fsm) prints the reference's lines."""
    case = [c for c in golden_cases() if c["name"] == "er3300" and c["min_support"] == 20][0]
    g = golden_graph(case)
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "g.bin")
        g.save(path)
        r = subprocess.run([os.path.join(ROOT, "gspan_gb300", "_lib", "fsm"), path, "20", "3"],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out = r.stdout.splitlines()
    assert out[-1].startswith("load:")
    assert out[:-1] == golden_lines(case)


def test_unsorted_adjacency_input(miner):
    """Adjacency lists not in (to, label) order take the rank-sort fallback of
    the upload; with one edge label the reference's output does not depend on
    that order."""
    import numpy as np
    from gspan_gb300 import datagen
    case = [c for c in golden_cases() if c["name"] == "er3300" and c["min_support"] == 50][0]
    g = golden_graph(case)
    rng = np.random.default_rng(3)
    edges = g.edges.copy()
    for v in range(g.n):
        b, e = g.offsets[v], g.offsets[v + 1]
        edges[b:e] = edges[b:e][rng.permutation(e - b)]
    shuffled = datagen.CSR(g.offsets, g.vlabels, edges)
    patterns, _ = miner.fsm(shuffled, case["k"], case["min_support"])
    assert lines_of(patterns) == golden_lines(case)


def test_wide_label_space(miner):
    """150 vertex labels x 2 edge labels (300 tuple keys): the upload ranks
    entries without the counting sort and the mask path uses its 16-word
    build; the output equals the oracle's on every kernel path."""
    from gspan_gb300 import datagen
    g = datagen.erdos_renyi(3000, 9000, 150, 41, nelabels=2)
    want, st = run_port(g, 3, 3, threads=4, with_stats=True)
    patterns, got = miner.fsm(g, 3, 3)
    assert lines_of(patterns) == want
    assert got["extended"] == st["extended"]


def test_wide_label_space_paths():
    """The mask path takes up to 512 tuple keys (16 mask words); beyond that
    only the per-candidate kernels run."""
    from gspan_gb300 import Miner, datagen
    g300 = datagen.erdos_renyi(3000, 9000, 150, 41, nelabels=2)
    g1k = datagen.erdos_renyi(4000, 12000, 330, 43, nelabels=3)
    with Miner(path=2) as m:
        p300, s300 = m.fsm(g300, 3, 3)
        p1k, s1k = m.fsm(g1k, 3, 2)
    assert s300["mask_parents"] > 0
    assert s1k["mask_parents"] == 0
    assert lines_of(p1k) == run_port(g1k, 2, 3, threads=4)


def test_fsm_cli_options():
    """Optional flags after the reference's three arguments: kernel path,
    domain representation, device-side text reading, JSON statistics."""
    import json
    from gspan_gb300 import datagen
    case = [c for c in golden_cases() if c["name"] == "er3300" and c["min_support"] == 20][0]
    g = golden_graph(case)
    fsm = os.path.join(ROOT, "gspan_gb300", "_lib", "fsm")
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "g.bin")
        g.save(path)
        txt = os.path.join(tmp, "g.txt")
        with open(txt, "w") as f:
            f.write(datagen.to_gspan_text(g))
        for args in (["--path", "candidate"], ["--path", "mask", "--domains", "bitmap"],
                     ["--domains", "hash", "--stats"], ["--text", "--stats"]):
            src = txt if "--text" in args else path
            r = subprocess.run([fsm, src, "20", "3", *args], capture_output=True, text=True)
            assert r.returncode == 0, (args, r.stderr)
            out = r.stdout.splitlines()
            assert out[-1].startswith("load:")
            assert out[:-1] == golden_lines(case), args
            if "--stats" in args:
                st = json.loads(r.stderr.strip().splitlines()[-1])
                assert st["patterns"] == len(out) - 1 and st["extended"] > 0
        r = subprocess.run([fsm, path, "20", "3", "--path", "fast"], capture_output=True, text=True)
        assert r.returncode == 1 and "--path" in r.stderr


def test_asymmetric_adjacency(miner):
    """A CSR whose entries lack their reverse (the text reader never makes one,
    but the C ABI accepts it): the symmetric shortcuts (entry columns, existence
    tests from the shorter side) are off; the output still equals the port's."""
    import numpy as np
    from gspan_gb300 import datagen
    rng = np.random.default_rng(11)
    n, m = 400, 2400
    u = rng.integers(0, n, m).astype(np.int32)
    v = rng.integers(0, n, m).astype(np.int32)
    el = rng.integers(0, 2, m).astype(np.int32)
    order = np.lexsort((el, v, u))
    u, v, el = u[order], v[order], el[order]
    offsets = np.zeros(n + 1, dtype=np.int32)
    np.add.at(offsets, u + 1, 1)
    offsets = np.cumsum(offsets).astype(np.int32)
    vlabels = rng.integers(0, 3, n).astype(np.int32)
    g = datagen.CSR(offsets, vlabels, np.stack([u, v, el], axis=1).astype(np.int32))
    want = run_port(g, 3, 3, threads=4)
    patterns, st = miner.fsm(g, 3, 3)
    assert lines_of(patterns) == want and len(want) > 0


@pytest.mark.parametrize("seed", range(6))
def test_deep_patterns(miner, seed):
    """Patterns of 5 and 6 edges (up to 7 pattern vertices): the row pass's
    general branches for more than 4 vertices, deep rightmost paths and many
    backward targets; the output equals the port's."""
    from gspan_gb300 import datagen
    g = datagen.random_multigraph(9 + seed, 18 + 3 * seed, 1 + seed % 2, 1 + seed % 2, 700 + seed,
                                  self_loops=seed % 3 == 0)
    dg = miner.upload(g)
    for sup, k in ((1, 5), (2, 6)):
        patterns, st = miner.mine(dg, k, sup)
        ref, ref_st = run_port(g, sup, k, threads=4, with_stats=True)
        assert lines_of(patterns) == ref, (seed, sup, k)
        assert st["extended"] == ref_st["extended"], (seed, sup, k)


@pytest.mark.parametrize("seed", range(3))
def test_wide_mask_build_deep(seed):
    """The row pass's 16-word build (129..512 tuple keys) at four edges, with
    parallel edges and self-loops, forced onto the mask path."""
    from gspan_gb300 import Miner, datagen
    g = datagen.random_multigraph(160 + 20 * seed, 700 + 60 * seed, 60, 3, 800 + seed, self_loops=True)
    ref, ref_st = run_port(g, 2, 4, threads=4, with_stats=True)
    with Miner(path=2) as m:
        patterns, st = m.fsm(g, 4, 2)
    assert st["mask_parents"] > 0
    assert lines_of(patterns) == ref and st["extended"] == ref_st["extended"]
