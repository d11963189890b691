"""Label-frequency pruning (graph.cc:216-266, the reference's prune_graph,
which its CLI leaves commented out at fsm.cu:28-29), on the CPU.

The host surface's prune_graph is called through its C++ ABI (the way a C++
caller links it) and checked against a numpy restatement of the reference's
steps.  Then the property that makes pruning safe inside the miner: the oracle
mines the pruned graph to exactly the patterns and supports of the full graph
(a frequent pattern's images all carry labels with at least min_support
vertices, because MNI support never exceeds a label's vertex count)."""
import ctypes

import numpy as np
import pytest

from helpers import golden_cases, golden_graph, golden_lines, numpy_prune, run_port
from gspan_gb300 import datagen


class _CSRGraph(ctypes.Structure):
    # include/graph.h CSRGraph: int nr_nodes, nr_edges; int *offsets, *vlabels; Edge* edges.
    _fields_ = [("nr_nodes", ctypes.c_int), ("nr_edges", ctypes.c_int), ("offsets", ctypes.POINTER(ctypes.c_int)),
                ("vlabels", ctypes.POINTER(ctypes.c_int)), ("edges", ctypes.POINTER(ctypes.c_int))]


def host_prune(g, min_sup):
    import gspan_gb300 as gs
    lib = ctypes.CDLL(gs.LIB_PATH)
    fn = getattr(lib, "_Z11prune_graphR8CSRGraphRKS_i")
    fn.argtypes = [ctypes.POINTER(_CSRGraph), ctypes.POINTER(_CSRGraph), ctypes.c_int]
    fn.restype = None
    off = np.ascontiguousarray(g.offsets, dtype=np.int32)
    vl = np.ascontiguousarray(g.vlabels, dtype=np.int32)
    ed = np.ascontiguousarray(g.edges, dtype=np.int32).reshape(-1)
    src = _CSRGraph(g.n, g.m, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                    vl.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), ed.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    out = _CSRGraph(0, 0, None, None, None)
    fn(ctypes.byref(out), ctypes.byref(src), min_sup)
    n, m = out.nr_nodes, out.nr_edges
    # The arrays were made with new[] by the library; copied out and left to the process.
    return datagen.CSR(np.ctypeslib.as_array(out.offsets, shape=(n + 1,)).copy(),
                       np.ctypeslib.as_array(out.vlabels, shape=(n,)).copy() if n else np.zeros(0, np.int32),
                       np.ctypeslib.as_array(out.edges, shape=(m * 3,)).reshape(m, 3).copy()
                       if m else np.zeros((0, 3), np.int32))


CASES = [("er3300", "datagen.er_3300(0)", [300, 200, 50, 20]),
         ("cl_2k", "datagen.chung_lu(2000, 6000, 2.1, 6, 1.0, 11, max_deg=120)", [150, 60]),
         ("multigraph_loops", "datagen.random_multigraph(30, 80, 3, 2, 21, self_loops=True)", [1, 2, 9]),
         ("negative_labels", "datagen.csr_from_edge_list(6, [-5,7,-5,100,7,-5], [0,1,2,3,4,5], [1,2,3,4,5,0], "
                             "[-2,9,-2,9,-2,9])", [1, 2, 3])]


@pytest.mark.parametrize("name,expr,sups", CASES, ids=[c[0] for c in CASES])
def test_host_prune_graph_matches_reference_steps(name, expr, sups):
    g = eval(expr, {"datagen": datagen})
    for sup in sups:
        got, want = host_prune(g, sup), numpy_prune(g, sup)
        assert np.array_equal(got.offsets, want.offsets), sup
        assert np.array_equal(got.vlabels, want.vlabels), sup
        assert np.array_equal(got.edges, want.edges), sup


@pytest.mark.parametrize("case", [c for c in golden_cases() if c["min_support"] > 1],
                         ids=lambda c: f"{c['name']}-s{c['min_support']}-k{c['k']}")
def test_pruned_graph_mines_to_the_same_patterns(case):
    g = golden_graph(case)
    pruned = numpy_prune(g, case["min_support"])
    lines, st = run_port(pruned, case["min_support"], case["k"], threads=4, with_stats=True)
    assert lines == golden_lines(case)
    _, full = run_port(g, case["min_support"], case["k"], threads=4, with_stats=True)
    assert st["extended"] <= full["extended"]


def test_headline_graph_prunes_most_vertices():
    """100,000-vertex Chung-Lu graph at min support 10,000: only two of the 29
    Zipf labels have that many vertices; the 2-edge job is unchanged."""
    g = datagen.chung_lu_100k(1)
    pruned = numpy_prune(g, 10000)
    assert pruned.n < 0.4 * g.n and len(set(pruned.vlabels.tolist())) == 2
    a, sa = run_port(g, 10000, 2, with_stats=True, stream_last=True)
    b, sb = run_port(pruned, 10000, 2, with_stats=True, stream_last=True)
    assert a == b and sb["extended"] < sa["extended"]
