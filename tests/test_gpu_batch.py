"""Batches: many independent mining instances in one device store, mined by
the same kernel launches.  Each instance's result must be exactly what mining
it alone gives (and what the oracle gives)."""
import numpy as np
import pytest

from helpers import lines_of, run_port

pytestmark = pytest.mark.gpu


def _instances():
    from gspan_gb300 import datagen
    gs_, sups = [], []
    for seed in range(6):
        gs_.append(datagen.random_multigraph(10 + seed, 25 + 4 * seed, 1 + seed % 3, 1 + seed % 2, 500 + seed,
                                             self_loops=seed % 2 == 0))
        sups.append(1 + seed % 2)
    for seed in range(4):
        gs_.append(datagen.erdos_renyi(200 + 40 * seed, 500 + 60 * seed, 3 + seed, 600 + seed, nelabels=1 + seed % 2))
        sups.append(4 + seed)
    gs_.append(datagen.chung_lu(1500, 5000, 2.1, 6, 1.0, 700, max_deg=80))
    sups.append(40)
    gs_.append(datagen.csr_from_edge_list(0, [], [], [], []))          # empty instance
    sups.append(1)
    gs_.append(datagen.csr_from_edge_list(3, [5, 6, 7], [], [], []))   # vertices only
    sups.append(1)
    return gs_, sups


@pytest.mark.parametrize("path", [0, 1, 2], ids=["auto", "per-candidate", "mask"])
def test_batch_equals_single_runs(path):
    from gspan_gb300 import Miner
    graphs, sups = _instances()
    with Miner(path=path) as m:
        bg = m.upload_batch(graphs)
        got, st = m.mine_batch(bg, 3, sups)
        ext = 0
        for i, (g, s) in enumerate(zip(graphs, sups)):
            want, st1 = m.fsm(g, 3, s)
            assert got[i] == want, i
            ext += st1["extended"]
        assert st["extended"] == ext


def test_batch_matches_oracle():
    from gspan_gb300 import Miner
    graphs, sups = _instances()
    with Miner() as m:
        got, _ = m.mine_batch(m.upload_batch(graphs), 4, sups)
    for i in (0, 3, 7, 10):
        assert lines_of(got[i]) == run_port(graphs[i], sups[i], 4, threads=4), i


def test_generated_batch_equals_single_runs():
    """The first 16 instances of the 256-instance workload (k = 3)."""
    from gspan_gb300 import Miner, datagen
    graphs, sups = datagen.batch_instances(2, 16)
    with Miner() as m:
        got, st = m.mine_batch(m.upload_batch(graphs), 3, sups)
        for i, (g, s) in enumerate(zip(graphs, sups)):
            assert got[i] == m.fsm(g, 3, s)[0], i
    assert st["patterns"] == sum(len(r) for r in got)


def test_edge_outside_its_instance_is_rejected():
    from gspan_gb300 import GspanError, Miner, datagen
    a = datagen.erdos_renyi(30, 60, 2, 1)
    b = datagen.erdos_renyi(30, 60, 2, 2)
    bad = datagen.CSR(b.offsets, b.vlabels, b.edges.copy())
    bad.edges[0, 1] = 45          # beyond instance b's 30 vertices
    with Miner() as m:
        with pytest.raises(GspanError) as e:
            m.upload_batch([a, bad])
        assert e.value.status == 1
        bg = m.upload_batch([a, b])
        with pytest.raises(GspanError):
            m.mine(bg, 2, 1)     # a batch is mined with mine_batch
        with pytest.raises(ValueError):
            m.mine_batch(bg, 2, [1])


def test_generated_last_level_in_a_batch():
    """A batch at 4 edges with the 3-edge level generated inside the 4-edge
    row pass (fused_last = 2): every instance equals the oracle, and the
    instances' windows keep generated rows apart."""
    from gspan_gb300 import Miner
    graphs, sups = _instances()
    with Miner(fused_last=2) as m:
        got, st = m.mine_batch(m.upload_batch(graphs), 4, sups)
    assert st["fused_rows"] > 0
    ext = 0
    for i, (g, s) in enumerate(zip(graphs, sups)):
        lines, ref = run_port(g, s, 4, threads=4, with_stats=True, stream_last=True)
        assert lines_of(got[i]) == lines, i
        ext += ref["extended"]
    assert st["extended"] == ext
