"""Serving: jobs submitted while others run overlap on the GPU; every result
must be the same alone and in the mix, and equal to the CPU oracle's."""
import random

import pytest

from helpers import lines_of, run_port

pytestmark = pytest.mark.gpu


def _pool():
    from gspan_gb300 import datagen
    graphs = [datagen.er_3300(s) for s in range(4)]
    graphs += [datagen.chung_lu(20000, 80000, 2.1, 12, 1.0, 40 + s, max_deg=400) for s in range(2)]
    graphs += [datagen.random_multigraph(20, 60, 3, 2, 50, self_loops=True)]
    return graphs


@pytest.mark.parametrize("slots,budget", [(4, 0.0), (2, 1.0)], ids=["4 slots", "budget forces one at a time"])
def test_results_same_alone_and_in_mix(slots, budget):
    from gspan_gb300 import Miner, Server
    graphs = _pool()
    rng = random.Random(9)
    jobs = []
    for _ in range(24):
        gi = rng.randrange(len(graphs))
        n = graphs[gi].n
        jobs.append((gi, rng.choice([2, 3, 4]) if n < 10000 else 3, max(1, int(n * rng.uniform(0.01, 0.05)))))
    with Server(slots=slots, budget_bytes=budget) as srv:
        ids = [srv.add_graph(g) for g in graphs]
        handles = [srv.submit(ids[gi], k, sup) for gi, k, sup in jobs]
        mixed = [srv.wait(h) for h in handles]
    with Miner() as m:
        alone = [m.fsm(graphs[gi], k, sup)[0] for gi, k, sup in jobs]
    for (got, info), want in zip(mixed, alone):
        assert got == want
        assert info["status"] == 0 and info["latency_ms"] >= info["run_ms"] >= 0
    # Served results against the oracle, one job per graph of the pool (the
    # oracle's 3-edge jobs on the 20,000-vertex graphs take seconds).
    checked = set()
    for (got, info), (gi, k, sup) in zip(mixed, jobs):
        if gi in checked:
            continue
        checked.add(gi)
        lines, st = run_port(graphs[gi], sup, k, with_stats=True, stream_last=True)
        assert lines_of(got) == lines, (gi, k, sup)
        assert info["stats"]["extended"] == st["extended"], (gi, k, sup)
    assert len(checked) >= 4


def test_bad_requests():
    from gspan_gb300 import GspanError, Server, datagen
    with Server(slots=1) as srv:
        gid = srv.add_graph(datagen.er_3300(0))
        with pytest.raises(GspanError):
            srv.submit(gid + 5, 3, 10)
        h = srv.submit(gid, 0, 10)            # k < 1: the job fails, the server goes on
        with pytest.raises(GspanError) as e:
            srv.wait(h)
        assert e.value.status == 1
        got, _ = srv.wait(srv.submit(gid, 2, 100))
        assert got


def test_out_of_memory_job_among_others():
    """A job too large for the device fails with NOMEM after its retry alone;
    the jobs around it are unaffected."""
    from gspan_gb300 import GspanError, Miner, Server, datagen
    small = datagen.er_3300(0)
    big = datagen.chung_lu_100k(1)
    with Miner() as m:
        want = m.fsm(small, 3, 20)[0]
    with Server(slots=3) as srv:
        gs_, gb = srv.add_graph(small), srv.add_graph(big)
        hs = [srv.submit(gs_, 3, 20) for _ in range(3)]
        hb = srv.submit(gb, 5, 1000)         # five-edge patterns at support 1,000: terabytes of embeddings
        hs += [srv.submit(gs_, 3, 20) for _ in range(3)]
        for h in hs:
            got, info = srv.wait(h)
            assert got == want and info["status"] == 0
        with pytest.raises(GspanError) as e:
            srv.wait(hb)
        assert e.value.status == 3
