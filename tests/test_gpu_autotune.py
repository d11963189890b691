"""Autotuner: every option set gives the same result, and the chosen set mines
the same patterns as the defaults."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("make,sup", [("er", 20), ("cl", 300)], ids=["er_3300", "chung_lu_20k"])
def test_autotune_builtin_grid(make, sup):
    from gspan_gb300 import Miner, datagen
    g = datagen.er_3300(0) if make == "er" else datagen.chung_lu(20000, 80000, 2.1, 12, 1.0, 5, max_deg=400)
    with Miner() as m:
        dg = m.upload(g)
        want, _ = m.mine(dg, 3, sup)
        best, ms = m.autotune(dg, 3, sup, repeats=1)
    assert len(ms) == 6 and all(t > 0 for t in ms)
    with Miner(**best) as m2:
        assert m2.fsm(g, 3, sup)[0] == want


def test_autotune_batch_and_candidates():
    from gspan_gb300 import Miner, datagen
    graphs, sups = datagen.batch_instances(2, 8)
    with Miner() as m:
        bg = m.upload_batch(graphs)
        want, _ = m.mine_batch(bg, 3, sups)
        best, ms = m.autotune(bg, 3, sups, candidates=[{"path": 1}, {"path": 2}, {"mask_bias": 0.5}], repeats=1)
    assert len(ms) == 3
    with Miner(**best) as m2:
        got, _ = m2.mine_batch(m2.upload_batch(graphs), 3, sups)
    assert got == want


def test_autotune_rejects_bad_arguments():
    from gspan_gb300 import GspanError, Miner, datagen
    with Miner() as m:
        dg = m.upload(datagen.er_3300(0))
        with pytest.raises(GspanError):
            m.autotune(dg, 3, 20, ncand=0)
        with pytest.raises(ValueError):
            m.autotune(dg, 3, 20, candidates=[{"device": 1}])
