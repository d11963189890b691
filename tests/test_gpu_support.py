"""MNI support of device-resident embedding tables (gspan_table_support), the
reference's support_gpu step, checked against distinct counts on the host and
against the miner's own 1-edge supports."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def miner():
    from gspan_gb300 import Miner
    m = Miner()
    yield m
    m.close()


@pytest.mark.parametrize("nrows,ncols,n", [(1, 1, 1), (1000, 2, 50), (100_000, 4, 100_000), (3_000_000, 5, 3_700_000),
                                           (77, 16, 64)])
def test_distinct_counts(miner, nrows, ncols, n):
    import torch
    rng = np.random.default_rng(nrows + ncols)
    host = [rng.integers(0, max(1, n // (c + 1)), size=nrows, dtype=np.int32) for c in range(ncols)]
    cols = [torch.from_numpy(h).cuda() for h in host]
    sizes, sup = miner.table_support(cols, n)
    want = [len(np.unique(h)) for h in host]
    assert sizes == want
    assert sup == min(want)


def test_empty_table(miner):
    import torch
    sizes, sup = miner.table_support([torch.empty(0, dtype=torch.int32, device="cuda")] * 3, 10)
    assert sizes == [0, 0, 0] and sup == 0x7FFFFFFF


def test_bad_id_rejected(miner):
    import torch
    from gspan_gb300 import GspanError
    with pytest.raises(GspanError):
        miner.table_support([torch.tensor([0, 5, 10], dtype=torch.int32, device="cuda")], 10)


def test_seed_tables_match_mined_supports(miner):
    """Tables of all 1-edge embeddings give the supports the miner reports."""
    import torch
    from gspan_gb300 import datagen
    g = datagen.er_3300(0)
    patterns, _ = miner.fsm(g, 1, 1)
    fl = g.vlabels[g.edges[:, 0]]
    tl = g.vlabels[g.edges[:, 1]]
    for code, sup in patterns:
        (_, _, a, el, b), = code
        sel = (fl == a) & (tl == b) & (g.edges[:, 2] == el)
        cols = [torch.from_numpy(np.ascontiguousarray(g.edges[sel, 0])).cuda(),
                torch.from_numpy(np.ascontiguousarray(g.edges[sel, 1])).cuda()]
        _, s = miner.table_support(cols, g.n)
        assert s == sup, code
