"""gspan_table_support_noalloc: the support step for callers that cannot let
the library allocate device memory (a fixed device-memory budget, a
latency-critical loop that cannot take cudaMalloc's synchronisation, or an
application that owns all device allocation).  Its scratch is an array built
into the library, so the test checks it against the allocating entry point,
gspan_table_support, through the C ABI, on two calls in a row: the second
call uses a smaller table than the first, so bits the first call left in the
shared array would show up if a call did not clear what it uses.

This file is collected last so that a run stopping at the first failure has
run every other test before it."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(cols, nr_nodes, stream):
    import torch
    from gspan_gb300 import _lib
    ptrs = (ctypes.c_void_p * len(cols))(*[c.data_ptr() for c in cols])
    out = torch.full((len(cols) + 1,), -7, dtype=torch.int32, device=cols[0].device)
    rc = _lib.gspan_table_support_noalloc(nr_nodes, ptrs, len(cols), int(cols[0].numel()), out.data_ptr(),
                                          ctypes.c_void_p(stream))
    return rc, out


def test_noalloc_matches_allocating_entry_point():
    import torch
    from gspan_gb300 import Miner
    rng = np.random.default_rng(11)
    stream = torch.cuda.current_stream().cuda_stream
    with Miner() as m:
        for n, ncols, nrows in [(120_000, 5, 400_000), (5_000, 3, 20_000)]:
            host = [rng.integers(0, n // (c + 1), size=nrows, dtype=np.int32) for c in range(ncols)]
            cols = [torch.from_numpy(h).cuda() for h in host]
            sizes, sup = m.table_support(cols, n)
            rc, out = _noalloc(cols, n, stream)
            torch.cuda.current_stream().synchronize()
            assert rc == 0
            got = [v & 0xFFFFFFFF for v in out.cpu().tolist()]
            assert got == sizes + [sup]
            assert sizes == [len(np.unique(h)) for h in host]


def test_noalloc_flags_a_bad_id_then_recovers():
    """An id outside [0, nr_nodes) sets out[ncols] to 0xFFFFFFFF (the call is
    asynchronous and cannot return it); the flag word lives in the shared
    array, so the next clean call must clear it and give the normal support."""
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    n = 1000
    good = [torch.arange(0, 300, dtype=torch.int32, device="cuda") % (c + 7) for c in range(3)]
    bad = [c.clone() for c in good]
    bad[1][17] = n                                   # one id equal to nr_nodes
    rc, out = _noalloc(bad, n, stream)
    torch.cuda.current_stream().synchronize()
    assert rc == 0 and (out[3].item() & 0xFFFFFFFF) == 0xFFFFFFFF
    rc, out = _noalloc(good, n, stream)
    torch.cuda.current_stream().synchronize()
    assert rc == 0 and [v & 0xFFFFFFFF for v in out.cpu().tolist()] == [7, 8, 9, 7]


def test_noalloc_empty_table():
    """nrows == 0: every domain is empty and the support is 0x7fffffff, even
    right after a call that left bits in the array."""
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    full = [torch.arange(0, 500, dtype=torch.int32, device="cuda") for _ in range(2)]
    rc, _ = _noalloc(full, 500, stream)
    assert rc == 0
    empty = [torch.empty(0, dtype=torch.int32, device="cuda") for _ in range(2)]
    rc, out = _noalloc(empty, 500, stream)
    torch.cuda.current_stream().synchronize()
    assert rc == 0 and out.cpu().tolist() == [0, 0, 0x7fffffff]


def test_noalloc_rejects_tables_beyond_its_array():
    import torch
    cols = [torch.zeros(4, dtype=torch.int32, device="cuda")] * 16
    rc, _ = _noalloc(cols, 5_000_000, torch.cuda.current_stream().cuda_stream)   # 16 x 156,250 words
    assert rc == 4   # GSPAN_ERR_LIMIT
