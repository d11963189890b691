"""Out of device memory is an ordinary error: the context stays usable and the
failed run gives back every device block it took."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu

_POOL_USED_MEM_CURRENT = 7      # CUmemPool_attribute: bytes of the pool handed out


def _pool_used_bytes(device=0):
    try:
        cu = ctypes.CDLL("libcuda.so.1")
    except OSError:
        return None
    pool = ctypes.c_void_p()
    if cu.cuDeviceGetDefaultMemPool(ctypes.byref(pool), ctypes.c_int(device)) != 0:
        return None
    v = ctypes.c_uint64()
    if cu.cuMemPoolGetAttribute(pool, ctypes.c_int(_POOL_USED_MEM_CURRENT), ctypes.byref(v)) != 0:
        return None
    return v.value


def test_out_of_memory_leaves_context_usable():
    import torch
    from gspan_gb300 import GSPAN_ERR_NOMEM, GspanError, Miner, datagen
    small = datagen.er_3300(0)
    big = datagen.chung_lu_100k(1)
    with Miner() as m:
        want = m.fsm(small, 3, 20)[0]
        dbig = m.upload(big)
        torch.cuda.synchronize()
        used0 = _pool_used_bytes()
        for _ in range(2):
            # Five-edge patterns at support 1,000: the stored three-edge table
            # alone would take terabytes (only the four-edge level is generated).
            with pytest.raises(GspanError) as e:
                m.mine(dbig, 5, 1000)
            assert e.value.status == GSPAN_ERR_NOMEM
            torch.cuda.synchronize()
            if used0 is not None:
                assert _pool_used_bytes() == used0
        assert m.fsm(small, 3, 20)[0] == want
        got, _ = m.mine(dbig, 3, 10000)
        assert len(got) > 0
        # What the failed runs freed is not kept from other processes.
        free_b, total_b = torch.cuda.mem_get_info()
        assert free_b > total_b // 2
