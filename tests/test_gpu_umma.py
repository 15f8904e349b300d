"""The tcgen05 digit-plane tile step (tensor-memory accumulators) against the mma.sync
tile step: the FP64 fold bit for bit for every orientation and plane shift the
selected inversion uses, and accumulation over two steps."""
import pytest

pytestmark = pytest.mark.gpu


def test_umma_tile_step_matches_mma_sync():
    from pyinla_gb300 import probes

    res = probes.umma_check(iters=64)
    mis = dict(res["mismatches"])
    mis.pop("trans_swapped_offsets")   # the other descriptor layout, not used by the kernels
    assert all(v == 0 for v in mis.values()), res
    assert res["cycles_per_step"]["tcgen05"] > 0


def test_tensor_memory_ctas_share_an_sm():
    """Two CTAs with 256 tensor-memory columns each run on one SM at the same time,
    although the occupancy calculator reports one CTA per SM for such kernels; the
    grid rule for tensor-memory kernels (resident_ctas) counts two."""
    import numpy as np
    from pyinla_gb300 import _lib

    lib = _lib.load()
    out = np.zeros(5, dtype=np.int64)
    _lib.check(lib.gbta_probe_tmem_pairs(out.ctypes.data))
    assert out[2] > 0 and out[1] == out[2], out
    assert out[4] == 2, out
