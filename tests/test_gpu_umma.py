"""The tcgen05 digit-plane tile step (tensor-memory accumulators) against the mma.sync
tile step: exact partial sums of every diagonal, every orientation and plane shift the
selected inversion uses, the FP64 fold bit for bit, and accumulation over two steps."""
import pytest

pytestmark = pytest.mark.gpu


def test_umma_tile_step_matches_mma_sync():
    from pyinla_gb300 import probes

    res = probes.umma_check(iters=64)
    assert all(v == 0 for v in res["mismatches"].values()), res
    assert res["cycles_per_step"]["tcgen05"] > 0
