"""GPU test of gbta_pobtaf_noalloc, the factorization for callers that cannot allocate
device memory (its scratch is a fixed array inside the library).

Collected last on purpose: if it fails, a run that stops at the first failure has
already run every other test.  Works alone in a fresh process and after the others.
"""
import ctypes

import numpy as np
import pytest

from oracle import bta_oracle as orc

pytestmark = pytest.mark.gpu
RTOL = 1e-10


def relerr(x, y):
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


@pytest.fixture(scope="module")
def lib():
    from pyinla_gb300 import _lib, build

    build.build()
    return _lib.load()


@pytest.mark.parametrize("seed,nt,b,a", [(31, 6, 70, 5), (32, 1, 40, 0), (33, 16, 128, 4)])
def test_noalloc_matches_pobtaf_on_two_calls(lib, seed, nt, b, a):
    import torch

    from pyinla_gb300 import _lib
    from pyinla_gb300.device import BtaHandle, current_stream_ptr

    stream = current_stream_ptr()
    # reference result: the existing entry point
    D, L, R, T, _ = orc.make_bta_c1(seed, nt=nt, b=b, a=a)
    h = BtaHandle.get(b, nt, a)
    h.set_stream(stream)
    ref = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (D, L, R, T)]
    _lib.check(lib.gbta_pobtaf(h.ptr, *[t.data_ptr() for t in ref]))
    ref = [t.cpu().numpy() for t in ref]
    assert lib.gbta_noalloc_scratch_bytes(b, nt, a) <= (64 << 20)
    for call in range(2):   # two calls in a row share (and reuse) the fixed scratch
        Dn, Ln, Rn, Tn, _ = orc.make_bta_c1(seed, nt=nt, b=b, a=a)
        dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (Dn, Ln, Rn, Tn)]
        ptrs = [t.data_ptr() for t in dev]
        if a == 0:
            ptrs[2] = ptrs[3] = None
        code = lib.gbta_pobtaf_noalloc(b, nt, a, *ptrs, stream)
        assert code == 0, _lib.last_error()
        for got, want in zip(dev, ref):
            g = got.cpu().numpy()
            if want.size:
                assert relerr(g, want) < RTOL, call


def test_noalloc_rejects_oversized_problem(lib):
    from pyinla_gb300 import _lib

    D = ctypes.c_void_p(1)   # never dereferenced: the size check comes first
    code = lib.gbta_pobtaf_noalloc(3072, 256, 9, D, D, D, D, None)
    assert code == _lib.GBTA_ERR_ARG
    assert "scratch" in _lib.last_error()


def test_noalloc_reports_non_spd_row(lib):
    import torch

    from pyinla_gb300 import _lib
    from pyinla_gb300.device import current_stream_ptr

    D, L, R, T, _ = orc.make_bta_c1(34, nt=3, b=40, a=2)
    D[1][5, 5] = -10.0
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (D, L, R, T)]
    code = lib.gbta_pobtaf_noalloc(40, 3, 2, *[t.data_ptr() for t in dev], current_stream_ptr())
    assert code == 46, (code, _lib.last_error())
