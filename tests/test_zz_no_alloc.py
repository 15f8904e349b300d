"""Tests of gbta_pobtaf_noalloc, the factorization for callers that cannot allocate
device memory when they factor (hosts with a fixed device-memory pool, loops that
cannot take cudaMalloc's implicit synchronisation); its scratch is a fixed 64 MiB
array inside the library.

The GPU tests compare it with gbta_pobtaf on two calls in a row and check that a call
after the first takes no device memory; a CPU test checks the task count behind
gbta_noalloc_scratch_bytes against the task list the kernel writes.  Collected last on
purpose: if a GPU test here fails, a run that stops at the first failure has already
run every other test.  Works alone in a fresh process and after the others.
"""
import ctypes

import numpy as np
import pytest

from oracle import bta_oracle as orc

RTOL = 1e-10
TS = 32


def relerr(x, y):
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


@pytest.fixture(scope="module")
def lib():
    from pyinla_gb300 import _lib, build

    build.build()
    return _lib.load()


@pytest.mark.gpu
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


@pytest.mark.gpu
def test_noalloc_rejects_oversized_problem(lib):
    from pyinla_gb300 import _lib

    D = ctypes.c_void_p(1)   # never dereferenced: the size check comes first
    code = lib.gbta_pobtaf_noalloc(3072, 256, 9, D, D, D, D, None)
    assert code == _lib.GBTA_ERR_ARG
    assert "scratch" in _lib.last_error()


@pytest.mark.gpu
def test_noalloc_reports_non_spd_row(lib):
    import torch

    from pyinla_gb300 import _lib
    from pyinla_gb300.device import current_stream_ptr

    D, L, R, T, _ = orc.make_bta_c1(34, nt=3, b=40, a=2)
    D[1][5, 5] = -10.0
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (D, L, R, T)]
    code = lib.gbta_pobtaf_noalloc(40, 3, 2, *[t.data_ptr() for t in dev], current_stream_ptr())
    assert code == 46, (code, _lib.last_error())


@pytest.mark.gpu
def test_noalloc_call_takes_no_device_memory(lib):
    """After the first call on the device (which loads the array), a call of a new
    geometry leaves the device's free memory unchanged."""
    import torch

    from pyinla_gb300 import _lib
    from pyinla_gb300.device import current_stream_ptr

    stream = current_stream_ptr()
    first = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in orc.make_bta_c1(35, nt=2, b=33, a=1)[:4]]
    assert lib.gbta_pobtaf_noalloc(33, 2, 1, *[t.data_ptr() for t in first], stream) == 0, _lib.last_error()
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in orc.make_bta_c1(36, nt=9, b=200, a=7)[:4]]
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    assert lib.gbta_pobtaf_noalloc(200, 9, 7, *[t.data_ptr() for t in dev], stream) == 0, _lib.last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 >= free0, (free0, free1)


def default_sep(nt):
    """Separator block of the solvers' elimination order (middle block for nt >= 3)."""
    return nt // 2 if nt >= 3 else nt - 1


def interleave(n1, n2, u):
    """(chain, index) of position u when n1 top-chain units and n2 bottom-chain units
    are interleaved one for one, the longer chain's rest last."""
    mn = min(n1, n2)
    if u < 2 * mn:
        return u & 1, u >> 1
    return (0 if n1 > mn else 1), mn + (u - 2 * mn)


def column_order(nt, B):
    """Block columns (i, c) in elimination order: both chains interleaved, then the
    separator block's columns."""
    sp = default_sep(nt)
    n1, n2 = sp * B, (nt - 1 - sp) * B
    out = []
    for u in range(n1 + n2):
        ch, k = interleave(n1, n2, u)
        out.append((k // B if ch == 0 else nt - 1 - k // B, k % B))
    return out + [(sp, c) for c in range(B)]


def plain_factor_tasks(nt, B, a):
    """The factorization task list without the feeder split, as (kind, i, r, c)."""
    sp = default_sep(nt)
    out = []
    for i, c in column_order(nt, B):
        out.append(("DIAG", i, c, c))
        out += [("OFFD", i, r, c) for r in range(c + 1, B)]
        if i != sp:
            out += [("LOW", i, r, c) for r in range(B)]
        if a > 0:
            out.append(("ARW", i, 0, c))
    if a > 0:
        out.append(("TIP", 0, 0, 0))
    return out


def kernel_column_offset(nt, B, a, q):
    """Offset of the q-th column's first task as k_gen_factor_tasks computes it."""
    ab = 1 if a > 0 else 0
    sp = default_sep(nt)
    n1, n2 = sp * B, (nt - 1 - sp) * B
    mn = min(n1, n2)

    def chain(n):   # tasks of the first n chain columns, f(c) = 2B + ab - c
        full, rem = divmod(n, B)
        fb = B * (2 * B + ab) - B * (B - 1) // 2
        return full * fb + rem * (2 * B + ab) - rem * (rem - 1) // 2

    if q < n1 + n2:
        _, k = interleave(n1, n2, q)
        c = k % B
        if q < 2 * mn:
            return 2 * chain(q >> 1) + ((2 * B + ab - c) if q & 1 else 0)
        return chain(mn) + chain(k)
    c = q - (n1 + n2)
    return chain(mn) + chain(n1 + n2 - mn) + c * (B + ab) - c * (c - 1) // 2


def align256(n):
    return (n + 255) // 256 * 256


@pytest.mark.parametrize("nt,b,a", [(1, 40, 0), (1, 70, 5), (6, 70, 0), (6, 70, 5), (3, 32, 1), (16, 128, 4),
                                    (2, 1, 0), (7, 33, 2), (9, 64, 0)])
def test_noalloc_task_count_and_offsets(lib, nt, b, a):
    """CPU: the kernel's per-column offsets tile the plain task list of the regular
    path's elimination order exactly (no gap, no overlap, TIP last), and
    gbta_noalloc_scratch_bytes sizes exactly that many tasks next to the control words,
    flags and tip partials."""
    B = (b + TS - 1) // TS
    tasks = plain_factor_tasks(nt, B, a)
    sp = default_sep(nt)
    pos = 0
    for q, (i, c) in enumerate(column_order(nt, B)):
        assert kernel_column_offset(nt, B, a, q) == pos, (q, i, c)
        assert tasks[pos] == ("DIAG", i, c, c)
        pos += 1 + (B - 1 - c) + (B if i != sp else 0) + (1 if a > 0 else 0)
    assert pos + (1 if a > 0 else 0) == len(tasks)
    nflags = (2 * nt - 1) * B * B + nt * B + 1
    want = align256(8 * 4) + align256(nflags * 4) + align256(len(tasks) * 16) + align256(nt * B * TS * TS * 8)
    assert lib.gbta_noalloc_scratch_bytes(b, nt, a) == want
