"""Both sweeps in one launch (gbta_pobtas trans = 2) and the selected inversion
overlapped with them (gbta_set_selinv_overlap).

The combined launch runs the same tile tasks as the forward and backward launches one
after the other, and the overlapped inversion the same pre-pass and product loops into a
workspace (written back afterwards) as the in-place one: results must be bit-identical
to the plain calls (the overlap is taken only while the sweeps are in flight, so the
stream is held by a short spin kernel first), and agree with the oracle (the reference's recurrence,
src/pyinla/solvers/structured_solver.py:83-190) at 1e-10.  b = 32 has one tile per block
row, where the flag array has no room for the second sweep's flags and trans = 2 falls
back to two launches.
"""
import numpy as np
import pytest

from oracle import bta_oracle as orc

pytestmark = pytest.mark.gpu
RTOL = 1e-10


def relerr(x, y):
    return float(np.max(np.abs(np.asarray(x) - np.asarray(y))) / max(np.max(np.abs(np.asarray(y))), 1e-300))


@pytest.fixture(scope="module")
def torch():
    import torch as _t

    from pyinla_gb300 import build

    build.build()
    return _t


def run(torch, D, L, R, T, rhs, b, nt, a, combined, overlap):
    from pyinla_gb300 import _lib
    from pyinla_gb300.device import BtaHandle

    h = BtaHandle(b, nt, a, True)
    h.set_selinv_overlap(overlap)
    lib = h.lib
    Dd, Ld, Rd, Td = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (D, L, R, T)]
    x = torch.from_numpy(np.ascontiguousarray(rhs)).cuda()
    nrhs = 1 if rhs.ndim == 1 else rhs.shape[1]
    Rp, Tp = (Rd.data_ptr(), Td.data_ptr()) if a else (None, None)
    # the inversion overlaps only sweeps that are still in flight when it is called:
    # hold the stream (a bounded spin kernel of ~10 ms) so that they are
    h.set_stream(torch.cuda.current_stream().cuda_stream)
    torch.cuda._sleep(20_000_000)
    _lib.check(lib.gbta_pobtaf_async(h.ptr, Dd.data_ptr(), Ld.data_ptr(), Rp, Tp))
    if a:
        if combined:
            _lib.check(lib.gbta_pobtas_async(h.ptr, Dd.data_ptr(), Ld.data_ptr(), Rp, Tp, x.data_ptr(), nrhs, 2))
        else:
            for tr in (0, 1):
                _lib.check(lib.gbta_pobtas_async(h.ptr, Dd.data_ptr(), Ld.data_ptr(), Rp, Tp, x.data_ptr(), nrhs, tr))
        _lib.check(lib.gbta_pobtasi(h.ptr, Dd.data_ptr(), Ld.data_ptr(), Rp, Tp))
    else:
        if combined:   # queued (the bt sweeps without the arrow), so that they are in flight
            _lib.check(lib.gbta_pobtas_async(h.ptr, Dd.data_ptr(), Ld.data_ptr(), None, None, x.data_ptr(), nrhs, 2))
        else:
            for tr in (0, 1):
                _lib.check(lib.gbta_pobts(h.ptr, Dd.data_ptr(), Ld.data_ptr(), x.data_ptr(), nrhs, tr))
        _lib.check(lib.gbta_pobtsi(h.ptr, Dd.data_ptr(), Ld.data_ptr()))
    h.status()
    out = [t.cpu().numpy() for t in (x, Dd, Ld, Rd, Td)]
    ws = h.workspace_bytes()
    h.close()
    return out, ws


@pytest.mark.parametrize("b,nt,a,nrhs", [(96, 6, 3, 1), (64, 5, 0, 1), (32, 5, 2, 1), (70, 4, 4, 6)])
def test_combined_sweeps_and_overlapped_inversion(torch, b, nt, a, nrhs):
    D, L, R, T, rhs = orc.make_bta_c1(7 + b, nt, b, a, nrhs)
    if not a:
        R, T = np.zeros((nt, 0, b)), np.zeros((0, 0))
        rhs = rhs[: nt * b]
    plain, ws_plain = run(torch, D, L, R, T, rhs, b, nt, a, combined=False, overlap=False)
    both, ws_both = run(torch, D, L, R, T, rhs, b, nt, a, combined=True, overlap=True)
    for got, want in zip(both, plain):
        assert np.array_equal(got, want)
    # the overlapped inversion ran (into its Sigma workspace; the plain one works in place)
    sig = 8 * (nt * b * b + (nt - 1) * b * b + nt * a * b + a * a)
    assert ws_both - ws_plain >= sig, (ws_both, ws_plain, sig)
    # against the oracle: solution and selected inverse
    Dn, Ln, Rn, Tn = [np.array(v, copy=True) for v in (D, L, R, T)]
    xo = np.array(rhs, copy=True)
    if a:
        orc.pobtaf(Dn, Ln, Rn, Tn)
        orc.pobtas(Dn, Ln, Rn, Tn, xo, "N")
        orc.pobtas(Dn, Ln, Rn, Tn, xo, "C")
        orc.pobtasi(Dn, Ln, Rn, Tn)
    else:
        orc.pobtf(Dn, Ln)
        orc.pobts(Dn, Ln, xo, "N")
        orc.pobts(Dn, Ln, xo, "C")
        orc.pobtsi(Dn, Ln)
    assert relerr(both[0], xo) < RTOL
    assert relerr(both[1], Dn) < RTOL
    if nt > 1:
        assert relerr(both[2], Ln) < RTOL
    if a:
        assert relerr(both[3], Rn) < RTOL
        assert relerr(both[4], Tn) < RTOL
