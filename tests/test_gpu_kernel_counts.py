"""Issued tensor-core work of the dataflow kernels (gbta_kernel_pairs).

The tensor-core product loops leave out the products of structurally zero coupling
tiles (factorization) and of zero factor tiles and zero leading digit planes (selected
inversion), and count the 32 x 32 x 32 plane-pair products they issue.  With dense
couplings the factorization issues exactly the dense DAG's 43 pairs on every tile step;
with the banded couplings of an SPDE x AR(1) precision it issues fewer, and so does the
selected inversion.  The results are checked against the oracle either way.
"""
import ctypes

import numpy as np
import pytest

from oracle import bta_oracle as orc
from oracle import model_oracle as mo

pytestmark = pytest.mark.gpu
TS = 32


def dense_factor_steps(nt, b, a):
    """Tile steps of the factorization DAG without skipping: tile (r, c) of a diagonal
    block sums over its c own-block columns and the B columns of each neighbour
    eliminated before it (nt - 1 neighbour blocks in all, in either order); coupling
    tiles over their c own-block columns; arrow tiles over both."""
    B = (b + TS - 1) // TS
    steps = 0
    for i in range(nt):
        nprev = B if i > 0 else 0
        for c in range(B):
            steps += (nprev + c) * (1 + (B - 1 - c) + (1 if a else 0))
            if i < nt - 1:
                steps += c * B
    return steps


def run_counts(torch, D, L, R, T, b, nt, a):
    from pyinla_gb300 import _lib
    from pyinla_gb300.device import BtaHandle

    h = BtaHandle(b, nt, a, True)
    lib = h.lib
    Dd, Ld, Rd, Td = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (D, L, R, T)]
    _lib.check(lib.gbta_set_kernel_timing(h.ptr, 1))
    _lib.check(lib.gbta_pobtaf(h.ptr, Dd.data_ptr(), Ld.data_ptr(), Rd.data_ptr(), Td.data_ptr()))
    _lib.check(lib.gbta_pobtasi(h.ptr, Dd.data_ptr(), Ld.data_ptr(), Rd.data_ptr(), Td.data_ptr()))
    pairs = (ctypes.c_longlong * 2)()
    _lib.check(lib.gbta_kernel_pairs(h.ptr, pairs))
    ms = np.zeros(3)
    _lib.check(lib.gbta_kernel_ms(h.ptr, ms.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
    out = [x.cpu().numpy() for x in (Dd, Ld, Rd, Td)]
    _lib.check(lib.gbta_set_kernel_timing(h.ptr, 0))
    return int(pairs[0]), int(pairs[1]), ms, out


def check_sigma(out, D, L, R, T):
    Dn, Ln, Rn, Tn = [x.copy() for x in (D, L, R, T)]
    orc.pobtaf(Dn, Ln, Rn, Tn)
    orc.pobtasi(Dn, Ln, Rn, Tn)
    for got, want in zip(out, (Dn, Ln, Rn, Tn)):
        assert np.max(np.abs(got - want)) <= 1e-10 * np.max(np.abs(want))


@pytest.fixture(scope="module")
def torch():
    import torch as _t

    from pyinla_gb300 import build

    build.build()
    return _t


def test_dense_couplings_issue_the_dense_dag(torch):
    b, nt, a = 96, 5, 3
    D, L, R, T, _ = orc.make_bta_c1(3, nt, b, a)
    fp, sp, ms, out = run_counts(torch, D, L, R, T, b, nt, a)
    assert fp == 43 * dense_factor_steps(nt, b, a)
    assert 0 < sp
    assert ms[0] > 0 and ms[1] > 0
    check_sigma(out, D, L, R, T)


def test_banded_couplings_skip_zero_tiles(torch):
    from pyinla_gb300.model import SeparableSpdeAr1

    spec = SeparableSpdeAr1.synthetic(16, 6, 4, 6000, seed=7)
    c = spec.coefficients(spec.theta0)
    _, Qc, _ = mo.conditional_system(spec.terms, spec.term_vw, spec.ns, spec.nv, spec.nt, spec.nb, spec.A, spec.y,
                                     spec.tip_prec, c.alpha, c.beta, c.tau_y, spec.obs_variates())
    D, L, R, T = mo.sparse_to_bta(Qc, spec.nt, spec.b, spec.nb)
    b, nt, a = spec.b, spec.nt, spec.nb
    fp, sp, ms, out = run_counts(torch, D, L, R, T, b, nt, a)
    dense = 43 * dense_factor_steps(nt, b, a)
    print("factor pairs", fp, "of", dense, "; selinv pairs", sp)
    assert 0 < fp < dense
    assert 0 < sp
    check_sigma(out, D, L, R, T)
