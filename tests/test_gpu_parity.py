"""GPU parity of the BTA kernels against the reference's own results and the oracle.

* golden fixtures (tests/golden/*.npz, made by the reference's DenseSolver and its
  SerinvSolver wrapper) pin logdet, solution and selected-inverse blocks;
* the oracle (oracle/bta_oracle.py) covers shapes without fixtures.

Tolerance: 1e-10 relative in FP64 (max-abs error over max-abs value).
"""
import ctypes

import numpy as np
import pytest

from oracle import bta_oracle as orc
from tests.conftest import GOLDEN
from tests.golden.make_golden import checksum

pytestmark = pytest.mark.gpu
RTOL = 1e-10


def relerr(x, y):
    x = np.asarray(x)
    y = np.asarray(y)
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


@pytest.fixture(scope="module")
def torch():
    import torch as _t

    from pyinla_gb300 import build

    build.build()
    return _t


METHODS = [0, 1]   # GBTA_METHOD_FP64, GBTA_METHOD_OZAKI


@pytest.fixture
def use_method(torch):
    """Set the product method of the cached solver handles the algs drop-ins use (in
    their current elimination order) for one test."""
    from pyinla_gb300 import algs
    from pyinla_gb300.device import BtaHandle

    touched = []

    def _set(b, nt, a, method):
        h = BtaHandle.get(b, nt, a, algs._TWIST)
        touched.append((h, h.method()))
        h.set_method(method)

    yield _set
    for h, m in touched:
        h.set_method(m)


TWIST = [False, True]   # Serinv's top-down order; both ends towards the middle block


@pytest.fixture
def order(torch):
    """Run the algs drop-ins in the given elimination order for one test."""
    from pyinla_gb300 import algs

    def _set(twisted):
        algs.set_twisted(twisted)

    yield _set
    algs.set_twisted(False)


def dev(torch, *arrs):
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]


def host(t):
    return t.cpu().numpy()


GOLDEN_CASES = ["tiny", "ragged", "single", "two", "c1"]


def _golden(name):
    g = np.load(GOLDEN / f"bta_{name}.npz")
    D, L, R, T, rhs = orc.make_bta_c1(int(g["seed"]), nt=int(g["nt"]), b=int(g["b"]), a=int(g["a"]))
    np.testing.assert_allclose(checksum(D, L, R, T, rhs), g["input_checksum"], rtol=1e-13, atol=0)
    return g, D, L, R, T, rhs


@pytest.mark.parametrize("twisted", TWIST)
@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_bta_against_reference_golden(torch, use_method, order, name, method, twisted):
    from pyinla_gb300 import algs

    order(twisted)
    g, D, L, R, T, rhs = _golden(name)
    use_method(int(g["b"]), int(g["nt"]), int(g["a"]), method)
    Dd, Ld, Rd, Td = dev(torch, D, L, R, T)
    algs.pobtaf(Dd, Ld, Rd, Td)
    ld = algs.logdet(Dd, Td, "bta")
    assert abs(ld - float(g["dense_logdet"])) <= RTOL * abs(float(g["dense_logdet"]))
    for i in range(D.shape[0]):   # factor's strict upper triangle is exactly zero
        assert np.all(np.triu(host(Dd[i]), 1) == 0.0)
    x = torch.from_numpy(rhs.copy()).cuda()
    algs.pobtas(Dd, Ld, Rd, Td, x, "N")
    algs.pobtas(Dd, Ld, Rd, Td, x, "C")
    assert relerr(host(x), g["dense_x"]) < RTOL
    algs.pobtasi(Dd, Ld, Rd, Td)
    SD, SL, SR, ST = map(host, (Dd, Ld, Rd, Td))
    if "dense_SD" in g:
        assert relerr(SD, g["dense_SD"]) < RTOL
        if D.shape[0] > 1:
            assert relerr(SL, g["dense_SL"]) < RTOL
    else:
        assert relerr(SD[0], g["dense_SD_first"]) < RTOL
        assert relerr(SD[-1], g["dense_SD_last"]) < RTOL
        assert relerr(SL[0], g["dense_SL_first"]) < RTOL
        assert relerr(SL[-1], g["dense_SL_last"]) < RTOL
        diag = np.concatenate([np.diagonal(SD[i]) for i in range(SD.shape[0])] + [np.diagonal(ST)])
        assert relerr(diag, g["dense_Sdiag"]) < RTOL
    assert relerr(SR, g["dense_SR"]) < RTOL
    assert relerr(ST, g["dense_ST"]) < RTOL
    # D and T of Sigma are full symmetric
    assert np.array_equal(SD, np.transpose(SD, (0, 2, 1)))
    assert np.array_equal(ST, ST.T)


@pytest.mark.parametrize("twisted", TWIST)
@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_bt_against_reference_golden(torch, use_method, order, name, method, twisted):
    from pyinla_gb300 import algs

    order(twisted)
    g, D, L, R, T, rhs = _golden(name)
    use_method(int(g["b"]), int(g["nt"]), 0, method)
    nt, b = D.shape[0], D.shape[1]
    Dd, Ld = dev(torch, D, L)
    algs.pobtf(Dd, Ld)
    ld = algs.logdet(Dd, None, "bt")
    assert abs(ld - float(g["dense_bt_logdet"])) <= RTOL * abs(float(g["dense_bt_logdet"]))
    x = torch.from_numpy(rhs[: nt * b].copy()).cuda()
    algs.pobts(Dd, Ld, x, "N")
    algs.pobts(Dd, Ld, x, "C")
    assert relerr(host(x), g["dense_bt_x"]) < RTOL
    algs.pobtsi(Dd, Ld)
    if "dense_bt_SD" in g:
        assert relerr(host(Dd), g["dense_bt_SD"]) < RTOL
        if nt > 1:
            assert relerr(host(Ld), g["dense_bt_SL"]) < RTOL
    else:
        diag = np.concatenate([np.diagonal(host(Dd[i])) for i in range(nt)])
        assert relerr(diag, g["dense_bt_Sdiag"]) < RTOL


SHAPES = [
    # (seed, nt, b, a): ragged tiles, single block, a = 0, a = TS, b < TS, b = k*TS
    (21, 5, 96, 6),
    (22, 3, 100, 1),
    (23, 1, 64, 0),
    (24, 6, 31, 32),
    (25, 2, 5, 3),
    (26, 9, 64, 9),
]


@pytest.mark.parametrize("twisted", TWIST)
@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("seed,nt,b,a", SHAPES)
def test_against_oracle_shapes(torch, use_method, order, seed, nt, b, a, method, twisted):
    """In Serinv's order the factor and the lone N sweep match the oracle's as well;
    in the two-sided order (a different factor of the same matrix) the logdet, the
    N-then-C solution and the selected inverse do."""
    from pyinla_gb300 import algs

    order(twisted)
    D, L, R, T, rhs = orc.make_bta_c1(seed, nt=nt, b=b, a=a, nrhs=5)
    use_method(b, nt, a, method)
    ref = [x.copy() for x in (D, L, R, T)]
    orc.pobtaf(*ref)
    Dd, Ld, Rd, Td = dev(torch, D, L, R, T)
    algs.pobtaf(Dd, Ld, Rd, Td)
    if not twisted:
        for d, r in zip((Dd, Ld, Rd, Td), ref):
            if r.size:
                assert relerr(host(d), r) < RTOL
    for i in range(nt):   # the factor's diagonal blocks are lower triangular either way
        assert np.all(np.triu(host(Dd[i]), 1) == 0.0)
    assert abs(algs.logdet(Dd, Td, "bta") - orc.logdet(ref[0], ref[3])) <= RTOL * abs(orc.logdet(ref[0], ref[3]))
    xr = rhs.copy()
    orc.pobtas(*ref, xr, "N")
    x = torch.from_numpy(rhs.copy()).cuda()
    algs.pobtas(Dd, Ld, Rd, Td, x, "N")
    if not twisted:
        assert relerr(host(x), xr) < RTOL
    orc.pobtas(*ref, xr, "C")
    algs.pobtas(Dd, Ld, Rd, Td, x, "C")
    assert relerr(host(x), xr) < RTOL
    orc.pobtasi(*ref)
    algs.pobtasi(Dd, Ld, Rd, Td)
    for d, r in zip((Dd, Ld, Rd, Td), ref):
        if r.size:
            assert relerr(host(d), r) < RTOL


def test_numpy_inputs_in_place(torch):
    """The serinv.algs drop-in also takes the reference's NumPy buffers, in place."""
    from pyinla_gb300 import algs

    D, L, R, T, rhs = orc.make_bta_c1(4, nt=3, b=40, a=2)
    ref = [x.copy() for x in (D, L, R, T)]
    orc.pobtaf(*ref)
    algs.pobtaf(D, L, R, T)
    for d, r in zip((D, L, R, T), ref):
        assert relerr(d, r) < RTOL
    x = rhs.copy()
    xr = rhs.copy()
    algs.pobtas(D, L, R, T, x, trans="N")
    algs.pobtas(D, L, R, T, x, trans="C")
    orc.pobtas(*ref, xr, "N")
    orc.pobtas(*ref, xr, "C")
    assert relerr(x, xr) < RTOL


@pytest.mark.parametrize("method", METHODS)
def test_not_positive_definite_raises_with_row(torch, use_method, method):
    from pyinla_gb300 import algs

    use_method(40, 4, 3, method)
    D, L, R, T, rhs = orc.make_bta_c1(5, nt=4, b=40, a=3)
    D[2][7, 7] = -50.0   # global row 2*40 + 7 (0-based) fails first
    Dd, Ld, Rd, Td = dev(torch, D, L, R, T)
    with pytest.raises(np.linalg.LinAlgError) as ei:
        algs.pobtaf(Dd, Ld, Rd, Td)
    assert "row 88" in str(ei.value)
    # the context stays usable: a good matrix factors afterwards
    D, L, R, T, rhs = orc.make_bta_c1(5, nt=4, b=40, a=3)
    Dd, Ld, Rd, Td = dev(torch, D, L, R, T)
    algs.pobtaf(Dd, Ld, Rd, Td)


def test_nan_input_raises(torch):
    from pyinla_gb300 import algs

    D, L, R, T, rhs = orc.make_bta_c1(6, nt=2, b=16, a=2)
    D[0][0, 0] = np.nan
    Dd, Ld, Rd, Td = dev(torch, D, L, R, T)
    with pytest.raises(ValueError):
        algs.pobtaf(Dd, Ld, Rd, Td)


def test_wait_limit_timeout_is_reported_and_recoverable(torch):
    """A wait limit too short for any dependency to arrive makes the kernel give up,
    record GBTA_ERR_TIMEOUT and return; the next launch on the same solver works."""
    from pyinla_gb300 import _lib
    from pyinla_gb300.device import BtaHandle, current_stream_ptr

    D, L, R, T, rhs = orc.make_bta_c1(8, nt=24, b=96, a=4)
    h = BtaHandle(96, 24, 4, twist=False)   # Serinv's order: the factor is compared below
    h.set_stream(current_stream_ptr())
    h.set_wait_limit_ms(1e-6)
    Dd, Ld, Rd, Td = dev(torch, D, L, R, T)
    code = h.lib.gbta_pobtaf(h.ptr, Dd.data_ptr(), Ld.data_ptr(), Rd.data_ptr(), Td.data_ptr())
    assert code == _lib.GBTA_ERR_TIMEOUT, (code, _lib.last_error())
    h.set_wait_limit_ms(20000)
    Dd, Ld, Rd, Td = dev(torch, D, L, R, T)
    ref = [x.copy() for x in (D, L, R, T)]
    orc.pobtaf(*ref)
    _lib.check(h.lib.gbta_pobtaf(h.ptr, Dd.data_ptr(), Ld.data_ptr(), Rd.data_ptr(), Td.data_ptr()))
    assert relerr(host(Dd), ref[0]) < RTOL
    h.close()


def test_drop_in_solver_against_reference_wrapper(torch):
    """GB300SerinvSolver (sparse input, device scatter / gather) against the
    reference SerinvSolver wrapper results stored in the fixtures."""
    import scipy.sparse as sps

    from pyinla_gb300.solver import GB300SerinvSolver

    g, D, L, R, T, rhs = _golden("ragged")
    A = sps.csc_matrix(orc.bta_to_dense(D, L, R, T))
    s = GB300SerinvSolver(None, diagonal_blocksize=int(g["b"]), n_diag_blocks=int(g["nt"]),
                          arrowhead_blocksize=int(g["a"]))
    s.cholesky(A, sparsity="bta")
    assert abs(s.logdet("bta") - float(g["wrapper_logdet"])) <= RTOL * abs(float(g["wrapper_logdet"]))
    x = s.solve(rhs.copy(), sparsity="bta")
    assert relerr(x, g["wrapper_x"]) < RTOL
    s.selected_inversion("bta")
    out = s._structured_to_spmatrix(A, "bta").tocoo()
    lower = out.row >= out.col
    got = {(r, c): v for r, c, v in zip(out.row[lower], out.col[lower], out.data[lower])}
    want = [got[(r, c)] for r, c in zip(g["wrapper_pattern_row"], g["wrapper_pattern_col"])]
    assert relerr(want, g["wrapper_pattern_val"]) < RTOL
    assert len(got) == len(g["wrapper_pattern_val"])
    s.cholesky(A, sparsity="bt")
    assert abs(s.logdet("bt") - float(g["wrapper_bt_logdet"])) <= RTOL * abs(float(g["wrapper_bt_logdet"]))
    assert s.t_cholesky > 0 and s.t_solve > 0
    assert s.get_solver_memory() > D.nbytes


def test_drop_in_solver_pattern_cache(torch):
    """Matrices with the sparsity pattern of an earlier call reuse its index work
    (new arrays, same pattern), a CSR input and a COO input take the other paths,
    and all give the results of a fresh conversion."""
    import scipy.sparse as sps

    from pyinla_gb300.solver import GB300SerinvSolver

    g, D, L, R, T, rhs = _golden("ragged")
    A = sps.csc_matrix(orc.bta_to_dense(D, L, R, T))
    s = GB300SerinvSolver(None, diagonal_blocksize=int(g["b"]), n_diag_blocks=int(g["nt"]),
                          arrowhead_blocksize=int(g["a"]))
    s.cholesky(A, sparsity="bta")
    ld1 = s.logdet("bta")
    s.selected_inversion("bta")
    S1 = s._structured_to_spmatrix(A, "bta")
    A2 = A.copy()
    A2.data = A2.data * 1.7
    s.cholesky(A2, sparsity="bta")
    ld2 = s.logdet("bta")
    s.selected_inversion("bta")
    S2 = s._structured_to_spmatrix(A2, "bta")
    n = A.shape[0]
    assert abs(ld2 - (ld1 + n * np.log(1.7))) <= 1e-10 * abs(ld2)
    assert S2.format == S1.format and np.array_equal(S2.indices, S1.indices) and np.array_equal(S2.indptr, S1.indptr)
    assert relerr(S2.data * 1.7, S1.data) < RTOL
    for B in (A2.tocsr(), A2.tocoo()):
        s2 = GB300SerinvSolver(None, diagonal_blocksize=int(g["b"]), n_diag_blocks=int(g["nt"]),
                               arrowhead_blocksize=int(g["a"]))
        s2.cholesky(B, sparsity="bta")
        s2.selected_inversion("bta")
        S3 = s2._structured_to_spmatrix(B, "bta")
        assert np.abs((S3 - S2).toarray()).max() <= RTOL * np.abs(S2.data).max()


def test_drop_in_solver_pattern_change_same_sizes(torch):
    """A matrix whose index arrays differ from the kept pattern's while its format,
    shape and sizes match (two entries of one column stored in the other order) is
    first scattered and factored with the kept indices while the arrays are compared,
    then redone with its own: the results are those of the matrix in its first order."""
    import scipy.sparse as sps

    from pyinla_gb300.solver import GB300SerinvSolver

    g, D, L, R, T, rhs = _golden("ragged")
    A = sps.csc_matrix(orc.bta_to_dense(D, L, R, T))
    s = GB300SerinvSolver(None, diagonal_blocksize=int(g["b"]), n_diag_blocks=int(g["nt"]),
                          arrowhead_blocksize=int(g["a"]))
    s.cholesky(A, sparsity="bta")
    ld1 = s.logdet("bta")
    s.selected_inversion("bta")
    S1 = s._structured_to_spmatrix(A, "bta")
    B = A.copy()
    j = next(j for j in range(B.shape[1]) if B.indptr[j + 1] - B.indptr[j] >= 2
             and B.data[B.indptr[j]] != B.data[B.indptr[j] + 1])
    p, q = B.indptr[j], B.indptr[j] + 1
    B.indices[[p, q]] = B.indices[[q, p]]
    B.data[[p, q]] = B.data[[q, p]]
    B.has_sorted_indices = False
    assert not np.array_equal(B.indices, A.indices)
    s.cholesky(B, sparsity="bta")
    ld2 = s.logdet("bta")
    s.selected_inversion("bta")
    S2 = s._structured_to_spmatrix(B, "bta")
    assert abs(ld2 - ld1) <= 1e-12 * abs(ld1)
    assert np.abs((S2 - S1).toarray()).max() <= RTOL * np.abs(S1.data).max()
    # and back to the first order
    s.cholesky(A, sparsity="bta")
    assert abs(s.logdet("bta") - ld1) <= 1e-12 * abs(ld1)
