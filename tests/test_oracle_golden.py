"""The oracle (oracle/bta_oracle.py) against fixtures produced by the reference itself.

Fixtures come from tests/golden/make_golden.py: the reference's DenseSolver
(src/pyinla/solvers/dense_solver.py:34-68) and the reference's SerinvSolver wrapper
(src/pyinla/solvers/structured_solver.py) driven by the oracle.
"""
import numpy as np
import pytest

from oracle import bta_oracle as orc
from tests.conftest import GOLDEN
from tests.golden.make_golden import checksum

CASES = ["tiny", "ragged", "single", "two", "c1"]
RTOL = 1e-10


def _load(name):
    g = np.load(GOLDEN / f"bta_{name}.npz")
    D, L, R, T, rhs = orc.make_bta_c1(int(g["seed"]), nt=int(g["nt"]), b=int(g["b"]), a=int(g["a"]))
    np.testing.assert_allclose(checksum(D, L, R, T, rhs), g["input_checksum"], rtol=1e-13, atol=0)
    return g, D, L, R, T, rhs


def relerr(x, y):
    x = np.asarray(x); y = np.asarray(y)
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


@pytest.mark.parametrize("name", CASES)
def test_oracle_factor_logdet_solve(name):
    g, D, L, R, T, rhs = _load(name)
    orc.pobtaf(D, L, R, T)
    ld = orc.logdet(D, T, "bta")
    assert abs(ld - float(g["dense_logdet"])) <= RTOL * abs(float(g["dense_logdet"]))
    x = rhs.copy()
    orc.pobtas(D, L, R, T, x, trans="N")
    orc.pobtas(D, L, R, T, x, trans="C")
    assert relerr(x, g["dense_x"]) < RTOL
    # upper triangles of the factor's diagonal blocks are exactly zero
    for i in range(D.shape[0]):
        assert np.all(np.triu(D[i], 1) == 0.0)


@pytest.mark.parametrize("name", CASES)
def test_oracle_selinv(name):
    g, D, L, R, T, rhs = _load(name)
    orc.pobtaf(D, L, R, T)
    orc.pobtasi(D, L, R, T)
    if "dense_SD" in g:
        assert relerr(D, g["dense_SD"]) < RTOL
        if D.shape[0] > 1:
            assert relerr(L, g["dense_SL"]) < RTOL
    else:
        assert relerr(D[0], g["dense_SD_first"]) < RTOL
        assert relerr(D[-1], g["dense_SD_last"]) < RTOL
        assert relerr(L[0], g["dense_SL_first"]) < RTOL
        assert relerr(L[-1], g["dense_SL_last"]) < RTOL
        diag = np.concatenate([np.diagonal(D[i]) for i in range(D.shape[0])] + [np.diagonal(T)])
        assert relerr(diag, g["dense_Sdiag"]) < RTOL
    assert relerr(R, g["dense_SR"]) < RTOL
    assert relerr(T, g["dense_ST"]) < RTOL


@pytest.mark.parametrize("name", CASES)
def test_oracle_bt(name):
    g, D, L, R, T, rhs = _load(name)
    nt, b = D.shape[0], D.shape[1]
    orc.pobtf(D, L)
    ld = orc.logdet(D, None, "bt")
    assert abs(ld - float(g["dense_bt_logdet"])) <= RTOL * abs(float(g["dense_bt_logdet"]))
    if "wrapper_bt_logdet" in g:
        assert abs(ld - float(g["wrapper_bt_logdet"])) <= RTOL * abs(ld)
    x = rhs[: nt * b].copy()
    orc.pobts(D, L, x, trans="N")
    orc.pobts(D, L, x, trans="C")
    assert relerr(x, g["dense_bt_x"]) < RTOL
    orc.pobtsi(D, L)
    if "dense_bt_SD" in g:
        assert relerr(D, g["dense_bt_SD"]) < RTOL
        if nt > 1:
            assert relerr(L, g["dense_bt_SL"]) < RTOL
    else:
        diag = np.concatenate([np.diagonal(D[i]) for i in range(nt)])
        assert relerr(diag, g["dense_bt_Sdiag"]) < RTOL


@pytest.mark.parametrize("name", ["tiny", "ragged", "single", "two"])
def test_reference_wrapper_pattern_matches_dense(name):
    """The reference's SerinvSolver wrapper (oracle inside) agrees with its DenseSolver
    on every selected-inverse entry of Q's lower pattern (structured_solver.py:470-538)."""
    g = np.load(GOLDEN / f"bta_{name}.npz")
    key_d = {(r, c): v for r, c, v in zip(g["dense_pattern_row"], g["dense_pattern_col"], g["dense_pattern_val"])}
    vals_w = g["wrapper_pattern_val"]
    vals_d = np.array([key_d[(r, c)] for r, c in zip(g["wrapper_pattern_row"], g["wrapper_pattern_col"])])
    assert relerr(vals_w, vals_d) < RTOL
    assert abs(float(g["wrapper_logdet"]) - float(g["dense_logdet"])) <= RTOL * abs(float(g["dense_logdet"]))
    assert relerr(g["wrapper_x"], g["dense_x"]) < RTOL


def test_logdet_nan_raises():
    D = np.full((1, 2, 2), np.nan)
    with pytest.raises(ValueError):
        orc.logdet(D, None, "bt")
