"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run in a container where the reference source tree is available (it is read from
``$PYINLA_REFERENCE_SRC``, required: the reference's ``src/`` directory); the fixtures it writes are
committed, so tests never need the reference at run time.

What is pinned, per case (all float64):

* ``DenseSolver`` (reference ``src/pyinla/solvers/dense_solver.py:34-68``) on the
  densified matrix: ``logdet`` (``:51-55``), the solution of ``Q x = rhs`` (``:41-49``)
  and the full inverse (``:58-68``), from which the BTA-pattern blocks of Sigma are
  stored.  For the ``bt`` sparsity the same is done on the block-tridiagonal part.
* ``SerinvSolver`` (reference ``src/pyinla/solvers/structured_solver.py``) with the
  oracle module injected as ``serinv.algs``: ``cholesky`` via the reference's own
  sparse-to-BTA mapping (``:192-250``), ``logdet`` (``:151-166``), ``solve``
  (``:102-149``), ``selected_inversion`` + ``_structured_to_spmatrix`` (``:470-538``).
  Those wrapper results are stored too, so a test can check that the oracle driven
  by the reference's wrapper agrees with the reference's dense solver.

Inputs are regenerated in the tests from the seed with ``oracle.bta_oracle.make_bta_c1``;
a checksum of the inputs is stored so that a change of random stream is detected.
"""

from __future__ import annotations

import os
import sys
import types
from pathlib import Path

import numpy as np
import scipy.sparse as sps

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))

from oracle import bta_oracle as orc  # noqa: E402


def _import_reference():
    src = os.environ.get("PYINLA_REFERENCE_SRC")
    if not src:
        raise SystemExit("set PYINLA_REFERENCE_SRC to the reference's src/ directory (the tree that holds "
                         "the pyinla package) to regenerate the fixtures")
    os.environ.setdefault("ARRAY_MODULE", "numpy")
    # matplotlib is imported at module level by the reference's
    # utils/sparse_diagABAt.py:11 but is not used on this path; it is not installed.
    mpl = types.ModuleType("matplotlib")
    mpl.pyplot = types.ModuleType("matplotlib.pyplot")
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", mpl.pyplot)
    # Serinv is absent: inject the oracle as serinv.algs so SerinvSolver runs.
    serinv = types.ModuleType("serinv")
    serinv.algs = orc
    sys.modules["serinv"] = serinv
    sys.modules["serinv.algs"] = orc
    sys.path.insert(0, src)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        from pyinla.configs.pyinla_config import SolverConfig
        from pyinla.solvers.dense_solver import DenseSolver
        from pyinla.solvers import structured_solver
    # structured_solver imported pobtaf & co. by name at import time.
    for name in ("pobtaf", "pobtas", "pobtasi", "pobtf", "pobts", "pobtsi"):
        setattr(structured_solver, name, getattr(orc, name))
    return SolverConfig, DenseSolver, structured_solver.SerinvSolver


def checksum(*arrs) -> np.ndarray:
    out = []
    for x in arrs:
        x = np.asarray(x, dtype=np.float64).ravel()
        out += [x.size, float(x.sum()), float(np.abs(x).sum()), float(x[:7].sum()) if x.size else 0.0]
    return np.array(out, dtype=np.float64)


CASES = {
    # name: (seed, nt, b, a, store_all_sigma_blocks)
    "tiny": (3, 3, 8, 2, True),
    "ragged": (5, 4, 40, 5, True),
    "single": (7, 1, 16, 3, True),
    "two": (11, 2, 33, 1, True),
    "c1": (0, 16, 128, 4, False),
}


def make_case(name, seed, nt, b, a, store_all, SolverConfig, DenseSolver, SerinvSolver):
    D, L, R, T, rhs = orc.make_bta_c1(seed, nt=nt, b=b, a=a)
    out = {"seed": seed, "nt": nt, "b": b, "a": a, "input_checksum": checksum(D, L, R, T, rhs)}
    A = orc.bta_to_dense(D, L, R, T)
    Asp = sps.csc_matrix(A)
    n = A.shape[0]
    cfg = SolverConfig(type="dense")

    # --- reference DenseSolver, bta matrix
    ds = DenseSolver(cfg, n=n)
    ds.cholesky(Asp)
    out["dense_logdet"] = float(ds.logdet())
    out["dense_x"] = ds.solve(rhs.copy())
    Sigma = ds.selected_inversion(Asp)
    SD, SL, SR, ST = orc.dense_to_bta(np.asarray(Sigma), nt, b, a)
    if store_all:
        out.update(dense_SD=SD, dense_SL=SL, dense_SR=SR, dense_ST=ST)
    else:
        out["dense_Sdiag"] = np.diagonal(np.asarray(Sigma)).copy()
        out["dense_SD_first"], out["dense_SD_last"] = SD[0], SD[-1]
        out["dense_SL_first"], out["dense_SL_last"] = SL[0], SL[-1]
        out.update(dense_SR=SR, dense_ST=ST)
    if store_all:
        # reference _structured_to_spmatrix of DenseSolver on Q's pattern (lower values)
        pat = ds._structured_to_spmatrix(sps.tril(Asp).tocoo())
        out["dense_pattern_row"], out["dense_pattern_col"] = pat.row, pat.col
        out["dense_pattern_val"] = pat.data

    # --- reference DenseSolver, bt part (arrow removed)
    Abt = orc.bta_to_dense(D, L)
    ds2 = DenseSolver(cfg, n=nt * b)
    ds2.cholesky(sps.csc_matrix(Abt))
    out["dense_bt_logdet"] = float(ds2.logdet())
    out["dense_bt_x"] = ds2.solve(rhs[: nt * b].copy())
    Sbt = np.asarray(ds2.selected_inversion(sps.csc_matrix(Abt)))
    SDb, SLb, _, _ = orc.dense_to_bta(Sbt, nt, b, 0)
    if store_all:
        out.update(dense_bt_SD=SDb, dense_bt_SL=SLb)
    else:
        out["dense_bt_Sdiag"] = np.diagonal(Sbt).copy()

    # --- reference SerinvSolver wrapper driven by the oracle (needs a > 0: its CPU
    #     mapping zero-fills the arrow buffers unconditionally, structured_solver.py:198-201)
    if a > 0:
        ss = SerinvSolver(SolverConfig(type="serinv"), diagonal_blocksize=b, n_diag_blocks=nt,
                          arrowhead_blocksize=a)
        ss.cholesky(Asp, sparsity="bta")
        out["wrapper_logdet"] = float(ss.logdet(sparsity="bta"))
        out["wrapper_x"] = ss.solve(rhs.copy(), sparsity="bta")
        ss.selected_inversion(sparsity="bta")
        if store_all:
            sp_out = ss._structured_to_spmatrix(Asp, sparsity="bta").tocoo()
            lower = sp_out.row >= sp_out.col
            out["wrapper_pattern_row"] = sp_out.row[lower]
            out["wrapper_pattern_col"] = sp_out.col[lower]
            out["wrapper_pattern_val"] = sp_out.data[lower]
        else:
            out["wrapper_SD_first"] = ss.A_diagonal_blocks[0].copy()
            out["wrapper_ST"] = ss.A_arrow_tip_block.copy()
        # bt factorization of the same matrix with the same wrapper (Q_prior path,
        # pyinla.py:1102-1103): arrow ignored, tip excluded from the logdet.
        ss.cholesky(Asp, sparsity="bt")
        out["wrapper_bt_logdet"] = float(ss.logdet(sparsity="bt"))
    return out


def main():
    SolverConfig, DenseSolver, SerinvSolver = _import_reference()
    for name, (seed, nt, b, a, store_all) in CASES.items():
        res = make_case(name, seed, nt, b, a, store_all, SolverConfig, DenseSolver, SerinvSolver)
        path = HERE / f"bta_{name}.npz"
        np.savez_compressed(path, **res)
        print(f"wrote {path.name}: {os.path.getsize(path) / 1024:.1f} KiB")


if __name__ == "__main__":
    main()
