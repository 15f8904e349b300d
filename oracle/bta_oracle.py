"""CPU oracle for the block-tridiagonal-arrowhead (BTA) solve -- TEST INFRASTRUCTURE ONLY.

This module is the parity checker of the repository.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import it;
the product path (``pyinla_gb300``) never does, and fails loudly when its CUDA
library is missing.

What it restates
----------------
The reference (pyINLA / DALIA) delegates the arithmetic of its ``SerinvSolver`` to
the third-party package Serinv (``serinv.algs``: ``pobtaf, pobtas, pobtasi, pobtf,
pobts, pobtsi``), imported at ``src/pyinla/solvers/structured_solver.py:12-15`` and
declared without any version or commit pin at ``pyproject.toml:40``
(``serinv @ git+https://github.com/vincent-maillou/serinv``).  Serinv is not present
in the reference tree and cannot be installed offline, so this file restates its
published algorithms -- sequential block Cholesky of a BTA matrix, the two block
triangular sweeps, and the Takahashi selected-inversion recurrence -- from the
mathematics, with the calling convention fixed by the reference's call sites:

* storage (``structured_solver.py:37-61``): ``D (nt,b,b)`` diagonal blocks,
  ``L (nt-1,b,b)`` with ``L[i]`` = block (i+1, i), ``R (nt,a,b)`` arrow bottom blocks
  (row block nt, column block i), ``T (a,a)`` arrow tip; float64, C-contiguous, full
  (not packed) blocks;
* all routines work **in place** and return nothing (``structured_solver.py:83-93,
  112-140, 176-186``);
* ``pobtas(..., trans="N")`` solves ``L y = b``, ``trans="C"`` solves ``L^T x = y``;
  the solver calls N then C (``structured_solver.py:112-127``);
* after ``pobtasi`` the block buffers hold ``Sigma = Q^{-1}`` restricted to the BTA
  pattern (``structured_solver.py:168-190``, read back by ``:470-538``);
* the "bt" variants ignore the arrow; ``logdet("bt")`` excludes the tip
  (``structured_solver.py:151-166``).

Pinning
-------
``tests/golden/make_golden.py`` runs the reference's own ``DenseSolver``
(``src/pyinla/solvers/dense_solver.py:34-68``: dense Cholesky, triangular solves,
full inverse) and the reference's own ``SerinvSolver`` wrapper (with this module
injected as ``serinv.algs``) on seeded inputs and stores the results under
``tests/golden/``.  ``tests/test_oracle_golden.py`` checks this module against those
fixtures.  Parity against Serinv itself is unpinned (Serinv is absent).
"""

from __future__ import annotations

import numpy as np
import scipy.linalg as sla

__all__ = [
    "pobtaf",
    "pobtas",
    "pobtasi",
    "pobtf",
    "pobts",
    "pobtsi",
    "logdet",
    "bta_to_dense",
    "dense_to_bta",
    "make_bta_c1",
]


def _chol(A: np.ndarray) -> np.ndarray:
    # numpy.linalg.cholesky returns the lower factor with an exactly-zero upper
    # triangle, which is what the reference's buffers hold after a factorization.
    return np.linalg.cholesky(A)


def _rsolve_lt(Lfac: np.ndarray, X: np.ndarray) -> np.ndarray:
    """Return X @ Lfac^{-T} (Lfac lower triangular)."""
    return sla.solve_triangular(Lfac, X.T, lower=True).T


def _tri_inv(Lfac: np.ndarray) -> np.ndarray:
    n = Lfac.shape[0]
    return sla.solve_triangular(Lfac, np.eye(n), lower=True)


# --------------------------------------------------------------------------- factor
def pobtaf(D, L, R, T) -> None:
    """In-place BTA Cholesky (Serinv ``pobtaf``; called at structured_solver.py:83-88).

    Block recurrence for i = 0 .. nt-1::

        D_i <- chol(D_i);  L_i <- L_i D_i^{-T};  R_i <- R_i D_i^{-T}
        D_{i+1} -= L_i L_i^T;  R_{i+1} -= R_i L_i^T;  T -= R_i R_i^T
        finally T <- chol(T)
    """
    nt = D.shape[0]
    has_arrow = R is not None and T is not None and T.shape[0] > 0
    for i in range(nt):
        D[i] = _chol(D[i])
        if has_arrow:
            R[i] = _rsolve_lt(D[i], R[i])
        if i < nt - 1:
            L[i] = _rsolve_lt(D[i], L[i])
            D[i + 1] -= L[i] @ L[i].T
            if has_arrow:
                R[i + 1] -= R[i] @ L[i].T
        if has_arrow:
            T -= R[i] @ R[i].T
    if has_arrow:
        T[:] = _chol(T)


def pobtf(D, L) -> None:
    """In-place block-tridiagonal Cholesky (Serinv ``pobtf``; structured_solver.py:90-93)."""
    pobtaf(D, L, None, None)


# --------------------------------------------------------------------------- solve
def _as2d(Bv: np.ndarray) -> np.ndarray:
    return Bv.reshape(Bv.shape[0], -1)


def pobtas(D, L, R, T, B, trans: str = "N") -> None:
    """In-place triangular sweep with the BTA factor (Serinv ``pobtas``).

    ``trans="N"`` solves ``L y = b`` (forward), ``trans="C"`` solves ``L^T x = y``
    (backward); the solver calls N then C (structured_solver.py:112-127).  ``B`` has
    shape ``(N,)`` or ``(N, nrhs)`` and is overwritten.
    """
    nt, b = D.shape[0], D.shape[1]
    has_arrow = R is not None and T is not None and T.shape[0] > 0
    X = _as2d(B)
    nb = nt * b
    if trans == "N":
        for i in range(nt):
            xi = X[i * b:(i + 1) * b]
            if i > 0:
                xi -= L[i - 1] @ X[(i - 1) * b:i * b]
            xi[:] = sla.solve_triangular(D[i], xi, lower=True)
        if has_arrow:
            xa = X[nb:]
            for i in range(nt):
                xa -= R[i] @ X[i * b:(i + 1) * b]
            xa[:] = sla.solve_triangular(T, xa, lower=True)
    elif trans in ("C", "T"):
        if has_arrow:
            xa = X[nb:]
            xa[:] = sla.solve_triangular(T, xa, lower=True, trans="T")
        for i in range(nt - 1, -1, -1):
            xi = X[i * b:(i + 1) * b]
            if i < nt - 1:
                xi -= L[i].T @ X[(i + 1) * b:(i + 2) * b]
            if has_arrow:
                xi -= R[i].T @ X[nb:]
            xi[:] = sla.solve_triangular(D[i], xi, lower=True, trans="T")
    else:
        raise ValueError(f"Unknown trans {trans!r}")


def pobts(D, L, B, trans: str = "N") -> None:
    """Block-tridiagonal sweep (Serinv ``pobts``; structured_solver.py:129-140)."""
    pobtas(D, L, None, None, B, trans=trans)


# --------------------------------------------------------------------------- selinv
def pobtasi(D, L, R, T) -> None:
    """In-place selected inversion (Serinv ``pobtasi``; structured_solver.py:176-181).

    Takahashi recurrence from the tip backwards, with ``Li = D_i^{-1}`` the inverse of
    the diagonal Cholesky block::

        S_T     = T^{-T} T^{-1}
        S_{i+1,i} = -(S_{i+1,i+1} L_i + S_{a,i+1}^T R_i) Li
        S_{a,i}   = -(S_{a,i+1}   L_i + S_T        R_i) Li
        S_{i,i}   = (Li^T - S_{i+1,i}^T L_i - S_{a,i}^T R_i) Li
    """
    nt = D.shape[0]
    has_arrow = R is not None and T is not None and T.shape[0] > 0
    if has_arrow:
        Ti = _tri_inv(T)
        S_T = Ti.T @ Ti
    for i in range(nt - 1, -1, -1):
        Li = _tri_inv(D[i])
        acc = Li.T.copy()
        if i < nt - 1:
            Lf = L[i].copy()
            S_next = D[i + 1] @ Lf
            if has_arrow:
                S_next += R[i + 1].T @ R[i]
            S_next = -S_next @ Li
            acc -= S_next.T @ Lf
        if has_arrow:
            Rf = R[i].copy()
            S_a = S_T @ Rf
            if i < nt - 1:
                S_a += R[i + 1] @ Lf
            S_a = -S_a @ Li
            acc -= S_a.T @ Rf
        S_ii = acc @ Li
        if i < nt - 1:
            L[i] = S_next
        if has_arrow:
            R[i] = S_a
        D[i] = S_ii
    if has_arrow:
        T[:] = S_T


def pobtsi(D, L) -> None:
    """Block-tridiagonal selected inversion (Serinv ``pobtsi``; structured_solver.py:183-186)."""
    pobtasi(D, L, None, None)


# --------------------------------------------------------------------------- logdet
def logdet(D, T=None, sparsity: str = "bta") -> float:
    """2 * sum(log diag) of the factor (structured_solver.py:151-166).

    For ``sparsity == "bt"`` the arrow tip is excluded; NaN raises ``ValueError``.
    """
    ld = 0.0
    for i in range(D.shape[0]):
        ld += float(np.sum(np.log(np.diagonal(D[i]))))
    if sparsity == "bta" and T is not None and T.shape[0] > 0:
        ld += float(np.sum(np.log(np.diagonal(T))))
    if np.isnan(ld):
        raise ValueError("Logdet is NaN. Check the input matrix.")
    return 2.0 * ld


# --------------------------------------------------------------------------- layout helpers
def bta_to_dense(D, L, R=None, T=None) -> np.ndarray:
    """Assemble the full symmetric matrix from BTA blocks (lower blocks mirrored)."""
    nt, b = D.shape[0], D.shape[1]
    a = 0 if T is None else T.shape[0]
    n = nt * b + a
    A = np.zeros((n, n))
    for i in range(nt):
        A[i * b:(i + 1) * b, i * b:(i + 1) * b] = D[i]
        if i < nt - 1:
            A[(i + 1) * b:(i + 2) * b, i * b:(i + 1) * b] = L[i]
            A[i * b:(i + 1) * b, (i + 1) * b:(i + 2) * b] = L[i].T
        if a:
            A[nt * b:, i * b:(i + 1) * b] = R[i]
            A[i * b:(i + 1) * b, nt * b:] = R[i].T
    if a:
        A[nt * b:, nt * b:] = T
    return A


def dense_to_bta(A: np.ndarray, nt: int, b: int, a: int):
    """Slice the BTA blocks out of a dense matrix (the inverse of :func:`bta_to_dense`)."""
    D = np.stack([A[i * b:(i + 1) * b, i * b:(i + 1) * b] for i in range(nt)])
    L = np.stack([A[(i + 1) * b:(i + 2) * b, i * b:(i + 1) * b] for i in range(nt - 1)]) \
        if nt > 1 else np.zeros((0, b, b))
    R = np.stack([A[nt * b:, i * b:(i + 1) * b] for i in range(nt)]) if a else np.zeros((nt, 0, b))
    T = A[nt * b:, nt * b:].copy() if a else np.zeros((0, 0))
    return np.ascontiguousarray(D), np.ascontiguousarray(L), np.ascontiguousarray(R), np.ascontiguousarray(T)


def make_bta_c1(seed: int, nt: int = 16, b: int = 128, a: int = 4, nrhs: int = 1):
    """Seeded diagonally dominant SPD BTA matrix (the plain-solve workload).

    ``L_i``, ``R_i`` ~ N(0,1)/sqrt(b); ``D_i = (G+G^T)/2`` with G ~ N(0,1)/sqrt(b); the
    tip likewise (a x a).  Each diagonal entry then gets (sum of |off-diagonal| in its
    row of the full symmetric matrix) + 1.  One (or ``nrhs``) right-hand side ~ N(0,1).
    Draw order: D, L, R, T, rhs from ``numpy.random.default_rng(seed)``.
    """
    rng = np.random.default_rng(seed)
    s = 1.0 / np.sqrt(b)
    G = rng.standard_normal((nt, b, b)) * s
    D = 0.5 * (G + np.transpose(G, (0, 2, 1)))
    L = rng.standard_normal((max(nt - 1, 0), b, b)) * s
    R = rng.standard_normal((nt, a, b)) * s
    Gt = rng.standard_normal((a, a)) * s
    T = 0.5 * (Gt + Gt.T)
    n = nt * b + a
    rhs = rng.standard_normal((n, nrhs)) if nrhs > 1 else rng.standard_normal(n)

    # Row sums of |off-diagonal| over the whole symmetric matrix.
    rows_d = np.zeros((nt, b))
    for i in range(nt):
        Di = np.abs(D[i]).copy()
        np.fill_diagonal(Di, 0.0)
        rows_d[i] += Di.sum(axis=1)
        if i > 0:
            rows_d[i] += np.abs(L[i - 1]).sum(axis=1)      # block (i, i-1)
        if i < nt - 1:
            rows_d[i] += np.abs(L[i]).sum(axis=0)          # block (i, i+1) = L_i^T
        if a:
            rows_d[i] += np.abs(R[i]).sum(axis=0)          # block (i, nt) = R_i^T
    rows_a = np.zeros(a)
    if a:
        Ta = np.abs(T).copy()
        np.fill_diagonal(Ta, 0.0)
        rows_a += Ta.sum(axis=1)
        for i in range(nt):
            rows_a += np.abs(R[i]).sum(axis=1)
    for i in range(nt):
        D[i][np.diag_indices(b)] += rows_d[i] + 1.0
    if a:
        T[np.diag_indices(a)] += rows_a + 1.0
    return (np.ascontiguousarray(D), np.ascontiguousarray(L), np.ascontiguousarray(R),
            np.ascontiguousarray(T), rhs)
