"""CPU oracle of the marginal variances -- TEST INFRASTRUCTURE ONLY.

Restates, on the blocks of a selected inverse Sigma (the output of ``pobtasi``,
oracle/bta_oracle.py), what the reference returns after an INLA run
(src/pyinla/core/pyinla.py:303-311):

* the latent marginal variances diag(Sigma): ``get_marginal_variances_latent_parameters``
  (pyinla.py:940-964) maps Sigma onto the identity's pattern with
  ``SerinvSolver._structured_to_spmatrix`` (src/pyinla/solvers/structured_solver.py:470-538)
  and takes ``extract_diagonal`` (src/pyinla/utils/spmatrix_utils.py:46-63), i.e. the
  diagonals of the diagonal blocks and of the tip, in latent order;
* the observation marginal variances diag(A Sigma_Q A^T): ``get_marginal_variances_observations``
  (pyinla.py:966-1018) maps Sigma onto the pattern of Q_cond and forms the dense
  product's diagonal.  Row r of A with nonzeros (c_j, a_j) gives
  sum_{j,k} a_j a_k Sigma(c_j, c_k); every pair (c_j, c_k) lies in the pattern of
  A^T A, hence of Q_cond, so the pattern restriction removes nothing.  A pair farther
  apart than adjacent time blocks is outside the block-tridiagonal-arrowhead pattern
  (such an A does not give a BTA Q_cond) and contributes 0.

Only tests, smoke() and the CPU baseline of bench.py may use this module.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sps


def latent_variances(SD: np.ndarray, ST: np.ndarray | None = None) -> np.ndarray:
    """diag(Sigma) in latent order: the diagonal blocks' diagonals, then the tip's."""
    parts = [np.diagonal(SD[t]) for t in range(SD.shape[0])]
    if ST is not None and ST.shape[0] > 0:
        parts.append(np.diagonal(ST))
    return np.concatenate(parts).astype(np.float64)


def sigma_entries(SD, SL, SR, ST, p: np.ndarray, q: np.ndarray) -> np.ndarray:
    """Sigma(p, q) for index arrays p, q, read from the BTA blocks (0 outside the pattern)."""
    nt, b = SD.shape[0], SD.shape[1]
    nb = nt * b
    p = np.asarray(p, dtype=np.int64)
    q = np.asarray(q, dtype=np.int64)
    out = np.zeros(p.shape, dtype=np.float64)
    pa, qa = p >= nb, q >= nb
    # tip
    m = pa & qa
    out[m] = ST[p[m] - nb, q[m] - nb]
    # arrow row x block column (R_t = Sigma(arrow, block t)), and its transpose
    m = pa & ~qa
    out[m] = SR[q[m] // b, p[m] - nb, q[m] % b]
    m = ~pa & qa
    out[m] = SR[p[m] // b, q[m] - nb, p[m] % b]
    # blocks
    m = ~pa & ~qa
    tp, tq = p // b, q // b
    s = m & (tp == tq)
    out[s] = SD[tp[s], p[s] % b, q[s] % b]
    s = m & (tp == tq + 1)           # L_t = Sigma(block t+1, block t)
    out[s] = SL[tq[s], p[s] % b, q[s] % b]
    s = m & (tq == tp + 1)
    out[s] = SL[tp[s], q[s] % b, p[s] % b]
    return out


def observation_variances(A, SD, SL, SR, ST) -> np.ndarray:
    """diag(A Sigma A^T) over the rows of the sparse observation matrix A."""
    A = sps.csr_matrix(A)
    A.sum_duplicates()
    n = A.shape[0]
    cnt = np.diff(A.indptr)
    rows = np.repeat(np.arange(n), cnt * cnt)
    # every ordered pair (j, k) of each row's nonzeros
    starts = np.repeat(A.indptr[:-1], cnt * cnt)
    off = np.concatenate([np.arange(c * c) for c in cnt]) if n else np.zeros(0, dtype=np.int64)
    cc = np.repeat(cnt, cnt * cnt)
    j = starts + off // np.maximum(cc, 1)
    k = starts + off % np.maximum(cc, 1)
    vals = A.data[j] * A.data[k] * sigma_entries(SD, SL, SR, ST, A.indices[j], A.indices[k])
    return np.bincount(rows, weights=vals, minlength=n).astype(np.float64)


def make_observation_matrix(seed: int, nt: int, b: int, a: int, n_obs: int, spread: float = 0.1) -> sps.csr_matrix:
    """Seeded observation matrix in latent (BTA) order, shaped like a spatio-temporal design.

    Each row picks a time block t and 1-3 distinct nodes of it with weights that sum
    to 1 (barycentric-like), plus every fixed effect (arrow column) with a N(0, 1)
    covariate; a fraction ``spread`` of the rows (t < nt - 1) also touches one node of
    block t + 1, so that Sigma's off-diagonal blocks are read.  Draw order from
    ``numpy.random.default_rng(seed)``: per row t, node count, nodes, weights,
    spread flag, neighbour node, covariates.
    """
    rng = np.random.default_rng(seed)
    rows, cols, vals = [], [], []
    for r in range(n_obs):
        t = int(rng.integers(nt))
        m = int(rng.integers(1, 4))
        nodes = rng.choice(b, size=min(m, b), replace=False)
        w = rng.random(nodes.size) + 0.05
        w /= w.sum()
        two = bool(rng.random() < spread)
        nb_node = int(rng.integers(b))
        cov = rng.standard_normal(a)
        for nd, wv in zip(nodes, w):
            rows.append(r); cols.append(t * b + int(nd)); vals.append(float(wv))
        if two and t < nt - 1:
            rows.append(r); cols.append((t + 1) * b + nb_node); vals.append(0.5)
        for j in range(a):
            rows.append(r); cols.append(nt * b + j); vals.append(float(cov[j]))
    A = sps.csr_matrix((vals, (rows, cols)), shape=(n_obs, nt * b + a))
    A.sum_duplicates()
    A.sort_indices()
    return A
