"""CPU oracle of the Gaussian spatio-temporal objective -- TEST INFRASTRUCTURE ONLY.

Restates, with SciPy sparse matrices, what the reference computes per objective
evaluation for a Gaussian likelihood:

* Q_prior as a sum of Kronecker products of tridiagonal temporal matrices and
  sparse spatial matrices, as in src/pyinla/submodels/spatio_temporal.py:139-147
  (``sp.sparse.kron(m_k, q_k)`` summed), with the fixed-effect block
  ``tip_prec * I`` of src/pyinla/submodels/regression.py:27-30 appended;
* Q_cond = Q_prior - A^T D A with D = -tau_y I (src/pyinla/core/model.py:421,
  src/pyinla/likelihoods/gaussian.py:127-129), or D = -diag(tau_y of each row's
  variate) for the coregional model's per-variate likelihoods
  (src/pyinla/models/coregional_model.py:599-643);
* the information vector at x = 0, A^T D y (model.py:445-447, gaussian.py:94);
* the sparse-to-BTA mapping of SerinvSolver (src/pyinla/solvers/structured_solver.py:192-250);
* f(theta) of PyINLA._evaluate_f for the Gaussian branch
  (src/pyinla/core/pyinla.py:631-688, 1076-1167) with the BTA oracle of
  oracle/bta_oracle.py in place of Serinv;
* the central finite-difference gradient of PyINLA._objective_function
  (pyinla.py:546-580).

Only tests, smoke() and the CPU baseline of bench.py may use this module.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sps

from . import bta_oracle as orc


def temporal_matrix(diag: np.ndarray, off: np.ndarray) -> sps.csr_matrix:
    nt = diag.size
    return sps.diags([off, diag, off], [-1, 0, 1], shape=(nt, nt)).tocsr() if nt > 1 else sps.csr_matrix(diag.reshape(1, 1))


def kron_prior(spatial_terms, term_vw, alpha, beta, ns, nv, nt, nb, tip_prec) -> sps.csr_matrix:
    """Q_prior = sum_k M_k (x) S_k placed at variate blocks (v_k, w_k), plus tip_prec I_nb."""
    b = nv * ns
    N = nt * b + nb
    Q = sps.csr_matrix((N, N))
    for k, S in enumerate(spatial_terms):
        v, w = term_vw[k]
        M = temporal_matrix(alpha[k], beta[k] if nt > 1 else np.zeros(0))
        K = sps.kron(M, S).tocoo()   # rows t*ns + r, cols t'*ns + c
        t, r = K.row // ns, K.row % ns
        tp, c = K.col // ns, K.col % ns
        Q = Q + sps.csr_matrix((K.data, (t * b + v * ns + r, tp * b + w * ns + c)), shape=(N, N))
    if nb:
        Q = Q + sps.block_diag([sps.csr_matrix((nt * b, nt * b)), tip_prec * sps.eye(nb)]).tocsr()
    return Q.tocsr()


def sparse_to_bta(Q, nt: int, b: int, a: int):
    """Dense BTA blocks of a symmetric sparse matrix (structured_solver.py:198-250)."""
    Qc = sps.csc_matrix(Q)
    D = np.zeros((nt, b, b))
    L = np.zeros((max(nt - 1, 0), b, b))
    R = np.zeros((nt, a, b))
    T = np.zeros((a, a))
    for i in range(nt):
        D[i] = Qc[i * b:(i + 1) * b, i * b:(i + 1) * b].toarray()
        if i < nt - 1:
            L[i] = Qc[(i + 1) * b:(i + 2) * b, i * b:(i + 1) * b].toarray()
        if a:
            R[i] = Qc[nt * b:, i * b:(i + 1) * b].toarray()
    if a:
        T[:] = Qc[nt * b:, nt * b:].toarray()
    return D, L, R, T


def _variate_arrays(y, tau_y, obs_variate):
    tau_y = np.atleast_1d(np.asarray(tau_y, dtype=np.float64))
    ov = np.zeros(y.size, dtype=np.int64) if obs_variate is None else np.asarray(obs_variate, dtype=np.int64)
    return tau_y, ov, tau_y[ov]


def conditional_system(spatial_terms, term_vw, ns, nv, nt, nb, A, y, tip_prec, alpha, beta, tau_y,
                       obs_variate=None):
    """Q_prior, Q_cond = Q_prior + A^T diag(tau_y of each row) A (model.py:421) and the
    information vector A^T (tau_y y) at x = 0 (model.py:445-447), as SciPy matrices."""
    _, _, tau_row = _variate_arrays(y, tau_y, obs_variate)
    Qp = kron_prior(spatial_terms, term_vw, alpha, beta, ns, nv, nt, nb, tip_prec)
    Qc = (Qp + A.T @ (sps.diags(tau_row) @ A)).tocsr()
    return Qp, Qc, np.asarray(A.T @ (tau_row * y), dtype=np.float64)


def objective(spatial_terms, term_vw, ns, nv, nt, nb, A, y, tip_prec, alpha, beta, tau_y, theta_y, log_prior,
              obs_variate=None):
    """f(theta) for the Gaussian branch of PyINLA._evaluate_f, on the CPU.

    ``tau_y`` and ``theta_y`` hold one noise precision (and its log) per variate and
    ``obs_variate`` the variate of each observation (default: all 0); several variates
    are the coregional model's per-variate likelihoods: D = -diag(tau_y of each row)
    (src/pyinla/models/coregional_model.py:599-643) and the likelihood summed over the
    variates (:664-677)."""
    b = nv * ns
    tau_y, ov, tau_row = _variate_arrays(y, tau_y, obs_variate)
    theta_y = np.atleast_1d(np.asarray(theta_y, dtype=np.float64))
    Qp, Qc, rhs = conditional_system(spatial_terms, term_vw, ns, nv, nt, nb, A, y, tip_prec, alpha, beta, tau_y,
                                     obs_variate)
    Dp, Lp, Rp, Tp = sparse_to_bta(Qp, nt, b, nb)
    orc.pobtf(Dp, Lp)
    logdet_p = orc.logdet(Dp, None, "bt")
    Dc, Lc, Rc, Tc = sparse_to_bta(Qc, nt, b, nb)
    orc.pobtaf(Dc, Lc, Rc, Tc)
    logdet_c = orc.logdet(Dc, Tc, "bta")
    mu = rhs.copy()
    orc.pobtas(Dc, Lc, Rc, Tc, mu, "N")
    orc.pobtas(Dc, Lc, Rc, Tc, mu, "C")
    quad = float(mu @ (Qc @ mu))                        # pyinla.py:1157-1158
    lik = 0.0                                           # gaussian.py:58-60 at eta = 0, per variate
    for v in range(tau_y.size):
        yv = y[ov == v]
        lik += 0.5 * theta_y[v] * yv.size - 0.5 * tau_y[v] * float(yv @ yv)
    f = -(log_prior + lik + 0.5 * logdet_p) + 0.5 * logdet_c - 0.5 * quad
    return f, dict(logdet_prior=logdet_p, logdet_cond=logdet_c, quad=quad, mu=mu, Qp=Qp, Qc=Qc)


def central_difference(fun, theta, eps):
    """Central FD gradient as in PyINLA._objective_function (pyinla.py:546-580)."""
    theta = np.asarray(theta, dtype=np.float64)
    g = np.zeros_like(theta)
    for i in range(theta.size):
        e = np.zeros_like(theta)
        e[i] = eps
        g[i] = (fun(theta + e) - fun(theta - e)) / (2.0 * eps)
    return g


def dense_gradient(spatial_terms, term_vw, ns, nv, nt, nb, A, y, tip_prec, coef, dcoef, theta_y_index,
                   log_prior_grad, obs_variate=None):
    """Exact gradient of f with dense FP64 linear algebra (small problems only):
    tr(Q^{-1} dQ) with the full inverses, mu from a dense solve.  ``theta_y_index``
    lists the index of log tau_y,v in theta for each variate v; ``dcoef.dtau_y[k, v]``
    is d tau_y,v / d theta_k."""
    b = nv * ns
    tau_y, ov, tau_row = _variate_arrays(y, coef.tau_y, obs_variate)
    nvar = tau_y.size
    dtau = np.asarray(dcoef.dtau_y, dtype=np.float64).reshape(dcoef.dalpha.shape[0], nvar)
    Qp = kron_prior(spatial_terms, term_vw, coef.alpha, coef.beta, ns, nv, nt, nb, tip_prec).toarray()
    AtA_v = [(A[ov == v].T @ A[ov == v]).toarray() for v in range(nvar)]
    Aty_v = [A[ov == v].T @ y[ov == v] for v in range(nvar)]
    Qc = Qp + sum(tau_y[v] * AtA_v[v] for v in range(nvar))
    nbk = nt * b
    Sp = np.linalg.inv(Qp[:nbk, :nbk])
    Sc = np.linalg.inv(Qc)
    rhs = sum(tau_y[v] * Aty_v[v] for v in range(nvar))
    mu = np.linalg.solve(Qc, rhs)
    d = dcoef.dalpha.shape[0]
    g = np.zeros(d)
    for k in range(d):
        dQp = kron_prior(spatial_terms, term_vw, dcoef.dalpha[k], dcoef.dbeta[k], ns, nv, nt, nb, 0.0).toarray()
        dQc = dQp + sum(dtau[k, v] * AtA_v[v] for v in range(nvar))
        tr_p = float(np.sum(Sp * dQp[:nbk, :nbk]))
        tr_c = float(np.sum(Sc * dQc))
        mdb = float(sum(dtau[k, v] * (mu @ Aty_v[v]) for v in range(nvar)))
        g[k] = -0.5 * tr_p + 0.5 * tr_c - mdb + 0.5 * float(mu @ dQc @ mu)
    for v, idx in enumerate(np.atleast_1d(theta_y_index)):
        yv = y[ov == v]
        g[idx] -= 0.5 * yv.size - 0.5 * tau_y[v] * float(yv @ yv)
    g -= log_prior_grad
    return g


def hessian_fd(fun, theta, eps):
    """FD Hessian of f as in PyINLA._evaluate_hessian_f (pyinla.py:767-910): f at theta,
    theta +- eps_i (diagonal: (f+ - 2 f + f-) / eps^2) and theta +- eps_i +- eps_j (upper
    triangle: (f++ - f+- - f-+ + f--) / (4 eps^2), mirrored); 1 + 2d + 2d(d-1) evaluations."""
    theta = np.asarray(theta, dtype=np.float64)
    d = theta.size
    E = eps * np.eye(d)
    f0 = fun(theta)
    H = np.zeros((d, d))
    for i in range(d):
        H[i, i] = (fun(theta + E[i]) - 2.0 * f0 + fun(theta - E[i])) / eps ** 2
        for j in range(i + 1, d):
            H[i, j] = (fun(theta + E[i] + E[j]) - fun(theta + E[i] - E[j]) - fun(theta - E[i] + E[j])
                       + fun(theta - E[i] - E[j])) / (4.0 * eps * eps)
            H[j, i] = H[i, j]
    return H


def hessian_from_gradient(grad, theta, eps):
    """Hessian by central differences of an exact gradient (2d gradient evaluations),
    symmetrised: H[:, k] = (g(theta + eps e_k) - g(theta - eps e_k)) / (2 eps)."""
    theta = np.asarray(theta, dtype=np.float64)
    d = theta.size
    H = np.zeros((d, d))
    for k in range(d):
        e = np.zeros(d)
        e[k] = eps
        H[:, k] = (np.asarray(grad(theta + e)) - np.asarray(grad(theta - e))) / (2.0 * eps)
    return 0.5 * (H + H.T)
