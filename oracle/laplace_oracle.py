"""CPU oracle of the non-Gaussian objective (Laplace approximation) -- TEST INFRASTRUCTURE ONLY.

Restates what the reference computes per objective evaluation for a Poisson or a
Binomial likelihood (src/pyinla/core/pyinla.py:692-729):

* the likelihood, its gradient and the negative diagonal of its Hessian in eta:
  Poisson (src/pyinla/likelihoods/poisson.py: l = eta . y - sum e exp(eta),
  l' = y - e exp(eta), -l'' = e exp(eta)) and Binomial with the sigmoid link
  (src/pyinla/likelihoods/binomial.py: l = y . log s + (n - y) . log(1 - s),
  l' = y - n s, -l'' = n s (1 - s), s = sigmoid(eta));
* the inner Newton iteration of PyINLA._inner_iteration (pyinla.py:1025-1074): from the
  stored x, repeat x += dx; eta = A x; Q_cond = Q_prior + A^T diag(-l''(eta)) A
  (model.py:384-423); rhs = -Q_prior x + A^T l'(eta) (model.py:425-449); dx = Q_cond^{-1}
  rhs, until |dx| < eps (the returned Q_cond, x and eta are those of the last pass,
  before its dx);
* f(theta) = -(log prior(theta) + l(eta) + 0.5 logdet Q_prior - 0.5 x^T Q_prior x
  - 0.5 logdet Q_cond), the non-Gaussian branch of PyINLA._evaluate_f with
  _evaluate_prior_latent_parameters (pyinla.py:1076-1110; "bt" logdet, the tip of the
  prior excluded) and the conditional term at its mean (pyinla.py:1112-1167).

Dense FP64 linear algebra: small problems only.  Only tests may use this module.
"""
from __future__ import annotations

import numpy as np

from . import model_oracle as mo


def poisson(eta, y, e):
    ex = e * np.exp(eta)
    return float(eta @ y - np.sum(ex)), y - ex, ex


def sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


def binomial(eta, y, n):
    s = sigmoid(eta)
    return float(y @ np.log(s) + (n - y) @ np.log(1.0 - s)), y - n * s, n * s * (1.0 - s)


def laplace_objective(spec, theta, lik, x0, eps=1e-3, max_iter=50, e=None, n_trials=None):
    """f(theta) and the new latent mode x* (start x0) of a KronSpec-like model with a
    Poisson (`e` exposures) or Binomial (`n_trials`) likelihood."""
    theta = np.asarray(theta, dtype=np.float64)
    A = spec.A
    y = np.asarray(spec.y, dtype=np.float64)
    n = y.size
    e = np.ones(n) if e is None else np.asarray(e, dtype=np.float64)
    n_trials = np.ones(n) if n_trials is None else np.asarray(n_trials, dtype=np.float64)
    fun = (lambda eta: poisson(eta, y, e)) if lik == "poisson" else (lambda eta: binomial(eta, y, n_trials))
    c = spec.coefficients(theta)
    Qp = mo.kron_prior(spec.terms, spec.term_vw, c.alpha, c.beta, spec.ns, spec.nv, spec.nt, spec.nb,
                       spec.tip_prec).toarray()
    Ad = A.toarray()
    x = np.array(x0, dtype=np.float64)
    dx = np.zeros_like(x)
    for it in range(max_iter + 2):
        if it > max_iter:
            raise ValueError("inner iteration did not converge")
        x = x + dx
        eta = Ad @ x
        _, g, w = fun(eta)
        Qc = Qp + Ad.T @ (w[:, None] * Ad)
        rhs = -Qp @ x + Ad.T @ g
        dx = np.linalg.solve(Qc, rhs)
        if np.linalg.norm(dx) < eps:
            break
    nbk = spec.nt * spec.nv * spec.ns
    ld_p = 2.0 * np.sum(np.log(np.diag(np.linalg.cholesky(Qp[:nbk, :nbk]))))
    ld_c = 2.0 * np.sum(np.log(np.diag(np.linalg.cholesky(Qc))))
    lik_val, _, _ = fun(eta)
    f = -(spec.log_prior(theta) + lik_val + 0.5 * ld_p - 0.5 * float(x @ Qp @ x) - 0.5 * ld_c)
    return float(f), x
