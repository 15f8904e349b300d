"""CPU checks of the model oracle (oracle/model_oracle.py) and of the adjoint formula.

The gradient formula used on the GPU -- traces of Q^{-1} dQ/dtheta plus the mean
terms -- is checked here with dense FP64 algebra against central differences of the
oracle objective, which restates PyINLA._evaluate_f for the Gaussian branch.
"""
import numpy as np
import pytest

from oracle import bta_oracle as orc
from oracle import model_oracle as mo
from pyinla_gb300 import spde
from pyinla_gb300.model import SeparableSpdeAr1, union_pattern


def small_spec(seed=0, n_side=5, nt=4, nb=2, n_obs=300):
    return SeparableSpdeAr1.synthetic(n_side, nt, nb, n_obs, seed)


def oracle_f(spec, theta):
    c = spec.coefficients(theta)
    f, _ = mo.objective(spec.terms, spec.term_vw, spec.ns, spec.nv, spec.nt, spec.nb, spec.A, spec.y,
                        spec.tip_prec, c.alpha, c.beta, c.tau_y, theta[spec.lik_theta_index()],
                        spec.log_prior(theta))
    return f


def test_oracle_objective_matches_dense():
    spec = small_spec()
    theta = spec.theta0 + np.array([0.1, -0.2, 0.3, 0.05])
    c = spec.coefficients(theta)
    f, aux = mo.objective(spec.terms, spec.term_vw, spec.ns, spec.nv, spec.nt, spec.nb, spec.A, spec.y,
                          spec.tip_prec, c.alpha, c.beta, c.tau_y, theta[3], spec.log_prior(theta))
    Qp = aux["Qp"].toarray()
    Qc = aux["Qc"].toarray()
    nbk = spec.nt * spec.b
    ld_p = np.linalg.slogdet(Qp[:nbk, :nbk])[1]
    ld_c = np.linalg.slogdet(Qc)[1]
    assert abs(aux["logdet_prior"] - ld_p) < 1e-9 * abs(ld_p)
    assert abs(aux["logdet_cond"] - ld_c) < 1e-9 * abs(ld_c)
    mu = np.linalg.solve(Qc, c.tau_y * (spec.A.T @ spec.y))
    assert np.max(np.abs(aux["mu"] - mu)) < 1e-10 * np.max(np.abs(mu))


def test_separable_prior_is_kronecker():
    spec = small_spec()
    theta = spec.theta0
    c = spec.coefficients(theta)
    Qp = mo.kron_prior(spec.terms, spec.term_vw, c.alpha, c.beta, spec.ns, 1, spec.nt, spec.nb, spec.tip_prec)
    kappa, r_t, rho, tau, _ = spec.unpack(theta)
    Qs = sum(w * S for w, S in zip(spde.spde_weights(kappa), spec.terms))
    d, o = spde.ar1_bands(rho, spec.nt)
    T = mo.temporal_matrix(d, o)
    import scipy.sparse as sps
    ref = tau * sps.kron(T, Qs)
    nbk = spec.nt * spec.ns
    assert abs(Qp[:nbk, :nbk] - ref).max() < 1e-12 * abs(ref).max()


def test_dense_gradient_matches_central_differences():
    spec = small_spec(seed=3)
    theta = spec.theta0 + np.array([0.2, 0.1, -0.3, 0.1])
    g = mo.dense_gradient(spec.terms, spec.term_vw, spec.ns, spec.nv, spec.nt, spec.nb, spec.A, spec.y,
                          spec.tip_prec, spec.coefficients(theta), spec.coefficient_derivatives(theta),
                          spec.lik_theta_index(), spec.log_prior_grad(theta))
    fd = mo.central_difference(lambda th: oracle_f(spec, th), theta, 1e-5)
    np.testing.assert_allclose(g, fd, rtol=1e-6, atol=1e-6 * np.max(np.abs(fd)))


def test_union_pattern_values():
    spec = small_spec()
    rp, col, uval = union_pattern(spec.terms)
    for k, S in enumerate(spec.terms):
        rows = np.repeat(np.arange(spec.ns), np.diff(rp))
        import scipy.sparse as sps
        R = sps.csr_matrix((uval[:, k], (rows, col)), shape=S.shape)
        assert abs(R - S).max() == 0.0
