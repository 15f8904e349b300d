"""The theta-Hessian oracle against the reference's own PyINLA._evaluate_hessian_f.

Fixture from tests/golden/make_hessian_golden.py (reference Hessian and covariance of
the hyperparameters, src/pyinla/core/pyinla.py:747-910, on the oracle objective).
"""
import numpy as np

from oracle import model_oracle as mo
from tests.conftest import GOLDEN
from tests.golden.make_hessian_golden import make_spec, oracle_objective


def relerr(x, y):
    return float(np.max(np.abs(np.asarray(x) - np.asarray(y))) / max(np.max(np.abs(y)), 1e-300))


def test_oracle_hessian_matches_reference_fixture():
    g = np.load(GOLDEN / "hessian_spde5x5_nt4.npz")
    spec, theta = make_spec()
    assert np.array_equal(theta, g["theta"])
    H = mo.hessian_fd(oracle_objective(spec), theta, float(g["eps"]))
    assert relerr(H, g["hessian"]) < 1e-12
    assert relerr(np.linalg.inv(H), g["cov"]) < 1e-10


def test_gradient_differences_agree_with_function_differences():
    """FD of the exact (dense) gradient and the reference's FD of f approximate the same
    Hessian: both are O(eps^2) accurate; at eps = 5e-3 they agree to ~1e-5 here."""
    g = np.load(GOLDEN / "hessian_spde5x5_nt4.npz")
    spec, theta = make_spec()

    def grad(th):
        return mo.dense_gradient(spec.terms, spec.term_vw, spec.ns, spec.nv, spec.nt, spec.nb, spec.A, spec.y,
                                 spec.tip_prec, spec.coefficients(th), spec.coefficient_derivatives(th),
                                 spec.lik_theta_indices(), spec.log_prior_grad(th))

    Hg = mo.hessian_from_gradient(grad, theta, float(g["eps"]))
    assert relerr(Hg, g["hessian"]) < 1e-4
