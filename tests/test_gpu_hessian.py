"""GPU check of the theta-Hessian (KronGaussianModel.hessian / covariance_hp).

* against the same central differences of the oracle's exact dense gradient (same
  step): the adjoint gradient matches the dense one to ~1e-8, so the two Hessians
  agree to ~1e-6;
* against the reference's own FD-of-f Hessian and covariance (fixture of
  tests/golden/make_hessian_golden.py): both are O(eps^2) approximations of the
  Hessian; at eps = 5e-3 they agree to ~1e-5 here.
"""
import numpy as np
import pytest

from oracle import model_oracle as mo
from tests.conftest import GOLDEN
from tests.golden.make_hessian_golden import make_spec

pytestmark = pytest.mark.gpu


def relerr(x, y):
    return float(np.max(np.abs(np.asarray(x) - np.asarray(y))) / max(np.max(np.abs(y)), 1e-300))


@pytest.fixture(scope="module")
def built():
    from pyinla_gb300 import build

    build.build()
    return True


def test_hessian_and_covariance(built):
    from pyinla_gb300.model import KronGaussianModel

    g = np.load(GOLDEN / "hessian_spde5x5_nt4.npz")
    spec, theta = make_spec()
    eps = float(g["eps"])
    m = KronGaussianModel(spec)
    H = m.hessian(theta, eps)

    def grad(th):
        return mo.dense_gradient(spec.terms, spec.term_vw, spec.ns, spec.nv, spec.nt, spec.nb, spec.A, spec.y,
                                 spec.tip_prec, spec.coefficients(th), spec.coefficient_derivatives(th),
                                 spec.lik_theta_indices(), spec.log_prior_grad(th))

    assert relerr(H, mo.hessian_from_gradient(grad, theta, eps)) < 1e-6
    assert relerr(H, g["hessian"]) < 1e-4
    assert np.array_equal(H, H.T)
    assert relerr(m.covariance_hp(theta, eps), g["cov"]) < 1e-3
