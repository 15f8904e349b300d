"""CPU checks of the model oracle (oracle/model_oracle.py) and of the adjoint formula.

The oracle objective, which restates PyINLA._evaluate_f for the Gaussian branch, is
pinned to the reference's own _evaluate_f (fixture tests/golden/gaussian_objective.npz,
made by tests/golden/make_gaussian_golden.py) for a univariate and a bivariate
coregional model.  The gradient formula used on the GPU -- traces of Q^{-1}
dQ/dtheta plus the mean terms -- is checked with dense FP64 algebra against central
differences of the oracle objective.
"""
import numpy as np
import pytest

from oracle import bta_oracle as orc
from oracle import model_oracle as mo
from pyinla_gb300 import spde
from pyinla_gb300.model import CoregionalSpdeAr1, SeparableSpdeAr1, union_pattern
from tests.conftest import GOLDEN


def small_spec(seed=0, n_side=5, nt=4, nb=2, n_obs=300):
    return SeparableSpdeAr1.synthetic(n_side, nt, nb, n_obs, seed)


def oracle_f(spec, theta):
    c = spec.coefficients(theta)
    f, _ = mo.objective(spec.terms, spec.term_vw, spec.ns, spec.nv, spec.nt, spec.nb, spec.A, spec.y,
                        spec.tip_prec, c.alpha, c.beta, c.tau_y, theta[spec.lik_theta_indices()],
                        spec.log_prior(theta), spec.obs_variates())
    return f


def test_oracle_objective_matches_reference_fixture():
    """f(theta) and the conditional mean against the reference's own Gaussian
    _evaluate_f (src/pyinla/core/pyinla.py:631-688, 1076-1167) at three theta points,
    univariate and coregional (per-variate noise precisions), at 1e-10."""
    from tests.golden import make_gaussian_golden as gg

    g = np.load(GOLDEN / "gaussian_objective.npz")
    for tag, spec in (("uni", gg.uni_spec()), ("coreg", gg.coreg_spec())):
        np.testing.assert_allclose(gg.input_checksum(spec), g[f"{tag}_checksum"], rtol=1e-13, atol=0)
        for k in range(3):
            theta = g[f"{tag}_theta{k}"]
            c = spec.coefficients(theta)
            f, aux = mo.objective(spec.terms, spec.term_vw, spec.ns, spec.nv, spec.nt, spec.nb, spec.A, spec.y,
                                  spec.tip_prec, c.alpha, c.beta, c.tau_y, theta[spec.lik_theta_indices()],
                                  spec.log_prior(theta), spec.obs_variates())
            fr = float(g[f"{tag}_f{k}"])
            assert abs(f - fr) <= 1e-10 * abs(fr), (tag, k, f, fr)
            xr = g[f"{tag}_x{k}"]
            assert np.max(np.abs(aux["mu"] - xr)) <= 1e-10 * np.max(np.abs(xr)), (tag, k)


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
    mu = np.linalg.solve(Qc, c.tau_y[0] * (spec.A.T @ spec.y))
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
                          spec.lik_theta_indices(), spec.log_prior_grad(theta))
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


# ---------------------------------------------------------------- coregional model
def coreg_spec(nv, seed=0, n_side=4, m_side=5, nt=4, nb_per=2, n_obs=600):
    return CoregionalSpdeAr1.synthetic(n_side, nt, nb_per, nv, n_obs, seed, m_side=m_side)


def reference_coregional_prior(spec, theta):
    """The reference's construction, restated: per-variate unit-variance priors Qu_k,
    the q_ij blocks of src/pyinla/models/coregional_model.py:297-420 (variate-major
    order), then the permutation to time-major interleaved blocks of
    _generate_permutation_indices (:826-851)."""
    import scipy.sparse as sps

    kappa, r_t, rho, _ = spec._unpack(theta)
    Qu = []
    for k in range(spec.nv):
        Qs = sum(w * S for w, S in zip(spde.spde_weights(kappa[k]), spde.spde_terms(spec.mesh)))
        d, o = spde.ar1_bands(rho[k], spec.nt)
        Qu.append(sps.kron(mo.temporal_matrix(d, o), Qs).tocsr())
    s = spec.sigma
    lam = spec.lam
    if spec.nv == 2:
        l01 = lam["0_1"]
        q11 = Qu[0] / s[0] ** 2 + l01 ** 2 / s[1] ** 2 * Qu[1]
        q21 = -l01 / s[1] ** 2 * Qu[1]
        q22 = Qu[1] / s[1] ** 2
        Q = sps.bmat([[q11, q21.T], [q21, q22]])
    else:
        l01, l02, l12 = lam["0_1"], lam["0_2"], lam["1_2"]
        q11 = Qu[0] / s[0] ** 2 + l01 ** 2 / s[1] ** 2 * Qu[1] + l12 ** 2 / s[2] ** 2 * Qu[2]
        q21 = -l01 / s[1] ** 2 * Qu[1] + l02 * l12 / s[2] ** 2 * Qu[2]
        q31 = -l12 / s[2] ** 2 * Qu[2]
        q22 = Qu[1] / s[1] ** 2 + l02 ** 2 / s[2] ** 2 * Qu[2]
        q32 = -l02 / s[2] ** 2 * Qu[2]
        q33 = Qu[2] / s[2] ** 2
        Q = sps.bmat([[q11, q21.T, q31.T], [q21, q22, q32.T], [q31, q32, q33]])
    n_re = spec.nt * spec.ns
    idx = np.arange(n_re).reshape(spec.nt, spec.ns)
    perm = np.hstack([idx + v * n_re for v in range(spec.nv)]).ravel()
    return Q.tocsr()[perm][:, perm]


@pytest.mark.parametrize("nv", [2, 3])
def test_coregional_prior_matches_reference_blocks(nv):
    spec = coreg_spec(nv)
    theta = spec.theta0 + 0.05 * np.arange(3 * nv)
    c = spec.coefficients(theta)
    Qp = mo.kron_prior(spec.terms, spec.term_vw, c.alpha, c.beta, spec.ns, spec.nv, spec.nt, spec.nb, spec.tip_prec)
    ref = reference_coregional_prior(spec, theta)
    nbk = spec.nt * spec.b
    assert abs(Qp[:nbk, :nbk] - ref).max() < 1e-12 * abs(ref).max()
    tip = Qp[nbk:, nbk:].toarray()
    assert np.array_equal(tip, spec.tip_prec * np.eye(spec.nb))
    assert np.all(np.linalg.eigvalsh(spec.mixing_precision()) > 0)


@pytest.mark.parametrize("nv", [2, 3])
def test_coregional_design_matrix_layout(nv):
    spec = coreg_spec(nv)
    A = spec.A.tocoo()
    ov = spec.obs_variates()
    nbk = spec.nt * spec.b
    field = A.col < nbk
    assert np.all((A.col[field] % spec.b) // spec.ns == ov[A.row[field]])
    assert np.all((A.col[~field] - nbk) // spec.nb_per == ov[A.row[~field]])
    assert np.all(np.diff(ov) >= 0)


@pytest.mark.parametrize("nv", [2, 3])
def test_coregional_dense_gradient_matches_central_differences(nv):
    spec = coreg_spec(nv, seed=4)
    theta = spec.theta0 + 0.1 * np.sin(np.arange(3 * nv))
    g = mo.dense_gradient(spec.terms, spec.term_vw, spec.ns, spec.nv, spec.nt, spec.nb, spec.A, spec.y,
                          spec.tip_prec, spec.coefficients(theta), spec.coefficient_derivatives(theta),
                          spec.lik_theta_indices(), spec.log_prior_grad(theta), spec.obs_variates())
    fd = mo.central_difference(lambda th: oracle_f(spec, th), theta, 1e-5)
    np.testing.assert_allclose(g, fd, rtol=1e-6, atol=1e-6 * np.max(np.abs(fd)))
