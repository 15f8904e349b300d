"""GPU checks of the model path: device assembly, objective and adjoint gradient.

* assembly: the BTA blocks written by gbta_assemble_kron against the oracle's
  reference-style sparse Kronecker assembly + sparse-to-BTA mapping;
* objective: f(theta) against the oracle restatement of PyINLA._evaluate_f;
* gradient: the adjoint against a dense FP64 gradient and against central finite
  differences of the GPU objective (step 1e-4), within 1e-6 relative.
"""
import numpy as np
import pytest

from oracle import model_oracle as mo
from pyinla_gb300.model import CoregionalSpdeAr1, KronGaussianModel, SeparableSpdeAr1

pytestmark = pytest.mark.gpu


def relerr(x, y):
    x = np.asarray(x)
    y = np.asarray(y)
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


@pytest.fixture(scope="module")
def built():
    from pyinla_gb300 import build

    build.build()
    return True


def oracle_f(spec, theta):
    c = spec.coefficients(theta)
    f, aux = mo.objective(spec.terms, spec.term_vw, spec.ns, spec.nv, spec.nt, spec.nb, spec.A, spec.y,
                          spec.tip_prec, c.alpha, c.beta, c.tau_y, theta[spec.lik_theta_indices()],
                          spec.log_prior(theta), spec.obs_variates())
    return f, aux


@pytest.mark.parametrize("n_side,nt,nb,n_obs", [(5, 4, 2, 300), (8, 3, 6, 2000), (6, 1, 3, 500)])
def test_device_assembly_matches_oracle(built, n_side, nt, nb, n_obs):
    import torch

    spec = SeparableSpdeAr1.synthetic(n_side, nt, nb, n_obs, seed=5)
    m = KronGaussianModel(spec)
    theta = spec.theta0 + np.array([0.1, -0.1, 0.2, 0.3])
    c = spec.coefficients(theta)
    check_assembly(m, spec, theta)


def check_assembly(m, spec, theta):
    import torch

    c = spec.coefficients(theta)
    ptrs = m._upload_coef(c)
    m.h.set_stream(torch.cuda.current_stream().cuda_stream)
    m._assemble(ptrs, m.Dc, m.Lc, m.Rc, m.Tc, with_lik=True)
    m._assemble(ptrs, m.Dp, m.Lp, m.Rp, m.Tp, with_lik=False)
    torch.cuda.synchronize()
    nt, nb = spec.nt, spec.nb
    Qp, Qc = spec.sparse_precisions(theta)
    Qp_o = mo.kron_prior(spec.terms, spec.term_vw, c.alpha, c.beta, spec.ns, spec.nv, nt, nb, spec.tip_prec)
    assert abs(Qp - Qp_o).max() <= 1e-13 * abs(Qp_o).max()
    for (D, L, R, T), Q in (((m.Dc, m.Lc, m.Rc, m.Tc), Qc), ((m.Dp, m.Lp, m.Rp, m.Tp), Qp)):
        Do, Lo, Ro, To = mo.sparse_to_bta(Q, nt, spec.b, nb)
        assert relerr(D.cpu().numpy(), Do) < 1e-13
        if nt > 1:
            assert relerr(L.cpu().numpy()[: nt - 1], Lo) < 1e-13
        if nb:
            assert relerr(R.cpu().numpy(), Ro) < 1e-13
            assert relerr(T.cpu().numpy(), To) < 1e-13
    # deterministic: a second assembly is bit-identical
    D1 = m.Dc.clone()
    m._assemble(ptrs, m.Dc, m.Lc, m.Rc, m.Tc, with_lik=True)
    torch.cuda.synchronize()
    assert torch.equal(D1, m.Dc)


def test_objective_matches_reference_fixture(built):
    """The device objective and mean against the reference's own Gaussian _evaluate_f
    (fixture made by tests/golden/make_gaussian_golden.py), univariate and coregional,
    at 1e-10."""
    from tests.conftest import GOLDEN
    from tests.golden import make_gaussian_golden as gg

    g = np.load(GOLDEN / "gaussian_objective.npz")
    for tag, spec in (("uni", gg.uni_spec()), ("coreg", gg.coreg_spec())):
        m = KronGaussianModel(spec)
        for k in range(3):
            theta = g[f"{tag}_theta{k}"]
            f = m.evaluate(theta)
            fr = float(g[f"{tag}_f{k}"])
            assert abs(f - fr) <= 1e-10 * abs(fr), (tag, k, f, fr)
            assert relerr(m.mu.cpu().numpy(), g[f"{tag}_x{k}"]) < 1e-10, (tag, k)


def test_objective_matches_oracle(built):
    spec = SeparableSpdeAr1.synthetic(8, 5, 6, 3000, seed=7)
    m = KronGaussianModel(spec)
    for dth in (np.zeros(4), np.array([0.3, -0.2, 0.5, -0.4])):
        theta = spec.theta0 + dth
        f = m.evaluate(theta)
        fo, aux = oracle_f(spec, theta)
        assert abs(f - fo) <= 1e-10 * abs(fo), (f, fo)
        assert abs(m.last["logdet_cond"] - aux["logdet_cond"]) <= 1e-10 * abs(aux["logdet_cond"])
        assert abs(m.last["logdet_prior"] - aux["logdet_prior"]) <= 1e-10 * abs(aux["logdet_prior"])
        assert relerr(m.mu.cpu().numpy(), aux["mu"]) < 1e-10


@pytest.mark.parametrize("n_side,nt,nb,n_obs", [(5, 4, 2, 400), (16, 16, 6, 20000)])
def test_adjoint_gradient_matches_dense_and_fd(built, n_side, nt, nb, n_obs):
    """Adjoint vs dense FP64 gradient; the second case is ns = 256, nt = 16, nb = 6."""
    spec = SeparableSpdeAr1.synthetic(n_side, nt, nb, n_obs, seed=9)
    m = KronGaussianModel(spec)
    theta = spec.theta0 + np.array([0.15, -0.1, 0.2, 0.1])
    f, g = m.evaluate(theta, gradient=True)
    gd = mo.dense_gradient(spec.terms, spec.term_vw, spec.ns, spec.nv, spec.nt, spec.nb, spec.A, spec.y,
                           spec.tip_prec, spec.coefficients(theta), spec.coefficient_derivatives(theta),
                           spec.lik_theta_indices(), spec.log_prior_grad(theta))
    assert relerr(g, gd) < 1e-8, (g, gd)
    check_fd(m, theta, g)


def check_fd(m, theta, g, h=1e-4):
    d = theta.size
    fd = np.zeros(d)
    for k in range(d):
        e = np.zeros(d)
        e[k] = h
        fd[k] = (m.evaluate(theta + e) - m.evaluate(theta - e)) / (2 * h)
    assert relerr(g, fd) < 1e-6, (g, fd)


def test_autograd_function(built):
    import torch

    from pyinla_gb300.autograd import LaplaceObjective

    spec = SeparableSpdeAr1.synthetic(5, 4, 2, 300, seed=2)
    m = KronGaussianModel(spec)
    th = torch.tensor(spec.theta0 + 0.1, dtype=torch.float64, requires_grad=True)
    f = LaplaceObjective.apply(th, m)
    f.backward()
    _, g = m.evaluate(th.detach().numpy(), gradient=True)
    assert relerr(th.grad.numpy(), g) < 1e-12


# ---------------------------------------------------------------- coregional model
@pytest.mark.parametrize("nv,n_side,m_side,nt,nb_per,n_obs", [(2, 4, 6, 4, 2, 800), (3, 5, 4, 3, 3, 1200),
                                                               (2, 16, 24, 3, 2, 6000)])
def test_coregional_assembly_matches_oracle(built, nv, n_side, m_side, nt, nb_per, n_obs):
    """Coregional layout (block t = [variate nodes...]) with per-variate noise; the
    last case is the 2-variate ns = 384 (b = 768) block of the mixed batch."""
    spec = CoregionalSpdeAr1.synthetic(n_side, nt, nb_per, nv, n_obs, seed=11, m_side=m_side)
    m = KronGaussianModel(spec)
    check_assembly(m, spec, spec.theta0 + 0.05 * np.cos(np.arange(3 * nv)))


@pytest.mark.parametrize("nv", [2, 3])
def test_coregional_objective_and_gradient(built, nv):
    spec = CoregionalSpdeAr1.synthetic(5, 4, 2, nv, 1500, seed=13, m_side=6)
    m = KronGaussianModel(spec)
    theta = spec.theta0 + 0.1 * np.sin(1.0 + np.arange(3 * nv))
    f, g = m.evaluate(theta, gradient=True)
    fo, aux = oracle_f(spec, theta)
    assert abs(f - fo) <= 1e-10 * abs(fo), (f, fo)
    assert relerr(m.mu.cpu().numpy(), aux["mu"]) < 1e-10
    gd = mo.dense_gradient(spec.terms, spec.term_vw, spec.ns, spec.nv, spec.nt, spec.nb, spec.A, spec.y,
                           spec.tip_prec, spec.coefficients(theta), spec.coefficient_derivatives(theta),
                           spec.lik_theta_indices(), spec.log_prior_grad(theta), spec.obs_variates())
    assert relerr(g, gd) < 1e-8, (g, gd)
    check_fd(m, theta, g)


@pytest.mark.parametrize("kind", ["separable", "coreg2", "coreg3"])
def test_separable_prior_logdet_and_trace(built, kind):
    """The spatial-factor logdet and prior trace of a separable prior equal the BTA
    factorization's logdet and the selected-inverse trace."""
    if kind == "separable":
        spec = SeparableSpdeAr1.synthetic(6, 5, 2, 400, seed=21)
        theta = spec.theta0 + np.array([0.2, -0.1, 0.3, 0.1])
    else:
        nv = 2 if kind == "coreg2" else 3
        spec = CoregionalSpdeAr1.synthetic(4, 4, 2, nv, 900, seed=23, m_side=5)
        theta = spec.theta0 + 0.1 * np.cos(np.arange(3 * nv))
    m = KronGaussianModel(spec)
    f_sep = m.evaluate(theta)                   # prior logdet from the spatial factors
    ld_sep = m.last["logdet_prior"]
    _, g_sep = m.evaluate(theta, gradient=True)
    m.prior_trace = "selinv"                    # the whole prior factored (bt), as the reference
    f_bt = m.evaluate(theta)
    assert abs(ld_sep - m.last["logdet_prior"]) <= 1e-10 * abs(m.last["logdet_prior"])
    assert abs(f_sep - f_bt) <= 1e-10 * abs(f_bt)
    _, g_sel = m.evaluate(theta, gradient=True)
    assert relerr(g_sep, g_sel) < 1e-9, (g_sep, g_sel)
