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
from pyinla_gb300.model import KronGaussianModel, SeparableSpdeAr1

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
                          spec.tip_prec, c.alpha, c.beta, c.tau_y, theta[spec.lik_theta_index()],
                          spec.log_prior(theta))
    return f, aux


@pytest.mark.parametrize("n_side,nt,nb,n_obs", [(5, 4, 2, 300), (8, 3, 6, 2000), (6, 1, 3, 500)])
def test_device_assembly_matches_oracle(built, n_side, nt, nb, n_obs):
    import torch

    spec = SeparableSpdeAr1.synthetic(n_side, nt, nb, n_obs, seed=5)
    m = KronGaussianModel(spec)
    theta = spec.theta0 + np.array([0.1, -0.1, 0.2, 0.3])
    c = spec.coefficients(theta)
    ap, bp = m._upload_coef(c)
    m.h.set_stream(torch.cuda.current_stream().cuda_stream)
    m._assemble(ap, bp, c.tau_y, m.Dc, m.Lc, m.Rc, m.Tc, with_lik=True)
    m._assemble(ap, bp, 0.0, m.Dp, m.Lp, m.Rp, m.Tp, with_lik=False)
    torch.cuda.synchronize()
    Qp = mo.kron_prior(spec.terms, spec.term_vw, c.alpha, c.beta, spec.ns, 1, nt, nb, spec.tip_prec)
    Qc = Qp + c.tau_y * (spec.A.T @ spec.A)
    for (D, L, R, T), Q in (((m.Dc, m.Lc, m.Rc, m.Tc), Qc), ((m.Dp, m.Lp, m.Rp, m.Tp), Qp)):
        Do, Lo, Ro, To = mo.sparse_to_bta(Q, nt, spec.b, nb)
        assert relerr(D.cpu().numpy(), Do) < 1e-13
        if nt > 1:
            assert relerr(L.cpu().numpy()[: nt - 1], Lo) < 1e-13
        assert relerr(R.cpu().numpy(), Ro) < 1e-13
        assert relerr(T.cpu().numpy(), To) < 1e-13
    # deterministic: a second assembly is bit-identical
    D1 = m.Dc.clone()
    m._assemble(ap, bp, c.tau_y, m.Dc, m.Lc, m.Rc, m.Tc, with_lik=True)
    torch.cuda.synchronize()
    assert torch.equal(D1, m.Dc)


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
                           spec.lik_theta_index(), spec.log_prior_grad(theta))
    assert relerr(g, gd) < 1e-8, (g, gd)
    h = 1e-4
    fd = np.zeros(4)
    for k in range(4):
        e = np.zeros(4)
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
