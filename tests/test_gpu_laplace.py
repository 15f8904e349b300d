"""GPU checks of the non-Gaussian Laplace objective (pyinla_gb300.laplace).

* against the reference's own objective path on the committed fixtures (Poisson and
  Binomial, two theta points in sequence so that the warm start is exercised);
* against the oracle on a larger problem (ragged block size b = 49, 3 fixed effects);
* the building blocks: gbta_bta_symv against the dense prior, gbta_weighted_gram
  against A^T W A.
"""
import numpy as np
import pytest
import scipy.sparse as sps

from oracle import laplace_oracle as lo
from oracle import model_oracle as mo
from tests.conftest import GOLDEN
from tests.golden.make_laplace_golden import make_problem

pytestmark = pytest.mark.gpu


def relerr(x, y):
    return float(np.max(np.abs(np.asarray(x) - np.asarray(y))) / max(np.max(np.abs(y)), 1e-300))


@pytest.fixture(scope="module")
def built():
    from pyinla_gb300 import build

    build.build()
    return True


@pytest.mark.parametrize("lik", ["poisson", "binomial"])
def test_laplace_matches_reference_fixture(built, lik):
    from pyinla_gb300.laplace import KronLaplaceModel

    g = np.load(GOLDEN / f"laplace_{lik}.npz")
    spec, aux = make_problem(lik)
    kw = {"e": aux} if lik == "poisson" else {"n_trials": aux}
    m = KronLaplaceModel(spec, lik, **kw)
    for k in range(2):
        f = m.evaluate(g[f"theta{k}"])
        assert abs(f - float(g[f"f{k}"])) <= 1e-10 * abs(float(g[f"f{k}"])), (f, float(g[f"f{k}"]))
        assert relerr(m.x_latent.cpu().numpy(), g[f"x{k}"]) < 1e-8


def test_laplace_larger_problem_matches_oracle(built):
    from pyinla_gb300.laplace import KronLaplaceModel
    from pyinla_gb300.model import SeparableSpdeAr1

    spec = SeparableSpdeAr1.synthetic(7, 5, 3, 3000, seed=21)
    rng = np.random.default_rng(5)
    eta = spec.A @ (0.2 * rng.standard_normal(spec.A.shape[1]))
    e = rng.integers(1, 3, spec.A.shape[0]).astype(np.float64)
    spec.y = rng.poisson(e * np.exp(eta)).astype(np.float64)
    m = KronLaplaceModel(spec, "poisson", e=e)
    theta = spec.theta0 + 0.1
    f = m.evaluate(theta)
    fo, xo = lo.laplace_objective(spec, theta, "poisson", np.zeros(spec.A.shape[1]), e=e)
    assert abs(f - fo) <= 1e-10 * abs(fo)
    assert relerr(m.x_latent.cpu().numpy(), xo) < 1e-8


def test_bta_symv_and_weighted_gram(built):
    import torch

    from pyinla_gb300 import _lib
    from pyinla_gb300.laplace import KronLaplaceModel
    from pyinla_gb300.model import SeparableSpdeAr1

    spec = SeparableSpdeAr1.synthetic(6, 4, 2, 600, seed=3)
    spec.y = np.ones(spec.A.shape[0])
    m = KronLaplaceModel(spec, "poisson")
    theta = spec.theta0
    c = spec.coefficients(theta)
    ptrs = m._upload_coef(c)
    m.h.set_stream(torch.cuda.current_stream().cuda_stream)
    m._assemble(ptrs, m.Dp, m.Lp, m.Rp, m.Tp, with_lik=False)
    x = torch.from_numpy(np.random.default_rng(1).standard_normal(m.N)).cuda()
    y = torch.empty_like(x)
    _lib.check(m.h.lib.gbta_bta_symv(m.h.ptr, m.Dp.data_ptr(), m.Lp.data_ptr(), m.Rp.data_ptr(), m.Tp.data_ptr(), 1,
                                     x.data_ptr(), y.data_ptr()))
    Qp = mo.kron_prior(spec.terms, spec.term_vw, c.alpha, c.beta, spec.ns, spec.nv, spec.nt, spec.nb, spec.tip_prec)
    assert relerr(y.cpu().numpy(), Qp @ x.cpu().numpy()) < 1e-13
    w = torch.from_numpy(np.random.default_rng(2).random(m.n_obs) + 0.5).cuda()
    _lib.check(m.h.lib.gbta_weighted_gram(m.h.ptr, m._n_out, m._wseg.data_ptr(), m._wobs.data_ptr(),
                                          m._wcoef.data_ptr(), w.data_ptr(), m._wout.data_ptr()))
    A = sps.csr_matrix(spec.A)
    G = (A.T @ sps.diags(w.cpu().numpy()) @ A).toarray()
    out = m._wout.cpu().numpy()
    nbk = m.nt * m.b
    Rw = out[m._nnz_d: m._nnz_d + m.nt * m.nb * m.b].reshape(m.nt, m.nb, m.b)
    Tw = out[m._nnz_d + m.nt * m.nb * m.b:].reshape(m.nb, m.nb)
    assert relerr(Rw.transpose(1, 0, 2).reshape(m.nb, nbk), G[nbk:, :nbk]) < 1e-13
    assert relerr(Tw, G[nbk:, nbk:]) < 1e-13
    rp, cl = m._lik_rowptr.cpu().numpy(), m._lik_col.cpu().numpy()
    rows = np.repeat(np.arange(nbk), np.diff(rp))
    cols = (rows // m.b) * m.b + cl
    assert relerr(out[: m._nnz_d], G[rows, cols]) < 1e-13
