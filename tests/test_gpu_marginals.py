"""GPU checks of the marginal variances (gbta_sigma_diagonal, gbta_obs_variances).

* against the fixtures of the reference's own PyINLA.get_marginal_variances_latent_parameters
  and PyINLA.get_marginal_variances_observations (tests/golden/make_marginals_golden.py);
* the drop-in PyINLA methods (pyinla_gb300.marginals) on a stand-in PyINLA object:
  values and the reference's error behaviour;
* edge cases against the oracle: no arrow, nt = 1, rows touching two time blocks,
  an empty observation matrix, a column outside the matrix (NaN for that row);
* the model path (KronGaussianModel.marginal_variances) against the dense inverse
  of the oracle's Q_cond.
"""
import types

import numpy as np
import pytest
import scipy.sparse as sps

from oracle import bta_oracle as orc
from oracle import marginals_oracle as mo
from tests.conftest import GOLDEN
from tests.golden.make_marginals_golden import CASES, make_inputs

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def relerr(x, y):
    x = np.asarray(x)
    y = np.asarray(y)
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


@pytest.fixture(scope="module")
def built():
    from pyinla_gb300 import build

    build.build()
    return True


def gpu_solver(Q, nt, b, a):
    from pyinla_gb300.solver import GB300SerinvSolver

    s = GB300SerinvSolver(None, diagonal_blocksize=b, n_diag_blocks=nt, arrowhead_blocksize=a)
    s.cholesky(sps.csc_matrix(Q), sparsity="bta")
    s.selected_inversion(sparsity="bta")
    return s


@pytest.mark.parametrize("name", list(CASES))
def test_marginal_variances_match_reference_fixtures(built, name):
    from pyinla_gb300 import marginals

    g = np.load(GOLDEN / f"marginals_{name}.npz")
    seed, nt, b, a, n_obs = (int(g[k]) for k in ("seed", "nt", "b", "a", "n_obs"))
    Q, A = make_inputs(seed, nt, b, a, n_obs)
    s = gpu_solver(Q, nt, b, a)
    assert relerr(marginals.solver_latent_variances(s), g["latent"]) < RTOL
    obs = marginals.solver_observation_variances(s, A)
    assert relerr(obs, g["observations"]) < RTOL
    # deterministic
    assert np.array_equal(obs, marginals.solver_observation_variances(s, A))


class _Model:
    def __init__(self, Q, A, gaussian=True):
        self.Q_conditional = sps.csc_matrix(Q)
        self.a = A
        self.theta = np.zeros(2)
        self.x = np.zeros(Q.shape[0])
        self._gaussian = gaussian

    def construct_Q_conditional(self, eta):
        return self.Q_conditional

    def is_likelihood_gaussian(self):
        return self._gaussian


def _stand_in(Q, A, nt, b, a, gaussian=True):
    from pyinla_gb300.solver import GB300SerinvSolver

    me = types.SimpleNamespace()
    me.model = _Model(Q, A, gaussian)
    me.solver = GB300SerinvSolver(None, diagonal_blocksize=b, n_diag_blocks=nt, arrowhead_blocksize=a)
    calls = []

    def compute(theta, x_star):          # PyINLA._compute_covariance_latent_parameters (pyinla.py:912-938)
        calls.append((theta, x_star))
        me.model.construct_Q_conditional(me.model.a @ x_star)
        me.solver.cholesky(me.model.Q_conditional, sparsity="bta")
        me.solver.selected_inversion(sparsity="bta")

    me._compute_covariance_latent_parameters = compute
    return me, calls


def test_dropin_pyinla_methods(built):
    from pyinla_gb300 import marginals

    g = np.load(GOLDEN / "marginals_ragged.npz")
    seed, nt, b, a, n_obs = (int(g[k]) for k in ("seed", "nt", "b", "a", "n_obs"))
    Q, A = make_inputs(seed, nt, b, a, n_obs)
    me, calls = _stand_in(Q, A, nt, b, a)
    theta, x = np.ones(2), np.zeros(Q.shape[0])
    lat = marginals.get_marginal_variances_latent_parameters(me, theta, x)
    obs = marginals.get_marginal_variances_observations(me, theta, x)
    assert relerr(lat, g["latent"]) < RTOL and relerr(obs, g["observations"]) < RTOL
    assert len(calls) == 2 and calls[0][0] is theta
    # neither given: the model's stored theta and x (pyinla.py:943-948)
    lat2 = marginals.get_marginal_variances_latent_parameters(me)
    assert calls[-1][0] is me.model.theta and relerr(lat2, g["latent"]) < RTOL
    with pytest.raises(ValueError):
        marginals.get_marginal_variances_latent_parameters(me, theta, None)
    with pytest.raises(ValueError):
        marginals.get_marginal_variances_observations(me, None, x)
    me_ng, _ = _stand_in(Q, A, nt, b, a, gaussian=False)
    with pytest.raises(NotImplementedError):
        marginals.get_marginal_variances_observations(me_ng, theta, x)
    # install() puts them on a class
    cls = type("PyINLA", (), {})
    marginals.install(cls)
    assert cls.get_marginal_variances_observations is marginals.get_marginal_variances_observations


@pytest.mark.parametrize("nt,b,a,n_obs", [(5, 24, 0, 200), (1, 40, 3, 60), (7, 33, 2, 500), (3, 64, 32, 300)])
def test_marginal_variances_edge_shapes(built, nt, b, a, n_obs):
    from pyinla_gb300 import marginals

    D, L, R, T, _ = orc.make_bta_c1(31 + nt, nt=nt, b=b, a=a)
    A = mo.make_observation_matrix(77 + b, nt, b, a, n_obs, spread=0.3)
    Q = orc.bta_to_dense(D, L, R if a else None, T if a else None) + (A.T @ A).toarray()
    S = np.linalg.inv(Q)
    s = gpu_solver(Q, nt, b, a)
    assert relerr(marginals.solver_latent_variances(s), np.diagonal(S)) < RTOL
    assert relerr(marginals.solver_observation_variances(s, A), np.diagonal(A @ S @ A.T)) < RTOL
    # empty observation matrix
    assert marginals.solver_observation_variances(s, sps.csr_matrix((0, Q.shape[0]))).shape == (0,)


def test_out_of_range_column_gives_nan(built):
    import torch

    from pyinla_gb300 import _lib, marginals

    nt, b, a = 3, 16, 2
    D, L, R, T, _ = orc.make_bta_c1(3, nt=nt, b=b, a=a)
    Q = orc.bta_to_dense(D, L, R, T)
    s = gpu_solver(Q, nt, b, a)
    N = nt * b + a
    rowptr = torch.tensor([0, 2, 4], dtype=torch.int64, device="cuda")
    col = torch.tensor([0, 5, 3, N], dtype=torch.int32, device="cuda")    # row 1 has column N (outside)
    val = torch.tensor([1.0, 2.0, 1.0, 1.0], dtype=torch.float64, device="cuda")
    out = torch.empty(2, dtype=torch.float64, device="cuda")
    h = s._h
    _lib.check(h.lib.gbta_obs_variances(h.ptr, 2, rowptr.data_ptr(), col.data_ptr(), val.data_ptr(),
                                        s.A_diagonal_blocks.data_ptr(), s.A_lower_diagonal_blocks.data_ptr(),
                                        s.A_arrow_bottom_blocks.data_ptr(), s.A_arrow_tip_block.data_ptr(),
                                        out.data_ptr()))
    o = out.cpu().numpy()
    S = np.linalg.inv(Q)
    assert abs(o[0] - (S[0, 0] + 4 * S[0, 5] + 4 * S[5, 5])) < 1e-12 * abs(S[0, 0])
    assert np.isnan(o[1])
    with pytest.raises(ValueError):
        marginals.solver_observation_variances(s, sps.csr_matrix((1, N + 1)))


@pytest.mark.parametrize("kind", ["univariate", "coregional"])
def test_model_marginal_variances(built, kind):
    from pyinla_gb300.model import CoregionalSpdeAr1, KronGaussianModel, SeparableSpdeAr1

    if kind == "univariate":
        spec = SeparableSpdeAr1.synthetic(6, 4, 3, 800, seed=11)
        theta = spec.theta0 + 0.1
    else:
        spec = CoregionalSpdeAr1.synthetic(5, 4, 2, 2, 900, seed=12, m_side=6)
        theta = spec.theta0 + 0.05
    m = KronGaussianModel(spec)
    lat, obs = m.marginal_variances(theta)
    _, Qc = spec.sparse_precisions(theta)
    S = np.linalg.inv(Qc.toarray())
    assert relerr(lat, np.diagonal(S)) < RTOL
    A = sps.csr_matrix(spec.A)
    assert relerr(obs, np.asarray((A @ S @ A.T).diagonal()).ravel()) < RTOL
