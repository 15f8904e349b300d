"""Generate the Gaussian objective fixture under tests/golden/ from the reference itself.

Run where the reference source tree is available (``$PYINLA_REFERENCE_SRC``, required:
the reference's ``src/`` directory); the fixture is committed, so tests never read the
reference.

What runs is the reference's own code for f(theta) with a Gaussian likelihood:

* ``PyINLA._evaluate_f``, Gaussian branch (src/pyinla/core/pyinla.py:631-688):
  Q_prior, Q_cond at eta = 0, cholesky "bta", information vector, solve for the mean,
  the conditional term, the hyperparameter prior, the likelihood and the prior term;
* ``PyINLA._evaluate_prior_latent_parameters`` (pyinla.py:1076-1110: cholesky "bt" of
  Q_prior and the "bt" logdet, which leaves out the arrow tip) and
  ``PyINLA._evaluate_conditional_latent_parameters`` (pyinla.py:1112-1167: the "bta"
  logdet, the tip symmetrisation and mu^T Q_cond mu);
* univariate model: ``Model.construct_Q_conditional``, ``Model.construct_information_vector``
  and ``Model.evaluate_likelihood`` (src/pyinla/core/model.py:384-449, 490-500) with the
  ``GaussianLikelihood`` methods (src/pyinla/likelihoods/gaussian.py:19-131);
* coregional model (two variates): ``CoregionalModel.construct_Q_conditional``,
  ``custom_Q_ATDA``, ``spgemm``, ``construct_information_vector`` and
  ``evaluate_likelihood`` (src/pyinla/models/coregional_model.py:557-686), one
  ``GaussianLikelihood`` per variate with its own noise precision;
* the solver is the reference's ``SerinvSolver`` with the oracle as Serinv.

One NumPy-version incompatibility is bridged: the univariate Model.evaluate_likelihood
returns a length-1 array (it slices theta), which NumPy 2 no longer converts with
float(); the stand-in passes on its single element.

The stand-in objects supply what those methods read: Q_prior from the oracle's
Kronecker assembly (oracle/model_oracle.py, itself pinned to the reference's
spatio-temporal and coregional prior formulas by the CPU tests), the hyperparameter
log-prior of the spec, the observations grouped by variate (the coregional model's
``n_observations_idx`` layout), and single-process communicators.

Per model, f and the conditional mean are stored at three theta points.
"""
from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np
import scipy.sparse as sps

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))

from oracle import model_oracle as mo  # noqa: E402
from tests.golden.make_golden import _import_reference, checksum  # noqa: E402

UNI = dict(n_side=6, nt=5, nb=3, n_obs=600, seed=17)
COREG = dict(n_side=4, m_side=5, nt=4, nb_per=2, nv=2, n_obs=800, seed=19)


def uni_spec():
    from pyinla_gb300.model import SeparableSpdeAr1

    return SeparableSpdeAr1.synthetic(UNI["n_side"], UNI["nt"], UNI["nb"], UNI["n_obs"], seed=UNI["seed"])


def coreg_spec():
    from pyinla_gb300.model import CoregionalSpdeAr1

    return CoregionalSpdeAr1.synthetic(COREG["n_side"], COREG["nt"], COREG["nb_per"], COREG["nv"], COREG["n_obs"],
                                       seed=COREG["seed"], m_side=COREG["m_side"])


def theta_points(spec):
    d = spec.theta0.size
    return [spec.theta0.copy(), spec.theta0 + 0.15 * np.sin(1.0 + np.arange(d)),
            spec.theta0 - 0.2 * np.cos(2.0 + np.arange(d))]


def input_checksum(spec):
    return checksum(spec.A.toarray() if sps.issparse(spec.A) else spec.A, spec.y)


def _gaussian_likelihood(GaussianLikelihood, n):
    like = types.SimpleNamespace(n_observations=n)
    for name in ("evaluate_likelihood", "evaluate_gradient_likelihood", "evaluate_hessian_likelihood"):
        setattr(like, name, types.MethodType(getattr(GaussianLikelihood, name), like))
    return like


def _stand_in_inla(model, solver, PyINLA, DummyCommunicator):
    me = types.SimpleNamespace()
    me.model = model
    me.solver = solver
    me.comm_feval = DummyCommunicator()
    me.comm_qeval = DummyCommunicator()
    me.qeval_world = DummyCommunicator()
    me.color_qeval = 0
    me.t_construction_qprior = 0.0
    me.t_construction_qconditional = 0.0
    me._evaluate_prior_latent_parameters = types.MethodType(PyINLA._evaluate_prior_latent_parameters, me)
    me._evaluate_conditional_latent_parameters = types.MethodType(PyINLA._evaluate_conditional_latent_parameters, me)
    return me


def _prior_builder(spec, model):
    def construct_Q_prior():
        c = spec.coefficients(model.theta)
        model.Q_prior = mo.kron_prior(spec.terms, spec.term_vw, c.alpha, c.beta, spec.ns, spec.nv, spec.nt, spec.nb,
                                      spec.tip_prec).tocsc()
        return model.Q_prior
    return construct_Q_prior


def run_uni(refs):
    SolverConfig, SerinvSolver, PyINLA, Model, GaussianLikelihood, _, DummyCommunicator = refs
    spec = uni_spec()
    N = spec.A.shape[1]
    model = types.SimpleNamespace()
    model.theta = np.zeros(spec.theta0.size)
    model.x = np.zeros(N)
    model.y = np.asarray(spec.y, dtype=np.float64)
    model.a = sps.csr_matrix(spec.A)
    model.likelihood = _gaussian_likelihood(GaussianLikelihood, spec.y.size)
    model.likelihood_config = types.SimpleNamespace(type="gaussian")
    model.submodels = [object()]
    model.hyperparameters_idx = [0, spec.lik_theta_indices()[0]]
    model.construct_Q_prior = _prior_builder(spec, model)
    for name in ("construct_Q_conditional", "construct_information_vector"):
        setattr(model, name, types.MethodType(getattr(Model, name), model))
    # Model.evaluate_likelihood hands the likelihood theta as a length-1 slice
    # (model.py:495-497), so it returns a length-1 array, which _evaluate_f passes to
    # float() (pyinla.py:681); NumPy 2 refuses float() of a 1-d array, so the stand-in
    # returns the element itself (the value is unchanged).
    model.evaluate_likelihood = lambda eta: np.asarray(Model.evaluate_likelihood(model, eta)).reshape(-1)[0]
    model.evaluate_log_prior_hyperparameters = lambda: spec.log_prior(model.theta)
    model.is_likelihood_gaussian = lambda: True
    model.total_number_fixed_effects = lambda: spec.nb
    solver = SerinvSolver(SolverConfig(type="serinv"), diagonal_blocksize=spec.b, n_diag_blocks=spec.nt,
                          arrowhead_blocksize=spec.nb)
    return spec, _stand_in_inla(model, solver, PyINLA, DummyCommunicator)


def run_coreg(refs):
    SolverConfig, SerinvSolver, PyINLA, _, GaussianLikelihood, CoregionalModel, DummyCommunicator = refs
    spec = coreg_spec()
    ov = np.asarray(spec.obs_variates())
    order = np.argsort(ov, kind="stable")             # observations grouped by variate
    A = sps.csr_matrix(spec.A)[order]
    y = np.asarray(spec.y, dtype=np.float64)[order]
    counts = np.bincount(ov, minlength=spec.nv)
    N = A.shape[1]
    model = types.SimpleNamespace()
    model.theta = np.zeros(spec.theta0.size)
    model.x = np.zeros(N)
    model.y = y
    model.a = A
    model.n_observations = y.size
    model.n_observations_idx = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    lik_idx = spec.lik_theta_indices()
    # CoregionalModel reads variate i's noise log-precision at hyperparameters_idx[i + 1] - 1
    model.hyperparameters_idx = [0] + [int(k) + 1 for k in lik_idx]
    model.models = []
    for v in range(spec.nv):
        sub = types.SimpleNamespace(likelihood=_gaussian_likelihood(GaussianLikelihood, int(counts[v])),
                                    likelihood_config=types.SimpleNamespace(type="gaussian"))
        sub.is_likelihood_gaussian = lambda: True
        model.models.append(sub)
    model.construct_Q_prior = _prior_builder(spec, model)
    for name in ("spgemm", "custom_Q_ATDA", "construct_Q_conditional", "construct_information_vector",
                 "evaluate_likelihood", "is_likelihood_gaussian"):
        setattr(model, name, types.MethodType(getattr(CoregionalModel, name), model))
    model.evaluate_log_prior_hyperparameters = lambda: spec.log_prior(model.theta)
    model.total_number_fixed_effects = lambda: spec.nb
    solver = SerinvSolver(SolverConfig(type="serinv"), diagonal_blocksize=spec.b, n_diag_blocks=spec.nt,
                          arrowhead_blocksize=spec.nb)
    return spec, _stand_in_inla(model, solver, PyINLA, DummyCommunicator)


def main():
    SolverConfig, _, SerinvSolver = _import_reference()
    from pyinla.core.model import Model
    from pyinla.core.pyinla import PyINLA
    from pyinla.likelihoods.gaussian import GaussianLikelihood
    from pyinla.models.coregional_model import CoregionalModel
    from pyinla.utils import DummyCommunicator

    refs = (SolverConfig, SerinvSolver, PyINLA, Model, GaussianLikelihood, CoregionalModel, DummyCommunicator)
    out = {}
    for tag, build in (("uni", run_uni), ("coreg", run_coreg)):
        spec, me = build(refs)
        out[f"{tag}_checksum"] = input_checksum(spec)
        for k, theta in enumerate(theta_points(spec)):
            f = float(PyINLA._evaluate_f(me, theta.copy(), comm=DummyCommunicator()))
            out[f"{tag}_theta{k}"] = theta
            out[f"{tag}_f{k}"] = f
            out[f"{tag}_x{k}"] = np.asarray(me.model.x, dtype=np.float64).copy()
            print(f"{tag} theta{k}: f = {f:.10f}")
    path = HERE / "gaussian_objective.npz"
    np.savez_compressed(path, **out)
    print(f"wrote {path.name}")


if __name__ == "__main__":
    main()
