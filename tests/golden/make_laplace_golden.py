"""Generate the non-Gaussian objective fixtures under tests/golden/ from the reference.

Run where the reference source tree is available (``$PYINLA_REFERENCE_SRC``, required: the reference's ``src/`` directory); the fixtures are committed, so tests never read the reference.

What runs is the reference's own code: PyINLA._evaluate_f (non-Gaussian branch,
src/pyinla/core/pyinla.py:692-729), PyINLA._inner_iteration (:1025-1074),
PyINLA._evaluate_prior_latent_parameters (:1076-1110), Model.construct_Q_conditional,
Model.construct_information_vector, Model.evaluate_likelihood (src/pyinla/core/model.py)
and the Poisson / Binomial likelihood methods (src/pyinla/likelihoods/), on stand-in
objects: the model's Q_prior comes from the oracle's Kronecker assembly
(oracle/model_oracle.py), its hyperparameter prior from the spec, and the solver is the
reference's SerinvSolver with the oracle as Serinv.  Two defects of the reference path
are bridged by the stand-ins and nothing else: _inner_iteration calls
``solver.cholesky(A=Q_conditional)`` without the ``sparsity`` argument (pyinla.py:1060;
the stand-in solver defaults it to "bta"), and _evaluate_conditional_latent_parameters
indexes ``x_mean`` although the non-Gaussian branch passes None (pyinla.py:1155; the
stand-in returns its value at x = x_mean, 0.5 logdet Q_cond).

Per likelihood, f is evaluated at two theta points in sequence (the inner iteration
starts from the previous mode, as the reference's stored model.x does); f and the
modes are stored.
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
from tests.golden.make_golden import _import_reference  # noqa: E402

SEED, N_SIDE, NT, NB, N_OBS = 6, 5, 4, 2, 400
THETA_SHIFTS = (np.array([0.1, -0.05, 0.15, 0.0]), np.array([0.2, 0.05, -0.1, 0.0]))


def make_problem(lik):
    """Spec (synthetic spatio-temporal design) with counts drawn from the likelihood at a
    seeded latent field; e (Poisson exposures) / n (Binomial trials) per observation."""
    from pyinla_gb300.model import SeparableSpdeAr1
    spec = SeparableSpdeAr1.synthetic(N_SIDE, NT, NB, N_OBS, seed=SEED)
    rng = np.random.default_rng(SEED + 100)
    x_true = 0.3 * rng.standard_normal(spec.A.shape[1])
    eta = spec.A @ x_true
    if lik == "poisson":
        aux = rng.integers(1, 4, N_OBS).astype(np.float64)        # exposures e
        y = rng.poisson(aux * np.exp(eta)).astype(np.float64)
    else:
        aux = rng.integers(1, 6, N_OBS).astype(np.float64)        # trials n
        y = rng.binomial(aux.astype(np.int64), 1.0 / (1.0 + np.exp(-eta))).astype(np.float64)
    spec.y = y
    return spec, aux


def main():
    SolverConfig, _, SerinvSolver = _import_reference()
    from pyinla.core.model import Model
    from pyinla.core.pyinla import PyINLA
    from pyinla.likelihoods.binomial import BinomialLikelihood
    from pyinla.likelihoods.poisson import PoissonLikelihood
    from pyinla.utils import DummyCommunicator, sigmoid
    for lik in ("poisson", "binomial"):
        spec, aux = make_problem(lik)
        N = spec.A.shape[1]
        like = types.SimpleNamespace()
        cls = PoissonLikelihood if lik == "poisson" else BinomialLikelihood
        if lik == "poisson":
            like.e = aux
        else:
            like.n_trials = aux
            like.link_function = sigmoid
        like.evaluate_likelihood = types.MethodType(cls.evaluate_likelihood, like)
        like.evaluate_gradient_likelihood = types.MethodType(cls.evaluate_gradient_likelihood, like)
        like.evaluate_hessian_likelihood = types.MethodType(cls.evaluate_hessian_likelihood, like)

        model = types.SimpleNamespace()
        model.theta = np.zeros(4)
        model.x = np.zeros(N)
        model.y = spec.y
        model.a = sps.csr_matrix(spec.A)
        model.likelihood = like
        model.likelihood_config = types.SimpleNamespace(type=lik)
        model.submodels = [object()]
        model.hyperparameters_idx = [0, 4]

        def construct_Q_prior(model=model):
            c = spec.coefficients(model.theta)
            model.Q_prior = mo.kron_prior(spec.terms, spec.term_vw, c.alpha, c.beta, spec.ns, spec.nv, spec.nt,
                                          spec.nb, spec.tip_prec).tocsc()
            return model.Q_prior

        model.construct_Q_prior = construct_Q_prior
        model.construct_Q_conditional = types.MethodType(Model.construct_Q_conditional, model)
        model.construct_information_vector = types.MethodType(Model.construct_information_vector, model)
        model.evaluate_likelihood = types.MethodType(Model.evaluate_likelihood, model)
        model.evaluate_log_prior_hyperparameters = lambda model=model: spec.log_prior(model.theta)
        model.is_likelihood_gaussian = lambda: False

        class StandInSolver(SerinvSolver):
            def cholesky(self, A, sparsity="bta"):
                return super().cholesky(A, sparsity=sparsity)

        me = types.SimpleNamespace()
        me.model = model
        me.solver = StandInSolver(SolverConfig(type="serinv"), diagonal_blocksize=spec.b, n_diag_blocks=spec.nt,
                                  arrowhead_blocksize=spec.nb)
        me.eps_inner_iteration = 1e-3
        me.inner_iteration_max_iter = 50
        me.comm_feval = DummyCommunicator()
        me._inner_iteration = types.MethodType(PyINLA._inner_iteration, me)
        me._evaluate_prior_latent_parameters = types.MethodType(PyINLA._evaluate_prior_latent_parameters, me)
        me._evaluate_conditional_latent_parameters = (
            lambda Q_conditional, x=None, x_mean=None: 0.5 * me.solver.logdet(sparsity="bta"))
        out = {"lik": lik, "aux": aux, "y": spec.y}
        for k, sh in enumerate(THETA_SHIFTS):
            theta = spec.theta0 + sh
            f = float(PyINLA._evaluate_f(me, theta.copy(), comm=DummyCommunicator()))
            out[f"theta{k}"] = theta
            out[f"f{k}"] = f
            out[f"x{k}"] = np.asarray(me.model.x, dtype=np.float64).copy()
        path = HERE / f"laplace_{lik}.npz"
        np.savez_compressed(path, **out)
        print(f"wrote {path.name}: f = {out['f0']:.6f}, {out['f1']:.6f}")


if __name__ == "__main__":
    main()
