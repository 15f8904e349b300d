"""Generate the theta-Hessian fixture under tests/golden/ from the reference itself.

Run where the reference source tree is available (``$PYINLA_REFERENCE_SRC``, required: the reference's ``src/`` directory); the fixture is committed, so tests never read the reference.

The reference's own ``PyINLA._evaluate_hessian_f`` (src/pyinla/core/pyinla.py:767-910)
and ``PyINLA.compute_covariance_hp`` (pyinla.py:747-765) run unmodified on a stand-in
``self`` whose ``_evaluate_f`` is the oracle objective (oracle/model_oracle.py, the
restatement of ``PyINLA._evaluate_f`` for the Gaussian case) of a small seeded
spatio-temporal model (5 x 5 mesh, nt = 4, 2 fixed effects, 300 observations), with
the reference's default step eps_hessian_f = 5e-3 (src/pyinla/configs/pyinla_config.py:52).
"""
from __future__ import annotations

import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))

from oracle import model_oracle as mo  # noqa: E402
from tests.golden.make_golden import _import_reference  # noqa: E402

SEED, N_SIDE, NT, NB, N_OBS = 4, 5, 4, 2, 300
EPS = 5e-3


def make_spec():
    from pyinla_gb300.model import SeparableSpdeAr1
    spec = SeparableSpdeAr1.synthetic(N_SIDE, NT, NB, N_OBS, seed=SEED)
    theta = spec.theta0 + np.array([0.1, -0.05, 0.15, 0.05])
    return spec, theta


def oracle_objective(spec):
    def f(theta):
        c = spec.coefficients(theta)
        val, _ = mo.objective(spec.terms, spec.term_vw, spec.ns, spec.nv, spec.nt, spec.nb, spec.A, spec.y,
                              spec.tip_prec, c.alpha, c.beta, c.tau_y, theta[spec.lik_theta_indices()],
                              spec.log_prior(theta), spec.obs_variates())
        return float(val)
    return f


def main():
    _import_reference()
    from pyinla.core.pyinla import PyINLA
    from pyinla.utils import DummyCommunicator
    spec, theta = make_spec()
    fun = oracle_objective(spec)
    me = types.SimpleNamespace()
    me.model = types.SimpleNamespace(theta=np.zeros(theta.size), n_hyperparameters=theta.size)
    me.eps_hessian_f = EPS
    me.world_size = 1
    me.comm_feval = DummyCommunicator()
    me.comm_world = DummyCommunicator()
    me.color_feval = 0
    me._evaluate_f = lambda th, comm=None: fun(np.asarray(th))
    me._evaluate_hessian_f = types.MethodType(PyINLA._evaluate_hessian_f, me)
    hess = np.asarray(PyINLA._evaluate_hessian_f(me, theta.copy()), dtype=np.float64)
    cov = np.asarray(PyINLA.compute_covariance_hp(me, theta.copy()), dtype=np.float64)
    path = HERE / "hessian_spde5x5_nt4.npz"
    np.savez_compressed(path, theta=theta, eps=EPS, hessian=hess, cov=cov)
    print(f"wrote {path.name}")


if __name__ == "__main__":
    main()
