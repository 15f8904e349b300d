"""Generate the marginal-variance fixtures under tests/golden/ from the reference itself.

Run where the reference source tree is available (``$PYINLA_REFERENCE_SRC``, required: the reference's ``src/`` directory); the fixtures are committed, so tests never read the
reference at run time.

Per case, Q_cond = (seeded SPD BTA matrix of ``oracle.bta_oracle.make_bta_c1``) +
A^T A with A from ``oracle.marginals_oracle.make_observation_matrix``.  The
reference's own methods ``PyINLA.get_marginal_variances_latent_parameters``
(src/pyinla/core/pyinla.py:940-964) and ``PyINLA.get_marginal_variances_observations``
(pyinla.py:966-1018) run unmodified on a stand-in ``self`` whose model holds Q_cond
and A (its ``construct_Q_conditional`` keeps the given Q_cond) and whose solver is
the reference's ``SerinvSolver`` with the oracle injected as ``serinv.algs``; their
outputs are stored.
"""
from __future__ import annotations

import os
import sys
import types
from pathlib import Path

import numpy as np
import scipy.sparse as sps

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))

from oracle import bta_oracle as orc  # noqa: E402
from oracle import marginals_oracle as mo  # noqa: E402
from tests.golden.make_golden import _import_reference, checksum  # noqa: E402

CASES = {
    # name: (seed, nt, b, a, n_obs)
    "tiny": (21, 3, 8, 2, 24),
    "ragged": (22, 4, 40, 5, 160),
    "single": (23, 1, 16, 3, 30),
    "wide": (24, 6, 33, 1, 400),
}


def make_inputs(seed, nt, b, a, n_obs):
    """Q_cond (dense) and A of one case; the same in the tests."""
    D, L, R, T, _ = orc.make_bta_c1(seed, nt=nt, b=b, a=a)
    A = mo.make_observation_matrix(seed + 1000, nt, b, a, n_obs)
    Q = orc.bta_to_dense(D, L, R, T) + (A.T @ A).toarray()
    return Q, A


class _StandInModel:
    def __init__(self, Q, A):
        self.Q_conditional = sps.csc_matrix(Q)
        self.a = A
        self.n_latent_parameters = Q.shape[0]
        self.theta = np.zeros(1)
        self.x = np.zeros(Q.shape[0])

    def construct_Q_conditional(self, eta):
        return self.Q_conditional

    def is_likelihood_gaussian(self):
        return True


def main():
    SolverConfig, _, SerinvSolver = _import_reference()
    from pyinla.core.pyinla import PyINLA
    for name, (seed, nt, b, a, n_obs) in CASES.items():
        Q, A = make_inputs(seed, nt, b, a, n_obs)
        me = types.SimpleNamespace()
        me.model = _StandInModel(Q, A)
        me.solver = SerinvSolver(SolverConfig(type="serinv"), diagonal_blocksize=b, n_diag_blocks=nt,
                                 arrowhead_blocksize=a)
        me._compute_covariance_latent_parameters = types.MethodType(PyINLA._compute_covariance_latent_parameters, me)
        theta, x = np.zeros(1), np.zeros(Q.shape[0])
        lat = np.asarray(PyINLA.get_marginal_variances_latent_parameters(me, theta, x), dtype=np.float64)
        obs = np.asarray(PyINLA.get_marginal_variances_observations(me, theta, x), dtype=np.float64).ravel()
        path = HERE / f"marginals_{name}.npz"
        np.savez_compressed(path, seed=seed, nt=nt, b=b, a=a, n_obs=n_obs, input_checksum=checksum(Q, A.toarray()),
                            latent=lat, observations=obs)
        print(f"wrote {path.name}: {os.path.getsize(path) / 1024:.1f} KiB")


if __name__ == "__main__":
    main()
