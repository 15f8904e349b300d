"""The marginal-variance oracle (oracle/marginals_oracle.py) against fixtures of the reference.

Fixtures come from tests/golden/make_marginals_golden.py: the reference's
``PyINLA.get_marginal_variances_latent_parameters`` and
``PyINLA.get_marginal_variances_observations`` (src/pyinla/core/pyinla.py:940-1018)
run on its SerinvSolver wrapper with the oracle as Serinv.
"""
import numpy as np
import pytest

from oracle import bta_oracle as orc
from oracle import marginals_oracle as mo
from tests.conftest import GOLDEN
from tests.golden.make_golden import checksum
from tests.golden.make_marginals_golden import CASES, make_inputs

RTOL = 1e-10


def relerr(x, y):
    x = np.asarray(x); y = np.asarray(y)
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


def oracle_sigma(Q, nt, b, a):
    D, L, R, T = orc.dense_to_bta(Q, nt, b, a)
    orc.pobtaf(D, L, R, T)
    orc.pobtasi(D, L, R, T)
    return D, L, R, T


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_marginal_variances(name):
    g = np.load(GOLDEN / f"marginals_{name}.npz")
    seed, nt, b, a, n_obs = (int(g[k]) for k in ("seed", "nt", "b", "a", "n_obs"))
    Q, A = make_inputs(seed, nt, b, a, n_obs)
    np.testing.assert_allclose(checksum(Q, A.toarray()), g["input_checksum"], rtol=1e-13, atol=0)
    SD, SL, SR, ST = oracle_sigma(Q, nt, b, a)
    assert relerr(mo.latent_variances(SD, ST), g["latent"]) < RTOL
    assert relerr(mo.observation_variances(A, SD, SL, SR, ST), g["observations"]) < RTOL


def test_oracle_sigma_entries_match_dense_inverse():
    Q, A = make_inputs(5, 3, 7, 2, 40)
    S = np.linalg.inv(Q)
    SD, SL, SR, ST = oracle_sigma(Q, 3, 7, 2)
    n = Q.shape[0]
    p, q = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    got = mo.sigma_entries(SD, SL, SR, ST, p.ravel(), q.ravel()).reshape(n, n)
    blk = np.minimum(p, 21) // 7, np.minimum(q, 21) // 7
    inside = (np.abs(blk[0] - blk[1]) <= 1) | (p >= 21) | (q >= 21)
    assert relerr(got[inside], S[inside]) < RTOL
    assert np.all(got[~inside] == 0.0)
    assert relerr(mo.observation_variances(A, SD, SL, SR, ST), np.diagonal(A @ S @ A.T)) < RTOL
