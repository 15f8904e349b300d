"""The non-Gaussian (Laplace) objective oracle against the reference's own code path.

Fixtures from tests/golden/make_laplace_golden.py: PyINLA._evaluate_f's non-Gaussian
branch with its inner Newton iteration (src/pyinla/core/pyinla.py:692-729, 1025-1110),
the reference's Model and likelihood methods, two theta points in sequence.
"""
import numpy as np
import pytest

from oracle import laplace_oracle as lo
from tests.conftest import GOLDEN
from tests.golden.make_laplace_golden import make_problem


def relerr(x, y):
    return float(np.max(np.abs(np.asarray(x) - np.asarray(y))) / max(np.max(np.abs(y)), 1e-300))


@pytest.mark.parametrize("lik", ["poisson", "binomial"])
def test_laplace_oracle_matches_reference(lik):
    g = np.load(GOLDEN / f"laplace_{lik}.npz")
    spec, aux = make_problem(lik)
    assert np.array_equal(spec.y, g["y"]) and np.array_equal(aux, g["aux"])
    kw = {"e": aux} if lik == "poisson" else {"n_trials": aux}
    x = np.zeros(spec.A.shape[1])
    for k in range(2):
        f, x = lo.laplace_objective(spec, g[f"theta{k}"], lik, x, **kw)
        assert abs(f - float(g[f"f{k}"])) <= 1e-10 * abs(float(g[f"f{k}"]))
        assert relerr(x, g[f"x{k}"]) < 1e-8
