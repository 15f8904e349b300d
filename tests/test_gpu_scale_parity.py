"""GPU parity at the block sizes the benchmark runs, against the oracle.

The golden fixtures stop at b = 128 (at most eight tile steps per product).  These
cases run the code paths of the benchmarked sizes -- products of 32 to 190 tile steps,
which fold the exact tensor-core partial sums several times, and selected-inversion
products whose left tiles change exponent along the sum -- on the precisions of the
benchmark's own models, not on diagonally dominant random blocks:

* ``spde32x32_nt32``: the conditional precision of the spatio-temporal benchmark model
  (SPDE on a 32 x 32 mesh, b = 1024, AR(1), 6 fixed effects, the benchmark's 1562
  observations per time step) with nt = 32 time blocks;
* ``coreg2x384_nt32``: a bivariate coregional model with 384 nodes per variate
  (b = 768), the coregional shape of the mixed batch;
* ``coreg3x1024_nt2``: the trivariate coregional model of the large benchmark
  (b = 3072, 9 fixed effects) with nt = 2.

Each is factored, solved (N then C), and inverted on the selected pattern with both
product methods and both elimination orders (both ends towards the middle block, the
solvers' default, and Serinv's top-down order), and logdet, solution and every Sigma
block are compared with the
oracle (oracle/bta_oracle.py, pinned to the reference's DenseSolver and SerinvSolver
wrapper by the golden fixtures) at 1e-10 relative: max-abs error over max-abs value of
each block array.  The reference path these replace is
src/pyinla/solvers/structured_solver.py:72-190.

The adjoint theta-gradient of the full benchmark model (nt = 128, dim theta = 4) and of
the large coregional model (nt = 64, dim theta = 9) is compared with central
differences of the GPU objective (step 1e-4; 9 and 19 evaluations) at 1e-6 relative;
the reference differentiates that way (src/pyinla/core/pyinla.py:512-600).
"""
import numpy as np
import pytest

from oracle import bta_oracle as orc
from oracle import model_oracle as mo

pytestmark = pytest.mark.gpu
RTOL = 1e-10
FD_RTOL = 1e-6


def relerr(x, y):
    x = np.asarray(x)
    y = np.asarray(y)
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


def _spec(name):
    from pyinla_gb300.model import CoregionalSpdeAr1, SeparableSpdeAr1

    if name == "spde32x32_nt32":
        return SeparableSpdeAr1.synthetic(32, 32, 6, 200000 * 32 // 128, seed=11)
    if name == "coreg2x384_nt32":
        return CoregionalSpdeAr1.synthetic(16, 32, 2, 2, 24000, seed=41, m_side=24)
    if name == "coreg3x1024_nt2":
        return CoregionalSpdeAr1.synthetic(32, 2, 3, 3, 300000 * 2 // 64, seed=5)
    raise KeyError(name)


CASES = ["spde32x32_nt32", "coreg2x384_nt32", "coreg3x1024_nt2"]
_ORACLE = {}


def oracle_case(name):
    """Q_cond blocks (oracle assembly + sparse-to-BTA mapping), the information vector,
    and the oracle's factor logdet, solution and selected inverse; computed once."""
    if name not in _ORACLE:
        spec = _spec(name)
        c = spec.coefficients(spec.theta0)
        _, Qc, rhs = mo.conditional_system(spec.terms, spec.term_vw, spec.ns, spec.nv, spec.nt, spec.nb, spec.A,
                                           spec.y, spec.tip_prec, c.alpha, c.beta, c.tau_y, spec.obs_variates())
        D, L, R, T = mo.sparse_to_bta(Qc, spec.nt, spec.b, spec.nb)
        inputs = [x.copy() for x in (D, L, R, T)]
        orc.pobtaf(D, L, R, T)
        ld = orc.logdet(D, T, "bta")
        x = rhs.copy()
        orc.pobtas(D, L, R, T, x, "N")
        orc.pobtas(D, L, R, T, x, "C")
        orc.pobtasi(D, L, R, T)
        _ORACLE[name] = dict(geom=(spec.b, spec.nt, spec.nb), inputs=inputs, rhs=rhs, logdet=ld, x=x,
                             sigma=(D, L, R, T))
    return _ORACLE[name]


@pytest.fixture(scope="module")
def torch():
    import torch as _t

    from pyinla_gb300 import build

    build.build()
    return _t


@pytest.mark.parametrize("twisted", [True, False])   # the solvers' default order; Serinv's
@pytest.mark.parametrize("method", [0, 1])            # GBTA_METHOD_FP64, GBTA_METHOD_OZAKI
@pytest.mark.parametrize("name", CASES)
def test_benchmark_sizes_match_oracle(torch, name, method, twisted):
    from pyinla_gb300 import algs
    from pyinla_gb300.device import BtaHandle

    o = oracle_case(name)
    b, nt, a = o["geom"]
    algs.set_twisted(twisted)
    h = BtaHandle.get(b, nt, a, twisted)
    old = h.method()
    h.set_method(method)
    try:
        Dd, Ld, Rd, Td = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in o["inputs"]]
        algs.pobtaf(Dd, Ld, Rd, Td)
        ld = algs.logdet(Dd, Td, "bta")
        x = torch.from_numpy(o["rhs"].copy()).cuda()
        algs.pobtas(Dd, Ld, Rd, Td, x, "N")
        algs.pobtas(Dd, Ld, Rd, Td, x, "C")
        algs.pobtasi(Dd, Ld, Rd, Td)
        torch.cuda.synchronize()
    finally:
        h.set_method(old)
        algs.set_twisted(False)
    errs = {"logdet": abs(ld - o["logdet"]) / abs(o["logdet"]), "x": relerr(x.cpu().numpy(), o["x"])}
    for key, got, want in zip(("SD", "SL", "SR", "ST"), (Dd, Ld, Rd, Td), o["sigma"]):
        errs[key] = relerr(got.cpu().numpy(), want)
    print(name, "method", method, "twisted", twisted, {k: f"{v:.2e}" for k, v in errs.items()})
    bad = {k: v for k, v in errs.items() if not v < RTOL}
    assert not bad, (name, method, errs)


def check_fd(model, theta, g, h=1e-4):
    d = theta.size
    fd = np.zeros(d)
    for k in range(d):
        e = np.zeros(d)
        e[k] = h
        fd[k] = (model.evaluate(theta + e) - model.evaluate(theta - e)) / (2 * h)
    err = relerr(g, fd)
    print("adjoint vs central differences:", f"{err:.2e}", g, fd)
    assert err < FD_RTOL, (g, fd)


def test_adjoint_matches_central_differences_on_benchmark_model(torch):
    """C2 model itself: 32 x 32 mesh, nt = 128, 6 fixed effects, 200 000 observations."""
    from pyinla_gb300.model import KronGaussianModel, SeparableSpdeAr1

    spec = SeparableSpdeAr1.synthetic(32, 128, 6, 200000, seed=11)
    m = KronGaussianModel(spec)
    theta = spec.theta0
    _, g = m.evaluate(theta, gradient=True)
    check_fd(m, theta, g)
    del m
    torch.cuda.empty_cache()


def test_adjoint_matches_central_differences_on_large_coregional_model(torch):
    """Trivariate coregional model: ns = 1024 per variate (b = 3072), nt = 64, nb = 9,
    300 000 observations, dim theta = 9 (19 evaluations)."""
    from pyinla_gb300.model import CoregionalSpdeAr1, KronGaussianModel

    spec = CoregionalSpdeAr1.synthetic(32, 64, 3, 3, 300000, seed=5)
    m = KronGaussianModel(spec)
    theta = spec.theta0
    _, g = m.evaluate(theta, gradient=True)
    check_fd(m, theta, g)
    del m
    torch.cuda.empty_cache()
