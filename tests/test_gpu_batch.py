"""GPU checks of the multi-instance launch (gbta_batch_*, pyinla_gb300.batch).

Every instance of a mixed batch -- different block sizes, ragged tiles, with and
without the arrowhead, both product methods -- must equal, bit for bit, the
single-instance entry points with the same method (the same task bodies run), and
the golden instances must match the reference's dense results within 1e-10.  The
merge orders and the CUDA-graph replay must not change any bit, and a failed pivot
in one instance must come back as that instance's info without a fault.
"""
import numpy as np
import pytest

from oracle import bta_oracle as orc
from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu
RTOL = 1e-10

# (seed, nt, b, a): golden cases first (their dense results are in tests/golden)
SHAPES = [(7, 2, 40, 3), (11, 5, 45, 5), (5, 3, 64, 0), (3, 6, 96, 4), (9, 1, 70, 2), (13, 4, 128, 0)]


def relerr(x, y):
    x = np.asarray(x)
    y = np.asarray(y)
    return float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))


@pytest.fixture(scope="module")
def torch():
    import torch as _t

    from pyinla_gb300 import build

    build.build()
    return _t


def single_reference(torch, D, L, R, T, rhs, method):
    """The single-instance path (algs + the C ABI) with the given product method, in the
    batch's elimination order (both ends towards the middle block)."""
    from pyinla_gb300 import algs
    from pyinla_gb300.device import BtaHandle

    nt, b, a = D.shape[0], D.shape[1], (R.shape[1] if R is not None else 0)
    algs.set_twisted(True)
    h = BtaHandle.get(b, nt, a, True)
    old = h.method()
    h.set_method(method)
    try:
        Dd = torch.from_numpy(D.copy()).cuda()
        Ld = torch.from_numpy(L.copy() if nt > 1 else np.zeros((1, b, b))).cuda()
        Rd = torch.from_numpy(R.copy()).cuda() if a else None
        Td = torch.from_numpy(T.copy()).cuda() if a else None
        x = torch.from_numpy(rhs.copy()).cuda()
        if a:
            algs.pobtaf(Dd, Ld, Rd, Td)
            ld = algs.logdet(Dd, Td, "bta")
            algs.pobtas(Dd, Ld, Rd, Td, x, "N")
            algs.pobtas(Dd, Ld, Rd, Td, x, "C")
            algs.pobtasi(Dd, Ld, Rd, Td)
        else:
            algs.pobtf(Dd, Ld)
            ld = algs.logdet(Dd, None, "bt")
            algs.pobts(Dd, Ld, x, "N")
            algs.pobts(Dd, Ld, x, "C")
            algs.pobtsi(Dd, Ld)
        out = dict(ld=ld, x=x.cpu().numpy(), D=Dd.cpu().numpy(), L=Ld.cpu().numpy()[: max(nt - 1, 0)])
        if a:
            out["R"] = Rd.cpu().numpy()
            out["T"] = Td.cpu().numpy()
        return out
    finally:
        h.set_method(old)
        algs.set_twisted(False)


def make_instances(shapes):
    out = []
    for (seed, nt, b, a) in shapes:
        D, L, R, T, rhs = orc.make_bta_c1(seed, nt=nt, b=b, a=a)
        out.append((D, L, R, T, rhs))
    return out


def load_all(bt, insts):
    for k, (D, L, R, T, rhs) in enumerate(insts):
        bt.load(k, D, L, R if R.shape[1] else None, T if T.shape[0] else None, rhs)


def batch_results(bt, k):
    b, nt, a = bt.shapes[k]
    out = dict(ld=float(bt.logdet[k].item()), x=bt.rhs[k].cpu().numpy(), D=bt.D[k].cpu().numpy(),
               L=bt.L[k].cpu().numpy()[: max(nt - 1, 0)])
    if a:
        out["R"] = bt.R[k].cpu().numpy()
        out["T"] = bt.T[k].cpu().numpy()
    return out


def assert_same(r1, r2):
    assert r1["ld"] == r2["ld"]
    for key in r1:
        if key != "ld":
            assert np.array_equal(r1[key], r2[key]), key


@pytest.mark.parametrize("methods", ["ozaki", "fp64", "mixed"])
def test_batch_matches_single_instance_bitwise(torch, methods):
    from pyinla_gb300.batch import BtaBatch

    shapes = [(b, nt, a) for (_, nt, b, a) in SHAPES]
    m = {"ozaki": [1] * len(shapes), "fp64": [0] * len(shapes), "mixed": [k % 2 for k in range(len(shapes))]}[methods]
    insts = make_instances(SHAPES)
    bt = BtaBatch(shapes, methods=m)
    load_all(bt, insts)
    bt.run(graph=False)
    for k, inst in enumerate(insts):
        ref = single_reference(torch, *inst, method=m[k])
        assert_same(batch_results(bt, k), ref)


def test_batch_golden_instances(torch):
    """The golden instances inside a batch match the reference's dense results."""
    from pyinla_gb300.batch import BtaBatch

    names = ["tiny", "ragged", "single", "two"]
    gs = [np.load(GOLDEN / f"bta_{n}.npz") for n in names]
    shapes = [(int(g["b"]), int(g["nt"]), int(g["a"])) for g in gs]
    insts = [orc.make_bta_c1(int(g["seed"]), nt=int(g["nt"]), b=int(g["b"]), a=int(g["a"])) for g in gs]
    bt = BtaBatch(shapes)
    load_all(bt, insts)
    lds = bt.run()
    for k, g in enumerate(gs):
        assert abs(lds[k] - float(g["dense_logdet"])) <= RTOL * abs(float(g["dense_logdet"]))
        r = batch_results(bt, k)
        assert relerr(r["x"], g["dense_x"]) < RTOL
        assert relerr(r["D"], g["dense_SD"]) < RTOL
        assert relerr(r["R"], g["dense_SR"]) < RTOL
        assert relerr(r["T"], g["dense_ST"]) < RTOL


def test_batch_orders_and_graph_replay_are_bit_identical(torch):
    from pyinla_gb300.batch import BtaBatch

    shapes = [(b, nt, a) for (_, nt, b, a) in SHAPES]
    insts = make_instances(SHAPES)
    bt = BtaBatch(shapes)
    results = {}
    for order in ("proportional", "round_robin", "sequential"):
        bt.set_order(order)
        for graph in (False, True, True):   # eager, capture + launch, replay
            load_all(bt, insts)
            bt.run(graph=graph)
            results[(order, graph)] = [batch_results(bt, k) for k in range(len(shapes))]
    base = results[("proportional", False)]
    for key, res in results.items():
        for k in range(len(shapes)):
            assert_same(res[k], base[k])
    assert bt.graph_kernels() > 0


def test_batch_reports_failed_pivot_per_instance(torch):
    """An indefinite instance aborts the launch and is reported in its info slot."""
    from pyinla_gb300.batch import BtaBatch

    shapes = [(b, nt, a) for (_, nt, b, a) in SHAPES[:3]]
    insts = make_instances(SHAPES[:3])
    D, L, R, T, rhs = insts[1]
    D = D.copy()
    D[2, 7, 7] = -50.0   # block 2, row 7: the pivot at global row 2*b + 8 fails
    insts[1] = (D, L, R, T, rhs)
    bt = BtaBatch(shapes)
    load_all(bt, insts)
    bt.run_async(graph=False)
    with pytest.raises(np.linalg.LinAlgError):
        bt.status()
    # the batch is reusable after the failure
    good = make_instances(SHAPES[:3])
    load_all(bt, good)
    bt.run(graph=False)
    for k, inst in enumerate(good):
        assert_same(batch_results(bt, k), single_reference(torch, *inst, method=1))


def test_autotuner_picks_and_caches(torch, tmp_path, monkeypatch):
    from pyinla_gb300 import autotune
    from pyinla_gb300.batch import BtaBatch

    monkeypatch.setenv("PYINLA_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    shapes = [(64, 3, 2), (96, 2, 0), (64, 4, 2)]
    m = autotune.choose_methods(shapes, nt_probe=3)
    assert len(m) == 3 and set(m) <= {0, 1} and m[0] == m[2]
    assert (tmp_path / "tune.json").exists()
    assert autotune.choose_methods(shapes, nt_probe=3) == m   # served from the cache
    bt = BtaBatch(shapes, methods=m)
    insts = make_instances([(1, 3, 64, 2), (2, 2, 96, 0), (3, 4, 64, 2)])

    def reload():
        load_all(bt, insts)

    times = autotune.choose_order(bt, reload=reload)
    assert set(times) == {"proportional", "round_robin", "sequential"}
    assert bt.order == min(times, key=times.get)
