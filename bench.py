#!/usr/bin/env python
"""Benchmark of the BTA hot path on one GB300 (and N replicas under torchrun).

Workload (one "step"): the plain INLA conditional precision of a Gaussian
spatio-temporal model -- SPDE on a 32 x 32 triangulated unit square (ns = 1024,
lumped C, stiffness G, Q_s = kappa^4 C + 2 kappa^2 G + G C^-1 G), AR1 over nt = 128
(rho = 0.9), nb = 6 fixed effects (prior precision 1e-3), 200 000 Gaussian
observations (3 barycentric weights + 6 N(0,1) covariates each, tau_y = 4).  Each step
assembles Q_cond on the device, factors it (pobtaf), takes its logdet, solves for the
conditional mean (pobtas N then C) and runs the selected inversion (pobtasi).  Inputs
are seeded synthetic data of those shapes (the reference's datasets are not
available).

metric: FP64 TFLOP/s of factor + selected inversion, counted with the fixed
algorithmic flop counts F_f + F_s of the BTA recurrences (LAPACK conventions),
divided by the device time of the whole step.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

METRIC = "BTA factor+selinv FP64 TFLOPS (% peak); theta-gradient/s adjoint vs FD, same GPU"
UNIT = "TFLOP/s"


# ----------------------------------------------------------------------------- shapes
def workload(small: bool):
    if small:   # a reduced case for profiler captures only
        return dict(name="spde32x32_ar1_nt16_nb6_obs25k", n_side=32, nt=16, nb=6, n_obs=25000, seed=11)
    return dict(name="spde32x32_ar1_nt128_nb6_obs200k", n_side=32, nt=128, nb=6, n_obs=200000, seed=11)


def bta_flops(nt: int, b: int, a: int) -> tuple[float, float]:
    """Algorithmic flops of pobtaf and pobtasi (POTRF n^3/3, TRSM/TRMM m n^2, SYRK n^2 k,
    GEMM 2mnk, TRTRI n^3/3, LAUUM n^3/3), the counts the throughput is quoted with."""
    ff = nt * b ** 3 / 3 + (nt - 1) * (2 * b ** 3) + (nt - 1) * 2 * a * b * b + nt * (a * b * b + a * a * b) + a ** 3 / 3
    fs = ((nt - 1) * (b ** 3 / 3 + b ** 3 + 2 * b ** 3 + b ** 3 / 3 + 2 * b ** 3)
          + (nt - 1) * (7 * a * b * b + 2 * a * a * b) + (2 * b ** 3 / 3 + 2 * a * b * b + 2 * a ** 3 / 3))
    return float(ff), float(fs)


# Tile steps of the digit-plane products and the fp16 tensor work of one step: four
# warps x two k16 slices x 43 digit-plane pairs x two n8 halves of mma.m16n8k16
# (4096 flops each) = 43 times the 2 * 32^3 FP64 flops of the tile product.
OZ_STEP_TENSOR_FLOPS = 4 * 2 * 43 * 2 * 4096


def oz_tile_steps(nt: int, b: int, a: int) -> tuple[int, int]:
    """Product steps of the tensor-core factorization and selected inversion (their
    task DAGs): factor tile (r, c) of block i sums over c earlier tiles, plus the B
    tiles of the previous block column except for L tiles; selected-inversion column
    (i, c) has |P| = arrow + B (block i+1, i < nt-1) + (B-1-c) pattern rows, and each
    of its |P| off-diagonal tasks and its diagonal task sums over all of them."""
    B = (b + 31) // 32
    fsteps = 0
    ssteps = 0
    for i in range(nt):
        nprev = B if i > 0 else 0
        for c in range(B):
            fsteps += (nprev + c) * (1 + (B - 1 - c) + (1 if a else 0))    # DIAG, OFFD, ARW
            if i < nt - 1:
                fsteps += c * B                                          # LOW
            npat = (1 if a else 0) + (B if i < nt - 1 else 0) + (B - 1 - c)
            ssteps += npat * (npat + 1)
    return fsteps, ssteps


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region (read-only queries)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ----------------------------------------------------------------------------- CPU baseline
def cpu_sample_tflops(b: int, a: int, nt_sample: int, seed: int = 3):
    """Time the oracle's block-level NumPy/OpenBLAS pobtaf + pobtasi (the restatement of
    the reference's Serinv CPU path) on a bounded sample with nt_sample blocks."""
    from oracle import bta_oracle as orc

    D, L, R, T, _ = orc.make_bta_c1(seed, nt=nt_sample, b=b, a=a)
    t0 = time.perf_counter()
    orc.pobtaf(D, L, R, T)
    orc.pobtasi(D, L, R, T)
    dt = time.perf_counter() - t0
    ff, fs = bta_flops(nt_sample, b, a)
    return (ff + fs) / dt / 1e12, dt


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ----------------------------------------------------------------------------- reference arm
def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    wl = workload(args.small)
    cores = host_cores()
    b, nt, a = wl["n_side"] ** 2, wl["nt"], wl["nb"]
    nt_sample = 8
    vals = []
    for _ in range(max(args.warmup, 0)):
        cpu_sample_tflops(b, a, nt_sample)
    for _ in range(args.steps):
        v, _ = cpu_sample_tflops(b, a, nt_sample)
        vals.append(v)
    value = statistics.median(vals)
    ff, fs = bta_flops(nt, b, a)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": (ff + fs) / (value * 1e12) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded; reference datasets unavailable)",
        "config": {"workload": wl["name"], "b": b, "nt": nt, "a": a,
                   "note": "Serinv is not installable offline; the reference arm times the oracle's "
                           "Serinv-equivalent NumPy/OpenBLAS restatement on the host cores"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"pobtaf+pobtasi on {nt_sample} of {nt} diagonal blocks (b={b}, a={a}); "
                                   f"ms_per_step extrapolates to the full {nt} blocks"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- our arm
def run_ours(args, rank: int, world: int, local_rank: int):
    import torch

    from pyinla_gb300 import _lib
    from pyinla_gb300 import build as _build
    from pyinla_gb300.model import KronGaussianModel, SeparableSpdeAr1
    from pyinla_gb300.solver import GB300SerinvSolver

    torch.cuda.set_device(local_rank)
    _build.build()
    lib = _lib.load()
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    wl = workload(args.small)
    spec = SeparableSpdeAr1.synthetic(wl["n_side"], wl["nt"], wl["nb"], wl["n_obs"], wl["seed"] + rank)
    model = KronGaussianModel(spec)
    theta = spec.theta0
    b, nt, a = model.b, model.nt, model.nb
    ff, fs = bta_flops(nt, b, a)
    h = model.h
    stream = torch.cuda.current_stream()
    h.set_stream(stream.cuda_stream)
    coef = spec.coefficients(theta)
    tau_dev = torch.from_numpy(coef.tau_y).cuda()

    Dc, Lc, Rc, Tc = model.Dc, model.Lc, model.Rc, model.Tc
    mu = model.mu
    ev = {k: [torch.cuda.Event(enable_timing=True) for _ in range(2)] for k in ("asm", "fac", "sol", "sel")}
    timings = {k: [] for k in ev}

    def step(record: bool):
        e = ev if record else None
        ptrs = model._upload_coef(coef)
        if e: e["asm"][0].record()
        model._assemble(ptrs, Dc, Lc, Rc, Tc, with_lik=True)
        if e: e["asm"][1].record(); e["fac"][0].record()
        _lib.check(lib.gbta_pobtaf_async(h.ptr, Dc.data_ptr(), Lc.data_ptr(), Rc.data_ptr(), Tc.data_ptr()))
        if e: e["fac"][1].record(); e["sol"][0].record()
        torch.mv(model._Aty_v.t(), tau_dev, out=mu)
        _lib.check(lib.gbta_pobtas_async(h.ptr, Dc.data_ptr(), Lc.data_ptr(), Rc.data_ptr(), Tc.data_ptr(),
                                         mu.data_ptr(), 1, 0))
        _lib.check(lib.gbta_pobtas_async(h.ptr, Dc.data_ptr(), Lc.data_ptr(), Rc.data_ptr(), Tc.data_ptr(),
                                         mu.data_ptr(), 1, 1))
        if e: e["sol"][1].record(); e["sel"][0].record()
        _lib.check(lib.gbta_pobtasi_async(h.ptr, Dc.data_ptr(), Lc.data_ptr(), Rc.data_ptr(), Tc.data_ptr()))
        if e: e["sel"][1].record()

    def collect():
        for k, (e0, e1) in ev.items():
            timings[k].append(e0.elapsed_time(e1))

    for _ in range(args.warmup):
        step(False)
    _lib.check(lib.gbta_status(h.ptr))
    torch.cuda.synchronize()
    peak = ctypes.c_double(0.0)
    _lib.check(lib.gbta_probe_fp64_peak(4000, ctypes.byref(peak)))
    peak_tf = float(peak.value)

    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local_rank)
    clocks.start()
    launches0 = lib.gbta_kernel_launches()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record()
    for s in range(args.steps):
        step(True)
        if s < args.steps - 1:
            torch.cuda.current_stream().synchronize()
            collect()
    t_end.record()
    torch.cuda.synchronize()
    collect()
    launches = lib.gbta_kernel_launches() - launches0
    clk = clocks.stop()
    _lib.check(lib.gbta_status(h.ptr))
    elapsed_ms = t_start.elapsed_time(t_end)
    if dist:
        tt = torch.tensor([elapsed_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        elapsed_ms = float(tt.item())
    ms_per_step = elapsed_ms / args.steps
    value = world * args.steps * (ff + fs) / (elapsed_ms * 1e-3) / 1e12

    avg = {k: statistics.mean(v) for k, v in timings.items()}
    dominant = "sel" if avg["sel"] >= avg["fac"] else "fac"
    dom_flops = fs if dominant == "sel" else ff
    achieved = dom_flops / (avg[dominant] * 1e-3) / 1e12
    traffic = None
    tfile = REPO / "profiles" / "traffic.json"
    if tfile.exists():
        try:
            traffic = json.loads(tfile.read_text()).get(wl["name"], {}).get("k_selinv" if dominant == "sel" else "k_factor")
        except (ValueError, OSError):
            traffic = None

    # the same launch seen from the tensor pipe: fp16 mma work of its digit-plane
    # products against the measured bf16 tensor peak of this machine (a kernel timed
    # inside back-to-back seconds-long steps: the sustained figure)
    fsteps, ssteps = oz_tile_steps(nt, b, a)
    tflops = (ssteps if dominant == "sel" else fsteps) * OZ_STEP_TENSOR_FLOPS
    tachieved = tflops / (avg[dominant] * 1e-3) / 1e12
    try:
        mp = json.loads((REPO / "MEASURED_PEAKS.json").read_text())
        tpeak, tsrc = float(mp["bf16_tflops_sustained"]), "MEASURED_PEAKS.json bf16_tflops_sustained (of measured)"
    except (OSError, ValueError, KeyError):
        tpeak, tsrc = 1700.0, "fallback sustained bf16 figure (MEASURED_PEAKS.json absent)"
    tensor_pipe = {"achieved": tachieved, "peak": tpeak, "unit": "TFLOP/s", "frac": tachieved / tpeak,
                   "peak_source": tsrc,
                   "work": "fp16 mma.sync work of the digit-plane tile products (43x their FP64 flops)"}

    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded; reference datasets unavailable)",
        "config": {"workload": wl["name"], "b": b, "nt": nt, "a": a, "n_obs": wl["n_obs"],
                   "parallelism": f"replicas{world}", "l2": "inputs larger than L2 (BTA blocks "
                   f"{(2 * nt - 1) * b * b * 8 / 1e9:.2f} GB)",
                   "step": "assemble Q_cond + pobtaf + pobtas(N,C) + pobtasi",
                   "flops_per_step": ff + fs, "flops_factor": ff, "flops_selinv": fs},
        "phases_ms": {"assemble": avg["asm"], "factor": avg["fac"], "solve": avg["sol"], "selinv": avg["sel"]},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak_tf, "unit": "TFLOP/s",
                     "frac": achieved / peak_tf if peak_tf else None, "traffic": traffic,
                     "kernel": "k_selinv" if dominant == "sel" else "k_factor",
                     "peak_source": "measured FP64 DFMA rate of this GPU (gbta_probe_fp64_peak; the "
                                    "pool's MEASURED_PEAKS.json carries no FP64 figure); GB300's FP64 "
                                    "tensor (DMMA) path measures below it"},
        "tensor_pipe": tensor_pipe,
        "frac_of_peak_step": value / world / peak_tf if peak_tf else None,
        "gpu_launches": int(launches),
        "clocks": clk,
    }

    # ---- e2e through the reference-facing drop-in (host sparse Q_cond in, host results out)
    if not args.no_e2e:
        Qp_host, Qc_host = spec.sparse_precisions(theta)
        rhs_host = np.asarray(spec.A.T @ (coef.tau_y[spec.obs_variates()] * spec.y), dtype=np.float64)
        solver = GB300SerinvSolver(None, diagonal_blocksize=b, n_diag_blocks=nt, arrowhead_blocksize=a)
        out_nnz = [0]

        def e2e_step():
            solver.cholesky(Qc_host, sparsity="bta")
            solver.logdet("bta")
            solver.solve(rhs_host.copy(), sparsity="bta")
            solver.selected_inversion("bta")
            out = solver._structured_to_spmatrix(Qc_host, sparsity="bta")
            out_nnz[0] = int(out.nnz)
            return out

        e2e_step()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        n_e2e = max(1, min(args.steps, 3))
        for _ in range(n_e2e):
            e2e_step()
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / n_e2e
        if dist:
            tt = torch.tensor([dt], device="cuda", dtype=torch.float64)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            dt = float(tt.item())
        result["e2e"] = {"value": world * (ff + fs) / dt / 1e12, "unit": UNIT,
                         # values of Q_cond and the right-hand side in; the solution, the
                         # selected inverse on Q_cond's pattern and the logdet out (the
                         # index arrays of a pattern seen before stay on the device)
                         "h2d_bytes_per_step": int(Qc_host.nnz * 8 + rhs_host.nbytes),
                         "d2h_bytes_per_step": int(rhs_host.nbytes + out_nnz[0] * 8 + 8),
                         "ms_per_step": dt * 1e3,
                         "path": "GB300SerinvSolver (drop-in SerinvSolver): cholesky(sparse) + logdet + "
                                 "solve + selected_inversion + _structured_to_spmatrix"}
        del solver

    # ---- adjoint gradient vs one plain evaluation and vs central differences
    if not args.no_adjoint:
        model.evaluate(theta)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f0 = model.evaluate(theta)
        torch.cuda.synchronize()
        t_plain = time.perf_counter() - t0
        t0 = time.perf_counter()
        f1, g = model.evaluate(theta, gradient=True)
        torch.cuda.synchronize()
        t_grad = time.perf_counter() - t0
        d = theta.size
        result["adjoint"] = {"plain_eval_ms": t_plain * 1e3, "value_and_grad_ms": t_grad * 1e3,
                             "ratio_vs_plain": t_grad / t_plain, "central_fd_ratio": 2 * d + 1,
                             "speedup_vs_fd": (2 * d + 1) * t_plain / t_grad,
                             "gradients_per_s": 1.0 / t_grad, "dim_theta": int(d)}
        # theta-Hessian: differences of 2d adjoint gradients, against the reference's
        # differences of f (1 + 2d + 2d(d-1) evaluations, pyinla.py:767-910)
        t0 = time.perf_counter()
        model.hessian(theta)
        torch.cuda.synchronize()
        t_hess = time.perf_counter() - t0
        n_fd = 1 + 2 * d + 2 * d * (d - 1)
        result["hessian"] = {"ms": t_hess * 1e3, "gradient_evaluations": 2 * int(d),
                             "reference_f_evaluations": int(n_fd),
                             "speedup_vs_fd_of_f": n_fd * t_plain / t_hess}

    # ---- CPU baseline (rank 0, N = 1 only): the oracle on the host cores
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        nt_sample = 8
        v, dt = cpu_sample_tflops(b, a, nt_sample)
        result["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": host_cores(), "kind": "port",
                                  "sample": f"oracle pobtaf+pobtasi (NumPy/OpenBLAS block restatement of "
                                            f"Serinv) on {nt_sample} of {nt} diagonal blocks, b={b}, a={a}; "
                                            f"{dt:.1f} s"}
    if rank == 0:
        print(json.dumps(result), flush=True)
    if dist:
        dist.destroy_process_group()


# ----------------------------------------------------------------------------- other workloads
def batch41_shapes(seed: int = 41):
    """41 instances (9 central-difference theta points + 32 grid points) of mixed
    sizes, drawn from the seed: block size from univariate ns in {256, 512, 768} or a
    2-variate coregional model with ns = 384 per variate (b = 768); nt in
    {32, 64, 128, 256}; nb in {2, 4, 8}."""
    rng = np.random.default_rng(seed)
    kinds = [("uni256", 256), ("uni512", 512), ("uni768", 768), ("coreg2x384", 768)]
    out = []
    for _ in range(41):
        kind, b = kinds[int(rng.integers(len(kinds)))]
        nt = int(rng.choice([32, 64, 128, 256]))
        nb = int(rng.choice([2, 4, 8]))
        out.append((b, nt, nb, kind))
    return out


def run_batch41(args):
    """All 41 instances in one graph-captured launch per run (factor, logdet, solve N+C,
    selinv), methods from the autotuner; against the same instances one at a time
    through the single-instance entry points."""
    import torch

    from pyinla_gb300 import _lib, autotune
    from pyinla_gb300 import build as _build
    from pyinla_gb300.batch import BtaBatch
    from pyinla_gb300.device import BtaHandle
    from pyinla_gb300.synthetic import random_bta

    _build.build()
    lib = _lib.load()
    shapes4 = batch41_shapes()
    shapes = [(b, nt, a) for (b, nt, a, _) in shapes4]
    flops = sum(sum(bta_flops(nt, b, a)) for (b, nt, a) in shapes)
    t0 = time.perf_counter()
    methods = autotune.choose_methods(shapes)
    t_tune_methods = time.perf_counter() - t0
    bt = BtaBatch(shapes, methods=methods)

    def refill():
        for k, (b, nt, a) in enumerate(shapes):
            D, L, R, T = random_bta(nt, b, a, seed=1000 + k)
            bt.D[k].copy_(D)
            bt.L[k].copy_(L)
            bt.R[k].copy_(R)
            bt.T[k].copy_(T)
            bt.rhs[k].fill_(1.0)
            del D, L, R, T

    t0 = time.perf_counter()
    order_ms = autotune.choose_order(bt, reload=refill)
    t_tune_order = time.perf_counter() - t0
    for _ in range(args.warmup):
        refill()
        bt.run(graph=True)
    clocks = ClockSampler(0)
    clocks.start()
    times = []
    launches0 = lib.gbta_kernel_launches()
    for _ in range(args.steps):
        refill()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        bt.run_async(graph=True)
        e1.record()
        bt.status()
        times.append(e0.elapsed_time(e1))
    launches = lib.gbta_kernel_launches() - launches0
    clk = clocks.stop()
    ms = statistics.median(times)
    ws = bt.workspace_bytes()
    graph_kernels = bt.graph_kernels()
    # the same instances one at a time (single-instance entry points, same methods)
    bt.close()
    seq_ms = 0.0
    stream = torch.cuda.current_stream()
    for k, (b, nt, a) in enumerate(shapes):
        h = BtaHandle(b, nt, a)
        h.set_stream(stream.cuda_stream)
        h.set_method(methods[k])
        for rep in range(2):
            D, L, R, T = random_bta(nt, b, a, seed=1000 + k)
            x = torch.ones(nt * b + a, dtype=torch.float64, device="cuda")
            ld = torch.zeros(1, dtype=torch.float64, device="cuda")
            Rp, Tp = (R.data_ptr(), T.data_ptr()) if a else (None, None)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            _lib.check(lib.gbta_pobtaf_async(h.ptr, D.data_ptr(), L.data_ptr(), Rp, Tp))
            _lib.check(lib.gbta_pobtas_async(h.ptr, D.data_ptr(), L.data_ptr(), Rp, Tp, x.data_ptr(), 1, 0))
            _lib.check(lib.gbta_pobtas_async(h.ptr, D.data_ptr(), L.data_ptr(), Rp, Tp, x.data_ptr(), 1, 1))
            _lib.check(lib.gbta_pobtasi_async(h.ptr, D.data_ptr(), L.data_ptr(), Rp, Tp))
            e1.record()
            h.status()
            if rep:
                seq_ms += e0.elapsed_time(e1)
            del D, L, R, T
        h.close()
    line = {
        "metric": METRIC, "value": flops / (ms * 1e-3) / 1e12, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded diagonally dominant SPD instances)",
        "config": {"workload": "batch41_mixed", "instances": len(shapes),
                   "shapes": [f"{kind}:b{b},nt{nt},nb{a}" for (b, nt, a, kind) in shapes4],
                   "methods": methods, "order": bt.order, "order_ms": order_ms,
                   "flops_per_step": flops, "workspace_bytes": ws,
                   "step": "one graph launch: factor + logdet + solve N,C + selinv of all 41 instances",
                   "tuning_s": {"methods": t_tune_methods, "order": t_tune_order}},
        "graph_kernels": graph_kernels, "gpu_launches": int(launches),
        "sequential_ms": seq_ms, "batch_speedup_vs_sequential": seq_ms / ms, "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def run_coreg3(args):
    """3-variate coregional model (ns = 1024 per variate, b = 3072, nt = 64, nb = 9,
    300 000 observations): factor and selected inversion throughput of Q_cond and the
    adjoint theta-gradient (d = 9) against one plain evaluation and central FD."""
    import torch

    from pyinla_gb300 import _lib
    from pyinla_gb300 import build as _build
    from pyinla_gb300.model import CoregionalSpdeAr1, KronGaussianModel

    _build.build()
    lib = _lib.load()
    t0 = time.perf_counter()
    spec = CoregionalSpdeAr1.synthetic(32, 64, 3, 3, 300000, seed=5)
    model = KronGaussianModel(spec)
    t_setup = time.perf_counter() - t0
    theta = spec.theta0
    b, nt, a = model.b, model.nt, model.nb
    ff, fs = bta_flops(nt, b, a)
    h = model.h
    h.set_stream(torch.cuda.current_stream().cuda_stream)
    coef = spec.coefficients(theta)
    Dc, Lc, Rc, Tc = model.Dc, model.Lc, model.Rc, model.Tc
    fac, sel = [], []
    for s in range(args.warmup + args.steps):
        ptrs = model._upload_coef(coef)
        model._assemble(ptrs, Dc, Lc, Rc, Tc, with_lik=True)
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        _lib.check(lib.gbta_pobtaf_async(h.ptr, Dc.data_ptr(), Lc.data_ptr(), Rc.data_ptr(), Tc.data_ptr()))
        e[1].record()
        _lib.check(lib.gbta_pobtasi_async(h.ptr, Dc.data_ptr(), Lc.data_ptr(), Rc.data_ptr(), Tc.data_ptr()))
        e[2].record()
        h.status()
        if s >= args.warmup:
            fac.append(e[0].elapsed_time(e[1]))
            sel.append(e[1].elapsed_time(e[2]))
    model.evaluate(theta)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    model.evaluate(theta)
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    t0 = time.perf_counter()
    model.evaluate(theta, gradient=True)
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0
    d = theta.size
    fm, sm = statistics.median(fac), statistics.median(sel)
    line = {
        "metric": METRIC, "value": (ff + fs) / ((fm + sm) * 1e-3) / 1e12, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": fm + sm, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": "coreg3_spde32x32_ar1_nt64_nb9_obs300k", "b": b, "nt": nt, "a": a,
                   "flops_factor": ff, "flops_selinv": fs, "host_setup_s": t_setup},
        "phases_ms": {"factor": fm, "selinv": sm},
        "adjoint": {"plain_eval_ms": t_plain * 1e3, "value_and_grad_ms": t_grad * 1e3,
                    "ratio_vs_plain": t_grad / t_plain, "central_fd_ratio": 2 * d + 1,
                    "speedup_vs_fd": (2 * d + 1) * t_plain / t_grad, "dim_theta": int(d)},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--small", action="store_true", help="reduced workload (profiler captures)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", choices=["spde", "batch41", "coreg3"], default="spde",
                    help="spde: the headline single-model step (default); batch41: the mixed 41-instance "
                         "graph-captured launch; coreg3: the 3-variate coregional model with adjoint")
    args = ap.parse_args()
    if args.impl == "ours" and args.workload == "batch41":
        return run_batch41(args)
    if args.impl == "ours" and args.workload == "coreg3":
        return run_coreg3(args)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus if args.impl == "reference" else 1)))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)   # OpenBLAS uses every host core by default
    else:
        run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
