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

The same line carries the adjoint theta-gradient against one plain evaluation and
against a measured central-difference gradient, the parity of the timed step's
results against the oracle, the CPU baseline, and two further workloads timed in the
same run: 41 mixed instances in one graph launch ("batch41") and the trivariate
coregional model with b = 3072 ("coreg3").
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
# (4096 flops each) = 43 times the 2 * 32^3 FP64 flops of the tile product.  The
# kernels leave out the products of zero tiles and zero leading digit planes and count
# the plane pairs they issue (gbta_kernel_pairs): OZ_PAIR_TENSOR_FLOPS each.
OZ_PAIR_TENSOR_FLOPS = 4 * 2 * 2 * 4096
OZ_STEP_TENSOR_FLOPS = 43 * OZ_PAIR_TENSOR_FLOPS


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
def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def oracle_qcond(spec, theta, nt_keep: int | None = None):
    """The workload's Q_cond as BTA blocks, from the oracle's own sparse assembly and
    sparse-to-BTA mapping, and the information vector.  nt_keep < nt keeps the leading
    nt_keep time blocks and the arrow: a principal submatrix, so still SPD."""
    from oracle import model_oracle as mo

    c = spec.coefficients(theta)
    _, Qc, rhs = mo.conditional_system(spec.terms, spec.term_vw, spec.ns, spec.nv, spec.nt, spec.nb, spec.A, spec.y,
                                       spec.tip_prec, c.alpha, c.beta, c.tau_y, spec.obs_variates())
    D, L, R, T = mo.sparse_to_bta(Qc, spec.nt, spec.b, spec.nb)
    if nt_keep is not None and nt_keep < spec.nt:
        b = spec.b
        rhs = np.concatenate([rhs[: nt_keep * b], rhs[spec.nt * b:]])
        D, L, R = D[:nt_keep].copy(), L[: nt_keep - 1].copy(), R[:nt_keep].copy()
    return D, L, R, T, rhs


def oracle_pass(D, L, R, T, rhs):
    """The oracle's pobtaf, logdet, pobtas N and C, pobtasi in place (the restatement
    of the reference's Serinv CPU path, NumPy/OpenBLAS on every host core); returns the
    seconds of pobtaf + pobtasi, the logdet and the solution."""
    from oracle import bta_oracle as orc

    t0 = time.perf_counter()
    orc.pobtaf(D, L, R, T)
    t_f = time.perf_counter() - t0
    ld = orc.logdet(D, T, "bta")
    x = rhs.copy()
    orc.pobtas(D, L, R, T, x, "N")
    orc.pobtas(D, L, R, T, x, "C")
    t0 = time.perf_counter()
    orc.pobtasi(D, L, R, T)
    t_s = time.perf_counter() - t0
    return t_f + t_s, ld, x


def relerr(x, y) -> float:
    x = np.asarray(x)
    y = np.asarray(y)
    return float(np.max(np.abs(x - y)) / max(float(np.max(np.abs(y))), 1e-300))


def cpu_baseline_and_parity(spec, theta, gpu: dict):
    """cpu_baseline: the oracle on this step's whole Q_cond (every time block), timed on
    the host cores.  Its results are the parity check of the timed step's GPU results
    (logdet, mean, every Sigma block), at the 1e-10 relative bar."""
    D, L, R, T, rhs = oracle_qcond(spec, theta)
    b, nt, a = spec.b, spec.nt, spec.nb
    dt, ld, x = oracle_pass(D, L, R, T, rhs)
    ff, fs = bta_flops(nt, b, a)
    diag_o = np.concatenate([np.diagonal(D, axis1=1, axis2=2).ravel(), np.diagonal(T)])
    diag_g = np.concatenate([np.diagonal(gpu["SD"], axis1=1, axis2=2).ravel(), np.diagonal(gpu["ST"])])
    blocks = {k: relerr(gpu[k], o) for k, o in (("SD", D), ("SL", L), ("SR", R), ("ST", T))}
    parity = {"rtol": 1e-10, "logdet": abs(gpu["logdet"] - ld) / abs(ld), "mu": relerr(gpu["mu"], x),
              "sigma_diag": relerr(diag_g, diag_o), "sigma_blocks": max(blocks.values()), "per_block": blocks,
              "against": f"oracle (NumPy/OpenBLAS restatement of Serinv) on the same Q_cond, all {nt} time "
                         "blocks; max-abs error over max-abs value per array"}
    parity["pass"] = all(parity[k] < 1e-10 for k in ("logdet", "mu", "sigma_diag", "sigma_blocks"))
    cpu = {"value": (ff + fs) / dt / 1e12, "unit": UNIT, "cores": host_cores(), "kind": "port",
           "sample": f"the whole workload: oracle pobtaf + pobtasi of this Q_cond (nt={nt}, b={b}, a={a}), "
                     f"{dt:.1f} s, no extrapolation"}
    return cpu, parity


# ----------------------------------------------------------------------------- reference arm
REF_NT_SAMPLE = 16


def run_reference(args, rank: int, world: int):
    """The reference's CPU implementation of the path on the host cores: the oracle
    port of Serinv's pobtaf + pobtasi (Serinv itself is absent), on a bounded sample of
    this workload's own Q_cond -- its leading 16 of 128 time blocks and the arrow."""
    if rank != 0:
        return
    from pyinla_gb300.model import SeparableSpdeAr1

    wl = workload(args.small)
    cores = host_cores()
    spec = SeparableSpdeAr1.synthetic(wl["n_side"], wl["nt"], wl["nb"], wl["n_obs"], wl["seed"])
    nts = min(REF_NT_SAMPLE, spec.nt)
    blocks = oracle_qcond(spec, spec.theta0, nts)
    b, a = spec.b, spec.nb
    ff, fs = bta_flops(nts, b, a)
    times = []
    for k in range(args.warmup + args.steps):
        D, L, R, T, rhs = [x.copy() for x in blocks]
        dt, _, _ = oracle_pass(D, L, R, T, rhs)
        if k >= args.warmup:
            times.append(dt)
    dt = statistics.median(times)
    value = (ff + fs) / dt / 1e12
    sample = (f"oracle pobtaf + pobtasi (NumPy/OpenBLAS restatement of Serinv) of the leading {nts} of "
              f"{spec.nt} time blocks of this workload's Q_cond with its arrow (b={b}, a={a}); "
              f"ms_per_step is that sample's time, not extrapolated")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded; reference datasets unavailable)",
        "config": {"workload": wl["name"], "b": b, "nt": spec.nt, "a": a, "nt_sample": nts,
                   "note": "Serinv is not installable offline; the reference arm times the oracle's "
                           "Serinv-equivalent NumPy/OpenBLAS restatement on the host cores"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- our arm
def tensor_peak():
    """Sustained bf16 tensor throughput of the GB300s (a kernel timed inside
    seconds-long back-to-back steps)."""
    try:
        mp = json.loads((REPO / "MEASURED_PEAKS.json").read_text())
        return float(mp["bf16_tflops_sustained"]), "MEASURED_PEAKS.json bf16_tflops_sustained (of measured)"
    except (OSError, ValueError, KeyError):
        return 1700.0, "fallback sustained bf16 figure, 1.7 PFLOP/s (of fallback: MEASURED_PEAKS.json absent)"


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
    kernel_ms = {"factor": [], "selinv": [], "solve": []}
    kernel_pairs = {"factor": [], "selinv": []}
    logdet = ctypes.c_double(0.0)

    def step(record: bool):
        e = ev if record else None
        ptrs = model._upload_coef(coef)
        if e: e["asm"][0].record()
        model._assemble(ptrs, Dc, Lc, Rc, Tc, with_lik=True)
        if e: e["asm"][1].record(); e["fac"][0].record()
        _lib.check(lib.gbta_pobtaf_async(h.ptr, Dc.data_ptr(), Lc.data_ptr(), Rc.data_ptr(), Tc.data_ptr()))
        _lib.check(lib.gbta_logdet(h.ptr, Dc.data_ptr(), Tc.data_ptr(), 1, ctypes.byref(logdet)))
        if e: e["fac"][1].record(); e["sol"][0].record()
        torch.mv(model._Aty_v.t(), tau_dev, out=mu)
        _lib.check(lib.gbta_pobtas_async(h.ptr, Dc.data_ptr(), Lc.data_ptr(), Rc.data_ptr(), Tc.data_ptr(),
                                         mu.data_ptr(), 1, 2))   # N then C in one launch
        if e: e["sol"][1].record(); e["sel"][0].record()
        _lib.check(lib.gbta_pobtasi_async(h.ptr, Dc.data_ptr(), Lc.data_ptr(), Rc.data_ptr(), Tc.data_ptr()))
        if e: e["sel"][1].record()

    def collect():
        for k, (e0, e1) in ev.items():
            timings[k].append(e0.elapsed_time(e1))
        km = np.zeros(3)
        _lib.check(lib.gbta_kernel_ms(h.ptr, km.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        for k, v in zip(("factor", "selinv", "solve"), km):
            kernel_ms[k].append(float(v))
        kp = (ctypes.c_longlong * 2)()
        _lib.check(lib.gbta_kernel_pairs(h.ptr, kp))
        for k, v in zip(("factor", "selinv"), kp):
            kernel_pairs[k].append(int(v))

    for _ in range(args.warmup):
        step(False)
    _lib.check(lib.gbta_status(h.ptr))
    torch.cuda.synchronize()
    peak = ctypes.c_double(0.0)
    _lib.check(lib.gbta_probe_fp64_peak(4000, ctypes.byref(peak)))
    dfma_peak = float(peak.value)
    _lib.check(lib.gbta_set_kernel_timing(h.ptr, 1))

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
    _lib.check(lib.gbta_set_kernel_timing(h.ptr, 0))
    elapsed_ms = t_start.elapsed_time(t_end)
    if dist:
        tt = torch.tensor([elapsed_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        elapsed_ms = float(tt.item())
    ms_per_step = elapsed_ms / args.steps
    value = world * args.steps * (ff + fs) / (elapsed_ms * 1e-3) / 1e12
    # results of the last timed step, for the parity check against the oracle
    gpu_out = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        gpu_out = {"logdet": float(logdet.value), "mu": mu.cpu().numpy(), "SD": Dc.cpu().numpy(),
                   "SL": Lc.cpu().numpy(), "SR": Rc.cpu().numpy(), "ST": Tc.cpu().numpy()}

    avg = {k: statistics.mean(v) for k, v in timings.items()}
    kavg = {k: statistics.mean(v) for k, v in kernel_ms.items()}
    dominant = "selinv" if kavg["selinv"] >= kavg["factor"] else "factor"
    kname = {"factor": "k_factor_oz", "selinv": "k_selinv_oz"}[dominant]
    # the dominant kernel against the tensor pipe: the fp16 mma work of the digit-plane
    # tile products it issued (its own count, per launch) over its CUDA-event time; the
    # dense count (43 plane pairs on every tile step of the DAG) for comparison
    fsteps, ssteps = oz_tile_steps(nt, b, a)
    dense_flop = (ssteps if dominant == "selinv" else fsteps) * OZ_STEP_TENSOR_FLOPS
    pairs_launch = statistics.mean(kernel_pairs[dominant])
    tflop_launch = pairs_launch * OZ_PAIR_TENSOR_FLOPS
    tachieved = tflop_launch / (kavg[dominant] * 1e-3) / 1e12
    tpeak, tsrc = tensor_peak()
    fp64_flops = fs if dominant == "selinv" else ff
    fp64_achieved = fp64_flops / (kavg[dominant] * 1e-3) / 1e12
    traffic, traffic_src = None, None
    tfile = REPO / "profiles" / "traffic.json"
    if tfile.exists():
        try:
            tj = json.loads(tfile.read_text()).get(wl["name"], {})
            traffic, traffic_src = tj.get(kname), tj.get("method")
        except (ValueError, OSError):
            pass

    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded; reference datasets unavailable)",
        "config": {"workload": wl["name"], "b": b, "nt": nt, "a": a, "n_obs": wl["n_obs"],
                   "parallelism": f"replicas{world}", "l2": "inputs larger than L2 (BTA blocks "
                   f"{(2 * nt - 1) * b * b * 8 / 1e9:.2f} GB)",
                   "step": "assemble Q_cond + pobtaf + logdet + pobtas(N,C) + pobtasi",
                   "flops_per_step": ff + fs, "flops_factor": ff, "flops_selinv": fs,
                   "flops_note": "dense block-operation counts of the recurrence (Serinv's own count); the "
                                 "kernels leave out the products of structurally zero tiles"},
        "phases_ms": {"assemble": avg["asm"], "factor_and_logdet": avg["fac"], "solve": avg["sol"],
                      "selinv": avg["sel"]},
        "kernels_ms": kavg,
        "roofline": {"bound": "tensor", "achieved": tachieved, "peak": tpeak, "unit": "TFLOP/s",
                     "frac": tachieved / tpeak, "traffic": traffic, "kernel": kname, "peak_source": tsrc,
                     "work": "fp16 mma.sync flops of the digit-plane tile products the kernel issued per "
                             f"launch ({pairs_launch:.0f} plane pairs of 32x32x32, {tflop_launch / 1e12:.2f} "
                             f"TFLOP; counted by the kernel); all 43 pairs on every tile step of the DAG "
                             f"would be {dense_flop / 1e12:.2f} TFLOP",
                     "traffic_source": traffic_src,
                     "fp64": {"achieved": fp64_achieved, "unit": "TFLOP/s", "dfma_peak": dfma_peak,
                              "frac_of_dfma": fp64_achieved / dfma_peak if dfma_peak else None,
                              "note": "algorithmic FP64 flops of the kernel's recurrence per launch against the "
                                      "measured FP64 FMA rate of this GPU (gbta_probe_fp64_peak)"}},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    # pobtas N and C: both sweeps read the factor once each (their algorithmic bytes)
    sb = solve_bytes(nt, b, a)
    result["solve_hbm"] = {"bytes": sb, "ms": avg["sol"], "achieved_gbs": sb / (avg["sol"] * 1e-3) / 1e9,
                           "peak_gbs": hbm_peak()[0], "frac": sb / (avg["sol"] * 1e-3) / 1e9 / hbm_peak()[0],
                           "peak_source": hbm_peak()[1]}

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
        n_e2e = max(1, min(args.steps, 5))   # (whole steps; more of them damp a slow host step)
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

    # ---- adjoint gradient vs one plain evaluation and vs measured central differences
    if not args.no_adjoint:
        result["adjoint"] = adjoint_figures(model, theta, reps=5, torch=torch)
        d = theta.size
        # theta-Hessian: differences of 2d adjoint gradients, against the reference's
        # differences of f (1 + 2d + 2d(d-1) evaluations, pyinla.py:767-910)
        t0 = time.perf_counter()
        model.hessian(theta)
        torch.cuda.synchronize()
        t_hess = time.perf_counter() - t0
        n_fd = 1 + 2 * d + 2 * d * (d - 1)
        result["hessian"] = {"ms": t_hess * 1e3, "gradient_evaluations": 2 * int(d),
                             "reference_f_evaluations": int(n_fd),
                             "speedup_vs_fd_of_f": n_fd * result["adjoint"]["plain_eval_ms"] / (t_hess * 1e3)}

    # ---- CPU baseline (rank 0, N = 1 only): the oracle on the host cores, which also
    # checks the timed step's results
    if gpu_out is not None:
        result["cpu_baseline"], result["parity"] = cpu_baseline_and_parity(spec, theta, gpu_out)
        del gpu_out

    del model, Dc, Lc, Rc, Tc, mu
    torch.cuda.empty_cache()
    if rank == 0 and world == 1 and not args.no_extra:
        sub = argparse.Namespace(**vars(args))
        sub.steps, sub.warmup = min(args.steps, 3), 3
        result["batch41"] = run_batch41(sub)
        torch.cuda.empty_cache()
        result["coreg3"] = run_coreg3(sub)
        torch.cuda.empty_cache()
    if rank == 0:
        print(json.dumps(result), flush=True)
    if dist:
        dist.destroy_process_group()


def solve_bytes(nt: int, b: int, a: int) -> float:
    """Algorithmic bytes of pobtas N + C with one right-hand side: the factor read once
    per sweep (lower triangles of the diagonal blocks, the off-diagonal and arrow blocks,
    the tip's triangle) plus four passes over the vector."""
    N = nt * b + a
    return 2 * 8.0 * (nt * b * (b + 1) / 2 + (nt - 1) * b * b + nt * a * b + a * (a + 1) / 2) + 4 * 8.0 * N


def hbm_peak():
    try:
        mp = json.loads((REPO / "MEASURED_PEAKS.json").read_text())
        return float(mp["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (of measured)"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback 6.8 TB/s (of fallback: MEASURED_PEAKS.json absent)"


def adjoint_figures(model, theta, reps: int, torch) -> dict:
    """Median times of reps plain evaluations and reps value-and-gradient evaluations,
    and one measured central-difference gradient (2 dim(theta) + 1 evaluations, step
    1e-4, as the reference's PyINLA._objective_function does with its own step,
    pyinla.py:546-580), with its relative distance from the adjoint gradient."""
    d = theta.size
    model.evaluate(theta)
    torch.cuda.synchronize()
    tp, tg = [], []
    g = None
    for _ in range(reps):
        t0 = time.perf_counter()
        model.evaluate(theta)
        torch.cuda.synchronize()
        tp.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        _, g = model.evaluate(theta, gradient=True)
        torch.cuda.synchronize()
        tg.append(time.perf_counter() - t0)
    t0 = time.perf_counter()
    model.evaluate(theta)
    fd = np.zeros(d)
    for k in range(d):
        e = np.zeros(d)
        e[k] = 1e-4
        fd[k] = (model.evaluate(theta + e) - model.evaluate(theta - e)) / 2e-4
    torch.cuda.synchronize()
    t_fd = time.perf_counter() - t0
    t_plain, t_grad = statistics.median(tp), statistics.median(tg)
    return {"plain_eval_ms": t_plain * 1e3, "value_and_grad_ms": t_grad * 1e3,
            "ratio_vs_plain": t_grad / t_plain, "reps": reps, "central_fd_evaluations": 2 * d + 1,
            "central_fd_ms": t_fd * 1e3, "speedup_vs_fd": t_fd / t_grad,
            "fd_rel_diff": relerr(g, fd), "gradients_per_s": 1.0 / t_grad, "dim_theta": int(d)}


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
            _lib.check(lib.gbta_pobtas_async(h.ptr, D.data_ptr(), L.data_ptr(), Rp, Tp, x.data_ptr(), 1, 2))
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
    return line


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
    clocks = ClockSampler(0)
    for s in range(args.warmup + args.steps):
        if s == args.warmup:
            clocks.start()
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
    clk = clocks.stop()
    adj = adjoint_figures(model, theta, reps=3, torch=torch)
    fm, sm = statistics.median(fac), statistics.median(sel)
    line = {
        "metric": METRIC, "value": (ff + fs) / ((fm + sm) * 1e-3) / 1e12, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": fm + sm, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": "coreg3_spde32x32_ar1_nt64_nb9_obs300k", "b": b, "nt": nt, "a": a,
                   "flops_factor": ff, "flops_selinv": fs, "host_setup_s": t_setup},
        "phases_ms": {"factor": fm, "selinv": sm},
        "adjoint": adj, "clocks": clk,
    }
    del model, Dc, Lc, Rc, Tc
    return line


def main():
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--small", action="store_true", help="reduced workload (profiler captures)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the oracle leg (CPU baseline and parity)")
    ap.add_argument("--no-extra", action="store_true", help="skip the batch41 and coreg3 workloads")
    ap.add_argument("--workload", choices=["spde", "batch41", "coreg3"], default="spde",
                    help="spde: the headline single-model step (default); batch41: the mixed 41-instance "
                         "graph-captured launch; coreg3: the 3-variate coregional model with adjoint")
    args = ap.parse_args()
    if args.impl == "ours" and args.workload == "batch41":
        print(json.dumps(run_batch41(args)), flush=True)
        return
    if args.impl == "ours" and args.workload == "coreg3":
        print(json.dumps(run_coreg3(args)), flush=True)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus if args.impl == "reference" else 1)))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)   # OpenBLAS uses every host core by default
    else:
        run_ours(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
