"""Measurement probes of the GPU at hand: ``python -m pyinla_gb300.probes``.

Prints the chip's FP64 FMA rate (the roofline denominator of the FP64 kernels), the
cycle counts of the 32 x 32 tile routines that sit on the dataflow critical paths
and of the primitives they are built from, and the check of the tcgen05 tile step
against the mma.sync one (gbta_probe_tiles, gbta_probe_latencies, gbta_probe_umma in
include/pyinla_gb300.h).
"""
from __future__ import annotations

import ctypes
import json

import numpy as np

from . import _lib


def fp64_peak_tflops(iters: int = 4000) -> float:
    lib = _lib.load()
    out = ctypes.c_double(0.0)
    _lib.check(lib.gbta_probe_fp64_peak(int(iters), ctypes.byref(out)))
    return float(out.value)


def tile_cycles(iters: int = 200) -> dict:
    lib = _lib.load()
    cyc = np.zeros(9, dtype=np.int64)
    _lib.check(lib.gbta_probe_tiles(int(iters), cyc.ctypes.data))
    names = ["reload", "potrf", "recip+trsm_rlt", "recip+trsm_rln", "digit_planes", "store",
             "recip+scale+trsm_rlt_8rows", "oz_tile_step", "oz_stage_2x16KB"]
    return {n: int(c) for n, c in zip(names, cyc)}


def umma_check(iters: int = 200) -> dict:
    """tcgen05 tile step against the mma.sync tile step (gbta_probe_umma)."""
    lib = _lib.load()
    mis = np.zeros(10, dtype=np.int32)
    cyc = np.zeros(4, dtype=np.int64)
    _lib.check(lib.gbta_probe_umma(int(iters), mis.ctypes.data, cyc.ctypes.data))
    names = ["plain_q0", "trans_q0", "plain_q2", "trans_q3", "plain_q5", "trans_q7", "plain_q7",
             "trans_swapped_offsets", "two_steps_trans", "two_steps_plain"]
    return {"mismatches": {n: int(m) for n, m in zip(names, mis)},
            "cycles_per_step": {"tcgen05": int(cyc[0]), "mma_sync": int(cyc[1])},
            "cycles_tcgen05_issue_one_step": int(cyc[2]), "cycles_fold": int(cyc[3])}


def primitive_cycles() -> dict:
    lib = _lib.load()
    cyc = np.zeros(9, dtype=np.int64)
    _lib.check(lib.gbta_probe_latencies(cyc.ctypes.data))
    names = ["dfma_dependent_1warp", "dfma_independent_1warp", "dfma_independent_4warps", "dfma_predicated_off",
             "rsqrt_approx_f64_plus_dadd", "shfl_f64", "lds_dependent", "bar_sync_4warps"]
    return {n: int(c) for n, c in zip(names, cyc)}


def tensor_rates(iters: int = 2000) -> dict:
    lib = _lib.load()
    out = np.zeros(3, dtype=np.float64)
    _lib.check(lib.gbta_probe_tensor_rates(int(iters), out.ctypes.data))
    return {"dmma_f64_tflops": float(out[0]), "hmma_f16_f32_tflops": float(out[1]), "ffma_tflops": float(out[2])}


def main() -> None:
    from . import build

    build.build()
    print(json.dumps({"fp64_dfma_tflops": fp64_peak_tflops(), **tensor_rates(), "tile_cycles": tile_cycles(),
                      "umma_tile_step": umma_check(), "primitive_cycles": primitive_cycles()}))


if __name__ == "__main__":
    main()
