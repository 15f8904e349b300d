"""Autotuner of the multi-instance launch.

Two choices are made by measurement on the GPU at hand and cached per device:

* the product method of every instance shape (block size b, arrow a): FP64 FMAs or
  tensor-core digit planes (``GBTA_METHOD_FP64`` / ``GBTA_METHOD_OZAKI``).  The tile
  edge is fixed at 32 by the kernels' layout; what differs between the methods is the
  shape of the product work per tile step (one FP64 32x32x32 update, or 43 integer
  m16n8k16 products over digit planes) and the data it stages.  Each candidate
  factorizes and inverts a synthetic SPD instance of that (b, a) with ``nt_probe``
  blocks; the faster wins;
* the ticket merge order of a concrete batch (proportional, round robin, sequential),
  timed on the batch itself with graph launches.

The cache is a JSON file (``$PYINLA_GB300_TUNE_CACHE``, default
``~/.cache/pyinla_gb300/tune.json``) keyed by device name, library version and shape.
"""
from __future__ import annotations

import json
import os
from pathlib import Path

from . import _lib
from .device import BtaHandle, require_torch_cuda
from .synthetic import random_bta

METHODS = (_lib.GBTA_METHOD_FP64, _lib.GBTA_METHOD_OZAKI)


def cache_path() -> Path:
    p = os.environ.get("PYINLA_GB300_TUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "pyinla_gb300" / "tune.json"


def _load_cache() -> dict:
    try:
        return json.loads(cache_path().read_text())
    except (OSError, ValueError):
        return {}


def _store_cache(c: dict) -> None:
    p = cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        tmp = p.with_suffix(".tmp")
        tmp.write_text(json.dumps(c, indent=1, sort_keys=True))
        tmp.replace(p)
    except OSError:
        pass   # an unwritable cache only costs re-tuning


def _device_key() -> str:
    torch = require_torch_cuda()
    lib = _lib.load()
    return f"{torch.cuda.get_device_name()}|v{lib.gbta_version()}"


def time_method(b: int, a: int, method: int, nt_probe: int = 8, reps: int = 2) -> float:
    """Milliseconds of factor + selected inversion of a synthetic (nt_probe, b, a)
    instance with the given product method (best of ``reps``)."""
    torch = require_torch_cuda()
    lib = _lib.load()
    h = BtaHandle(b, nt_probe, a)
    try:
        h.set_stream(torch.cuda.current_stream().cuda_stream)
        h.set_method(method)
        D0, L0, R0, T0 = random_bta(nt_probe, b, a, seed=1)
        best = float("inf")
        for rep in range(reps + 1):
            D, L, R, T = D0.clone(), L0.clone(), R0.clone(), T0.clone()
            Rp, Tp = (R.data_ptr(), T.data_ptr()) if a else (None, None)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            if a:
                _lib.check(lib.gbta_pobtaf_async(h.ptr, D.data_ptr(), L.data_ptr(), Rp, Tp))
                _lib.check(lib.gbta_pobtasi_async(h.ptr, D.data_ptr(), L.data_ptr(), Rp, Tp))
            else:
                _lib.check(lib.gbta_pobtf_async(h.ptr, D.data_ptr(), L.data_ptr()))
                _lib.check(lib.gbta_pobtsi(h.ptr, D.data_ptr(), L.data_ptr()))
            e1.record()
            h.status()
            if rep:   # the first run warms up
                best = min(best, e0.elapsed_time(e1))
        return best
    finally:
        h.close()


def choose_methods(shapes, nt_probe: int = 8, use_cache: bool = True) -> list[int]:
    """Product method per instance of ``shapes`` [(b, nt, a), ...]."""
    cache = _load_cache() if use_cache else {}
    dev = _device_key()
    table = cache.setdefault(dev, {}).setdefault("method", {})
    out = []
    dirty = False
    for (b, nt, a) in shapes:
        key = f"b{int(b)}_a{int(a)}_p{int(nt_probe)}"
        if key not in table:
            times = {str(m): time_method(int(b), int(a), m, nt_probe) for m in METHODS}
            best = min(times, key=times.get)
            table[key] = {"method": int(best), "ms": times}
            dirty = True
        out.append(int(table[key]["method"]))
    if dirty and use_cache:
        _store_cache(cache)
    return out


def choose_order(batch, phases: int = _lib.GBTA_PHASE_ALL, reps: int = 1, reload=None) -> dict:
    """Time every merge order on ``batch`` (graph launches; ``reload()`` refills the
    inputs before each run) and keep the fastest.  Returns {order: ms}."""
    torch = require_torch_cuda()
    from .batch import ORDERS

    times = {}
    for order in ORDERS:
        batch.set_order(order)
        best = float("inf")
        for rep in range(reps + 1):
            if reload is not None:
                reload()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            batch.run_async(phases, graph=True)
            e1.record()
            batch.status()
            if rep:
                best = min(best, e0.elapsed_time(e1))
        times[order] = best
    batch.set_order(min(times, key=times.get))
    return times


def tuned_batch(shapes, nt_probe: int = 8):
    """A :class:`~pyinla_gb300.batch.BtaBatch` with autotuned product methods."""
    from .batch import BtaBatch

    return BtaBatch(shapes, methods=choose_methods(shapes, nt_probe))
