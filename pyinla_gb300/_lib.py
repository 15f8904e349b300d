"""ctypes binding of libpyinla_gb300.so (the C ABI in include/pyinla_gb300.h).

The library is the only compute path of this package: if it is missing or cannot
be loaded, every entry point raises -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libpyinla_gb300.so"

GBTA_OK = 0
GBTA_ERR_ARG = -1
GBTA_ERR_CUDA = -2
GBTA_ERR_TIMEOUT = -3
GBTA_ERR_ALLOC = -5
GBTA_METHOD_FP64 = 0
GBTA_METHOD_OZAKI = 1
GBTA_MAX_VARIATES = 8        # include/pyinla_gb300.h
GBTA_PHASE_FACTOR = 1
GBTA_PHASE_LOGDET = 2
GBTA_PHASE_SOLVE = 4
GBTA_PHASE_SELINV = 8
GBTA_PHASE_ALL = 15
GBTA_BATCH_ORDER_PROPORTIONAL = 0
GBTA_BATCH_ORDER_ROUND_ROBIN = 1
GBTA_BATCH_ORDER_SEQUENTIAL = 2

_lib = None
_lock = threading.Lock()

_c_int = ctypes.c_int
_c_ll = ctypes.c_longlong
_vp = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)

# name -> (restype, argtypes); the exact list of symbols declared in the header.
SIGNATURES = {
    "gbta_version": (_c_int, []),
    "gbta_kernel_launches": (_c_ll, []),
    "gbta_probe_fp64_peak": (_c_int, [_c_int, _dp]),
    "gbta_last_error": (ctypes.c_char_p, []),
    "gbta_geometry": (_c_int, [_vp, ctypes.POINTER(_c_int), ctypes.POINTER(_c_int), ctypes.POINTER(_c_int),
                               ctypes.POINTER(_vp)]),
    "gbta_set_error": (_c_int, [_c_int, ctypes.c_char_p]),
    "gbta_create": (_c_int, [_c_int, _c_int, _c_int, ctypes.POINTER(_vp)]),
    "gbta_destroy": (_c_int, [_vp]),
    "gbta_set_stream": (_c_int, [_vp, _vp]),
    "gbta_set_wait_limit_ms": (_c_int, [_vp, ctypes.c_double]),
    "gbta_set_method": (_c_int, [_vp, _c_int]),
    "gbta_get_method": (_c_int, [_vp]),
    "gbta_set_ctas_per_sm": (_c_int, [_vp, _c_int]),
    "gbta_set_trace": (_c_int, [_vp, _c_int]),
    "gbta_get_trace": (_c_ll, [_vp, _vp, _c_ll]),
    "gbta_get_task_list": (_c_ll, [_vp, _c_int, _vp, _c_ll]),
    "gbta_set_selinv_overlap": (_c_int, [_vp, _c_int]),
    "gbta_set_twist": (_c_int, [_vp, _c_int]),
    "gbta_get_twist": (_c_int, [_vp]),
    "gbta_set_kernel_timing": (_c_int, [_vp, _c_int]),
    "gbta_kernel_ms": (_c_int, [_vp, _dp]),
    "gbta_kernel_pairs": (_c_int, [_vp, ctypes.POINTER(ctypes.c_longlong)]),
    "gbta_workspace_bytes": (ctypes.c_size_t, [_vp]),
    "gbta_status": (_c_int, [_vp]),
    "gbta_pobtaf": (_c_int, [_vp, _vp, _vp, _vp, _vp]),
    "gbta_pobtf": (_c_int, [_vp, _vp, _vp]),
    "gbta_pobtaf_async": (_c_int, [_vp, _vp, _vp, _vp, _vp]),
    "gbta_pobtf_async": (_c_int, [_vp, _vp, _vp]),
    "gbta_noalloc_scratch_bytes": (ctypes.c_size_t, [_c_int, _c_int, _c_int]),
    "gbta_pobtaf_noalloc": (_c_int, [_c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp]),
    "gbta_pobtas": (_c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _c_int, _c_int]),
    "gbta_pobts": (_c_int, [_vp, _vp, _vp, _vp, _c_int, _c_int]),
    "gbta_pobtas_async": (_c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _c_int, _c_int]),
    "gbta_logdet": (_c_int, [_vp, _vp, _vp, _c_int, _dp]),
    "gbta_pobtasi": (_c_int, [_vp, _vp, _vp, _vp, _vp]),
    "gbta_pobtsi": (_c_int, [_vp, _vp, _vp]),
    "gbta_pobtasi_async": (_c_int, [_vp, _vp, _vp, _vp, _vp]),
    "gbta_scatter_coo": (_c_int, [_vp, _vp, _vp, _vp, _c_ll, _vp, _vp, _vp, _vp, _c_int]),
    "gbta_gather_coo": (_c_int, [_vp, _vp, _vp, _c_ll, _vp, _vp, _vp, _vp, _c_int, _vp]),
    "gbta_assemble_kron": (_c_int, [_vp, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                    _vp, _vp, _vp, _vp, ctypes.c_double, _vp, _vp, _vp, _vp]),
    "gbta_contract_kron": (_c_int, [_vp, _c_int, _c_int, _c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                    _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gbta_sigma_diagonal": (_c_int, [_vp, _vp, _vp, _vp]),
    "gbta_obs_variances": (_c_int, [_vp, _c_ll, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gbta_weighted_gram": (_c_int, [_vp, _c_ll, _vp, _vp, _vp, _vp, _vp]),
    "gbta_bta_symv": (_c_int, [_vp, _vp, _vp, _vp, _vp, _c_int, _vp, _vp]),
    "gbta_batch_create": (_c_int, [_c_int, _vp, _vp, _vp, _vp, ctypes.POINTER(_vp)]),
    "gbta_batch_destroy": (_c_int, [_vp]),
    "gbta_batch_workspace_bytes": (ctypes.c_size_t, [_vp]),
    "gbta_batch_set_stream": (_c_int, [_vp, _vp]),
    "gbta_batch_set_order": (_c_int, [_vp, _c_int]),
    "gbta_batch_set_ctas_per_sm": (_c_int, [_vp, _c_int]),
    "gbta_batch_set_wait_limit_ms": (_c_int, [_vp, ctypes.c_double]),
    "gbta_batch_bind": (_c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "gbta_batch_run_async": (_c_int, [_vp, _c_int, _vp]),
    "gbta_batch_graph_launch": (_c_int, [_vp, _c_int, _vp]),
    "gbta_batch_graph_kernels": (_c_ll, [_vp]),
    "gbta_batch_status": (_c_int, [_vp, _vp]),
}


class GBTAError(RuntimeError):
    """A CUDA, argument or timeout error reported by the library."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[gbta {code}] {msg}")
        self.code = code


def load(path: str | os.PathLike | None = None):
    """Load the shared library (once).  Raises if it is absent: build it with
    ``python -m pyinla_gb300.build``."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise RuntimeError(f"{p} is missing: build the CUDA library with `python -m pyinla_gb300.build`")
        lib = ctypes.CDLL(str(p))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def last_error() -> str:
    return load().gbta_last_error().decode(errors="replace")


def check(code: int) -> int:
    """Translate a return code: > 0 (non-positive pivot) raises numpy's LinAlgError
    (a ValueError, like numpy.linalg.cholesky on a non-SPD block); < 0 raises GBTAError."""
    if code == GBTA_OK:
        return code
    msg = last_error()
    if code > 0:
        raise np.linalg.LinAlgError(msg or f"Matrix is not positive definite (pivot at row {code})")
    raise GBTAError(code, msg)


def ptr(t) -> int | None:
    """Device address of a torch tensor (None passes NULL)."""
    if t is None:
        return None
    return t.data_ptr()
