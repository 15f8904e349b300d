"""Drop-in for ``serinv.algs`` on the reference's single-process path.

The reference imports ``pobtaf, pobtas, pobtasi, pobtf, pobts, pobtsi`` from Serinv
(src/pyinla/solvers/structured_solver.py:12-15) and calls them positionally, in
place, on its block buffers (``:83-93, 112-140, 176-186``).  These functions keep
those names, argument orders and in-place semantics and run on the GB300 through
libpyinla_gb300.so:

* torch CUDA float64 tensors are used in place (zero copy);
* NumPy arrays (the reference's ``ARRAY_MODULE=numpy`` buffers) are copied to the
  device, processed, and written back into the same arrays.

A non-positive pivot raises ``numpy.linalg.LinAlgError`` (a ``ValueError``), as
``numpy.linalg.cholesky`` does inside Serinv's NumPy path.  Injecting this module
as ``serinv.algs`` (see :func:`install_as_serinv`) makes the reference's own
``SerinvSolver`` run on the GPU unchanged.
"""
from __future__ import annotations

import sys
import types
from typing import Any

import numpy as np

from . import _lib
from .device import BtaHandle, current_stream_ptr, require_torch_cuda

__all__ = ["pobtaf", "pobtas", "pobtasi", "pobtf", "pobts", "pobtsi", "logdet", "install_as_serinv",
           "set_twisted"]

# Elimination order of these drop-ins.  False (the default) is Serinv's top-down block
# recurrence, so the factor blocks and each half-sweep hold what Serinv's would; True
# eliminates from both ends towards the middle block (half the critical path of the
# dataflow kernels), which changes the factor and the intermediate of a lone "N" sweep
# but not the logdet, the solution of an N-then-C solve or the selected inverse.
_TWIST = False


def set_twisted(enable: bool) -> None:
    """Choose the elimination order of the functions of this module (see _TWIST); a
    factor must be swept and inverted under the order it was made with."""
    global _TWIST
    _TWIST = bool(enable)


class _Staged:
    """A block buffer on the device; remembers the host array to write back."""

    def __init__(self, x: Any, torch, writable: bool = True):
        self.host = None
        if x is None:
            self.dev = None
        elif isinstance(x, torch.Tensor):
            if x.device.type != "cuda" or x.dtype != torch.float64 or not x.is_contiguous():
                raise ValueError("device buffers must be contiguous float64 CUDA tensors")
            self.dev = x
        else:
            arr = np.asarray(x)
            if arr.dtype != np.float64:
                raise ValueError("BTA buffers must be float64")
            self.host = arr if writable else None
            self.dev = torch.from_numpy(np.ascontiguousarray(arr)).to("cuda", non_blocking=False)

    def ptr(self):
        return None if self.dev is None else self.dev.data_ptr()

    def write_back(self):
        if self.host is not None:
            self.host[...] = self.dev.cpu().numpy().reshape(self.host.shape)


def _geometry(D, R, T):
    nt, b = int(D.shape[0]), int(D.shape[1])
    a = 0
    if T is not None and R is not None and int(T.shape[0]) > 0:
        a = int(T.shape[0])
    return b, nt, a


def pobtaf(A_diagonal_blocks, A_lower_diagonal_blocks, A_arrow_bottom_blocks, A_arrow_tip_block) -> None:
    """In-place BTA Cholesky (Serinv ``pobtaf``; structured_solver.py:83-88)."""
    torch = require_torch_cuda()
    b, nt, a = _geometry(A_diagonal_blocks, A_arrow_bottom_blocks, A_arrow_tip_block)
    bufs = [_Staged(x, torch) for x in (A_diagonal_blocks, A_lower_diagonal_blocks,
                                        A_arrow_bottom_blocks if a else None, A_arrow_tip_block if a else None)]
    h = BtaHandle.get(b, nt, a, _TWIST)
    h.set_stream(current_stream_ptr())
    code = h.lib.gbta_pobtaf(h.ptr, *[s.ptr() for s in bufs])
    _lib.check(code)
    for s in bufs:
        s.write_back()


def pobtf(A_diagonal_blocks, A_lower_diagonal_blocks) -> None:
    """In-place block-tridiagonal Cholesky (Serinv ``pobtf``; structured_solver.py:90-93)."""
    torch = require_torch_cuda()
    b, nt, _ = _geometry(A_diagonal_blocks, None, None)
    bufs = [_Staged(x, torch) for x in (A_diagonal_blocks, A_lower_diagonal_blocks)]
    h = BtaHandle.get(b, nt, 0, _TWIST)
    h.set_stream(current_stream_ptr())
    _lib.check(h.lib.gbta_pobtf(h.ptr, bufs[0].ptr(), bufs[1].ptr()))
    for s in bufs:
        s.write_back()


def _trans_code(trans: str) -> int:
    if trans == "N":
        return 0
    if trans in ("C", "T"):
        return 1
    raise ValueError(f"Unknown trans {trans!r}; use 'N' or 'C'")


def pobtas(A_diagonal_blocks, A_lower_diagonal_blocks, A_arrow_bottom_blocks, A_arrow_tip_block, B,
           trans: str = "N") -> None:
    """In-place triangular sweep (Serinv ``pobtas``; structured_solver.py:112-127).

    ``B`` is (N,) or (N, nrhs); ``trans="N"`` solves L y = b, ``"C"`` solves L^T x = y.
    """
    torch = require_torch_cuda()
    b, nt, a = _geometry(A_diagonal_blocks, A_arrow_bottom_blocks, A_arrow_tip_block)
    n = nt * b + a
    if int(B.shape[0]) != n:
        raise ValueError(f"rhs has {B.shape[0]} rows, expected {n}")
    nrhs = 1 if B.ndim == 1 else int(np.prod(B.shape[1:]))
    fac = [_Staged(x, torch, writable=False) for x in (A_diagonal_blocks, A_lower_diagonal_blocks,
                                                       A_arrow_bottom_blocks if a else None,
                                                       A_arrow_tip_block if a else None)]
    rhs = _Staged(B, torch)
    h = BtaHandle.get(b, nt, a, _TWIST)
    h.set_stream(current_stream_ptr())
    _lib.check(h.lib.gbta_pobtas(h.ptr, *[s.ptr() for s in fac], rhs.ptr(), nrhs, _trans_code(trans)))
    rhs.write_back()


def pobts(A_diagonal_blocks, A_lower_diagonal_blocks, B, trans: str = "N") -> None:
    """In-place block-tridiagonal sweep (Serinv ``pobts``; structured_solver.py:129-140)."""
    torch = require_torch_cuda()
    b, nt, _ = _geometry(A_diagonal_blocks, None, None)
    n = nt * b
    if int(B.shape[0]) != n:
        raise ValueError(f"rhs has {B.shape[0]} rows, expected {n}")
    nrhs = 1 if B.ndim == 1 else int(np.prod(B.shape[1:]))
    fac = [_Staged(x, torch, writable=False) for x in (A_diagonal_blocks, A_lower_diagonal_blocks)]
    rhs = _Staged(B, torch)
    h = BtaHandle.get(b, nt, 0, _TWIST)
    h.set_stream(current_stream_ptr())
    _lib.check(h.lib.gbta_pobts(h.ptr, fac[0].ptr(), fac[1].ptr(), rhs.ptr(), nrhs, _trans_code(trans)))
    rhs.write_back()


def pobtasi(A_diagonal_blocks, A_lower_diagonal_blocks, A_arrow_bottom_blocks, A_arrow_tip_block) -> None:
    """In-place selected inversion (Serinv ``pobtasi``; structured_solver.py:176-181)."""
    torch = require_torch_cuda()
    b, nt, a = _geometry(A_diagonal_blocks, A_arrow_bottom_blocks, A_arrow_tip_block)
    bufs = [_Staged(x, torch) for x in (A_diagonal_blocks, A_lower_diagonal_blocks,
                                        A_arrow_bottom_blocks if a else None, A_arrow_tip_block if a else None)]
    h = BtaHandle.get(b, nt, a, _TWIST)
    h.set_stream(current_stream_ptr())
    _lib.check(h.lib.gbta_pobtasi(h.ptr, *[s.ptr() for s in bufs]))
    for s in bufs:
        s.write_back()


def pobtsi(A_diagonal_blocks, A_lower_diagonal_blocks) -> None:
    """In-place block-tridiagonal selected inversion (Serinv ``pobtsi``; structured_solver.py:183-186)."""
    torch = require_torch_cuda()
    b, nt, _ = _geometry(A_diagonal_blocks, None, None)
    bufs = [_Staged(x, torch) for x in (A_diagonal_blocks, A_lower_diagonal_blocks)]
    h = BtaHandle.get(b, nt, 0, _TWIST)
    h.set_stream(current_stream_ptr())
    _lib.check(h.lib.gbta_pobtsi(h.ptr, bufs[0].ptr(), bufs[1].ptr()))
    for s in bufs:
        s.write_back()


def logdet(A_diagonal_blocks, A_arrow_tip_block=None, sparsity: str = "bta") -> float:
    """2 * sum(log diag) of a factor (structured_solver.py:151-166); "bt" excludes the tip.
    Raises ``ValueError`` when the result is NaN."""
    torch = require_torch_cuda()
    if sparsity not in ("bt", "bta"):
        raise ValueError(f"Unknown sparsity pattern: {sparsity}. Use 'bt' or 'bta'.")
    nt, b = int(A_diagonal_blocks.shape[0]), int(A_diagonal_blocks.shape[1])
    a = int(A_arrow_tip_block.shape[0]) if (A_arrow_tip_block is not None and sparsity == "bta") else 0
    D = _Staged(A_diagonal_blocks, torch, writable=False)
    T = _Staged(A_arrow_tip_block if a else None, torch, writable=False)
    h = BtaHandle.get(b, nt, a, _TWIST)
    h.set_stream(current_stream_ptr())
    import ctypes
    out = ctypes.c_double(0.0)
    code = h.lib.gbta_logdet(h.ptr, D.ptr(), T.ptr(), 1 if a else 0, ctypes.byref(out))
    if code == _lib.GBTA_ERR_ARG and np.isnan(out.value):
        raise ValueError("Logdet is NaN. Check the input matrix.")
    _lib.check(code)
    return float(out.value)


def install_as_serinv() -> types.ModuleType:
    """Register this module as ``serinv.algs`` (and a ``serinv`` package) in
    ``sys.modules`` so that ``from serinv.algs import pobtaf, ...`` resolves here."""
    mod = sys.modules[__name__]
    pkg = sys.modules.get("serinv")
    if pkg is None:
        pkg = types.ModuleType("serinv")
        sys.modules["serinv"] = pkg
    pkg.algs = mod
    sys.modules["serinv.algs"] = mod
    return mod
