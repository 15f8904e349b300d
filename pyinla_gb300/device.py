"""Device plumbing: solver handles of libpyinla_gb300.so and the torch stream they use.

PyTorch provides device memory and the current CUDA stream; all arithmetic runs in
the library's kernels.
"""
from __future__ import annotations

import ctypes
import threading

from . import _lib

_handles: dict = {}
_hlock = threading.Lock()


def require_torch_cuda():
    """Return the torch module, raising if no CUDA device is usable (no CPU fallback)."""
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("pyinla_gb300 needs a CUDA device (GB300); none is visible")
    _lib.load()
    return torch


def current_stream_ptr() -> int:
    import torch

    return torch.cuda.current_stream().cuda_stream


class BtaHandle:
    """Owns one ``gbta_solver`` (geometry b, nt, a on the current device).

    ``twist`` selects the elimination order of the block recurrences (gbta_set_twist):
    True, the library's default, eliminates from both ends towards the middle block
    (half the critical path); False keeps Serinv's top-down order, whose factor blocks
    and half-sweeps match Serinv's own.  Logdet, full solves and the selected inverse
    agree either way."""

    def __init__(self, b: int, nt: int, a: int, twist: bool = True):
        self.lib = _lib.load()
        self.b, self.nt, self.a = int(b), int(nt), int(a)
        h = ctypes.c_void_p()
        _lib.check(self.lib.gbta_create(self.b, self.nt, self.a, ctypes.byref(h)))
        self.ptr = h
        _lib.check(self.lib.gbta_set_twist(self.ptr, 1 if twist else 0))
        self.twist = bool(twist)

    @classmethod
    def get(cls, b: int, nt: int, a: int, twist: bool = True) -> "BtaHandle":
        import torch

        key = (int(b), int(nt), int(a), bool(twist), torch.cuda.current_device())
        with _hlock:
            h = _handles.get(key)
            if h is None:
                h = cls(b, nt, a, twist)
                _handles[key] = h
            return h

    def set_stream(self, stream_ptr: int | None) -> None:
        _lib.check(self.lib.gbta_set_stream(self.ptr, stream_ptr))

    def set_method(self, method: int) -> None:
        """GBTA_METHOD_FP64 (0) or GBTA_METHOD_OZAKI (1, default): how the
        factorization computes its tile products."""
        _lib.check(self.lib.gbta_set_method(self.ptr, int(method)))

    def set_ctas_per_sm(self, n: int) -> None:
        """Persistent CTAs per SM of the dataflow launches (0: as many as fit)."""
        _lib.check(self.lib.gbta_set_ctas_per_sm(self.ptr, int(n)))

    def set_selinv_overlap(self, enable: bool) -> None:
        """Run a (tensor-core) selected inversion that follows this handle's
        factorization concurrently with the sweeps enqueued in between, into a
        workspace of the size of the blocks (gbta_set_selinv_overlap)."""
        _lib.check(self.lib.gbta_set_selinv_overlap(self.ptr, 1 if enable else 0))

    def method(self) -> int:
        return int(self.lib.gbta_get_method(self.ptr))

    def set_wait_limit_ms(self, ms: float) -> None:
        _lib.check(self.lib.gbta_set_wait_limit_ms(self.ptr, float(ms)))

    def workspace_bytes(self) -> int:
        return int(self.lib.gbta_workspace_bytes(self.ptr))

    def status(self) -> int:
        return _lib.check(self.lib.gbta_status(self.ptr))

    def close(self) -> None:
        if self.ptr:
            self.lib.gbta_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
