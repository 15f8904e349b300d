"""Many BTA instances in one persistent launch per phase (``gbta_batch_*`` of the C ABI).

The instances of a theta-gradient's central-difference points, a Hessian or a theta
grid -- the Q(theta) the reference factors one after the other
(src/pyinla/core/pyinla.py:512-600, 747-910) -- are held side by side, each in the
Serinv block layout, and every phase (factor, logdet, solve N then C, selected
inversion) of all of them runs as one persistent kernel whose ticket order merges
the instances' task lists.  A run can be captured once into a CUDA graph and
replayed, so a whole sweep is one graph launch.

Per instance the results are those of ``pobtaf`` / ``logdet`` / ``pobtas`` /
``pobtasi`` with the same product method (bit for bit: the same task bodies run).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .device import require_torch_cuda

ORDERS = {"proportional": _lib.GBTA_BATCH_ORDER_PROPORTIONAL, "round_robin": _lib.GBTA_BATCH_ORDER_ROUND_ROBIN,
          "sequential": _lib.GBTA_BATCH_ORDER_SEQUENTIAL}


def _ptr_array(ptrs):
    arr = (ctypes.c_void_p * len(ptrs))()
    for i, p in enumerate(ptrs):
        arr[i] = p
    return arr


class BtaBatch:
    """n BTA instances of shapes ``[(b, nt, a), ...]`` with device-resident blocks.

    ``D[k]`` (nt, b, b), ``L[k]`` (max(nt-1, 1), b, b), ``R[k]`` (nt, a, b), ``T[k]``
    (a, a) and ``rhs[k]`` (nt*b + a,) are torch CUDA tensors owned by the batch (their
    addresses are bound once, so captured graphs stay valid); fill them, then call
    :meth:`run`.  ``methods`` gives each instance's product method
    (``_lib.GBTA_METHOD_FP64`` / ``_lib.GBTA_METHOD_OZAKI``, default Ozaki).
    """

    def __init__(self, shapes, methods=None, order: str = "proportional"):
        torch = require_torch_cuda()
        self.torch = torch
        self.lib = _lib.load()
        self.shapes = [(int(b), int(nt), int(a)) for (b, nt, a) in shapes]
        n = self.n = len(self.shapes)
        if n < 1:
            raise ValueError("a batch needs at least one instance")
        self.methods = [(_lib.GBTA_METHOD_OZAKI if methods is None else int(methods[k])) for k in range(n)]
        bs = (ctypes.c_int * n)(*[s[0] for s in self.shapes])
        nts = (ctypes.c_int * n)(*[s[1] for s in self.shapes])
        as_ = (ctypes.c_int * n)(*[s[2] for s in self.shapes])
        ms = (ctypes.c_int * n)(*self.methods)
        h = ctypes.c_void_p()
        _lib.check(self.lib.gbta_batch_create(n, bs, nts, as_, ms, ctypes.byref(h)))
        self.ptr = h
        f64 = torch.float64
        self.D, self.L, self.R, self.T, self.rhs = [], [], [], [], []
        for (b, nt, a) in self.shapes:
            self.D.append(torch.zeros((nt, b, b), dtype=f64, device="cuda"))
            self.L.append(torch.zeros((max(nt - 1, 1), b, b), dtype=f64, device="cuda"))
            self.R.append(torch.zeros((nt, max(a, 1), b), dtype=f64, device="cuda"))
            self.T.append(torch.zeros((max(a, 1), max(a, 1)), dtype=f64, device="cuda"))
            self.rhs.append(torch.zeros(nt * b + a, dtype=f64, device="cuda"))
        self.logdet = torch.zeros(n, dtype=f64, device="cuda")
        # the batch works on its own stream, ordered after / before the caller's stream
        # by stream waits (a graph cannot be captured on the legacy default stream)
        self.stream = torch.cuda.Stream()
        _lib.check(self.lib.gbta_batch_set_stream(self.ptr, self.stream.cuda_stream))
        _lib.check(self.lib.gbta_batch_bind(
            self.ptr, _ptr_array([t.data_ptr() for t in self.D]), _ptr_array([t.data_ptr() for t in self.L]),
            _ptr_array([t.data_ptr() for t in self.R]), _ptr_array([t.data_ptr() for t in self.T]),
            _ptr_array([t.data_ptr() for t in self.rhs])))
        self.ctas_per_sm = 0
        self.set_order(order)

    # ------------------------------------------------------------------ settings
    def set_order(self, order: str) -> None:
        if order not in ORDERS:
            raise ValueError(f"unknown order {order!r}; one of {sorted(ORDERS)}")
        _lib.check(self.lib.gbta_batch_set_order(self.ptr, ORDERS[order]))
        self.order = order

    def set_ctas_per_sm(self, n: int) -> None:
        """Persistent CTAs per SM of the batch's launches (0: as many as fit)."""
        _lib.check(self.lib.gbta_batch_set_ctas_per_sm(self.ptr, int(n)))
        self.ctas_per_sm = int(n)

    def set_wait_limit_ms(self, ms: float) -> None:
        _lib.check(self.lib.gbta_batch_set_wait_limit_ms(self.ptr, float(ms)))

    def workspace_bytes(self) -> int:
        return int(self.lib.gbta_batch_workspace_bytes(self.ptr))

    def graph_kernels(self) -> int:
        return int(self.lib.gbta_batch_graph_kernels(self.ptr))

    # ------------------------------------------------------------------ data
    def load(self, k: int, D, L, R=None, T=None, rhs=None) -> None:
        """Copy instance k's blocks (numpy or torch, Serinv layout) into the batch."""
        torch = self.torch
        b, nt, a = self.shapes[k]

        def put(dst, src):
            src = torch.as_tensor(src, dtype=torch.float64)
            dst.copy_(src.reshape(dst.shape))

        put(self.D[k], D)
        if nt > 1:
            put(self.L[k][: nt - 1], L)
        if a > 0:
            put(self.R[k], R)
            put(self.T[k], T)
        if rhs is not None:
            put(self.rhs[k], rhs)

    # ------------------------------------------------------------------ runs
    def run_async(self, phases: int = _lib.GBTA_PHASE_ALL, graph: bool = True) -> None:
        """Enqueue the phases of every instance (on the batch's stream); with
        ``graph`` the sequence is captured once and replayed as one graph launch."""
        torch = self.torch
        fn = self.lib.gbta_batch_graph_launch if graph else self.lib.gbta_batch_run_async
        caller = torch.cuda.current_stream()
        self.stream.wait_stream(caller)
        _lib.check(fn(self.ptr, int(phases), self.logdet.data_ptr()))
        caller.wait_stream(self.stream)

    def status(self) -> np.ndarray:
        """Wait; raise on a timeout or a failed pivot; return every instance's info."""
        info = (ctypes.c_int * self.n)()
        code = self.lib.gbta_batch_status(self.ptr, info)
        _lib.check(code)
        return np.frombuffer(info, dtype=np.int32).copy()

    def run(self, phases: int = _lib.GBTA_PHASE_ALL, graph: bool = True) -> np.ndarray:
        """Run and wait; returns the logdets (when the logdet phase ran)."""
        self.run_async(phases, graph)
        self.status()
        return self.logdet.cpu().numpy()

    def close(self) -> None:
        if getattr(self, "ptr", None):
            self.lib.gbta_batch_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
