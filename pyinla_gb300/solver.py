"""``GB300SerinvSolver``: drop-in for the reference's ``SerinvSolver``.

Mirrors src/pyinla/solvers/structured_solver.py:19-550 method for method --
``cholesky``, ``solve``, ``logdet``, ``selected_inversion``,
``_structured_to_spmatrix``, ``get_solver_memory`` and the ``t_cholesky`` /
``t_solve`` timers that ``PyINLA`` resets and reads (src/pyinla/core/pyinla.py:216-217,
531-532, 588) -- with the block buffers resident in GB300 memory as torch float64
tensors and every step (sparse-to-BTA scatter, factorization, sweeps, logdet,
selected inversion, pattern gather) running in libpyinla_gb300.so.

It does not import pyinla.  To use it inside the reference, replace the class the
driver instantiates (``pyinla.core.pyinla.SerinvSolver``) with this one, or inject
:mod:`pyinla_gb300.algs` as ``serinv.algs`` (``sys.modules["serinv.algs"]``) before the
reference's solver module is imported.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np
import scipy.sparse as sps

from . import _lib
from .device import BtaHandle, current_stream_ptr, require_torch_cuda


class GB300SerinvSolver:
    """BTA solver on one GB300 (reference: ``SerinvSolver``, structured_solver.py:19)."""

    def __init__(self, config=None, diagonal_blocksize: int = None, n_diag_blocks: int = None,
                 arrowhead_blocksize: int = 0, **kwargs) -> None:
        torch = require_torch_cuda()
        self.config = config
        self.diagonal_blocksize = int(diagonal_blocksize)
        self.arrowhead_blocksize = int(arrowhead_blocksize)
        self.n_diag_blocks = int(n_diag_blocks)
        b, nt, a = self.diagonal_blocksize, self.n_diag_blocks, self.arrowhead_blocksize
        dev = torch.device("cuda", torch.cuda.current_device())
        f64 = torch.float64
        # structured_solver.py:37-61
        self.A_diagonal_blocks = torch.empty((nt, b, b), dtype=f64, device=dev)
        self.A_lower_diagonal_blocks = torch.empty((max(nt - 1, 0), b, b), dtype=f64, device=dev)
        self.A_arrow_bottom_blocks = torch.empty((nt, a, b), dtype=f64, device=dev) if a > 0 else None
        self.A_arrow_tip_block = torch.empty((a, a), dtype=f64, device=dev) if a > 0 else None
        self._h = BtaHandle.get(b, nt, a)
        # selected_inversion follows cholesky and solve (structured_solver.py's order): it
        # runs next to the sweeps
        self._h.set_selinv_overlap(True)
        self._torch = torch
        # index structures derived from the sparsity pattern of the matrices passed in
        # (the same at every theta): input scatter indices, output gather indices and
        # the permutation that yields the CSC data of the symmetric result
        self._in_cache = None
        self._out_cache = {}
        self._pinned = {}
        self.total_bytes = 0
        self.t_cholesky = 0.0
        self.t_solve = 0.0

    # ------------------------------------------------------------------ helpers
    def _ptrs(self, sparsity: str):
        D = self.A_diagonal_blocks.data_ptr()
        L = self.A_lower_diagonal_blocks.data_ptr() if self.n_diag_blocks > 1 else None
        if sparsity == "bta" and self.arrowhead_blocksize > 0:
            return D, L, self.A_arrow_bottom_blocks.data_ptr(), self.A_arrow_tip_block.data_ptr()
        return D, L, None, None

    @staticmethod
    def _check_sparsity(sparsity: str) -> None:
        if sparsity not in ("bt", "bta"):
            raise ValueError(f"Unknown sparsity pattern: {sparsity}. Use 'bt' or 'bta'.")

    def _sync(self) -> None:
        self._torch.cuda.current_stream().synchronize()

    # ------------------------------------------------------------------ API
    def cholesky(self, A, sparsity: str) -> None:
        """Map the sparse matrix into BTA blocks and factor it (structured_solver.py:72-100).

        For a CSR / CSC matrix whose format, shape and sizes match the pattern seen
        before, the scatter and the factorization are queued with that pattern's
        indices first and the full comparison of the index arrays runs on the host
        while the device works; on a mismatch both are redone with the new pattern."""
        self._check_sparsity(sparsity)
        tic = time.perf_counter()
        h = self._h
        h.set_stream(current_stream_ptr())
        verify = self._spmatrix_to_structured(A, sparsity, verify_later=True)
        self._factor_async(sparsity)
        if verify is not None and not self._same_pattern(A, verify):
            h.lib.gbta_status(h.ptr)   # drain the queued work; its result is discarded
            self._in_cache = None
            self._spmatrix_to_structured(A, sparsity)
            self._factor_async(sparsity)
        h.status()
        self.t_cholesky += time.perf_counter() - tic

    def _factor_async(self, sparsity: str) -> None:
        h = self._h
        D, L, R, T = self._ptrs(sparsity)
        if sparsity == "bta" and self.arrowhead_blocksize > 0:
            _lib.check(h.lib.gbta_pobtaf_async(h.ptr, D, L, R, T))
        else:
            _lib.check(h.lib.gbta_pobtf_async(h.ptr, D, L))

    def solve(self, rhs, sparsity: str):
        """Forward then backward sweep, overwriting and returning ``rhs``
        (structured_solver.py:102-149)."""
        self._check_sparsity(sparsity)
        torch = self._torch
        tic = time.perf_counter()
        self._sync()
        on_dev = isinstance(rhs, torch.Tensor) and rhs.device.type == "cuda"
        nb = self.n_diag_blocks * self.diagonal_blocksize
        n = nb + (self.arrowhead_blocksize if sparsity == "bta" else 0)
        if on_dev:
            x = rhs[:n] if rhs.is_contiguous() else rhs[:n].contiguous()
        else:
            x = torch.from_numpy(np.ascontiguousarray(np.asarray(rhs, dtype=np.float64)[:n])).cuda()
        nrhs = 1 if x.ndim == 1 else int(np.prod(x.shape[1:]))
        h = self._h
        h.set_stream(current_stream_ptr())
        D, L, R, T = self._ptrs(sparsity)
        if R is not None:
            _lib.check(h.lib.gbta_pobtas(h.ptr, D, L, R, T, x.data_ptr(), nrhs, 2))   # N then C, one launch
        else:
            _lib.check(h.lib.gbta_pobts(h.ptr, D, L, x.data_ptr(), nrhs, 2))
        if on_dev:
            if x.data_ptr() != rhs.data_ptr():
                rhs[:n].copy_(x)
        else:
            rhs[:n] = x.cpu().numpy()
        self._sync()
        self.t_solve += time.perf_counter() - tic
        return rhs

    def logdet(self, sparsity: str) -> float:
        """2 * sum(log diag) of the factor; "bt" excludes the tip (structured_solver.py:151-166)."""
        self._check_sparsity(sparsity)
        h = self._h
        h.set_stream(current_stream_ptr())
        D, _, _, T = self._ptrs(sparsity)
        out = ctypes.c_double(0.0)
        code = h.lib.gbta_logdet(h.ptr, D, T, 1 if T is not None else 0, ctypes.byref(out))
        if code == _lib.GBTA_ERR_ARG and np.isnan(out.value):
            raise ValueError("Logdet is NaN. Check the input matrix.")
        _lib.check(code)
        return float(out.value)

    def selected_inversion(self, sparsity: str) -> None:
        """Overwrite the factor blocks with Sigma on the BTA pattern (structured_solver.py:168-190).

        The bta form returns once the work is queued on the current stream (as the
        reference's device backend does): stream-ordered readers of the blocks see
        Sigma, and a failure is raised by the next call that waits for the device
        (``_structured_to_spmatrix``, ``cholesky``, ``solve``, ``logdet``)."""
        self._check_sparsity(sparsity)
        h = self._h
        h.set_stream(current_stream_ptr())
        D, L, R, T = self._ptrs(sparsity)
        if R is not None:
            _lib.check(h.lib.gbta_pobtasi_async(h.ptr, D, L, R, T))
        else:
            _lib.check(h.lib.gbta_pobtsi(h.ptr, D, L))

    def _same_pattern(self, A, key) -> bool:
        """A (CSR or CSC) has the sparsity pattern recorded in key (the index arrays
        compared by torch's multi-threaded CPU kernels where the dtypes agree)."""
        fmt, shape, indptr, indices = key
        if not self._same_shape(A, key):
            return False
        return self._equal(A.indptr, indptr) and self._equal(A.indices, indices)

    def _equal(self, x: np.ndarray, y: np.ndarray) -> bool:
        if x.dtype == y.dtype and x.flags.c_contiguous and y.flags.c_contiguous:
            return bool(self._torch.equal(self._torch.from_numpy(x), self._torch.from_numpy(y)))
        return bool(np.array_equal(x, y))

    def _host_copy(self, x):
        """A fresh host copy (numpy) of a host tensor or array, by torch's multi-threaded copy."""
        t = x if isinstance(x, self._torch.Tensor) else self._torch.from_numpy(x)
        return t.clone().numpy()

    @staticmethod
    def _pattern_key(A):
        return (A.format, A.shape, A.indptr.copy(), A.indices.copy())

    def _to_device(self, x: np.ndarray, slot: str):
        """Host array to a device tensor through a pinned staging buffer kept per slot."""
        torch = self._torch
        src = torch.from_numpy(np.ascontiguousarray(x))
        buf = self._pinned.get(slot)
        if buf is None or buf.numel() < src.numel() or buf.dtype != src.dtype:
            buf = torch.empty(src.numel(), dtype=src.dtype, pin_memory=True)
            self._pinned[slot] = buf
        stage = buf[: src.numel()]
        stage.copy_(src)
        return stage.to("cuda")   # (blocking: the staging buffer is reused by the next call)

    @staticmethod
    def _same_shape(A, key) -> bool:
        """The cheap part of _same_pattern: format, shape and array sizes."""
        fmt, shape, indptr, indices = key
        return A.format == fmt and A.shape == shape and A.indptr.size == indptr.size and A.indices.size == indices.size

    def _spmatrix_to_structured(self, A, sparsity: str, verify_later: bool = False):
        """Zero-fill and scatter the symmetric sparse matrix into the BTA blocks
        (structured_solver.py:192-250) with one device scatter.  For CSR / CSC input
        the scatter indices are kept per sparsity pattern, so a matrix with the
        pattern of an earlier call moves only its values.  With ``verify_later`` a
        matrix whose format, shape and sizes match the kept pattern is scattered with
        it at once and the pattern key is returned: the caller compares the index
        arrays (``_same_pattern``) while the device works.  Returns None otherwise."""
        self._check_sparsity(sparsity)
        torch = self._torch
        verify = None
        if sps.issparse(A) and A.format in ("csr", "csc"):
            if verify_later and self._in_cache is not None and self._same_shape(A, self._in_cache[0]):
                verify = self._in_cache[0]
            elif self._in_cache is None or not self._same_pattern(A, self._in_cache[0]):
                coo = A.tocoo()   # entries in the order of A.data
                rows = torch.from_numpy(coo.row.astype(np.int64)).cuda()
                cols = torch.from_numpy(coo.col.astype(np.int64)).cuda()
                self._in_cache = (self._pattern_key(A), rows, cols)
            _, rows, cols = self._in_cache
            vals = self._to_device(np.asarray(A.data, dtype=np.float64), "in")
            nnz = int(A.data.size)
        else:
            coo = sps.coo_matrix(A)
            rows = torch.from_numpy(coo.row.astype(np.int64)).cuda()
            cols = torch.from_numpy(coo.col.astype(np.int64)).cuda()
            vals = torch.from_numpy(np.ascontiguousarray(coo.data, dtype=np.float64)).cuda()
            nnz = int(coo.nnz)
        h = self._h
        h.set_stream(current_stream_ptr())
        D, L, R, T = self._ptrs("bta")
        _lib.check(h.lib.gbta_scatter_coo(h.ptr, rows.data_ptr(), cols.data_ptr(), vals.data_ptr(), nnz,
                                          D, L, R, T, 1 if R is not None else 0))
        return verify

    def _output_structure(self, A, sparsity: str):
        """Gather indices of the lower BTA pattern of A and the structure of the
        symmetrised result: the result's data is vals[perm] for the gathered vals."""
        torch = self._torch
        Bl = sps.tril(sps.csc_matrix(A)).tocoo()
        b, nt = self.diagonal_blocksize, self.n_diag_blocks
        nb = nt * b
        r, c = Bl.row.astype(np.int64), Bl.col.astype(np.int64)
        in_bt = (r < nb) & (c < nb) & ((r // b == c // b) | (r // b == c // b + 1))
        keep = in_bt | ((r >= nb) if sparsity == "bta" else np.zeros_like(in_bt))
        r, c = r[keep], c[keep]
        # the reference's construction, run once on markers 1..m (exact in float64)
        marks = np.arange(1, r.size + 1, dtype=np.float64)
        out = sps.coo_matrix((marks, (r, c)), shape=Bl.shape).tocsc()
        res = out + sps.tril(out, k=-1).T
        perm = res.data.astype(np.int64) - 1
        return {
            "rows": torch.from_numpy(r).cuda(), "cols": torch.from_numpy(c).cuda(),
            "perm": torch.from_numpy(perm).cuda(), "format": res.format, "shape": res.shape,
            "indices": res.indices.copy(), "indptr": res.indptr.copy(),
        }

    def _structured_to_spmatrix(self, A, sparsity: str):
        """Sigma (or the factor) on the lower pattern of ``A``, symmetrised, as CSC
        (structured_solver.py:470-538).  The index work depends only on the sparsity
        pattern of A and is kept per pattern; each call gathers the values on the
        device, orders them as the result's data and copies them to the host."""
        self._check_sparsity(sparsity)
        torch = self._torch
        A = A if (sps.issparse(A) and A.format in ("csr", "csc")) else sps.csc_matrix(A)
        ent = self._out_cache.get(sparsity)
        if ent is None or not self._same_pattern(A, ent[0]):
            ent = (self._pattern_key(A), self._output_structure(A, sparsity))
            self._out_cache[sparsity] = ent
        st = ent[1]
        rows, cols = st["rows"], st["cols"]
        vals = torch.empty(rows.numel(), dtype=torch.float64, device="cuda")
        h = self._h
        h.set_stream(current_stream_ptr())
        D, L, R, T = self._ptrs(sparsity)
        _lib.check(h.lib.gbta_gather_coo(h.ptr, rows.data_ptr(), cols.data_ptr(), int(rows.numel()), D, L, R, T,
                                         1 if R is not None else 0, vals.data_ptr()))
        data = vals[st["perm"]]
        host = self._pinned.get("out")
        if host is None or host.numel() < data.numel():
            host = torch.empty(data.numel(), dtype=torch.float64, pin_memory=True)
            self._pinned["out"] = host
        host[: data.numel()].copy_(data, non_blocking=True)
        # (while the device works)
        indices, indptr = self._host_copy(st["indices"]), self._host_copy(st["indptr"])
        h.status()   # waits for the copy; raises a failure of the queued work
        cls = sps.csc_matrix if st["format"] == "csc" else sps.csr_matrix
        return cls((self._host_copy(host[: data.numel()]), indices, indptr), shape=st["shape"])

    def get_solver_memory(self) -> int:
        """Bytes of the block buffers plus the library workspace (structured_solver.py:540-550)."""
        n = self.A_diagonal_blocks.nbytes + self.A_lower_diagonal_blocks.nbytes
        if self.A_arrow_bottom_blocks is not None:
            n += self.A_arrow_bottom_blocks.nbytes + self.A_arrow_tip_block.nbytes
        self.total_bytes = n + self._h.workspace_bytes()
        return self.total_bytes
