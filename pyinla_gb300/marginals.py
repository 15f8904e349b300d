"""Marginal variances of the latent field and of the observations, on the device.

After an INLA run the reference returns diag(Sigma) and diag(A Sigma A^T)
(src/pyinla/core/pyinla.py:303-311) through ``PyINLA.get_marginal_variances_latent_parameters``
(pyinla.py:940-964) and ``PyINLA.get_marginal_variances_observations`` (pyinla.py:966-1018).
Both re-factor Q_cond at (theta, x*), run the selected inversion, map Sigma onto a
sparse pattern on the host and, for the observations, form the dense product
``a @ Sigma @ a.T`` to take its diagonal.  Here the two diagonals are read straight
from the Sigma blocks in GB300 memory (``gbta_sigma_diagonal``, ``gbta_obs_variances``):

* :func:`latent_variances` / :func:`observation_variances` work on any Sigma blocks
  (torch CUDA tensors in the Serinv layout);
* :func:`solver_latent_variances` / :func:`solver_observation_variances` read a
  :class:`~pyinla_gb300.solver.GB300SerinvSolver` after ``selected_inversion("bta")``;
* :func:`get_marginal_variances_latent_parameters` and
  :func:`get_marginal_variances_observations` are drop-ins for the two ``PyINLA``
  methods (same arguments, same errors); :func:`install` puts them on the class.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sps

from . import _lib
from .device import current_stream_ptr, require_torch_cuda


class DeviceCSR:
    """A SciPy sparse matrix as device CSR arrays (int64 row pointers, int32 columns)."""

    def __init__(self, A):
        torch = require_torch_cuda()
        A = sps.csr_matrix(A)
        A.sum_duplicates()
        if A.shape[1] >= 2 ** 31:
            raise ValueError("observation matrix has too many columns for int32 indices")
        self.shape = A.shape
        self.rowptr = torch.from_numpy(A.indptr.astype(np.int64)).cuda()
        self.col = torch.from_numpy(A.indices.astype(np.int32)).cuda()
        self.val = torch.from_numpy(np.ascontiguousarray(A.data, dtype=np.float64)).cuda()


def _ptr(t):
    return None if t is None else t.data_ptr()


def _blocks_ok(SD, SL, SR, ST, b, nt, a):
    torch = require_torch_cuda()
    for name, t, shape in (("SD", SD, (nt, b, b)), ("SL", SL if nt > 1 else None, (nt - 1, b, b)),
                           ("SR", SR if a > 0 else None, (nt, a, b)), ("ST", ST if a > 0 else None, (a, a))):
        if t is None:
            if name == "SD" or (name == "SL" and nt > 1) or (name in ("SR", "ST") and a > 0):
                raise ValueError(f"{name} is required")
            continue
        if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous()):
            raise ValueError(f"{name} must be a contiguous float64 CUDA tensor")
        if t.numel() < int(np.prod(shape)):
            raise ValueError(f"{name} holds {t.numel()} elements, expected {shape}")


def latent_variances(h, SD, ST=None):
    """diag(Sigma) (length nt*b + a, latent order) as a CUDA tensor, from the blocks of
    the handle's geometry ``h`` (a :class:`~pyinla_gb300.device.BtaHandle`)."""
    torch = require_torch_cuda()
    b, nt, a = h.b, h.nt, h.a
    for name, t, n in (("SD", SD, nt * b * b), ("ST", ST if a > 0 else None, a * a)):
        if n == 0:
            continue
        if t is None:
            raise ValueError(f"{name} is required")
        if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous() and t.numel() >= n):
            raise ValueError(f"{name} must be a contiguous float64 CUDA tensor of {n} elements")
    out = torch.empty(nt * b + a, dtype=torch.float64, device=SD.device)
    h.set_stream(current_stream_ptr())
    _lib.check(h.lib.gbta_sigma_diagonal(h.ptr, SD.data_ptr(), _ptr(ST) if a > 0 else None, out.data_ptr()))
    return out


def observation_variances(h, A, SD, SL, SR=None, ST=None):
    """diag(A Sigma A^T) as a CUDA tensor; ``A`` a SciPy matrix or a :class:`DeviceCSR`
    with columns in latent order."""
    torch = require_torch_cuda()
    b, nt, a = h.b, h.nt, h.a
    dA = A if isinstance(A, DeviceCSR) else DeviceCSR(A)
    if dA.shape[1] != nt * b + a:
        raise ValueError(f"A has {dA.shape[1]} columns, expected {nt * b + a}")
    _blocks_ok(SD, SL, SR, ST, b, nt, a)
    out = torch.empty(dA.shape[0], dtype=torch.float64, device=SD.device)
    h.set_stream(current_stream_ptr())
    _lib.check(h.lib.gbta_obs_variances(h.ptr, int(dA.shape[0]), dA.rowptr.data_ptr(), dA.col.data_ptr(),
                                        dA.val.data_ptr(), SD.data_ptr(), _ptr(SL) if nt > 1 else None,
                                        _ptr(SR) if a > 0 else None, _ptr(ST) if a > 0 else None,
                                        out.data_ptr()))
    return out


def _solver_blocks(solver):
    return (solver.A_diagonal_blocks, solver.A_lower_diagonal_blocks if solver.n_diag_blocks > 1 else None,
            solver.A_arrow_bottom_blocks, solver.A_arrow_tip_block)


def solver_latent_variances(solver) -> np.ndarray:
    """diag(Sigma) of a GB300SerinvSolver whose blocks hold the selected inverse."""
    SD, _, _, ST = _solver_blocks(solver)
    return latent_variances(solver._h, SD, ST).cpu().numpy()


def solver_observation_variances(solver, A) -> np.ndarray:
    """diag(A Sigma A^T) of a GB300SerinvSolver whose blocks hold the selected inverse."""
    SD, SL, SR, ST = _solver_blocks(solver)
    return observation_variances(solver._h, A, SD, SL, SR, ST).cpu().numpy()


def _require_gb300_solver(solver):
    from .solver import GB300SerinvSolver
    if not isinstance(solver, GB300SerinvSolver):
        raise TypeError("the device marginal variances need PyINLA.solver to be a GB300SerinvSolver")


def _theta_x(self, theta, x_star):
    # pyinla.py:943-953 / 990-1001
    if theta is None and x_star is None:
        return self.model.theta, self.model.x
    if theta is None or x_star is None:
        raise ValueError("BOTH or NEITHER theta and x_star must be provided to compute the marginal variances.")
    return theta, x_star


def get_marginal_variances_latent_parameters(self, theta=None, x_star=None) -> np.ndarray:
    """Drop-in for ``PyINLA.get_marginal_variances_latent_parameters`` (pyinla.py:940-964)."""
    theta, x_star = _theta_x(self, theta, x_star)
    _require_gb300_solver(self.solver)
    self._compute_covariance_latent_parameters(theta, x_star)
    return solver_latent_variances(self.solver)


def get_marginal_variances_observations(self, theta, x_star) -> np.ndarray:
    """Drop-in for ``PyINLA.get_marginal_variances_observations`` (pyinla.py:966-1018)."""
    if not self.model.is_likelihood_gaussian():
        raise NotImplementedError(
            "in compute marginals observations: Only Gaussian likelihood is currently supported.")
    theta, x_star = _theta_x(self, theta, x_star)
    _require_gb300_solver(self.solver)
    self._compute_covariance_latent_parameters(theta, x_star)
    return solver_observation_variances(self.solver, self.model.a)


def install(pyinla_cls) -> None:
    """Replace the two methods on the reference's ``PyINLA`` class (or a subclass)."""
    pyinla_cls.get_marginal_variances_latent_parameters = get_marginal_variances_latent_parameters
    pyinla_cls.get_marginal_variances_observations = get_marginal_variances_observations
