"""Laplace-approximation objective for non-Gaussian likelihoods (Poisson, Binomial).

For a likelihood that is not Gaussian the reference finds the latent mode x* of every
objective evaluation with a Newton iteration (PyINLA._inner_iteration,
src/pyinla/core/pyinla.py:1025-1074) -- repeat x += dx; eta = A x;
Q_cond = Q_prior + A^T W(eta) A (W = -diag l''(eta), model.py:384-423);
rhs = -Q_prior x + A^T l'(eta) (model.py:425-449); dx = Q_cond^{-1} rhs -- until
|dx| < eps_inner_iteration, and then evaluates (pyinla.py:692-729)

    f(theta) = -(log pi(theta) + l(eta) + 1/2 logdet Q_prior - 1/2 x^T Q_prior x
                 - 1/2 logdet Q_cond).

:class:`KronLaplaceModel` runs all of it on the device for the Kronecker-sum models of
:mod:`pyinla_gb300.model`: each Newton step forms the weights W(eta) and the gradient
l'(eta) element-wise, the entries of A^T W A with ``gbta_weighted_gram`` (fixed-order
sums over precomputed (observation, A_rp A_rq) lists), assembles Q_cond straight into
the BTA blocks (``gbta_assemble_kron``), forms Q_prior x with ``gbta_bta_symv`` on the
unfactored prior blocks, and factors and solves with ``gbta_pobtaf`` / ``gbta_pobtas``.
As in the reference the mode is kept between evaluations and warm-starts the next one.

The likelihoods follow src/pyinla/likelihoods/poisson.py (l = eta.y - sum e exp(eta))
and binomial.py (sigmoid link, l = y.log s + (n - y).log(1 - s)); their defaults are
e = 1 and n = 1.  Two defects of the reference's path are not reproduced: its inner
iteration calls ``solver.cholesky`` without the sparsity argument (pyinla.py:1060), and
its conditional term indexes a missing mean (pyinla.py:1155); here Q_cond is factored
as "bta" and the conditional term is its value at the mean, 1/2 logdet Q_cond.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sps

from . import _lib
from .device import current_stream_ptr
from .model import KronGaussianModel, KronSpec

LIKELIHOODS = ("poisson", "binomial")


class KronLaplaceModel(KronGaussianModel):
    """Device-resident Laplace objective of a univariate :class:`KronSpec` whose ``y``
    holds counts; ``likelihood`` is "poisson" (``e``: exposures) or "binomial"
    (``n_trials``).  Only f(theta) is provided (the reference differentiates it by
    central differences, PyINLA._objective_function, pyinla.py:512-600)."""

    def __init__(self, spec: KronSpec, likelihood: str, e=None, n_trials=None, eps_inner: float = 1e-3,
                 max_iter: int = 50):
        if likelihood not in LIKELIHOODS:
            raise ValueError(f"likelihood must be one of {LIKELIHOODS}")
        if int(spec.nv) != 1:
            raise ValueError("the Laplace objective supports univariate models")
        super().__init__(spec)
        torch = self.torch
        self.likelihood = likelihood
        self.eps_inner = float(eps_inner)
        self.max_iter = int(max_iter)
        n = self.n_obs
        dev = "cuda"
        f64 = torch.float64
        self._y = torch.from_numpy(np.asarray(spec.y, dtype=np.float64)).to(dev)
        aux = e if likelihood == "poisson" else n_trials
        aux = np.ones(n) if aux is None else np.asarray(aux, dtype=np.float64).reshape(n)
        self._aux = torch.from_numpy(aux).to(dev)
        A = sps.csr_matrix(spec.A, dtype=np.float64)
        A.sum_duplicates()
        A.sort_indices()
        At = A.T.tocsr()
        self._A = torch.sparse_csr_tensor(torch.from_numpy(A.indptr.astype(np.int64)),
                                          torch.from_numpy(A.indices.astype(np.int64)),
                                          torch.from_numpy(A.data), size=A.shape, dtype=f64).to(dev)
        self._At = torch.sparse_csr_tensor(torch.from_numpy(At.indptr.astype(np.int64)),
                                           torch.from_numpy(At.indices.astype(np.int64)),
                                           torch.from_numpy(At.data), size=At.shape, dtype=f64).to(dev)
        self._build_pairs(A)
        self._ones = torch.ones(self.nv, dtype=f64, device=dev)
        self.x_latent = torch.zeros(self.N, dtype=f64, device=dev)
        self.last_iterations = 0

    # ------------------------------------------------------------ A^T W A pairs
    def _build_pairs(self, A: sps.csr_matrix):
        """Per output entry of A^T W A (the assembly's diagonal-block CSR entries, then
        the dense arrow rows R (nt, nb, b), then the tip (nb, nb)), the list of
        (observation, A_rp A_rq) pairs, sorted by entry."""
        torch = self.torch
        b, nt, nb = self.b, self.nt, self.nb
        nbk = nt * b
        rowptr = self._lik_rowptr.cpu().numpy()
        col = self._lik_col.cpu().numpy().astype(np.int64)
        nnz_d = col.size
        keys_d = np.repeat(np.arange(nbk, dtype=np.int64), np.diff(rowptr)) * b + col
        m = np.diff(A.indptr).astype(np.int64)
        tot = m * m
        npair = int(tot.sum())
        row_of = np.repeat(np.arange(A.shape[0], dtype=np.int64), tot)
        off = np.arange(npair, dtype=np.int64) - np.repeat(np.cumsum(tot) - tot, tot)
        mm = np.repeat(m, tot)
        st = np.repeat(A.indptr[:-1].astype(np.int64), tot)
        ia, ib = st + off // mm, st + off % mm
        p, q = A.indices[ia].astype(np.int64), A.indices[ib].astype(np.int64)
        cv = A.data[ia] * A.data[ib]
        out = np.full(npair, -1, dtype=np.int64)
        dd = (p < nbk) & (q < nbk)
        if np.any(dd & ((p // b) != (q // b))):
            raise ValueError("A^T A couples different time blocks: each observation must touch one time step")
        kq = p[dd] * b + (q[dd] % b)
        pos = np.searchsorted(keys_d, kq)
        if np.any(pos >= nnz_d) or np.any(keys_d[np.minimum(pos, nnz_d - 1)] != kq):
            raise ValueError("an A^T A entry is missing from the assembly pattern")
        out[dd] = pos
        rr = (p >= nbk) & (q < nbk)
        out[rr] = nnz_d + ((q[rr] // b) * nb + (p[rr] - nbk)) * b + (q[rr] % b)
        tt = (p >= nbk) & (q >= nbk)
        out[tt] = nnz_d + nt * nb * b + (p[tt] - nbk) * nb + (q[tt] - nbk)
        keep = out >= 0
        out, row_of, cv = out[keep], row_of[keep], cv[keep]
        order = np.argsort(out, kind="stable")
        n_out = nnz_d + nt * nb * b + nb * nb
        seg = np.zeros(n_out + 1, dtype=np.int64)
        np.cumsum(np.bincount(out, minlength=n_out), out=seg[1:])
        dev = "cuda"
        self._wseg = torch.from_numpy(seg).to(dev)
        self._wobs = torch.from_numpy(row_of[order].astype(np.int32)).to(dev)
        self._wcoef = torch.from_numpy(np.ascontiguousarray(cv[order])).to(dev)
        self._wout = torch.zeros(n_out, dtype=torch.float64, device=dev)
        self._n_out, self._nnz_d = n_out, nnz_d

    # ------------------------------------------------------------ pieces
    def _likelihood(self, eta):
        """(l(eta), l'(eta), -l''(eta)) on the device."""
        torch = self.torch
        y, aux = self._y, self._aux
        if self.likelihood == "poisson":
            ee = aux * torch.exp(eta)
            return torch.dot(eta, y) - torch.sum(ee), y - ee, ee
        s = torch.sigmoid(eta)
        lik = torch.dot(y, torch.log(s)) + torch.dot(aux - y, torch.log(1.0 - s))
        return lik, y - aux * s, aux * s * (1.0 - s)

    def _spmv(self, M, v):
        return (M @ v.unsqueeze(1)).squeeze(1)

    def _assemble_cond(self, coef_ptrs):
        alpha_p, beta_p, _ = coef_ptrs
        lib, h = self.h.lib, self.h
        w0 = self._wout.data_ptr()
        has_arrow = self.nb > 0
        _lib.check(lib.gbta_assemble_kron(
            h.ptr, self.ns, self.nv, self.K, self._upat_rowptr.data_ptr(), self._upat_col.data_ptr(),
            self._uval.data_ptr(), self._term_vw.data_ptr(), alpha_p, beta_p, self._lik_rowptr.data_ptr(),
            self._lik_col.data_ptr(), w0, w0 + 8 * self._nnz_d if has_arrow else None,
            w0 + 8 * (self._nnz_d + self.nt * self.nb * self.b) if has_arrow else None, self._ones.data_ptr(),
            self._ptr(self._arrow_var), self.tip_prec, self.Dc.data_ptr(), self.Lc.data_ptr(), self.Rc.data_ptr(),
            self.Tc.data_ptr()))

    # ------------------------------------------------------------ public
    def evaluate(self, theta, gradient: bool = False):
        """f(theta) of the Laplace approximation (the mode from the previous call starts
        the inner iteration)."""
        if gradient:
            raise NotImplementedError("the Laplace objective has no adjoint gradient; difference f")
        torch = self.torch
        theta = np.asarray(theta, dtype=np.float64)
        h = self.h
        h.set_stream(current_stream_ptr())
        lib = h.lib
        has_arrow = self.nb > 0
        ptrs = self._upload_coef(self.coefficients(theta))
        self._assemble(ptrs, self.Dp, self.Lp, self.Rp, self.Tp, with_lik=False)
        R, T = (self.Rc.data_ptr(), self.Tc.data_ptr()) if has_arrow else (None, None)
        Rp, Tp = (self.Rp.data_ptr(), self.Tp.data_ptr()) if has_arrow else (None, None)
        x = self.x_latent.clone()
        dx = torch.zeros_like(x)
        qpx = torch.empty_like(x)
        it = 0
        while True:
            if it > self.max_iter:
                raise ValueError(f"Inner iteration did not converge after {it} iterations.")
            x += dx
            eta = self._spmv(self._A, x)
            lik, grad, w = self._likelihood(eta)
            _lib.check(lib.gbta_weighted_gram(h.ptr, self._n_out, self._wseg.data_ptr(), self._wobs.data_ptr(),
                                              self._wcoef.data_ptr(), w.data_ptr(), self._wout.data_ptr()))
            self._assemble_cond(ptrs)
            _lib.check(lib.gbta_bta_symv(h.ptr, self.Dp.data_ptr(), self.Lp.data_ptr(), Rp, Tp,
                                         1 if has_arrow else 0, x.data_ptr(), qpx.data_ptr()))
            dx = self._spmv(self._At, grad) - qpx
            _lib.check(lib.gbta_pobtaf_async(h.ptr, self.Dc.data_ptr(), self.Lc.data_ptr(), R, T))
            _lib.check(lib.gbta_pobtas(h.ptr, self.Dc.data_ptr(), self.Lc.data_ptr(), R, T, dx.data_ptr(), 1, 2))
            it += 1
            if float(torch.linalg.vector_norm(dx)) < self.eps_inner:
                break
        self.last_iterations = it
        logdet_c = self._logdet(self.Dc, self.Tc, with_tip=has_arrow)
        xqx = float(torch.dot(x, qpx))
        logdet_p = self._prior_logdet(theta, ptrs)
        self.x_latent = x
        lik = float(lik)
        lp = self.log_prior(theta)
        f = -(lp + lik + 0.5 * logdet_p - 0.5 * xqx - 0.5 * logdet_c)
        self.last = dict(logdet_prior=logdet_p, logdet_cond=logdet_c, quad_prior=xqx, lik=lik, log_prior=lp,
                         iterations=it)
        return f
