"""Gaussian spatio-temporal models with a Kronecker-sum prior, evaluated on the GB300.

A model here is the reference's Gaussian-likelihood ``Model`` reduced to what the
BTA path needs (src/pyinla/core/model.py:306-449):

    Q_prior(theta) = sum_k  M_k(theta) (x) S_k   (+ tip_prec * I on the fixed effects)
    Q_cond(theta)  = Q_prior(theta) + tau_y(theta) A^T A
    b(theta)       = tau_y(theta) A^T y

with fixed sparse spatial matrices ``S_k`` and tridiagonal temporal coefficient
matrices ``M_k(theta)`` given by their diagonal ``alpha[k, t]`` and sub-diagonal
``beta[k, t]``.  The objective is the reference's ``_evaluate_f`` for a Gaussian
likelihood evaluated at x = 0 (src/pyinla/core/pyinla.py:602-745, 1076-1167):

    f(theta) = -log pi(theta) - l(y | eta=0) - 1/2 logdet_bt Q_prior
               + 1/2 logdet Q_cond - 1/2 mu^T Q_cond mu,      mu = Q_cond^{-1} b

and its gradient is computed by the adjoint (no counterpart in the reference, which
spends 2 dim(theta) + 1 evaluations on central differences, pyinla.py:512-600):

    df/dtheta = -dlog pi - dl - 1/2 tr(Q_prior^{-1} dQ_prior) + 1/2 tr(Q_cond^{-1} dQ_cond)
                - mu^T db + 1/2 mu^T dQ_cond mu

where the traces only need Q^{-1} on the BTA pattern -- exactly what the selected
inversion produces -- contracted against the sparse dQ blocks on the device.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sps

from . import _lib, spde
from .device import BtaHandle, current_stream_ptr, require_torch_cuda


@dataclass
class Coefficients:
    alpha: np.ndarray        # (K, nt)
    beta: np.ndarray         # (K, nt-1)
    tau_y: np.ndarray        # (nv,) noise precision of each variate's observations

    def __post_init__(self):
        self.tau_y = np.atleast_1d(np.asarray(self.tau_y, dtype=np.float64))


@dataclass
class CoefficientDerivatives:
    dalpha: np.ndarray       # (d, K, nt)
    dbeta: np.ndarray        # (d, K, nt-1)
    dtau_y: np.ndarray       # (d, nv)

    def __post_init__(self):
        dt = np.asarray(self.dtau_y, dtype=np.float64)
        self.dtau_y = dt.reshape(dt.shape[0], -1)


@dataclass
class SeparablePart:
    """One block c * T_AR1(rho) (x) Q_s of a separable prior, Q_s = sum_j w_j S_j over the
    spec's base spatial matrices; derivatives are with respect to theta."""
    c: float
    dlogc: np.ndarray        # (d,)
    rho: float
    drho: np.ndarray         # (d,)
    w: np.ndarray            # (J,)
    dw: np.ndarray           # (d, J)


def union_pattern(mats: list[sps.csr_matrix]):
    """Union CSR pattern of same-shape sparse matrices and each matrix's values on it."""
    n = mats[0].shape[0]
    U = sum(abs(m) for m in mats).tocsr()
    U.sum_duplicates()
    U.sort_indices()
    rowptr = U.indptr.astype(np.int32)
    col = U.indices.astype(np.int32)
    vals = np.zeros((col.size, len(mats)))
    rows = np.repeat(np.arange(n), np.diff(U.indptr))
    for k, m in enumerate(mats):
        mc = m.tocsr()
        mc.sum_duplicates()
        vals[:, k] = np.asarray(mc[rows, col]).ravel()
    return rowptr, col, vals


class KronSpec:
    """Host description of a Kronecker-sum Gaussian model (no device state).

    Subclasses define the theta -> coefficient maps.  Fields: ``terms`` (spatial
    matrices S_k), ``term_vw`` (variate block of each term), ``ns``, ``nv``, ``nt``,
    ``nb``, ``A`` (n_obs x N design matrix, time-major field then fixed effects),
    ``y``, ``tip_prec`` and, for several variates, ``obs_variate`` (variate of each
    observation) and ``arrow_variate`` (variate of each fixed effect); both default
    to variate 0.
    """

    terms: list
    term_vw: list
    ns: int
    nv: int
    nt: int
    nb: int
    A: sps.csr_matrix
    y: np.ndarray
    tip_prec: float

    @property
    def K(self) -> int:
        return len(self.terms)

    @property
    def b(self) -> int:
        return self.ns * self.nv

    @property
    def N(self) -> int:
        return self.nt * self.b + self.nb

    def coefficients(self, theta: np.ndarray) -> Coefficients:
        raise NotImplementedError

    def coefficient_derivatives(self, theta: np.ndarray) -> CoefficientDerivatives:
        raise NotImplementedError

    def log_prior(self, theta: np.ndarray) -> float:
        raise NotImplementedError

    def log_prior_grad(self, theta: np.ndarray) -> np.ndarray:
        raise NotImplementedError

    def lik_theta_indices(self) -> list[int]:
        """Index in theta of theta_y,v = log tau_y,v for each variate v."""
        raise NotImplementedError

    def separable_prior(self, theta):
        """For priors that are, up to a mixing of unit determinant, a block diagonal of
        separable blocks c_k T_AR1(rho_k) (x) Q_s,k: (base spatial matrices S_j, list of
        SeparablePart).  None when the prior has no such structure."""
        return None

    def obs_variates(self) -> np.ndarray:
        v = getattr(self, "obs_variate", None)
        return np.zeros(self.y.shape[0], dtype=np.int64) if v is None else np.asarray(v, dtype=np.int64)

    def arrow_variates(self) -> np.ndarray:
        v = getattr(self, "arrow_variate", None)
        return np.zeros(self.nb, dtype=np.int32) if v is None else np.asarray(v, dtype=np.int32)

    def sparse_precisions(self, theta: np.ndarray):
        """Host sparse (CSR) Q_prior and Q_cond at theta, in the form the reference's
        Model hands to its solver (src/pyinla/core/model.py:306-423): the input of
        the sparse drop-in path (``GB300SerinvSolver.cholesky``)."""
        c = self.coefficients(theta)
        b, nt, ns = self.b, self.nt, self.ns
        N = self.N
        rows, cols, vals = [], [], []
        for k, S in enumerate(self.terms):
            v, w = self.term_vw[k]
            Sc = S.tocoo()
            for t in range(nt):
                rows.append(t * b + v * ns + Sc.row)
                cols.append(t * b + w * ns + Sc.col)
                vals.append(c.alpha[k, t] * Sc.data)
                if t < nt - 1:
                    for (r0, c0) in ((t + 1, t), (t, t + 1)):
                        rows.append(r0 * b + v * ns + Sc.row)
                        cols.append(c0 * b + w * ns + Sc.col)
                        vals.append(c.beta[k, t] * Sc.data)
        if self.nb:
            rows.append(nt * b + np.arange(self.nb))
            cols.append(nt * b + np.arange(self.nb))
            vals.append(np.full(self.nb, self.tip_prec))
        Qp = sps.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))
        Qp.sum_duplicates()
        DA = sps.diags(c.tau_y[self.obs_variates()]) @ self.A
        Qc = (Qp + (self.A.T @ DA)).tocsr()
        Qc.sum_duplicates()
        return Qp, Qc


class KronGaussianModel:
    """Device-resident evaluation of a :class:`KronSpec` model (see module docstring)."""

    def __init__(self, spec: KronSpec):
        torch = require_torch_cuda()
        self.spec = spec
        self.torch = torch
        self.ns, self.nv, self.nt, self.nb = int(spec.ns), int(spec.nv), int(spec.nt), int(spec.nb)
        self.b = self.ns * self.nv
        self.N = self.nt * self.b + self.nb
        self.K = spec.K
        self.tip_prec = float(spec.tip_prec)
        A, y = spec.A, spec.y
        self.n_obs = int(y.shape[0])
        if A.shape != (self.n_obs, self.N):
            raise ValueError(f"A has shape {A.shape}, expected {(self.n_obs, self.N)}")
        if self.nv > _lib.GBTA_MAX_VARIATES:
            raise ValueError(f"at most {_lib.GBTA_MAX_VARIATES} variates")
        ov = spec.obs_variates()
        av = spec.arrow_variates()
        if ov.shape != (self.n_obs,) or (ov.size and (ov.min() < 0 or ov.max() >= self.nv)):
            raise ValueError("obs_variate must give a variate in [0, nv) per observation")
        if av.shape != (self.nb,) or (av.size and (av.min() < 0 or av.max() >= self.nv)):
            raise ValueError("arrow_variate must give a variate in [0, nv) per fixed effect")
        self._check_variate_support(A, ov, av)
        # --- theta-independent device data (built once, like the reference's pattern reuse,
        #     src/pyinla/core/model.py:356-380)
        dev = "cuda"
        rowptr, col, uval = union_pattern(spec.terms)
        self._upat_rowptr = torch.from_numpy(rowptr).to(dev)
        self._upat_col = torch.from_numpy(col).to(dev)
        self._uval = torch.from_numpy(np.ascontiguousarray(uval)).to(dev)
        self._term_vw = torch.from_numpy(np.asarray(spec.term_vw, dtype=np.int32).reshape(-1)).to(dev)
        At = A.T.tocsr()
        AtA = (At @ A).tocsr()
        AtA.sum_duplicates()
        nbk = self.nt * self.b
        # diagonal-block rows of A^T A as CSR with block-local columns
        blk = AtA[:nbk, :nbk].tocoo()
        keep = (blk.row // self.b) == (blk.col // self.b)
        if int(np.count_nonzero(~keep)):
            raise ValueError("A^T A couples different time blocks: each observation must touch one time step")
        D_lik = sps.csr_matrix((blk.data[keep], (blk.row[keep], blk.col[keep] % self.b)), shape=(nbk, self.b))
        D_lik.sum_duplicates()
        D_lik.sort_indices()
        self._lik_rowptr = torch.from_numpy(D_lik.indptr.astype(np.int64)).to(dev)
        self._lik_col = torch.from_numpy(D_lik.indices.astype(np.int32)).to(dev)
        self._lik_val = torch.from_numpy(D_lik.data.astype(np.float64)).to(dev)
        if self.nb > 0:
            Rl = np.asarray(AtA[nbk:, :nbk].todense()).reshape(self.nb, self.nt, self.b).transpose(1, 0, 2)
            Tl = np.asarray(AtA[nbk:, nbk:].todense())
            self._lik_R = torch.from_numpy(np.ascontiguousarray(Rl)).to(dev)
            self._lik_T = torch.from_numpy(np.ascontiguousarray(Tl)).to(dev)
        else:
            self._lik_R = self._lik_T = None
        Aty_v = np.zeros((self.nv, self.N))
        for v in range(self.nv):
            sel = ov == v
            Aty_v[v] = A[sel].T @ y[sel]
        self._Aty_v = torch.from_numpy(Aty_v).to(dev)
        self.yty_v = np.array([float(y[ov == v] @ y[ov == v]) for v in range(self.nv)])
        self.nobs_v = np.array([int(np.count_nonzero(ov == v)) for v in range(self.nv)])
        self._arrow_var = torch.from_numpy(np.ascontiguousarray(av, dtype=np.int32)).to(dev) if self.nb else None
        # --- block buffers: conditional (bta) and prior (bt) precisions
        f64 = torch.float64
        b, nt, a = self.b, self.nt, self.nb
        self.Dc = torch.empty((nt, b, b), dtype=f64, device=dev)
        self.Lc = torch.empty((max(nt - 1, 1), b, b), dtype=f64, device=dev)
        self.Rc = torch.empty((nt, max(a, 1), b), dtype=f64, device=dev)
        self.Tc = torch.empty((max(a, 1), max(a, 1)), dtype=f64, device=dev)
        self.Dp = torch.empty_like(self.Dc)
        self.Lp = torch.empty_like(self.Lc)
        self.Rp = torch.empty_like(self.Rc)
        self.Tp = torch.empty_like(self.Tc)
        self.mu = torch.empty(self.N, dtype=f64, device=dev)
        self._coef = torch.empty(2 * self.K * nt + self.nv, dtype=f64, device=dev)
        self._contract_out = torch.empty(4 * self.K * nt + 2 * self.nv * (nt + 1), dtype=f64, device=dev)
        self.h = BtaHandle.get(b, nt, a)
        # an evaluation with the gradient runs the selected inversion after the mean's
        # sweeps: let it run next to them
        self.h.set_selinv_overlap(True)
        self.last = {}
        # separable priors: logdet and tr(Q_prior^-1 dQ_prior) from the ns x ns spatial
        # factors (see _separable_prior_terms); "selinv" factors the whole prior (bt) for
        # its logdet and takes the trace from its selected inverse, as the reference does
        self.prior_trace = "separable"
        self._sep_prior_grad = None
        sep = spec.separable_prior(spec.theta0) if hasattr(spec, "theta0") else None
        self._sep_base = None
        if sep is not None:
            base, _ = sep
            rp, cl, uv = union_pattern(base)
            self._sep_base = base
            self._sep_rowptr = torch.from_numpy(rp).to(dev)
            self._sep_col = torch.from_numpy(cl).to(dev)
            self._sep_uval = torch.from_numpy(np.ascontiguousarray(uv)).to(dev)
            self._sep_vw = torch.zeros(2 * len(base), dtype=torch.int32, device=dev)
            self._sep_D = torch.empty((1, self.ns, self.ns), dtype=f64, device=dev)
            self._sep_coef = torch.empty(len(base), dtype=f64, device=dev)
            self._sep_out = torch.empty(4 * len(base) + 4, dtype=f64, device=dev)
            self._sep_h = BtaHandle.get(self.ns, 1, 0)

    def coefficients(self, theta):
        return self.spec.coefficients(theta)

    def coefficient_derivatives(self, theta):
        return self.spec.coefficient_derivatives(theta)

    def log_prior(self, theta):
        return self.spec.log_prior(theta)

    def log_prior_grad(self, theta):
        return self.spec.log_prior_grad(theta)

    def lik_theta_indices(self):
        return self.spec.lik_theta_indices()

    def _check_variate_support(self, A, ov, av):
        """Every observation must touch only its own variate's nodes and fixed effects
        (the block-diagonal A of the reference's CoregionalModel, coregional_model.py:
        203-214); the per-variate scaling of A^T A relies on it."""
        if self.nv == 1:
            return
        Ac = A.tocoo()
        col = Ac.col.astype(np.int64)
        nbk = self.nt * self.b
        field = col < nbk
        cv = np.empty(col.size, dtype=np.int64)
        cv[field] = (col[field] % self.b) // self.ns
        cv[~field] = av[col[~field] - nbk]
        if np.any(cv != ov[Ac.row]):
            raise ValueError("an observation touches another variate's latent parameters")

    # ---------------------------------------------------------------- device steps
    def _ptr(self, t):
        return None if t is None else t.data_ptr()

    def _upload_coef(self, c: Coefficients):
        """Copy alpha, beta and the per-variate tau_y into one device buffer; returns
        the device pointers (alpha, beta, tau_y)."""
        K, nt = self.K, self.nt
        buf = np.zeros(2 * K * nt + self.nv)
        buf[: K * nt] = c.alpha.reshape(-1)
        if nt > 1:
            buf[K * nt: K * nt + K * (nt - 1)] = c.beta.reshape(-1)
        buf[2 * K * nt:] = c.tau_y
        self._coef.copy_(self.torch.from_numpy(buf), non_blocking=False)
        p0 = self._coef.data_ptr()
        return p0, p0 + 8 * K * nt, p0 + 8 * 2 * K * nt

    def _assemble(self, coef_ptrs, D, L, R, T, with_lik: bool):
        alpha_p, beta_p, tau_p = coef_ptrs
        lib, h = self.h.lib, self.h
        _lib.check(lib.gbta_assemble_kron(
            h.ptr, self.ns, self.nv, self.K, self._upat_rowptr.data_ptr(), self._upat_col.data_ptr(),
            self._uval.data_ptr(), self._term_vw.data_ptr(), alpha_p, beta_p,
            self._lik_rowptr.data_ptr() if with_lik else None, self._lik_col.data_ptr() if with_lik else None,
            self._lik_val.data_ptr() if with_lik else None, self._ptr(self._lik_R) if with_lik else None,
            self._ptr(self._lik_T) if with_lik else None, tau_p if with_lik else None,
            self._ptr(self._arrow_var), self.tip_prec, D.data_ptr(), L.data_ptr(), R.data_ptr(), T.data_ptr()))

    def _contract(self, SD, SL, SR, ST, mu) -> np.ndarray:
        lib, h = self.h.lib, self.h
        _lib.check(lib.gbta_contract_kron(
            h.ptr, self.ns, self.nv, self.K, self._upat_rowptr.data_ptr(), self._upat_col.data_ptr(),
            self._uval.data_ptr(), self._term_vw.data_ptr(), self._lik_rowptr.data_ptr(), self._lik_col.data_ptr(),
            self._lik_val.data_ptr(), self._ptr(self._lik_R), self._ptr(self._lik_T), self._ptr(self._arrow_var),
            self._ptr(SD), self._ptr(SL), self._ptr(SR), self._ptr(ST), self._ptr(mu),
            self._contract_out.data_ptr()))
        return self._contract_out.cpu().numpy()

    def _logdet(self, D, T, with_tip: bool) -> float:
        out = ctypes.c_double(0.0)
        code = self.h.lib.gbta_logdet(self.h.ptr, D.data_ptr(), T.data_ptr() if with_tip else None,
                                      1 if with_tip else 0, ctypes.byref(out))
        if code == _lib.GBTA_ERR_ARG and np.isnan(out.value):
            raise ValueError("Logdet is NaN. Check the input matrix.")
        _lib.check(code)
        return float(out.value)

    def _spatial_logdet_and_traces(self, w: np.ndarray, traces: bool = True):
        """logdet Q_s and tr(Q_s^-1 S_j) for Q_s = sum_j w_j S_j (ns x ns), on the device:
        Kronecker assembly with one time block, factorization, logdet, selected
        inversion (the full inverse of a single block) and the trace contractions (the
        last two only with ``traces``; the traces are None without)."""
        h, lib = self._sep_h, self._sep_h.lib
        h.set_stream(current_stream_ptr())
        J = len(self._sep_base)
        self._sep_coef.copy_(self.torch.from_numpy(np.asarray(w, dtype=np.float64)))
        _lib.check(lib.gbta_assemble_kron(
            h.ptr, self.ns, 1, J, self._sep_rowptr.data_ptr(), self._sep_col.data_ptr(), self._sep_uval.data_ptr(),
            self._sep_vw.data_ptr(), self._sep_coef.data_ptr(), None, None, None, None, None, None, None, None, 0.0,
            self._sep_D.data_ptr(), None, None, None))
        _lib.check(lib.gbta_pobtf(h.ptr, self._sep_D.data_ptr(), None))
        out = ctypes.c_double(0.0)
        _lib.check(lib.gbta_logdet(h.ptr, self._sep_D.data_ptr(), None, 0, ctypes.byref(out)))
        if not traces:
            return float(out.value), None
        _lib.check(lib.gbta_pobtsi(h.ptr, self._sep_D.data_ptr(), None))
        _lib.check(lib.gbta_contract_kron(
            h.ptr, self.ns, 1, J, self._sep_rowptr.data_ptr(), self._sep_col.data_ptr(), self._sep_uval.data_ptr(),
            self._sep_vw.data_ptr(), None, None, None, None, None, None, self._sep_D.data_ptr(), None, None, None,
            None, self._sep_out.data_ptr()))
        tr = self._sep_out.cpu().numpy()[:J].copy()
        return float(out.value), tr

    def _separable_prior_terms(self, theta, gradient: bool = True):
        """logdet_bt Q_prior and (with ``gradient``, else None) its theta-gradient for a
        separable prior:
        Q_re = (W^T (x) I) blockdiag_k(c_k T_k (x) Q_s,k) (W (x) I) with |det W| = 1 gives
            logdet = sum_k nt ns log c_k + ns logdet T_k + nt logdet Q_s,k,
            d logdet = sum_k nt ns dlog c_k + ns dlogdet T_k + nt sum_j dw_kj tr(Q_s,k^-1 S_j),
        with the stationary AR1 logdet T(rho) = -(nt-1) log(1 - rho^2).  Equal to the
        BTA factorization's logdet of the time-major prior and to its adjoint trace
        tr(Q_prior^-1 dQ_prior), at the cost of one ns x ns factor per block."""
        _, parts = self.spec.separable_prior(theta)
        nt, ns = self.nt, self.ns
        d = np.asarray(theta).size
        logdet = 0.0
        grad = np.zeros(d)
        cache = {}
        for part in parts:
            key = tuple(np.asarray(part.w, dtype=np.float64).tolist())
            if key not in cache:
                cache[key] = self._spatial_logdet_and_traces(part.w, traces=gradient)
            ld_s, tr_s = cache[key]
            r = part.rho
            logdet += nt * ns * np.log(part.c) - ns * (nt - 1) * np.log1p(-r * r) + nt * ld_s
            if gradient:
                dlogdet_t = 2.0 * r * (nt - 1) / (1.0 - r * r)
                grad += nt * ns * part.dlogc + ns * dlogdet_t * part.drho + nt * (part.dw @ tr_s)
        return logdet, (grad if gradient else None)

    def _prior_logdet(self, theta, ptrs, gradient: bool = False) -> float:
        """logdet_bt Q_prior, the tip excluded (pyinla.py:1102-1103).  A separable prior
        takes it from its ns x ns spatial factors (with ``gradient`` also the trace the
        adjoint needs, kept for _adjoint_gradient), with no factorization of the whole
        prior; otherwise the prior is assembled and factored (bt) as the reference does."""
        self._sep_prior_grad = None
        if self._sep_base is not None and self.prior_trace == "separable":
            logdet, self._sep_prior_grad = self._separable_prior_terms(theta, gradient=gradient)
            return logdet
        h = self.h
        self._assemble(ptrs, self.Dp, self.Lp, self.Rp, self.Tp, with_lik=False)
        _lib.check(h.lib.gbta_pobtf(h.ptr, self.Dp.data_ptr(), self.Lp.data_ptr()))
        return self._logdet(self.Dp, self.Tp, with_tip=False)

    def _split(self, out: np.ndarray):
        K, nt = self.K, self.nt
        KN = K * nt
        c = out[0:KN].reshape(K, nt)
        d = out[KN:2 * KN].reshape(K, nt)[:, : nt - 1]
        qc = out[2 * KN:3 * KN].reshape(K, nt)
        qd = out[3 * KN:4 * KN].reshape(K, nt)[:, : nt - 1]
        lik = out[4 * KN:4 * KN + 2 * self.nv * (nt + 1)].reshape(self.nv, 2, nt + 1).sum(axis=2)
        return c, d, qc, qd, lik[:, 0], lik[:, 1]

    # ---------------------------------------------------------------- public
    def evaluate(self, theta, gradient: bool = False):
        """f(theta) (and, with ``gradient=True``, its adjoint gradient)."""
        theta = np.asarray(theta, dtype=np.float64)
        h = self.h
        h.set_stream(current_stream_ptr())
        lib = h.lib
        coef = self.coefficients(theta)
        ptrs = self._upload_coef(coef)
        has_arrow = self.nb > 0
        # prior logdet, tip excluded (pyinla.py:1102-1103)
        logdet_p = self._prior_logdet(theta, ptrs, gradient=gradient)
        # conditional: bta factorization (pyinla.py:650-662)
        self._assemble(ptrs, self.Dc, self.Lc, self.Rc, self.Tc, with_lik=True)
        R, T = (self.Rc.data_ptr(), self.Tc.data_ptr()) if has_arrow else (None, None)
        _lib.check(lib.gbta_pobtaf(h.ptr, self.Dc.data_ptr(), self.Lc.data_ptr(), R, T))
        logdet_c = self._logdet(self.Dc, self.Tc, with_tip=has_arrow)
        # mean: mu = Q_cond^{-1} sum_v tau_y,v A_v^T y_v (model.py:425-449 at x = 0;
        # per-variate likelihoods as in coregional_model.py:645-668)
        tau_t = self.torch.from_numpy(coef.tau_y).to(self.mu.device)
        self.mu.copy_(tau_t @ self._Aty_v)
        bvec = self.mu.clone()
        # N then C in one launch (trans = 2)
        if gradient:
            # the conditional's selected inverse (for the gradient's traces) is queued right
            # behind the sweeps: it reads the factor only, so it runs on the solver's side
            # stream next to them, and Sigma lands in the blocks after both
            _lib.check(lib.gbta_pobtas_async(h.ptr, self.Dc.data_ptr(), self.Lc.data_ptr(), R, T,
                                             self.mu.data_ptr(), 1, 2))
            _lib.check(lib.gbta_pobtasi_async(h.ptr, self.Dc.data_ptr(), self.Lc.data_ptr(), R, T))
            h.status()
        else:
            _lib.check(lib.gbta_pobtas(h.ptr, self.Dc.data_ptr(), self.Lc.data_ptr(), R, T, self.mu.data_ptr(), 1, 2))
        quad = float(self.torch.dot(self.mu, bvec))   # mu^T Q_cond mu = mu^T b
        ty = np.asarray(self.lik_theta_indices(), dtype=np.int64)
        # gaussian.py:58-60 at eta = 0, summed over the variates' likelihoods
        lik = float(np.sum(0.5 * self.nobs_v * theta[ty] - 0.5 * coef.tau_y * self.yty_v))
        lp = self.log_prior(theta)
        f = -(lp + lik + 0.5 * logdet_p) + 0.5 * logdet_c - 0.5 * quad
        self.last = dict(logdet_prior=logdet_p, logdet_cond=logdet_c, quad=quad, lik=lik, log_prior=lp)
        if not gradient:
            return f
        return f, self._adjoint_gradient(theta, coef, quad)

    def hessian(self, theta, eps: float = 5e-3) -> np.ndarray:
        """Hessian of f at theta by central differences of the adjoint gradient, symmetrised:
        2 d gradient evaluations (each a factorization, a solve and a selected inversion)
        where the reference differences f itself with 1 + 2d + 2d(d-1) evaluations
        (PyINLA._evaluate_hessian_f, pyinla.py:767-910; default step eps_hessian_f = 5e-3,
        configs/pyinla_config.py:52)."""
        theta = np.asarray(theta, dtype=np.float64)
        d = theta.size
        H = np.zeros((d, d))
        for k in range(d):
            e = np.zeros(d)
            e[k] = eps
            _, gp = self.evaluate(theta + e, gradient=True)
            _, gm = self.evaluate(theta - e, gradient=True)
            H[:, k] = (gp - gm) / (2.0 * eps)
        return 0.5 * (H + H.T)

    def covariance_hp(self, theta, eps: float = 5e-3) -> np.ndarray:
        """Covariance of the hyperparameters, the inverse of the Hessian of f
        (PyINLA.compute_covariance_hp, pyinla.py:747-765)."""
        return np.linalg.inv(self.hessian(theta, eps))

    def marginal_variances(self, theta):
        """(diag(Sigma), diag(A Sigma A^T)) at theta, Sigma = Q_cond^-1: the two outputs of
        the reference's run() (pyinla.py:303-311; get_marginal_variances_latent_parameters
        and get_marginal_variances_observations, pyinla.py:940-1018).  For a Gaussian
        likelihood Q_cond does not depend on x*, so theta alone fixes them."""
        from .marginals import DeviceCSR, latent_variances, observation_variances
        theta = np.asarray(theta, dtype=np.float64)
        h = self.h
        h.set_stream(current_stream_ptr())
        ptrs = self._upload_coef(self.coefficients(theta))
        self._assemble(ptrs, self.Dc, self.Lc, self.Rc, self.Tc, with_lik=True)
        has_arrow = self.nb > 0
        R, T = (self.Rc.data_ptr(), self.Tc.data_ptr()) if has_arrow else (None, None)
        _lib.check(h.lib.gbta_pobtaf(h.ptr, self.Dc.data_ptr(), self.Lc.data_ptr(), R, T))
        _lib.check(h.lib.gbta_pobtasi(h.ptr, self.Dc.data_ptr(), self.Lc.data_ptr(), R, T))
        if getattr(self, "_A_dev", None) is None:
            self._A_dev = DeviceCSR(self.spec.A)
        SL = self.Lc if self.nt > 1 else None
        SR, ST = (self.Rc, self.Tc) if has_arrow else (None, None)
        lat = latent_variances(h, self.Dc, ST)
        obs = observation_variances(h, self._A_dev, self.Dc, SL, SR, ST)
        return lat.cpu().numpy(), obs.cpu().numpy()

    def _adjoint_gradient(self, theta, coef: Coefficients, quad: float) -> np.ndarray:
        h = self.h
        lib = h.lib
        dc = self.coefficient_derivatives(theta)
        has_arrow = self.nb > 0
        # contractions of the conditional's selected inverse (over the factor's blocks,
        # computed in evaluate) with mu
        cc, dd, qc, qd, lc, lq = self._split(self._contract(
            self.Dc, self.Lc if self.nt > 1 else None, self.Rc if has_arrow else None,
            self.Tc if has_arrow else None, self.mu))
        # prior trace tr(Q_prior^-1 dQ_prior): from the spatial factors for a separable
        # prior, else from the prior's selected inverse (bt)
        tr_prior = None
        if self._sep_prior_grad is not None:   # from evaluate's separable prior terms
            tr_prior = self._sep_prior_grad
        elif self._sep_base is not None and self.prior_trace == "separable":
            _, tr_prior = self._separable_prior_terms(theta)
        else:
            _lib.check(lib.gbta_pobtsi(h.ptr, self.Dp.data_ptr(), self.Lp.data_ptr()))
            pc, pd, _, _, _, _ = self._split(self._contract(self.Dp, self.Lp if self.nt > 1 else None, None, None,
                                                            None))
        mAty = (self._Aty_v @ self.mu).cpu().numpy()      # mu^T A_v^T y_v per variate
        d = dc.dalpha.shape[0]
        grad = np.zeros(d)
        for k in range(d):
            da, db, dt = dc.dalpha[k], dc.dbeta[k], dc.dtau_y[k]
            tr_c = float(np.sum(da * cc) + 2.0 * np.sum(db * dd) + dt @ lc)
            tr_p = float(tr_prior[k]) if tr_prior is not None else float(np.sum(da * pc) + 2.0 * np.sum(db * pd))
            mqm = float(np.sum(da * qc) + 2.0 * np.sum(db * qd) + dt @ lq)
            mdb = float(dt @ mAty)                         # mu^T d(b), b = sum_v tau_y,v A_v^T y_v
            grad[k] = -0.5 * tr_p + 0.5 * tr_c - mdb + 0.5 * mqm
        ty = np.asarray(self.lik_theta_indices(), dtype=np.int64)
        grad[ty] -= 0.5 * self.nobs_v - 0.5 * coef.tau_y * self.yty_v
        grad -= self.log_prior_grad(theta)
        return grad


class SeparableSpdeAr1(KronSpec):
    """Q_prior = tau * (T_AR1(rho) (x) Q_s(kappa)) (+) tip_prec * I_nb, Gaussian likelihood.

    theta = (log kappa, log r_t, log tau, log tau_y) with rho = exp(-1 / r_t);
    Gaussian priors N(theta0, 1 / prior_prec) on every component (the form of the
    reference's GaussianPriorHyperparameters, src/pyinla/prior_hyperparameters/gaussian.py:26-29).
    """

    def __init__(self, mesh: spde.Mesh, nt: int, nb: int, obs: spde.Observations, theta0: np.ndarray,
                 prior_prec: float = 0.5, tip_prec: float = 1e-3):
        self.mesh = mesh
        self.theta0 = np.asarray(theta0, dtype=np.float64)
        self.prior_prec = float(prior_prec)
        self.terms = spde.spde_terms(mesh)
        self.term_vw = [(0, 0)] * len(self.terms)
        self.ns, self.nv, self.nt, self.nb = mesh.ns, 1, int(nt), int(nb)
        self.A = spde.design_matrix(obs, mesh.ns, nt, nb)
        self.y = obs.y
        self.tip_prec = float(tip_prec)

    @staticmethod
    def unpack(theta):
        kappa = np.exp(theta[0])
        r_t = np.exp(theta[1])
        rho = np.exp(-1.0 / r_t)
        return kappa, r_t, rho, np.exp(theta[2]), np.exp(theta[3])

    def coefficients(self, theta) -> Coefficients:
        kappa, r_t, rho, tau, tau_y = self.unpack(theta)
        w = spde.spde_weights(kappa)
        tdiag, toff = spde.ar1_bands(rho, self.nt)
        return Coefficients(alpha=tau * np.outer(w, tdiag), beta=tau * np.outer(w, toff).reshape(len(w), -1),
                            tau_y=tau_y)

    def coefficient_derivatives(self, theta) -> CoefficientDerivatives:
        kappa, r_t, rho, tau, tau_y = self.unpack(theta)
        w = spde.spde_weights(kappa)
        dw = spde.spde_weights_dlogkappa(kappa)
        tdiag, toff = spde.ar1_bands(rho, self.nt)
        ddiag, doff = spde.ar1_bands_drho(rho, self.nt)
        drho = rho / r_t                         # d rho / d log r_t
        dalpha = np.stack([tau * np.outer(dw, tdiag), tau * drho * np.outer(w, ddiag),
                           tau * np.outer(w, tdiag), np.zeros((self.K, self.nt))])
        dbeta = np.stack([tau * np.outer(dw, toff), tau * drho * np.outer(w, doff),
                          tau * np.outer(w, toff), np.zeros((self.K, max(self.nt - 1, 0)))])
        return CoefficientDerivatives(dalpha=dalpha, dbeta=dbeta, dtau_y=np.array([[0.0], [0.0], [0.0], [tau_y]]))

    @classmethod
    def synthetic(cls, n_side: int, nt: int, nb: int, n_obs: int, seed: int, theta0=None):
        """The benchmark's synthetic instance: n_side x n_side mesh, n_obs observations."""
        mesh = spde.unit_square_mesh(n_side)
        obs = spde.make_observations(mesh, nt, n_obs, nb, seed)
        th = default_theta() if theta0 is None else np.asarray(theta0, dtype=np.float64)
        return cls(mesh, nt, nb, obs, th)

    def log_prior(self, theta) -> float:
        return float(-0.5 * self.prior_prec * np.sum((theta - self.theta0) ** 2))

    def log_prior_grad(self, theta) -> np.ndarray:
        return -self.prior_prec * (theta - self.theta0)

    def lik_theta_indices(self) -> list[int]:
        return [3]

    def separable_prior(self, theta):
        kappa, r_t, rho, tau, _ = self.unpack(theta)
        d = 4
        dlogc = np.zeros(d)
        dlogc[2] = 1.0
        drho = np.zeros(d)
        drho[1] = rho / r_t
        dw = np.zeros((d, 3))
        dw[0] = spde.spde_weights_dlogkappa(kappa)
        return self.terms, [SeparablePart(c=tau, dlogc=dlogc, rho=rho, drho=drho, w=spde.spde_weights(kappa), dw=dw)]


def default_theta(rho: float = 0.9, kappa: float = None, tau: float = 1.0, tau_y: float = 4.0, ns: int = 1024):
    """theta = (log kappa, log r_t, log tau, log tau_y) for the benchmark model; kappa
    defaults to a spatial range of a third of the domain (kappa = sqrt(8) / 0.33)."""
    if kappa is None:
        kappa = np.sqrt(8.0) / 0.33
    r_t = -1.0 / np.log(rho)
    return np.array([np.log(kappa), np.log(r_t), np.log(tau), np.log(tau_y)])


def coregional_loadings(lam: dict, nv: int) -> np.ndarray:
    """Rows v_k of the coregional mixing: Q_re = sum_k sigma_k^-2 (v_k v_k^T) (x) Qu_k.

    Read off the reference's block formulas (src/pyinla/models/coregional_model.py:
    297-327 for two variates, :349-399 for three): v_0 = e_0, v_1 = (-l01, 1, 0),
    v_2 = (-l12, -l02, 1), e.g. q21 = -l01/s1^2 Qu_1 + l02 l12/s2^2 Qu_2.
    """
    if nv == 1:
        return np.ones((1, 1))
    V = np.eye(nv)
    V[1, 0] = -lam["0_1"]
    if nv == 3:
        V[2, 0] = -lam["1_2"]
        V[2, 1] = -lam["0_2"]
    elif nv != 2:
        raise ValueError("the reference's coregional model has 2 or 3 variates")
    return V


class CoregionalSpdeAr1(KronSpec):
    """nv-variate coregional spatio-temporal model with per-variate Gaussian likelihoods.

    Mirrors the reference's CoregionalModel (src/pyinla/models/coregional_model.py):
    each variate k has a unit-variance separable prior Qu_k = T_AR1(rho_k) (x)
    Q_s(kappa_k) (its ``sigma`` hyperparameter is removed, coregional_model.py:107-118);
    the mixing gives

        Q_re = sum_k sigma_k^-2 (v_k v_k^T) (x) Qu_k          (coregional_loadings)

    permuted to the BTA layout: block t = [variate 0 nodes, ..., variate nv-1 nodes]
    (coregional_model.py:217-231, 754-786), fixed effects ordered per variate, each with
    prior precision ``tip_prec`` (the regression submodel's block, appended with
    bdiag_tiling at :490-497).  Q_cond = Q_prior + sum_v tau_y,v A_v^T A_v with the
    block-diagonal A of the variates' design matrices (:203-214, 574-643).

    The mixing (sigma_k, lambda) is held fixed; theta = (log kappa_k, log r_t,k,
    log tau_y,k) for k = 0..nv-1 in that order (each variate's own parameters in
    the reference's per-model order), with Gaussian priors N(theta0, 1/prior_prec).
    The Kronecker terms are (S_j at variate block (p, q)) for the three spatial
    matrices S_j and every pair (p, q): 3 nv^2 terms.
    """

    def __init__(self, mesh: spde.Mesh, nt: int, nb_per: int, nv: int, obs: spde.Observations, sigma, lam: dict,
                 theta0: np.ndarray, prior_prec: float = 0.5, tip_prec: float = 1e-3):
        self.mesh = mesh
        self.nv, self.ns, self.nt = int(nv), mesh.ns, int(nt)
        self.nb_per = int(nb_per)
        self.nb = self.nv * self.nb_per
        self.sigma = np.asarray(sigma, dtype=np.float64).reshape(self.nv)
        self.lam = dict(lam)
        self.V = coregional_loadings(self.lam, self.nv)
        self.theta0 = np.asarray(theta0, dtype=np.float64).reshape(3 * self.nv)
        self.prior_prec = float(prior_prec)
        base = spde.spde_terms(mesh)
        self.base_terms = base
        self.terms, self.term_vw, self._term_jpq = [], [], []
        for j, S in enumerate(base):
            for p in range(self.nv):
                for q in range(self.nv):
                    self.terms.append(S)
                    self.term_vw.append((p, q))
                    self._term_jpq.append((j, p, q))
        self.A = spde.design_matrix(obs, mesh.ns, nt, self.nb_per, nv=self.nv)
        self.y = obs.y
        self.obs_variate = np.zeros(obs.y.shape[0], dtype=np.int64) if obs.v is None else np.asarray(obs.v)
        self.arrow_variate = np.repeat(np.arange(self.nv), self.nb_per).astype(np.int32)
        self.tip_prec = float(tip_prec)

    def mixing_precision(self) -> np.ndarray:
        """The nv x nv mixing precision sum_k sigma_k^-2 v_k v_k^T (SPD by construction)."""
        return self.V.T @ np.diag(self.sigma ** -2.0) @ self.V

    def _unpack(self, theta):
        th = np.asarray(theta, dtype=np.float64).reshape(self.nv, 3)
        kappa = np.exp(th[:, 0])
        r_t = np.exp(th[:, 1])
        rho = np.exp(-1.0 / r_t)
        return kappa, r_t, rho, np.exp(th[:, 2])

    def _mix(self, k, p, q):
        return self.V[k, p] * self.V[k, q] / self.sigma[k] ** 2

    def coefficients(self, theta) -> Coefficients:
        kappa, r_t, rho, tau_y = self._unpack(theta)
        nt, K = self.nt, self.K
        alpha = np.zeros((K, nt))
        beta = np.zeros((K, max(nt - 1, 0)))
        for k in range(self.nv):
            w = spde.spde_weights(kappa[k])
            tdiag, toff = spde.ar1_bands(rho[k], nt)
            for i, (j, p, q) in enumerate(self._term_jpq):
                m = self._mix(k, p, q)
                if m != 0.0:
                    alpha[i] += m * w[j] * tdiag
                    beta[i] += m * w[j] * toff
        return Coefficients(alpha=alpha, beta=beta, tau_y=tau_y)

    def coefficient_derivatives(self, theta) -> CoefficientDerivatives:
        kappa, r_t, rho, tau_y = self._unpack(theta)
        nt, K, nv = self.nt, self.K, self.nv
        d = 3 * nv
        dalpha = np.zeros((d, K, nt))
        dbeta = np.zeros((d, K, max(nt - 1, 0)))
        dtau = np.zeros((d, nv))
        for k in range(nv):
            w = spde.spde_weights(kappa[k])
            dw = spde.spde_weights_dlogkappa(kappa[k])
            tdiag, toff = spde.ar1_bands(rho[k], nt)
            ddiag, doff = spde.ar1_bands_drho(rho[k], nt)
            drho = rho[k] / r_t[k]
            for i, (j, p, q) in enumerate(self._term_jpq):
                m = self._mix(k, p, q)
                if m == 0.0:
                    continue
                dalpha[3 * k, i] = m * dw[j] * tdiag
                dbeta[3 * k, i] = m * dw[j] * toff
                dalpha[3 * k + 1, i] = m * w[j] * drho * ddiag
                dbeta[3 * k + 1, i] = m * w[j] * drho * doff
            dtau[3 * k + 2, k] = tau_y[k]
        return CoefficientDerivatives(dalpha=dalpha, dbeta=dbeta, dtau_y=dtau)

    def log_prior(self, theta) -> float:
        return float(-0.5 * self.prior_prec * np.sum((np.asarray(theta) - self.theta0) ** 2))

    def log_prior_grad(self, theta) -> np.ndarray:
        return -self.prior_prec * (np.asarray(theta) - self.theta0)

    def lik_theta_indices(self) -> list[int]:
        return [3 * k + 2 for k in range(self.nv)]

    def separable_prior(self, theta):
        """Q_re = P (V^T (x) I) blockdiag_k(sigma_k^-2 Qu_k) (V (x) I) P^T with V unit lower
        triangular and P the time-major permutation: separable blocks, unit mixing."""
        kappa, r_t, rho, _ = self._unpack(theta)
        d = 3 * self.nv
        parts = []
        for k in range(self.nv):
            drho = np.zeros(d)
            drho[3 * k + 1] = rho[k] / r_t[k]
            dw = np.zeros((d, 3))
            dw[3 * k] = spde.spde_weights_dlogkappa(kappa[k])
            parts.append(SeparablePart(c=float(self.sigma[k] ** -2.0), dlogc=np.zeros(d), rho=float(rho[k]), drho=drho,
                                       w=spde.spde_weights(kappa[k]), dw=dw))
        return self.base_terms, parts

    @classmethod
    def synthetic(cls, n_side: int, nt: int, nb_per: int, nv: int, n_obs: int, seed: int, m_side: int = 0,
                  theta0=None):
        """Seeded synthetic instance: n_side x m_side mesh per variate, n_obs observations
        split evenly over the variates, mixing sigma_k = exp(N(0, 0.2^2)) and
        lambda ~ N(0, 0.5^2) drawn from the seed (so the nv x nv mixing precision is a
        seeded SPD matrix)."""
        mesh = spde.unit_square_mesh(n_side, m_side)
        obs = spde.make_coregional_observations(mesh, nt, n_obs, nb_per, nv, seed)
        rng = np.random.default_rng(seed + 7919)
        sigma = np.exp(0.2 * rng.standard_normal(nv))
        lam = {"0_1": 0.5 * rng.standard_normal(), "0_2": 0.5 * rng.standard_normal(),
               "1_2": 0.5 * rng.standard_normal()}
        if theta0 is None:
            base = default_theta()
            th = []
            for k in range(nv):
                th += [base[0] + 0.1 * k, base[1] - 0.1 * k, base[3] - 0.2 * k]
            theta0 = np.array(th)
        return cls(mesh, nt, nb_per, nv, obs, sigma, lam, np.asarray(theta0, dtype=np.float64))
