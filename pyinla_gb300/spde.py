"""Synthetic spatio-temporal model inputs: SPDE mesh matrices, AR1 temporal precision
and Gaussian observations -- the data that feeds the BTA assembly.

The reference reads these from ``.npz`` files of real meshes
(src/pyinla/submodels/spatio_temporal.py:26-35: c0, g1, g2, g3, m0, m1, m2, and
src/pyinla/core/submodel.py:24-30: the design matrix ``a``); its example datasets are
not available, so seeded synthetic inputs of the benchmark's shapes stand in:

* a regular ``n x n`` node grid on the unit square, each cell split into two
  triangles; P1 finite elements give the lumped mass matrix ``C`` (diagonal) and
  the stiffness matrix ``G``;
* the Matern (alpha = 2) SPDE precision ``Q_s(kappa) = kappa^4 C + 2 kappa^2 G + G C^-1 G``;
* the stationary AR1 precision ``T(rho)`` over ``nt`` time steps;
* observations at uniform random locations and time steps: each row of ``A`` holds
  the 3 barycentric weights of its triangle at its time step, plus ``nb`` N(0,1)
  covariates for the fixed effects (latent order: time-major field, then fixed
  effects, as the reference's Model orders its submodels, src/pyinla/core/model.py:49-55).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.sparse as sps


@dataclass
class Mesh:
    n: int                   # nodes along x
    nodes: np.ndarray        # (ns, 2)
    tris: np.ndarray         # (ntri, 3)
    C: sps.csr_matrix        # lumped mass (diagonal)
    G: sps.csr_matrix        # P1 stiffness
    m: int = 0               # nodes along y (0: same as n)

    @property
    def ny(self) -> int:
        return self.m or self.n

    @property
    def ns(self) -> int:
        return self.n * self.ny


def unit_square_mesh(n: int, m: int = 0) -> Mesh:
    """Regular n x m node grid (m = n by default) on [0,1]^2, two triangles per cell,
    P1 FEM matrices."""
    m = m or n
    xs = np.linspace(0.0, 1.0, n)
    ys = np.linspace(0.0, 1.0, m)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    nodes = np.stack([X.ravel(), Y.ravel()], axis=1)
    idx = np.arange(n * m).reshape(m, n)   # idx[iy, ix]
    a = idx[:-1, :-1].ravel()
    b = idx[:-1, 1:].ravel()
    c = idx[1:, :-1].ravel()
    d = idx[1:, 1:].ravel()
    tris = np.concatenate([np.stack([a, b, d], 1), np.stack([a, d, c], 1)])
    p0, p1, p2 = nodes[tris[:, 0]], nodes[tris[:, 1]], nodes[tris[:, 2]]
    e0, e1, e2 = p2 - p1, p0 - p2, p1 - p0          # edge opposite each vertex
    area = 0.5 * np.abs(e2[:, 0] * (-e1[:, 1]) - e2[:, 1] * (-e1[:, 0]))
    E = np.stack([e0, e1, e2], axis=1)              # (ntri, 3, 2)
    K = np.einsum("tid,tjd->tij", E, E) / (4.0 * area)[:, None, None]
    rows = np.repeat(tris, 3, axis=1).ravel()
    cols = np.tile(tris, (1, 3)).ravel()
    ns = n * m
    G = sps.csr_matrix((K.ravel(), (rows, cols)), shape=(ns, ns))
    G.sum_duplicates()
    cdiag = np.zeros(ns)
    np.add.at(cdiag, tris.ravel(), np.repeat(area / 3.0, 3))
    C = sps.diags(cdiag).tocsr()
    return Mesh(n=n, nodes=nodes, tris=tris, C=C, G=G, m=0 if m == n else m)


def spde_terms(mesh: Mesh) -> list[sps.csr_matrix]:
    """The three fixed spatial matrices of Q_s(kappa): C, G, G C^-1 G."""
    Cinv = sps.diags(1.0 / mesh.C.diagonal())
    GCG = (mesh.G @ Cinv @ mesh.G).tocsr()
    GCG.sum_duplicates()
    return [mesh.C.tocsr(), mesh.G.tocsr(), GCG]


def spde_weights(kappa: float) -> np.ndarray:
    """Coefficients of (C, G, G C^-1 G) in Q_s(kappa)."""
    return np.array([kappa ** 4, 2.0 * kappa ** 2, 1.0])


def spde_weights_dlogkappa(kappa: float) -> np.ndarray:
    return np.array([4.0 * kappa ** 4, 4.0 * kappa ** 2, 0.0])


def ar1_bands(rho: float, nt: int) -> tuple[np.ndarray, np.ndarray]:
    """Diagonal and sub-diagonal of the stationary AR1 precision T(rho) (unit variance)."""
    s = 1.0 / (1.0 - rho * rho)
    diag = np.full(nt, (1.0 + rho * rho) * s)
    if nt >= 1:
        diag[0] = s
        diag[-1] = s
    if nt == 1:
        diag[0] = 1.0
    off = np.full(max(nt - 1, 0), -rho * s)
    return diag, off


def ar1_bands_drho(rho: float, nt: int) -> tuple[np.ndarray, np.ndarray]:
    """Derivative of :func:`ar1_bands` with respect to rho."""
    q = (1.0 - rho * rho) ** 2
    diag = np.full(nt, 4.0 * rho / q)
    if nt >= 1:
        diag[0] = 2.0 * rho / q
        diag[-1] = 2.0 * rho / q
    if nt == 1:
        diag[0] = 0.0
    off = np.full(max(nt - 1, 0), -(1.0 + rho * rho) / q)
    return diag, off


def ar1_logdet(rho: float, nt: int) -> float:
    return -(nt - 1) * np.log(1.0 - rho * rho)


@dataclass
class Observations:
    t: np.ndarray            # (nobs,) time step
    nodes: np.ndarray        # (nobs, 3) spatial node indices
    w: np.ndarray            # (nobs, 3) barycentric weights
    z: np.ndarray            # (nobs, nb) covariates (nb per variate)
    y: np.ndarray            # (nobs,)
    v: np.ndarray | None = None   # (nobs,) variate of each observation (None: all 0)


def locate(mesh: Mesh, pts: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Containing triangle's nodes and barycentric weights for points in [0,1]^2."""
    n, m = mesh.n, mesh.ny
    hx = 1.0 / (n - 1)
    hy = 1.0 / (m - 1)
    ix = np.clip((pts[:, 0] / hx).astype(np.int64), 0, n - 2)
    iy = np.clip((pts[:, 1] / hy).astype(np.int64), 0, m - 2)
    u = pts[:, 0] / hx - ix
    v = pts[:, 1] / hy - iy
    a = iy * n + ix
    b = a + 1
    c = a + n
    d = c + 1
    lower = u >= v                       # triangle (a, b, d) else (a, d, c)
    nodes = np.where(lower[:, None], np.stack([a, b, d], 1), np.stack([a, d, c], 1))
    w = np.where(lower[:, None], np.stack([1.0 - u, u - v, v], 1), np.stack([1.0 - v, u, v - u], 1))
    return nodes, w


def make_observations(mesh: Mesh, nt: int, nobs: int, nb: int, seed: int) -> Observations:
    rng = np.random.default_rng(seed)
    pts = rng.random((nobs, 2))
    t = rng.integers(0, nt, size=nobs)
    nodes, w = locate(mesh, pts)
    z = rng.standard_normal((nobs, nb))
    y = rng.standard_normal(nobs)
    return Observations(t=t, nodes=nodes, w=w, z=z, y=y)


def make_coregional_observations(mesh: Mesh, nt: int, nobs: int, nb_per: int, nv: int, seed: int) -> Observations:
    """nobs observations split evenly over nv variates (ordered by variate, as the
    reference concatenates its models' data, coregional_model.py:189-201); each has
    the 3 barycentric weights of a uniform random location at a uniform random time
    step of its own variate's field, nb_per N(0,1) covariates for its variate's fixed
    effects, and y ~ N(0,1)."""
    rng = np.random.default_rng(seed)
    counts = [nobs // nv + (1 if v < nobs % nv else 0) for v in range(nv)]
    v = np.repeat(np.arange(nv), counts)
    pts = rng.random((nobs, 2))
    t = rng.integers(0, nt, size=nobs)
    nodes, w = locate(mesh, pts)
    z = rng.standard_normal((nobs, nb_per))
    y = rng.standard_normal(nobs)
    return Observations(t=t, nodes=nodes, w=w, z=z, y=y, v=v)


def design_matrix(obs: Observations, ns: int, nt: int, nb: int, nv: int = 1) -> sps.csr_matrix:
    """The observation matrix A (nobs x (nt*nv*ns + nv*nb)), latent order time-major
    (block t = [variate 0 nodes, ..., variate nv-1 nodes]) then the fixed effects
    ordered per variate -- the coregional BTA layout (coregional_model.py:217-231,
    754-786, 853-919).  ``nb`` is the number of fixed effects per variate."""
    nobs = obs.y.shape[0]
    b = nv * ns
    v = np.zeros(nobs, dtype=np.int64) if obs.v is None else np.asarray(obs.v, dtype=np.int64)
    rows = np.concatenate([np.repeat(np.arange(nobs), 3), np.repeat(np.arange(nobs), nb)])
    cols = np.concatenate([(obs.t[:, None] * b + v[:, None] * ns + obs.nodes).ravel(),
                           (nt * b + v[:, None] * nb + np.arange(nb)[None, :]).ravel()])
    vals = np.concatenate([obs.w.ravel(), obs.z.ravel()])
    A = sps.csr_matrix((vals, (rows, cols)), shape=(nobs, nt * b + nv * nb))
    A.sum_duplicates()
    return A
