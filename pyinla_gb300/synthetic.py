"""Seeded synthetic BTA matrices generated on the device.

The same construction as the plain-solve workload (diagonally dominant SPD: L_i, R_i
~ N(0,1)/sqrt(b), D_i = (G + G^T)/2, tip likewise, each diagonal entry raised by
its row's off-diagonal absolute sum + 1), drawn with torch's CUDA generator so that
large instances never pass through host memory.  Used by the autotuner and the
benchmarks; the NumPy twin with a fixed draw order is the oracle's make_bta_c1.
"""
from __future__ import annotations

from .device import require_torch_cuda


def random_bta(nt: int, b: int, a: int, seed: int = 0):
    """(D, L, R, T) torch CUDA float64 tensors; L has max(nt-1, 1) blocks, R and T
    at least one row/column (zero-sized arrowheads are not allocated)."""
    torch = require_torch_cuda()
    g = torch.Generator(device="cuda")
    g.manual_seed(int(seed))
    s = 1.0 / float(b) ** 0.5
    f64 = torch.float64
    G = torch.randn((nt, b, b), generator=g, device="cuda", dtype=f64) * s
    D = 0.5 * (G + G.transpose(1, 2))
    del G
    L = torch.randn((max(nt - 1, 1), b, b), generator=g, device="cuda", dtype=f64) * s
    if nt == 1:
        L.zero_()
    R = torch.randn((nt, max(a, 1), b), generator=g, device="cuda", dtype=f64) * s
    T = torch.randn((max(a, 1), max(a, 1)), generator=g, device="cuda", dtype=f64) * s
    T = 0.5 * (T + T.T)
    if a == 0:
        R.zero_()
        T.zero_()
    rows = D.abs().sum(2) - D.diagonal(dim1=1, dim2=2).abs()
    if nt > 1:
        rows[1:] += L[: nt - 1].abs().sum(2)
        rows[:-1] += L[: nt - 1].abs().sum(1)
    if a:
        rows += R.abs().sum(1)
    D += torch.diag_embed(rows + 1.0)
    if a:
        ra = T.abs().sum(1) - T.diagonal().abs() + R.abs().sum((0, 2))
        T += torch.diag(ra + 1.0)
    else:
        T.fill_diagonal_(1.0)
    return D.contiguous(), L.contiguous(), R.contiguous(), T.contiguous()
