"""CPU checks of the tile-level schedules and recurrences of the dataflow kernels.

The tile Cholesky's warp schedule (csrc/bta_common.cuh, smem_potrf):

The kernel splits a 32 x 32 Cholesky between a pivot warp and three update warps that
hold columns in register slots; pivots travel through an eight-slot ring of shared
memory guarded by eight rotating named-barrier ids.  These tests read the slot
constants from the CUDA source, check the invariant that makes the rotation safe, and
replay the kernel's exact sequence of operations (lane by lane, with the same slot
layout and hand-over order) against numpy's Cholesky.  They run on the CPU and test
the schedule, not the GPU code's arithmetic (the GPU parity tests do that).

The selected inversion's tile recurrences (csrc/bta_selinv_task.cuh) are checked on a
dense matrix, including the two-product form of a diagonal-chain step.
"""
import re

import numpy as np
import pytest

from tests.conftest import REPO

SRC = (REPO / "pyinla_gb300" / "csrc" / "bta_common.cuh").read_text()
TS = 32


def _const(name: str) -> int:
    m = re.search(rf"\b{name}\s*=\s*(\d+)", SRC)
    assert m, name
    return int(m.group(1))


SLOTS, FULL = _const("POTRF_SLOTS"), _const("POTRF_FULL")


def slot_col(s):
    return s + 2 if s < FULL else 16 + 2 * (s - FULL)


def slot_last(s):
    return s + 2 if s < FULL else 17 + 2 * (s - FULL)


def slot_owner(s):
    return s % 3 if s < FULL else (s - 12) % 3


def column_owner(c):
    for s in range(SLOTS):
        if slot_col(s) <= c <= slot_last(s):
            return slot_owner(s)
    raise AssertionError(c)


def test_slot_maps_match_the_kernel():
    """The three slot maps above restate the constexpr functions of the kernel."""
    for body in ("s < POTRF_FULL ? s + 2 : 16 + 2 * (s - POTRF_FULL)",
                 "s < POTRF_FULL ? s + 2 : 17 + 2 * (s - POTRF_FULL)",
                 "s < POTRF_FULL ? s % 3 : (s - 12) % 3"):
        assert body in SRC, body


def test_slots_cover_columns_2_to_31_once():
    cols = [c for s in range(SLOTS) for c in range(slot_col(s), slot_last(s) + 1)]
    assert sorted(cols) == list(range(2, TS))
    # a pair slot holds rows 16..31 only: both of its columns must start at row >= 16
    assert all(slot_col(s) >= 16 for s in range(FULL, SLOTS))


def test_ring_slot_consumed_before_reuse():
    """Before the pivot warp publishes pivot p+8 (ring slot and barrier id p & 7 again)
    it has received the look-ahead columns p+2 .. p+8; each came from a warp that had
    consumed pivot >= p.  That covers every update warp iff any seven consecutive
    columns have all three owners."""
    for p in range(0, TS - 2 - 8):
        owners = {column_owner(c) for c in range(p + 2, p + 9)}
        assert owners == {0, 1, 2}, p


def _replay(A):
    """The kernel's operation order: pivot warp (lane = row) and update-warp slots."""
    S = A.copy()
    lanes = np.arange(TS)
    prow, half = 16 + (lanes & 15), lanes >> 4
    acc = {}
    for s in range(SLOTS):
        acc[s] = S[lanes, slot_col(s)].copy() if s < FULL else S[prow, slot_col(s) + half].copy()
    ring = {}

    def update_warps(j):
        wf, wp = ring[j], ring[j][prow]
        for s in range(SLOTS):   # the look-ahead column j + 2 first
            if s < FULL and slot_col(s) == j + 2:
                acc[s] = acc[s] - wf * S[j + 2, j]
                S[lanes, j + 2] = acc[s]
            elif s >= FULL and j + 2 in (slot_col(s), slot_col(s) + 1):
                acc[s] = acc[s] - wp * S[slot_col(s) + half, j]
                m = (slot_col(s) + half) == j + 2
                S[prow[m], j + 2] = acc[s][m]
        for s in range(SLOTS):
            if slot_last(s) <= j + 2:
                continue
            if s < FULL:
                acc[s] = acc[s] - wf * S[slot_col(s), j]
            elif slot_col(s) > j + 2:
                acc[s] = acc[s] - wp * S[slot_col(s) + half, j]

    u0 = S[:, 0].copy()
    d = np.zeros(TS)
    d[0] = u0[0]
    w = u0 / d[0]
    ring[0] = w.copy()
    update_warps(0)
    a, ub = S[:, 1].copy(), u0[1]
    for k in range(1, TS):
        a = a - w * ub
        u = np.where(lanes >= k, a, 0.0)
        d[k] = a[k]
        S[:, k] = u
        if k < TS - 1:
            an = S[:, k + 1].copy()
            w = u / d[k]
            ub = u[k + 1]
            if k < TS - 2:
                ring[k] = w.copy()
                update_warps(k)
            a = an
    return S / np.sqrt(d)[None, :]


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_replayed_schedule_is_cholesky(seed):
    rng = np.random.default_rng(seed)
    M = rng.standard_normal((TS, TS))
    A = M @ M.T + TS * np.eye(TS)
    L = _replay(A)
    np.testing.assert_allclose(L, np.linalg.cholesky(A), rtol=0, atol=1e-12 * np.abs(A).max())
    assert not np.triu(L, 1).any()


def test_selected_inversion_tile_recurrences():
    """The tile Takahashi recurrences of the selected inversion (csrc/bta_selinv_task.cuh)
    on a dense SPD matrix cut into 8 x 8 tiles, with G(l, c) = F(l, c) F(c, c)^-1 and
    C_c = F(c, c)^-T F(c, c)^-1:
      Sigma(j, c) = -sum_{l>c} Sigma(j, l) G(l, c)            (j > c)
      Sigma(c, c) = C_c - sum_{l>c} Sigma(l, c)^T G(l, c)
    and the two-product form of one column step of the diagonal chain: with
    G = G(c, c-1) and P = -sum_{l>c} Sigma(c, l) G(l, c-1) (the partial sum of the
    sub-diagonal tile), Sigma(c, c-1) = P - Sigma(c, c) G and
      Sigma(c-1, c-1) = C_{c-1} - Z' - P^T G + G^T Sigma(c, c) G,
    Z' = sum_{l>c} Sigma(l, c-1)^T G(l, c-1)."""
    t, nb = 8, 6
    rng = np.random.default_rng(7)
    M = rng.standard_normal((t * nb, t * nb))
    A = M @ M.T + t * nb * np.eye(t * nb)
    F = np.linalg.cholesky(A)
    S = np.linalg.inv(A)
    blk = lambda X, r, c: X[r * t:(r + 1) * t, c * t:(c + 1) * t]
    Finv = [np.linalg.inv(blk(F, c, c)) for c in range(nb)]
    G = {(l, c): blk(F, l, c) @ Finv[c] for c in range(nb) for l in range(c + 1, nb)}
    C = [Finv[c].T @ Finv[c] for c in range(nb)]
    tol = 1e-12 * np.abs(S).max()
    for c in range(nb):
        for j in range(c + 1, nb):
            rhs = -sum(blk(S, j, l) @ G[(l, c)] for l in range(c + 1, nb))
            np.testing.assert_allclose(blk(S, j, c), rhs, atol=tol)
        diag = C[c] - sum((blk(S, l, c).T @ G[(l, c)] for l in range(c + 1, nb)), np.zeros((t, t)))
        np.testing.assert_allclose(blk(S, c, c), diag, atol=tol)
    for c in range(1, nb):
        Gc = G[(c, c - 1)]
        P = -sum((blk(S, c, l) @ G[(l, c - 1)] for l in range(c + 1, nb)), np.zeros((t, t)))
        np.testing.assert_allclose(blk(S, c, c - 1), P - blk(S, c, c) @ Gc, atol=tol)
        Zp = sum((blk(S, l, c - 1).T @ G[(l, c - 1)] for l in range(c + 1, nb)), np.zeros((t, t)))
        two_product = C[c - 1] - Zp - P.T @ Gc + Gc.T @ blk(S, c, c) @ Gc
        np.testing.assert_allclose(blk(S, c - 1, c - 1), two_product, atol=tol)
