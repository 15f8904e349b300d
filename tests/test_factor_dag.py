"""CPU replay of the factorization's task DAG.

The dataflow kernels hand out tasks in ticket order and a task only ever waits for
flags published by tasks with smaller tickets, which is what keeps the persistent
grid from deadlocking whatever its size.  This restates the task list of
factor_task_list (csrc/bta_api.cu) -- both elimination orders (top-down, and both ends
towards the middle block), with and without the split of the diagonal and feeder tiles'
product loops into partial and tail tasks -- together with the flags each task body
waits on (the product steps of step_range / step_src in csrc/bta_factor_task.cuh, the
diagonal factor tile, the feeder and partial flags), and checks that every waited flag
is published, by a smaller ticket.  With structurally zero coupling tiles (the kf
array of launch_coupling_kfirst) the loops leave out the terms on them, and an L tile
that is itself structurally zero skips its solve: the tests also check that the split
loops then still cover exactly the live terms.
"""
import pytest


def geom(nt, b, a, twist=True):
    B = (b + 31) // 32
    sep = (nt // 2 if nt >= 3 else nt - 1) if twist else nt - 1

    def nxt(i): return i + 1 if i < sep else (i - 1 if i > sep else -1)

    def lslot(i): return i if i < sep else (i - 1 if i > sep else -1)

    def nprev(i):
        if i < sep: return 1 if i > 0 else 0
        if i > sep: return 1 if i < nt - 1 else 0
        return (1 if sep > 0 else 0) + (1 if sep < nt - 1 else 0)

    def prev(i, k):
        if i < sep: return i - 1
        if i > sep: return i + 1
        return sep - 1 if (k == 0 and sep > 0) else sep + 1

    def vrows(r): return min(32, b - r * 32)

    def feeder_kind(i, c): return 1 if c + 1 < B else (2 if nxt(i) >= 0 else 0)

    def quarters(i, c):
        fk = feeder_kind(i, c)
        if not fk: return 0
        rows = vrows(c + 1) if fk == 1 else vrows(0)
        return (rows + 7) // 8

    return dict(nt=nt, b=b, a=a, B=B, sep=sep, nxt=nxt, lslot=lslot, nprev=nprev, prev=prev, fk=feeder_kind,
                nq=quarters)


def has_partial(g, i, c):
    if c >= 1: return g["nprev"](i) * g["B"] + c - 1 > 0
    return g["nprev"](i) > 0 and g["B"] >= 2


def feeder_has_partial(g, i, c):
    fk = g["fk"](i, c)
    if fk == 1: return has_partial(g, i, c)
    return fk == 2 and g["B"] >= 3


def interleave(n1, n2, u):
    mn = min(n1, n2)
    if u < 2 * mn: return u & 1, u >> 1
    return (0 if n1 > mn else 1), mn + (u - 2 * mn)


def task_list(g, split=True):
    B, nt = g["B"], g["nt"]
    t = []

    def partials(i, c):
        if has_partial(g, i, c): t.append(("DPART", i, c, c))
        if feeder_has_partial(g, i, c):
            t.append(("FPARTO", i, c + 1, c) if g["fk"](i, c) == 1 else ("FPARTL", i, 0, c))

    def col(i, c):
        fk = g["fk"](i, c)
        if split and c == 0 and g["nprev"](i) > 1: partials(i, 0)
        if split and c == 0 and B >= 2: partials(i, 1)
        ft = "T" if split and feeder_has_partial(g, i, c) else ""
        if fk == 1: t.append(("PREO" + ft, i, c + 1, c))
        if fk == 2: t.append(("PREL" + ft, i, 0, c))
        t.append(("TAIL" if split and has_partial(g, i, c) else "DIAG", i, c, c))
        for q in range(g["nq"](i, c)): t.append(("FEEDQ", i, q, c))
        for r in range(c + 1 + (1 if fk == 1 else 0), B): t.append(("OFFD", i, r, c))
        if g["nxt"](i) >= 0:
            for r in range(1 if fk == 2 else 0, B): t.append(("LOW", i, r, c))
        if g["a"] > 0: t.append(("ARW", i, 0, c))
        if split and c + 2 < B: partials(i, c + 2)
        n = g["nxt"](i)
        if split and n >= 0 and g["nprev"](n) == 1 and c == (B - 2 if B >= 2 else 0): partials(n, 0)

    s = g["sep"]
    n1, n2 = s * B, (nt - 1 - s) * B
    for u in range(n1 + n2):
        ch, k = interleave(n1, n2, u)
        col(k // B if ch == 0 else nt - 1 - k // B, k % B)
    for c in range(B): col(s, c)
    if g["a"] > 0: t.append(("TIP", 0, 0, 0))
    return t


def steps(g, ttype, mode, i, col, r=None, kf=None):
    """(isprev, pb, k) of each product step, mirroring step_range / step_src: a
    neighbour's term k uses its coupling tiles (r, k), (col, k) (the arrow's only
    (col, k)), an L target's own-block term k its own tile (r, k); terms on a
    structurally zero tile (k < kf[slot][row]) are left out."""
    B = g["B"]
    r = col if r is None else r
    kfirst = (lambda ls, row: 0) if kf is None else (lambda ls, row: kf[ls][row])
    np_ = g["nprev"](i) if ttype != "LOW" else 0
    out = []
    for q in range(np_):
        pb = g["prev"](i, q)
        ls = g["lslot"](pb)
        k0, k1 = kfirst(ls, col), B
        if ttype != "ARW":
            k0 = max(k0, kfirst(ls, r))
        if mode == 1 and col == 0:
            k1 = B - 1
        if mode == 2:
            k0 = max(k0, B - 1) if col == 0 else B
        out += [(True, pb, k) for k in range(k0, k1)]
    kin = kfirst(g["lslot"](i), r) if ttype == "LOW" else 0
    kend = col
    if mode == 1:
        kend = col - 1
    if mode == 2:
        kin = col if col == 0 else max(kin, col - 1)
    out += [(False, i, k) for k in range(kin, kend)]
    return out


def full_steps_unskipped(g, ttype, i, col):
    """The loop without skipping, written out directly: every neighbour column, then
    the own block's columns k < col."""
    B = g["B"]
    np_ = g["nprev"](i) if ttype != "LOW" else 0
    return [(True, g["prev"](i, q), k) for q in range(np_) for k in range(B)] + [(False, i, k) for k in range(col)]


def check(nt, b, a, twist=True, split=True, kf=None):
    g = geom(nt, b, a, twist)
    B = g["B"]
    tl = task_list(g, split)
    prod = {}

    def pub(flag, t):
        prod.setdefault(flag, t)

    for t, (ty, i, r, c) in enumerate(tl):
        if ty in ("DIAG", "TAIL"): pub(("fD", i, c, c), t)
        elif ty == "OFFD": pub(("fD", i, r, c), t)
        elif ty == "LOW": pub(("fL", g["lslot"](i), r, c), t)
        elif ty == "ARW": pub(("fR", i, c), t)
        elif ty in ("PREO", "PREL", "PREOT", "PRELT"): pub(("feed", i, c), t)
        elif ty == "DPART": pub(("dpart", i, c), t)
        elif ty in ("FPARTO", "FPARTL"): pub(("fpart", i, c), t)
        elif ty == "FEEDQ":
            fk = g["fk"](i, c)
            fl = ("fD", i, c + 1, c) if fk == 1 else ("fL", g["lslot"](i), 0, c)
            if r == g["nq"](i, c) - 1: prod[fl] = t   # the flag is complete with the last group
        elif ty == "TIP": pub(("fT",), t)
    bad = []
    for t, (ty, i, r, c) in enumerate(tl):
        waits = []
        if ty == "FEEDQ":
            waits = [("feed", i, c), ("fD", i, c, c)]
        elif ty == "TIP":
            waits = [("fR", k // B, k % B) for k in range(nt * B)]
        else:
            mode = {"DPART": 1, "FPARTO": 1, "FPARTL": 1, "TAIL": 2, "PREOT": 2, "PRELT": 2}.get(ty, 0)
            kind = {"PREO": "OFFD", "PREL": "LOW", "PREOT": "OFFD", "PRELT": "LOW", "FPARTO": "OFFD",
                    "FPARTL": "LOW", "DPART": "DIAG", "TAIL": "DIAG"}.get(ty, ty)
            if ty == "TAIL": waits.append(("dpart", i, c))
            if ty in ("PREOT", "PRELT"): waits.append(("fpart", i, c))
            for isprev, pb, k in steps(g, kind, mode, i, c, r, kf):
                if isprev:
                    ls = g["lslot"](pb)
                    sa = ("fR", pb, k) if kind == "ARW" else ("fL", ls, r, k)
                    sb = ("fL", ls, c, k)
                else:
                    lsi = g["lslot"](i)
                    sa = ("fR", i, k) if kind == "ARW" else (("fL", lsi, r, k) if kind == "LOW" else ("fD", i, r, k))
                    sb = ("fD", i, c, k)
                waits += [sa, sb]
            if ty in ("OFFD", "ARW") or (ty == "LOW" and (kf is None or c >= kf[g["lslot"](i)][r])):
                waits.append(("fD", i, c, c))
        for w in waits:
            if w not in prod:
                bad.append(("never published", w, t, tl[t]))
            elif prod[w] >= t:
                bad.append(("later ticket", w, prod[w], t, tl[t]))
    tails = {(i, c) for (ty, i, r, c) in tl if ty == "TAIL"}
    parts = {(i, c) for (ty, i, r, c) in tl if ty == "DPART"}
    ftails = {(i, c) for (ty, i, r, c) in tl if ty in ("PREOT", "PRELT")}
    fparts = {(i, c) for (ty, i, r, c) in tl if ty in ("FPARTO", "FPARTL")}
    assert tails == parts, tails ^ parts
    assert ftails == fparts, ftails ^ fparts
    assert not bad, bad[:5]
    return True


SHAPES = [(1, 40, 0), (1, 70, 5), (2, 33, 1), (2, 64, 0), (3, 32, 1), (3, 96, 2), (4, 40, 3), (5, 45, 5),
          (6, 70, 5), (7, 33, 2), (9, 64, 0), (16, 128, 4), (24, 96, 4), (8, 1, 0), (6, 5, 2), (17, 100, 3)]


@pytest.mark.parametrize("split", [True, False])
@pytest.mark.parametrize("twist", [True, False])
@pytest.mark.parametrize("nt,b,a", SHAPES)
def test_factor_tasks_wait_only_on_earlier_tickets(nt, b, a, twist, split):
    assert check(nt, b, a, twist, split)


def test_two_sided_order_halves_the_chain():
    """The two chains of the two-sided order have about nt/2 blocks each."""
    g = geom(128, 1024, 6, True)
    assert g["sep"] == 64
    top = [i for i in range(128) if g["nxt"](i) == i + 1]
    bottom = [i for i in range(128) if g["nxt"](i) == i - 1]
    assert len(top) == 64 and len(bottom) == 63 and g["nprev"](64) == 2


def random_kf(g, seed):
    """First nonzero column tile per coupling-slot row tile: banded (row tile r starts
    near r - 2), with some empty row tiles (B) and some starting at 0."""
    rng = __import__("random").Random(seed)
    B = g["B"]
    out = []
    for _ in range(max(g["nt"] - 1, 0)):
        row = []
        for r in range(B):
            u = rng.random()
            row.append(B if u < 0.1 else (0 if u < 0.2 else max(0, r - rng.randint(0, 3))))
        out.append(row)
    return out


@pytest.mark.parametrize("nt,b,a", SHAPES)
def test_skipped_structural_zeros_keep_the_dag(nt, b, a):
    g = geom(nt, b, a, True)
    assert check(nt, b, a, True, True, random_kf(g, nt * 1000 + b))


@pytest.mark.parametrize("nt,b,a", [(3, 96, 2), (5, 45, 5), (16, 128, 4), (17, 100, 3), (6, 5, 2)])
def test_partial_and_tail_cover_the_live_steps(nt, b, a):
    """Partial + tail = the full loop's steps, and the full loop = the unskipped loop
    minus exactly the terms on structurally zero tiles."""
    for twist in (True, False):
        g = geom(nt, b, a, twist)
        kf = random_kf(g, nt + b)
        B = g["B"]
        for i in range(nt):
            for col in range(B):
                for ttype, r in (("DIAG", col), ("OFFD", min(col + 1, B - 1)), ("LOW", 0), ("LOW", B - 1),
                                 ("ARW", 0)):
                    full = steps(g, ttype, 0, i, col, r, kf)
                    split = steps(g, ttype, 1, i, col, r, kf) + steps(g, ttype, 2, i, col, r, kf)
                    assert sorted(split) == sorted(full), (i, col, ttype, r)

                    def live(st):
                        isprev, pb, k = st
                        if isprev:
                            ls = g["lslot"](pb)
                            ok = k >= kf[ls][col]
                            return ok and (ttype == "ARW" or k >= kf[ls][r])
                        return ttype != "LOW" or k >= kf[g["lslot"](i)][r]

                    want = [st for st in full_steps_unskipped(g, ttype, i, col) if live(st)]
                    assert full == want, (i, col, ttype, r)
