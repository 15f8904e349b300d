"""CPU replay of the factorization's task DAG.

The dataflow kernels hand out tasks in ticket order and a task only ever waits for
flags published by tasks with smaller tickets, which is what keeps the persistent
grid from deadlocking whatever its size.  This restates the task list of
factor_task_list (csrc/bta_api.cu) -- both elimination orders (top-down, and both ends
towards the middle block), with and without the split of the diagonal and feeder tiles'
product loops into partial and tail tasks -- together with the flags each task body
waits on (the product steps of step_range / step_src in csrc/bta_factor_task.cuh, the
diagonal factor tile, the feeder and partial flags), and checks that every waited flag
is published, by a smaller ticket.
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


def steps(g, ttype, mode, i, col):
    """(isprev, pb, k) of each product step, mirroring step_range / step_src."""
    B = g["B"]
    np_ = g["nprev"](i) if ttype != "LOW" else 0
    out = []
    if mode == 1:
        if col == 0:
            for s in range(np_ * (B - 1)): out.append((True, g["prev"](i, s // (B - 1)), s % (B - 1)))
        else:
            for s in range(np_ * B): out.append((True, g["prev"](i, s // B), s % B))
            for k in range(col - 1): out.append((False, i, k))
    elif mode == 2:
        if col == 0:
            for s in range(np_): out.append((True, g["prev"](i, s), B - 1))
        else:
            out.append((False, i, col - 1))
    else:
        for s in range(np_ * B): out.append((True, g["prev"](i, s // B), s % B))
        for k in range(col): out.append((False, i, k))
    return out


def check(nt, b, a, twist=True, split=True):
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
            for isprev, pb, k in steps(g, kind, mode, i, c):
                if isprev:
                    ls = g["lslot"](pb)
                    sa = ("fR", pb, k) if kind == "ARW" else ("fL", ls, r, k)
                    sb = ("fL", ls, c, k)
                else:
                    lsi = g["lslot"](i)
                    sa = ("fR", i, k) if kind == "ARW" else (("fL", lsi, r, k) if kind == "LOW" else ("fD", i, r, k))
                    sb = ("fD", i, c, k)
                waits += [sa, sb]
            if ty in ("OFFD", "LOW", "ARW"):
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
