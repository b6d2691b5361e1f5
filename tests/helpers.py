"""Shared helpers for the tests: golden fixture loading and scheme I/O."""
import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return os.path.join(GOLDEN, name)


def walk_fixtures():
    return sorted(glob.glob(os.path.join(GOLDEN, "walk_*.bin.gz")))


def load_into(batch, w, s, ring, with_lists=True):
    """Copies a golden scheme record into slot w of an oracle/library batch."""
    batch.n[w] = s["n"]
    batch.m[w] = s["m"]
    m = s["m"]
    batch.fac[w] = 0
    if ring == "z2":
        batch.fac[w, :, :m] = s["uvw"]
    else:
        batch.sgn[w] = 0
        batch.valid[w] = 0
        batch.fac[w, :, :m] = s["values"]
        batch.sgn[w, :, :m] = s["signs"]
        batch.valid[w, :, :m] = s["valid"]
    if with_lists:
        batch.list_pairs[w] = 0
        for c in range(3):
            L = len(s["flips"][c])
            batch.list_size[w, c] = L
            batch.list_pairs[w, c, :L] = s["flips"][c]


def diff_walk(batch, w, e, ring):
    """Differences between slot w of a batch and a golden per-launch record."""
    s = e["scheme"]
    errs = []
    m = s["m"]
    if list(batch.n[w]) != list(s["n"]):
        return [f"sizes {list(batch.n[w])} != {list(s['n'])}"]
    if batch.m[w] != m:
        return [f"m {batch.m[w]} != {m}"]
    if ring == "z2":
        if not np.array_equal(batch.fac[w, :, :m], s["uvw"]):
            errs.append("factors")
    else:
        for name, key in (("fac", "values"), ("sgn", "signs"), ("valid", "valid")):
            if not np.array_equal(getattr(batch, name)[w, :, :m], s[key]):
                errs.append(key)
    for c in range(3):
        L = batch.list_size[w, c]
        if L != len(s["flips"][c]) or not np.array_equal(batch.list_pairs[w, c, :L], s["flips"][c]):
            errs.append(f"list {c}")
    if batch.flips[w] != e["flips"]:
        errs.append(f"flips {batch.flips[w]} != {e['flips']}")
    if batch.best_rank[w] != e["best_rank"]:
        errs.append("best_rank")
    b = e["best"]
    best_n = getattr(batch, "best_n", None)
    if best_n is not None and best_n.any() and list(best_n[w]) != list(b["n"]):
        errs.append("best sizes")
    if batch.best_m[w] != b["m"]:
        errs.append("best_m")
    elif ring == "z2" and not np.array_equal(batch.best_fac[w, :, :b["m"]], b["uvw"]):
        errs.append("best factors")
    elif ring == "zt" and not np.array_equal(batch.best_fac[w, :, :b["m"]], b["values"]):
        errs.append("best values")
    return errs


def read_scheme_text(text):
    """Parses 'n1 n2 n3 m' + U,V,W rows into ((n1,n2,n3), m, coef[3][m][64])."""
    vals = [int(x) for x in text.split()]
    n1, n2, n3, m = vals[:4]
    p = 4
    nn = [n1 * n2, n2 * n3, n3 * n1]
    coef = np.zeros((3, m, 64), np.int8)
    for c in range(3):
        for t in range(m):
            coef[c, t, :nn[c]] = vals[p:p + nn[c]]
            p += nn[c]
    return (n1, n2, n3), m, coef


def strassen_blocks(k):
    """A ternary scheme for 2 x 2 x 2k of rank 7k (Strassen's seven products on each 2 x 2 block
    of B's and C's columns), signs canonical (first nonzero of u and v positive): the walks start
    below the naive rank, so random splits (two 16-bit chunks for factors of 20 entries) occur."""
    n1, n2, n3 = 2, 2, 2 * k
    A = lambda i, c: i * n2 + c  # noqa: E731
    terms = []
    for blk in range(k):
        B = lambda r, jj: r * n3 + 2 * blk + jj  # noqa: E731
        C = lambda i, jj: (2 * blk + jj) * n1 + i  # noqa: E731
        terms += [({A(0, 0): 1, A(1, 1): 1}, {B(0, 0): 1, B(1, 1): 1}, {C(0, 0): 1, C(1, 1): 1}),
                  ({A(1, 0): 1, A(1, 1): 1}, {B(0, 0): 1}, {C(1, 0): 1, C(1, 1): -1}),
                  ({A(0, 0): 1}, {B(0, 1): 1, B(1, 1): -1}, {C(0, 1): 1, C(1, 1): 1}),
                  ({A(1, 1): 1}, {B(1, 0): 1, B(0, 0): -1}, {C(0, 0): 1, C(1, 0): 1}),
                  ({A(0, 0): 1, A(0, 1): 1}, {B(1, 1): 1}, {C(0, 0): -1, C(0, 1): 1}),
                  ({A(1, 0): 1, A(0, 0): -1}, {B(0, 0): 1, B(0, 1): 1}, {C(1, 1): 1}),
                  ({A(0, 1): 1, A(1, 1): -1}, {B(1, 0): 1, B(1, 1): 1}, {C(0, 0): 1})]
    neg = lambda d: {e: -x for e, x in d.items()}  # noqa: E731
    out = []
    for u, v, w in terms:
        pu, pv = u[min(u)] > 0, v[min(v)] > 0
        if not pu and not pv:
            u, v = neg(u), neg(v)
        elif not pu:
            u, w = neg(u), neg(w)
        elif not pv:
            v, w = neg(v), neg(w)
        out.append((u, v, w))
    return (n1, n2, n3), out
