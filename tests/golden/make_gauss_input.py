#!/usr/bin/env python3
"""Writes tests/golden/gauss_input_z2.txt.gz: Z2 schemes on which the reference's
SchemeZ2::tryReduceGauss is run (make_golden.py --run, `ref_harness gauss`).

Walk states rarely hold a Gauss candidate, so the input mixes
  * schemes the reference's own walks produced (tests/golden/walk_z2_*.bin.gz:
    current and best schemes after each launch), which mostly have none, and
  * the same schemes with planted candidates: for a random term factor a in a
    random component p, terms (a, x_1, c), ..., (a, x_k, c), (a, x_1 ^ ... ^ x_k, c')
    with k = 2, 3 or 4, inserted at random positions (c' = c keeps the scheme
    exact: the planted terms sum to zero; a random c' does not, which the search
    does not look at).
Deterministic (numpy seed 2024).  Text layout: flip_graph's (a count, then per
scheme "n1 n2 n3 m" and the U, V, W rows).
"""
import glob
import gzip
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import golden_io  # noqa: E402

MAX_RANK = 350


def fixture_schemes():
    out = []
    for path in sorted(glob.glob(os.path.join(HERE, "walk_z2_*.bin.gz"))):
        d = golden_io.read_walk(path)
        for launch in d["launches"]:
            for w in launch:
                for key in ("scheme", "best"):
                    s = w[key]
                    out.append((list(s["n"]), [list(map(int, s["uvw"][c][:s["m"]])) for c in range(3)]))
    return out


def plant(n, uvw, rng):
    nn = [n[0] * n[1], n[1] * n[2], n[2] * n[0]]
    m = len(uvw[0])
    p = int(rng.integers(3))
    j, i = (p + 1) % 3, (p + 2) % 3
    if rng.integers(2):
        j, i = i, j
    k = int(rng.integers(2, 5))
    if m + k + 1 > MAX_RANK:
        return None
    a = uvw[p][int(rng.integers(m))]

    def rand(c):
        return int(rng.integers(1, 1 << nn[c]))

    xs = [rand(j) for _ in range(k)]
    target = 0
    for x in xs:
        target ^= x
    if target == 0:
        return None
    c = rand(i)
    last = c if rng.integers(2) else rand(i)
    new = [(x, c) for x in xs] + [(target, last)]
    terms = [tuple(uvw[q][t] for q in range(3)) for t in range(m)]
    for x, y in new:
        term = [0, 0, 0]
        term[p], term[j], term[i] = a, x, y
        terms.insert(int(rng.integers(len(terms) + 1)), tuple(term))
    return [[t[q] for t in terms] for q in range(3)]


def to_text(n, uvw):
    nn = [n[0] * n[1], n[1] * n[2], n[2] * n[0]]
    lines = [f"{n[0]} {n[1]} {n[2]} {len(uvw[0])}"]
    for c in range(3):
        for v in uvw[c]:
            lines.append(" ".join(str((v >> e) & 1) for e in range(nn[c])))
    return "\n".join(lines) + "\n"


def main():
    rng = np.random.default_rng(2024)
    base = fixture_schemes()
    chosen = [base[q] for q in sorted(rng.choice(len(base), 24, replace=False))]
    planted = []
    while len(planted) < 72:
        n, uvw = base[int(rng.integers(len(base)))]
        got = plant(n, uvw, rng)
        if got is not None:
            planted.append((n, got))
    schemes = chosen + planted
    order = rng.permutation(len(schemes))
    text = f"{len(schemes)}\n" + "".join(to_text(*schemes[q]) for q in order)
    with open(os.path.join(HERE, "gauss_input_z2.txt.gz"), "wb") as raw:
        with gzip.GzipFile(fileobj=raw, mode="wb", compresslevel=9, mtime=0) as f:
            f.write(text.encode())
    print(len(schemes), "schemes")


if __name__ == "__main__":
    main()
