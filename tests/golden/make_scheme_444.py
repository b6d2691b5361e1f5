"""Writes scheme_444_z2_r47.txt: a Z2 scheme for 4x4x4 matrix multiplication of
rank 47 (or --target), found by this engine's fast-mode search from the naive
rank-64 scheme (65,536 walks, plus transition after 10^5 flips without a rank
drop) and verified exactly (Brent equations on the GPU and again here on the
CPU).  The file is in the reference's text format ("n1 n2 n3 m", then the m
rows of U, V and W) and feeds the post-search (reducer / minimizer) tests and
benchmark.  Needs a GPU:

    python tests/golden/make_scheme_444.py --target 47 --seconds 600 --seed 1
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import flipgraphgpu_gb300 as fg  # noqa: E402


def brent_ok(n, m, fac):
    """Exact Z2 check of the 4x4x4-style Brent equations (scheme_z2.cu:3-29 layout)."""
    n1, n2, n3 = n
    nn0, nn1, nn2 = n1 * n2, n2 * n3, n3 * n1
    for i in range(nn0):
        for j in range(nn1):
            acc = 0
            for t in range(m):
                if (int(fac[0, t]) >> i) & (int(fac[1, t]) >> j) & 1:
                    acc ^= int(fac[2, t])
            target = (1 << ((j % n3) * n1 + i // n2)) if (i % n2 == j // n3) else 0
            if acc & ((1 << nn2) - 1) != target:
                return False
    return True


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--target", type=int, default=47)
    ap.add_argument("--seconds", type=float, default=600.0)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--walks", type=int, default=65536)
    ap.add_argument("--out", default=os.path.join(HERE, "scheme_444_z2_r47.txt"))
    a = ap.parse_args()
    n = (4, 4, 4)
    t0 = time.time()
    with fg.Engine(a.walks, 64, "z2", "fast", a.seed, 5000, 100000, 0.01, 0.0) as eng:
        eng.init_naive(*n)
        best = 64
        while time.time() - t0 < a.seconds:
            st = eng.run(1)
            best = min(best, st["min_best_rank"])
            if best <= a.target:
                break
        rec = eng.records()
        ok = eng.validate(best=True)
    order = np.argsort(rec.best_m, kind="stable")
    for w in order:
        m = int(rec.best_m[w])
        if not ok[w] or not brent_ok(n, m, rec.best_fac[w]):
            continue
        nn = [n[0] * n[1], n[1] * n[2], n[2] * n[0]]
        lines = [f"{n[0]} {n[1]} {n[2]} {m}"]
        for c in range(3):
            for t in range(m):
                word = int(rec.best_fac[w, c, t])
                lines.append(" ".join(str((word >> b) & 1) for b in range(nn[c])))
        with open(a.out, "w") as f:
            f.write("\n".join(lines) + "\n")
        print(f"rank {m} (walk {w}) after {time.time() - t0:.1f} s -> {a.out}")
        return 0
    print("no verified scheme", file=sys.stderr)
    return 1


if __name__ == "__main__":
    sys.exit(main())
