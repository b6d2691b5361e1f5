"""One batch of additions reducers from the command line (profiling and quick checks).

    python -m flipgraphgpu_gb300.reduce_run --scheme tests/golden/scheme_444_z2_r47.txt --count 8192

Reads one scheme in the additions_reducer text layout ("n1 n2 n3 m" and its
rows), runs --launches launches of --count reducers over it and prints runs/s
and the best addition count.  With --max-flips F each launch after the warm-up
is preceded by the flip pass (schemes 1..--schemes-1 become copies of the
scheme with up to F ternary flips) and reduces with independent=false, as the
additions_reducer executable's --max-flips iterations do.
"""
import argparse
import json
import time

import numpy as np

from . import Reducer


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scheme", required=True)
    ap.add_argument("--count", type=int, default=4096)
    ap.add_argument("--launches", type=int, default=2)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--threads", type=int, default=512, help="threads per reducer block (0: the library's 128)")
    ap.add_argument("--schemes", type=int, default=1, help="schemes side by side (reducer r reduces scheme r %% schemes)")
    ap.add_argument("--max-flips", type=int, default=0, help="flip pass before each timed launch (0: none)")
    a = ap.parse_args()
    if a.max_flips > 0 and a.schemes > a.count:
        ap.error("--schemes must not exceed --count with --max-flips (one stream per scheme)")
    tok = [int(x) for x in open(a.scheme).read().split()]
    n, m = tok[:3], tok[3]
    nn = [n[0] * n[1], n[1] * n[2], n[2] * n[0]]
    coef = np.zeros((1, 3, m, 64), np.int8)
    p = 4
    for c in range(3):
        for t in range(m):
            coef[0, c, t, :nn[c]] = tok[p:p + nn[c]]
            p += nn[c]
    coef = np.tile(coef, (a.schemes, 1, 1, 1))
    independent = a.max_flips == 0
    red = Reducer(n, m, coef, count=a.count, schemes=a.schemes, seed=a.seed, threads=a.threads)
    red.run(independent=independent)  # warm-up
    t = time.perf_counter()
    best = None
    for _ in range(a.launches):
        if a.max_flips > 0:
            red.flip(a.max_flips)
        out = red.run(independent=independent)
        adds = out["additions"].sum(axis=1)
        best = int(adds.min()) if best is None else min(best, int(adds.min()))
    dt = time.perf_counter() - t
    red.close()
    print(json.dumps({"scheme": a.scheme, "count": a.count, "schemes": a.schemes, "max_flips": a.max_flips,
                      "launches": a.launches, "runs_per_s": a.count * a.launches / dt, "best_additions": best}))


if __name__ == "__main__":
    main()
