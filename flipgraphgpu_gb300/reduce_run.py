"""One batch of additions reducers from the command line (profiling and quick checks).

    python -m flipgraphgpu_gb300.reduce_run --scheme tests/golden/scheme_444_z2_r47.txt --count 8192

Reads one scheme in the additions_reducer text layout ("n1 n2 n3 m" and its
rows), runs --launches launches of --count reducers over it and prints runs/s
and the best addition count.
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
    a = ap.parse_args()
    tok = [int(x) for x in open(a.scheme).read().split()]
    n, m = tok[:3], tok[3]
    nn = [n[0] * n[1], n[1] * n[2], n[2] * n[0]]
    coef = np.zeros((1, 3, m, 64), np.int8)
    p = 4
    for c in range(3):
        for t in range(m):
            coef[0, c, t, :nn[c]] = tok[p:p + nn[c]]
            p += nn[c]
    red = Reducer(n, m, coef, count=a.count, schemes=1, seed=a.seed, threads=a.threads)
    red.run()  # warm-up
    t = time.perf_counter()
    best = None
    for _ in range(a.launches):
        out = red.run()
        adds = out["additions"].sum(axis=1)
        best = int(adds.min()) if best is None else min(best, int(adds.min()))
    dt = time.perf_counter() - t
    red.close()
    print(json.dumps({"scheme": a.scheme, "count": a.count, "launches": a.launches,
                      "runs_per_s": a.count * a.launches / dt, "best_additions": best}))


if __name__ == "__main__":
    main()
