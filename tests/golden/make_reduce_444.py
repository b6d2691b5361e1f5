"""Writes reduce_444_r47.json: the reference's own additions-reducer results
(runReducersKernel, scheme_additions_reducer.cu:433-540, built from the
reference sources by oracle/build_ref.sh) on scheme_444_z2_r47.txt -- per
reducer the additions, fresh variables and naive additions of U, V, W and the
selection modes -- for 32 reducers and seeds 5 and 6.  Runs on a GPU machine:

    ./oracle/build_ref.sh && python tests/golden/make_reduce_444.py

or, from dumps the harness already wrote (FGR1 files):

    python tests/golden/make_reduce_444.py --dump 5:ref5.bin --dump 6:ref6.bin
"""
import argparse
import json
import os
import platform
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import golden_io  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(HERE))
SCHEME = os.path.join(HERE, "scheme_444_z2_r47.txt")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dump", action="append", default=[], help="SEED:FILE of an existing FGR1 dump")
    ap.add_argument("--count", type=int, default=32)
    ap.add_argument("--out", default=os.path.join(HERE, "reduce_444_r47.json"))
    a = ap.parse_args()
    dumps = {}
    for d in a.dump:
        seed, path = d.split(":", 1)
        dumps[int(seed)] = path
    if not dumps:
        exe = os.path.join(ROOT, "oracle", "_ref", f"zt-{platform.machine()}", "ref_harness")
        tmp = tempfile.mkdtemp()
        for seed in (5, 6):
            path = os.path.join(tmp, f"ref{seed}.bin")
            subprocess.run([exe, "reduce", SCHEME, str(a.count), "1", str(seed), path], check=True)
            dumps[seed] = path
    out = {"scheme": os.path.basename(SCHEME), "count": a.count, "seeds": {}}
    for seed, path in sorted(dumps.items()):
        d = golden_io.read_reduce(path)
        out["seeds"][str(seed)] = [{"u": list(r["u"]), "v": list(r["v"]), "w": list(r["w"]), "modes": r["modes"]}
                                  for r in d["reducers"][:d["count"]]]
    with open(a.out, "w") as f:
        json.dump(out, f, indent=1)
    print(a.out)


if __name__ == "__main__":
    main()
