"""One batch of walks from the command line (profiling and quick checks).

    python -m flipgraphgpu_gb300.run --shape 4x4x4 --walks 9728 --iterations 500 --mode fast

Runs `--launches` walk launches on naive starting schemes and prints the
library's statistics (accepted / verified flips, ranks, device times).
"""
import argparse
import json

from . import Engine


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--shape", default="3x3x3")
    ap.add_argument("--ring", default="z2", choices=["z2", "zt", "zb"],
                    help="zb (integers, |c| <= 2) runs in the fast mode only")
    ap.add_argument("--walks", type=int, default=1024)
    ap.add_argument("--iterations", type=int, default=1000)
    ap.add_argument("--plus-iterations", type=int, default=100000)
    ap.add_argument("--launches", type=int, default=1)
    ap.add_argument("--mode", default="fast", choices=["fast", "philox", "reference", "learned"])
    ap.add_argument("--candidates", type=int, default=1,
                    help="learned mode: candidates per step, scored by a freshly initialised network when > 1")
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--fast-kernel", default=None, choices=["auto", "thread", "group", "warp"])
    ap.add_argument("--lanes", type=int, default=0, help="group kernel: lanes per walk (4, 8, 16, 32; 0 = auto)")
    ap.add_argument("--fast-split", type=int, default=None,
                    help="fast mode: one thread per walk up to this many slots, one warp per walk above")
    a = ap.parse_args()
    n = tuple(int(x) for x in a.shape.split("x"))
    cap = n[0] * n[1] * n[2] + (4 if a.ring == "zb" else 0)
    with Engine(a.walks, cap, a.ring, a.mode, a.seed, a.iterations, a.plus_iterations) as eng:
        if a.fast_split is not None:
            eng.set_fast_split(a.fast_split)
        if a.fast_kernel is not None:
            eng.set_fast_kernel(a.fast_kernel, a.lanes)
        net = None
        if a.mode == "learned" and a.candidates > 1:
            from . import Mlp
            net = Mlp(seed=a.seed)
            eng.set_proposal(net, candidates=a.candidates)
        eng.init_naive(*n)
        eng.run(1)  # warm-up
        st = eng.run(a.launches)
        if net is not None:
            eng.set_proposal(None, candidates=1)
            net.close()
    print(json.dumps({"shape": a.shape, "ring": a.ring, "walks": a.walks, "iterations": a.iterations, "mode": a.mode,
                      "fast_split": a.fast_split, "fast_kernel": a.fast_kernel, "lanes": a.lanes, **st}))


if __name__ == "__main__":
    main()
