#!/usr/bin/env python3
"""Generates the golden fixtures under tests/golden/ from the reference itself.

The reference (dronperminov/FlipGraphGPU) has no tests and ships no fixtures,
so its behaviour is pinned by running its own CUDA code on a GB300 and
recording what it does.  This script is run in two steps:

  --run DIR   (on a GPU machine; needs the staged reference sources that
              oracle/build_ref.sh puts under oracle/_ref/)
              builds the reference, runs oracle/ref_harness (which drives the
              reference's unmodified kernels) and the reference's three
              executables, and writes raw outputs to DIR.
  --pack DIR  (anywhere) copies the raw outputs into tests/golden/ as gzip
              files plus a manifest.

Walk dumps hold the complete per-walk state after each launch (scheme,
FlipSet lists, flips counter, best rank, best scheme) and the exact XORWOW
draw tape each walk consumed; the CPU oracle replays the tape and must
reproduce every byte.  Binary layout: see tests/golden/golden_io.py.
"""
import argparse
import glob
import gzip
import json
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
import golden_io  # noqa: E402

# (name, ring, n1, n2, n3, walks, iterations, plus_iterations, expand_p, reduce_p, seed, launches)
WALK_CASES = [
    ("z2_333", "z2", 3, 3, 3, 6, 300, 50, 0.01, 0.0, 11, 2),
    ("z2_222", "z2", 2, 2, 2, 6, 200, 20, 0.01, 0.0, 12, 2),
    ("z2_444", "z2", 4, 4, 4, 3, 300, 100, 0.01, 0.0, 13, 1),
    ("z2_234_expand", "z2", 2, 3, 4, 4, 300, 30, 60.0, 0.0, 14, 1),
    ("z2_345_reduce", "z2", 3, 4, 5, 3, 200, 60, 0.01, 40.0, 15, 1),
    ("zt_333", "zt", 3, 3, 3, 4, 100, 40, 0.01, 0.0, 21, 2),
    ("zt_223_expand", "zt", 2, 2, 3, 6, 150, 20, 40.0, 0.0, 22, 1),
    ("zt_444", "zt", 4, 4, 4, 2, 30, 100, 0.01, 0.0, 23, 1),
    ("zt_233_reduce", "zt", 2, 3, 3, 4, 150, 30, 0.01, 40.0, 24, 1),
]

# Walks with the resize meta-operators on (FlipGraph::run's resize loop):
# (name, ring, n1, n2, n3, walks, iterations, plus_iterations, expand_p, reduce_p, seed, launches, resize_p)
RESIZE_CASES = [
    ("z2_222_resize", "z2", 2, 2, 2, 12, 150, 40, 0.01, 0.0, 41, 4, 0.5),
    ("z2_233_resize", "z2", 2, 3, 3, 8, 200, 60, 0.01, 0.0, 42, 3, 0.8),
    ("zt_222_resize", "zt", 2, 2, 2, 6, 50, 30, 0.01, 0.0, 51, 4, 0.6),
    ("zt_223_resize", "zt", 2, 2, 3, 6, 60, 40, 0.01, 0.0, 52, 3, 0.9),
]

# Walks with the sandwiching and basis-change moves (no resizing):
# (name, ring, n1, n2, n3, walks, iterations, plus_iterations, expand_p, reduce_p, seed, launches,
#  resize_p, sandwiching_p, basis_p)
MOVE_CASES = [
    ("z2_333_moves", "z2", 3, 3, 3, 8, 300, 80, 0.01, 0.0, 61, 2, 0.0, 30.0, 30.0),
    ("z2_234_moves", "z2", 2, 3, 4, 8, 300, 80, 0.01, 0.0, 62, 2, 0.0, 60.0, 10.0),
    ("zt_333_moves", "zt", 3, 3, 3, 4, 60, 40, 0.01, 0.0, 63, 2, 0.0, 10.0, 20.0),
]

# Long walks used only to produce low-rank input schemes for the reducer and
# minimizer runs (their dumps are not kept as fixtures).
SOURCE_WALKS = [
    ("src_zt_333", "zt", 3, 3, 3, 64, 3000, 2000, 0.01, 0.0, 31, 2),
    ("src_z2_333", "z2", 3, 3, 3, 64, 4000, 2000, 0.01, 0.0, 32, 3),
]


def run(cmd, **kw):
    print("+", " ".join(cmd), flush=True)
    return subprocess.run(cmd, check=True, **kw)


def binary(ring, name):
    return os.path.join(ROOT, "oracle", "_ref", f"{ring}-{os.uname().machine}", name)


def harness(ring):
    return binary(ring, "ref_harness")


def walk(out_dir, case, tape=True):
    name, ring, n1, n2, n3, S, iters, plus, ep, rp, seed, launches = case[:12]
    path = os.path.join(out_dir, f"walk_{name}.bin")
    env = dict(os.environ)
    if not tape:
        env["FG_NO_TAPE"] = "1"
    extra = [repr(x) for x in case[12:]]
    run([harness(ring), "walk", str(n1), str(n2), str(n3), str(S), str(iters), str(plus),
         repr(ep), repr(rp), str(seed), str(launches), path] + extra, env=env)
    return path


def best_scheme_text(dump, header=True):
    """Lowest-rank best scheme of a walk dump as reference input text."""
    last = dump["launches"][-1]
    k = min(range(len(last)), key=lambda w: last[w]["best"]["m"])
    s = last[k]["best"]
    return golden_io.scheme_to_text(s, dump["ring"], header=header), s


# flip_graph with resizing (Z2 build): the run is bounded by time, so only files
# saved in iterations below RESIZE_CLI_ITERATIONS are kept as the fixture.
RESIZE_CLI_ARGS = ["-n1", "2", "-n2", "2", "-n3", "3", "--schemes", "64", "--max-iterations", "300",
                   "--plus-iterations", "100", "--resize-probability", "0.3", "--seed", "73"]
RESIZE_CLI_ITERATIONS = 4
# The reference's default configuration: the ZT build with its default resize
# probability (0.2) -- no resize flag at all.  Its ternary products are slow in
# the reference, which completes only 3 full iterations in the time limit.
RESIZE_CLI_ARGS_ZT = ["-n1", "2", "-n2", "2", "-n3", "3", "--schemes", "48", "--max-iterations", "200",
                      "--plus-iterations", "100", "--seed", "75"]
RESIZE_CLI_ITERATIONS_ZT = 3
# Sandwiching and basis-change moves through the executables: with resizing
# (Z2) and without (ZT, whose sandwiching is empty in the reference).
MOVES_CLI_ARGS = ["-n1", "2", "-n2", "3", "-n3", "3", "--schemes", "64", "--max-iterations", "300",
                  "--plus-iterations", "100", "--resize-probability", "0.3", "--sandwiching-probability", "20",
                  "--basis-probability", "30", "--seed", "77"]
MOVES_CLI_ITERATIONS = 3
MOVES_CLI_ARGS_ZT = ["-n1", "3", "-n2", "3", "-n3", "3", "--schemes", "48", "--max-iterations", "200",
                     "--plus-iterations", "100", "--resize-probability", "0", "--sandwiching-probability", "10",
                     "--basis-probability", "40", "--seed", "79"]
MOVES_CLI_ITERATIONS_ZT = 4

# (ring, fixture directory, flags, iterations kept)
CLI_CASES = [
    ("z2", "cli_flip_graph_resize", RESIZE_CLI_ARGS, RESIZE_CLI_ITERATIONS),
    ("zt", "cli_flip_graph_resize_zt", RESIZE_CLI_ARGS_ZT, RESIZE_CLI_ITERATIONS_ZT),
    ("z2", "cli_flip_graph_moves", MOVES_CLI_ARGS, MOVES_CLI_ITERATIONS),
    ("zt", "cli_flip_graph_moves_zt", MOVES_CLI_ARGS_ZT, MOVES_CLI_ITERATIONS_ZT),
]


def cli_resize(out_dir):
    for ring, sub, args, K in CLI_CASES:
        fg_dir = os.path.join(out_dir, sub)
        os.makedirs(fg_dir, exist_ok=True)
        with open(os.path.join(out_dir, sub + ".log"), "w") as log:
            subprocess.run(["timeout", "20", binary(ring, "flip_graph")] + args + ["--path", fg_dir],
                           stdout=log, stderr=subprocess.STDOUT)
        for name in os.listdir(fg_dir):
            it = int(name.split("_iteration")[1].split("_")[0])
            if it >= K:
                os.remove(os.path.join(fg_dir, name))


# SchemeZ2::tryReduceGauss (never called by the reference's walk) on the schemes
# of gauss_input_z2.txt.gz (made by make_gauss_input.py), one call per scheme.
GAUSS_SEEDS = [91, 92]


def gauss(out_dir):
    inp = os.path.join(out_dir, "gauss_input_z2.txt")
    with gzip.open(os.path.join(HERE, "gauss_input_z2.txt.gz"), "rb") as f, open(inp, "wb") as o:
        o.write(f.read())
    for seed in GAUSS_SEEDS:
        run([harness("z2"), "gauss", inp, str(seed), os.path.join(out_dir, f"gauss_z2_s{seed}.bin")])
    os.remove(inp)


# The reducer's --max-flips mode (flipSchemesKernel + runReducersKernel with
# independent=false + updateBestTogether) on input_zt_333.txt:
# (count, schemes, seed, max_flips, iterations).
REDUCE_FLIP_CASES = [(12, 6, 43, 20, 3)]


def reduce_flips(out_dir):
    inp = os.path.join(out_dir, "input_zt_333.txt")
    if not os.path.exists(inp):
        with gzip.open(os.path.join(HERE, "input_zt_333.txt.gz"), "rb") as f, open(inp, "wb") as o:
            o.write(f.read())
    for count, schemes, seed, flips, iterations in REDUCE_FLIP_CASES:
        run([harness("zt"), "reduce", inp, str(count), str(schemes), str(seed),
             os.path.join(out_dir, f"flipreduce_zt_333_f{flips}.bin"), str(flips), str(iterations)])


def do_run(out_dir, resize_only=False, cli_only=False, gauss_only=False, flips_only=False):
    os.makedirs(out_dir, exist_ok=True)
    run([os.path.join(ROOT, "oracle", "build_ref.sh")])
    if flips_only:
        reduce_flips(out_dir)
        os.remove(os.path.join(out_dir, "input_zt_333.txt"))
        return
    if gauss_only:
        gauss(out_dir)
        return
    if cli_only:
        cli_resize(out_dir)
        return
    for case in RESIZE_CASES + MOVE_CASES:
        walk(out_dir, case)
    gauss(out_dir)
    cli_resize(out_dir)
    if resize_only:
        return
    for case in WALK_CASES:
        walk(out_dir, case)

    # Input schemes for the reducer / minimizer / CLI runs.
    inputs = {}
    for case in SOURCE_WALKS:
        path = walk(out_dir, case, tape=False)
        dump = golden_io.read_walk(path)
        os.remove(path)
        text, s = best_scheme_text(dump)
        inputs[case[1]] = (text, s)
        with open(os.path.join(out_dir, f"input_{case[1]}_333.txt"), "w") as f:
            f.write(text)

    # Reducer kernel, one iteration, per-reducer counts + tapes.
    for ring in ("zt", "z2"):
        inp = os.path.join(out_dir, f"input_{ring}_333.txt")
        run([harness("zt"), "reduce", inp, "12", "1", "41", os.path.join(out_dir, f"reduce_{ring}_333.bin")])

    reduce_flips(out_dir)

    # End-to-end executables (outputs compared file for file).
    ref_reduced = os.path.join(out_dir, "cli_additions_reducer")
    os.makedirs(ref_reduced, exist_ok=True)
    with open(os.path.join(out_dir, "cli_additions_reducer.log"), "w") as log:
        run([binary("zt", "additions_reducer"), "-i", os.path.join(out_dir, "input_zt_333.txt"),
             "-o", ref_reduced, "--count", "64", "--seed", "51"], stdout=log, stderr=subprocess.STDOUT)

    # The minimizer reads "n1 n2 n3 m count" followed by the bodies.
    text, s = inputs["z2"]
    body = golden_io.scheme_to_text(s, "z2", header=False)
    with open(os.path.join(out_dir, "input_minimizer_z2_333.txt"), "w") as f:
        f.write(f"{s['n'][0]} {s['n'][1]} {s['n'][2]} {s['m']} 1\n" + body)
    cm_dir = os.path.join(out_dir, "cli_complexity_minimizer")
    os.makedirs(cm_dir, exist_ok=True)
    with open(os.path.join(out_dir, "cli_complexity_minimizer.log"), "w") as log:
        run([binary("z2", "complexity_minimizer"), "--input-path",
             os.path.join(out_dir, "input_minimizer_z2_333.txt"), "--path", cm_dir,
             "--schemes", "256", "--max-iterations", "2000", "--seed", "61"],
            stdout=log, stderr=subprocess.STDOUT)

    # flip_graph never returns (flip_graph.cu:286): run it for a bounded time;
    # files named with iterations that completed are deterministic.
    fg_dir = os.path.join(out_dir, "cli_flip_graph")
    os.makedirs(fg_dir, exist_ok=True)
    with open(os.path.join(out_dir, "cli_flip_graph.log"), "w") as log:
        subprocess.run(["timeout", "20", binary("z2", "flip_graph"), "-n1", "3", "-n2", "3", "-n3", "3",
                        "--schemes", "128", "--max-iterations", "1000", "--plus-iterations", "300",
                        "--resize-probability", "0", "--path", fg_dir, "--seed", "71"],
                       stdout=log, stderr=subprocess.STDOUT)
    print("golden raw outputs written to", out_dir)


# Reducer tapes above this many draws are dropped from the committed fixture
# (their counts stay; tests skip reducers without a tape).
MAX_REDUCER_TAPE = 4000


def trimmed_reduce(path):
    """Re-serialises a reduce dump, dropping tapes longer than MAX_REDUCER_TAPE."""
    import struct
    d = golden_io.read_reduce(path)
    out = bytearray(struct.pack("<iii", 0x46475231, d["count"], d["seed"]))
    for r in d["reducers"]:
        out += struct.pack("<9i", *r["u"], *r["v"], *r["w"])
        modes = ",".join(r["modes"]).encode()
        out += struct.pack("<i", len(modes)) + modes
    for t in d["tapes"]:
        if t["used"] > MAX_REDUCER_TAPE or t["used"] < 0:
            out += struct.pack("<i", -1)
        else:
            out += struct.pack("<i", t["used"]) + t["draws"].tobytes() + t["uniforms"].tobytes()
    return bytes(out)


def do_pack(raw_dir):
    manifest = {"walk_cases": [list(c) for c in WALK_CASES], "resize_cases": [list(c) for c in RESIZE_CASES],
                "move_cases": [list(c) for c in MOVE_CASES],
                "files": []}
    old = os.path.join(HERE, "manifest.json")
    if os.path.exists(old):  # packing a partial run keeps the fixtures already recorded
        with open(old) as f:
            manifest["files"] = json.load(f).get("files", [])
    for path in sorted(glob.glob(os.path.join(raw_dir, "*.bin")) + glob.glob(os.path.join(raw_dir, "*.txt"))
                       + glob.glob(os.path.join(raw_dir, "*.log"))):
        base = os.path.basename(path)
        dst = os.path.join(HERE, base + ".gz")
        data = trimmed_reduce(path) if base.startswith("reduce_") else open(path, "rb").read()
        with gzip.open(dst, "wb", compresslevel=9) as fo:
            fo.write(data)
        if base not in manifest["files"]:
            manifest["files"].append(base)
    for sub in ["cli_additions_reducer", "cli_complexity_minimizer", "cli_flip_graph"] + [c[1] for c in CLI_CASES]:
        src = os.path.join(raw_dir, sub)
        if os.path.isdir(src):
            dst = os.path.join(HERE, sub)
            shutil.rmtree(dst, ignore_errors=True)
            shutil.copytree(src, dst)
            manifest["files"] += [f"{sub}/{x}" for x in sorted(os.listdir(dst)) if f"{sub}/{x}" not in manifest["files"]]
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--run")
    ap.add_argument("--pack")
    ap.add_argument("--resize-only", action="store_true", help="with --run: only the resize walks")
    ap.add_argument("--cli-only", action="store_true", help="with --run: only the flip_graph runs of CLI_CASES")
    ap.add_argument("--gauss-only", action="store_true", help="with --run: only the tryReduceGauss calls")
    ap.add_argument("--flips-only", action="store_true", help="with --run: only the reducer's --max-flips iterations")
    a = ap.parse_args()
    if a.run:
        do_run(a.run, a.resize_only, a.cli_only, a.gauss_only, a.flips_only)
    if a.pack:
        do_pack(a.pack)
