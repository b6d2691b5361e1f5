"""The three executables against the reference's own executables' outputs.

tests/golden/cli_* hold the files the reference's flip_graph (Z2 build),
complexity_minimizer (Z2 build) and additions_reducer (ZT build) saved for
the argument lists below; this project's executables, given the same
arguments (plus --ring for the compile-time ring choice), must save the same
files with the same names and byte-identical contents.
"""
import gzip
import os
import platform
import subprocess

import pytest

from helpers import GOLDEN

pytestmark = pytest.mark.gpu
fg = pytest.importorskip("flipgraphgpu_gb300")

BIN = os.path.join(os.path.dirname(fg.__file__), "_lib", platform.machine())


def unpack(name, dst):
    with gzip.open(os.path.join(GOLDEN, name + ".gz"), "rb") as f:
        data = f.read()
    path = os.path.join(dst, name)
    with open(path, "wb") as o:
        o.write(data)
    return path


def run(args, cwd, timeout=300):
    r = subprocess.run(args, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=timeout)
    assert r.returncode == 0, r.stdout[-3000:]
    return r.stdout


def same_files(out_dir, golden_dir):
    want = sorted(os.listdir(os.path.join(GOLDEN, golden_dir)))
    got = sorted(os.listdir(out_dir))
    assert got[:len(want)] == want, (got, want)
    for name in want:
        with open(os.path.join(GOLDEN, golden_dir, name)) as a, open(os.path.join(out_dir, name)) as b:
            assert a.read() == b.read(), name


@pytest.fixture
def work(tmp_path):
    return str(tmp_path)


def test_flip_graph_matches_reference_executable(work):
    out = os.path.join(work, "fg")
    os.makedirs(out)
    log = run([os.path.join(BIN, "flip_graph"), "-n1", "3", "-n2", "3", "-n3", "3", "--schemes", "128",
               "--max-iterations", "1000", "--plus-iterations", "300", "--resize-probability", "0", "--path", out,
               "--seed", "71", "--ring", "Z2", "--max-launches", "5"], work)
    assert "Best rank of 3x3x3 was improved" in log
    same_files(out, "cli_flip_graph")


@pytest.mark.parametrize("case", [0, 1, 2, 3], ids=["resize_z2", "resize_zt_default", "moves_z2", "moves_zt"])
def test_flip_graph_with_resizing_matches_reference_executable(work, case):
    """Resizing, sandwiching and basis changes on: walks change size and basis between launches;
    every scheme the reference saved in its first iterations (report and best-rank table saves) is
    saved here identically.  The second case is the reference's default configuration (ZT build,
    resize probability 0.2, no flag)."""
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden
    ring, sub, args, K = make_golden.CLI_CASES[case]
    if not os.path.isdir(os.path.join(GOLDEN, sub)):
        pytest.skip(f"fixture {sub} not recorded")
    out = os.path.join(work, "fgr")
    os.makedirs(out)
    run([os.path.join(BIN, "flip_graph")] + args + ["--path", out, "--ring", ring.upper(), "--max-launches", str(K)],
        work)
    want = sorted(os.listdir(os.path.join(GOLDEN, sub)))
    got = sorted(x for x in os.listdir(out) if int(x.split("_iteration")[1].split("_")[0]) < K)
    assert want and got == want, (got, want)
    for name in want:
        with open(os.path.join(GOLDEN, sub, name)) as a, open(os.path.join(out, name)) as b:
            assert a.read() == b.read(), name


def test_complexity_minimizer_matches_reference_executable(work):
    inp = unpack("input_minimizer_z2_333.txt", work)
    out = os.path.join(work, "cm")
    os.makedirs(out)
    run([os.path.join(BIN, "complexity_minimizer"), "--input-path", inp, "--path", out, "--schemes", "256",
         "--max-iterations", "2000", "--seed", "61", "--ring", "Z2"], work)
    same_files(out, "cli_complexity_minimizer")


def test_additions_reducer_matches_reference_executable(work):
    inp = unpack("input_zt_333.txt", work)
    out = os.path.join(work, "ar")
    os.makedirs(out)
    run([os.path.join(BIN, "additions_reducer"), "-i", inp, "-o", out, "--count", "64", "--seed", "51"], work)
    same_files(out, "cli_additions_reducer")


def test_additions_reducer_rejects_z2_only_scheme(work):
    inp = unpack("input_z2_333.txt", work)
    r = subprocess.run([os.path.join(BIN, "additions_reducer"), "-i", inp, "-o", work, "--seed", "3"], cwd=work,
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=120)
    assert "Error: readed scheme is invalid" in r.stdout
    # The additive --z2-input flag lifts the integer validity check.
    out = os.path.join(work, "z2")
    os.makedirs(out)
    run([os.path.join(BIN, "additions_reducer"), "-i", inp, "-o", out, "--seed", "3", "--z2-input", "1",
         "--count", "8", "--max-no-improvements", "1"], work)
    assert os.listdir(out)


# ---------------------------------------------------------------- JSON input
# The executables read the JSON they save (a file, or a directory of files) wherever they
# read the reference's text: the same run from JSON and from the equivalent text is
# identical, and on the reference's own inputs it still matches the reference's outputs.

def to_json(src, dst):
    run([os.path.join(BIN, "scheme_converter"), "-i", src, "-o", dst, "--to", "json"], os.path.dirname(dst))
    return dst


def test_complexity_minimizer_reads_json_input(work):
    js = to_json(unpack("input_minimizer_z2_333.txt", work), os.path.join(work, "in.json"))
    out = os.path.join(work, "cm")
    os.makedirs(out)
    run([os.path.join(BIN, "complexity_minimizer"), "--input-path", js, "--path", out, "--schemes", "256",
         "--max-iterations", "2000", "--seed", "61", "--ring", "Z2"], work)
    same_files(out, "cli_complexity_minimizer")


def test_additions_reducer_reads_json_input(work):
    js = to_json(unpack("input_zt_333.txt", work), os.path.join(work, "in.json"))
    out = os.path.join(work, "ar")
    os.makedirs(out)
    run([os.path.join(BIN, "additions_reducer"), "-i", js, "-o", out, "--count", "64", "--seed", "51"], work)
    same_files(out, "cli_additions_reducer")
    # Its own output, expanded back, is a valid input again.
    again = os.path.join(work, "ar2")
    os.makedirs(again)
    reduced = os.path.join(out, sorted(os.listdir(out))[0])
    run([os.path.join(BIN, "additions_reducer"), "-i", reduced, "-o", again, "--count", "64", "--seed", "51"], work)
    same_files(again, "cli_additions_reducer")


def test_flip_graph_resumes_from_its_own_json(work):
    first = os.path.join(work, "first")
    os.makedirs(first)
    base = [os.path.join(BIN, "flip_graph"), "-n1", "3", "-n2", "3", "-n3", "3", "--schemes", "128",
            "--max-iterations", "1000", "--plus-iterations", "300", "--resize-probability", "0", "--ring", "Z2"]
    run(base + ["--path", first, "--seed", "71", "--max-launches", "5"], work)
    saved = sorted(os.listdir(first))
    ranks = [int(x.split("_m")[1].split("_")[0]) for x in saved]
    # Resume from the directory of JSON files, and from the same schemes as text.
    text = os.path.join(work, "resume.txt")
    run([os.path.join(BIN, "scheme_converter"), "-i", first, "-o", text], work)
    outs = []
    for src in (first, text):
        out = os.path.join(work, "resumed_" + os.path.basename(src))
        os.makedirs(out)
        log = run(base + ["--path", out, "--seed", "72", "--max-launches", "3", "--input-path", src], work)
        assert f"Start reading {len(saved)} schemes" in log
        outs.append((out, sorted(os.listdir(out))))
    (a, fa), (b, fb) = outs
    assert fa == fb
    for name in fa:
        with open(os.path.join(a, name)) as x, open(os.path.join(b, name)) as y:
            assert x.read() == y.read(), name
    # The resumed walks start from the saved schemes: nothing above the best saved rank is saved again.
    assert all(int(x.split("_m")[1].split("_")[0]) <= min(ranks) for x in fa)


def test_flip_graph_zb_ring_saves_exact_schemes(work):
    """The |c| <= 2 ring (no reference counterpart) through flip_graph: fast mode, naive starts;
    every saved scheme is exact over the integers, within the bound, named with the ring."""
    import json
    import numpy as np
    from oracle import oracle as O
    out = os.path.join(work, "zb")
    os.makedirs(out)
    log = run([os.path.join(BIN, "flip_graph"), "-n1", "2", "-n2", "2", "-n3", "3", "--ring", "ZB", "--schemes", "512",
               "--max-iterations", "3000", "--plus-iterations", "3000", "--resize-probability", "0", "--seed", "5",
               "--max-launches", "3", "--path", out], work)
    assert "runs in the fast mode" in log
    files = sorted(os.listdir(out))
    assert files and all(f.endswith("_ZB.json") for f in files)
    for name in files:
        d = json.load(open(os.path.join(out, name)))
        assert d["z2"] is False and d["m"] < 12
        n, m = d["n"], d["m"]
        fac = np.zeros((1, 3, m), np.uint64)
        sgn = np.zeros((1, 3, m), np.uint64)
        two = np.zeros((1, 3, m), np.uint64)
        for c, key_ in enumerate("uvw"):
            for t, row in enumerate(d[key_]):
                for e, x in enumerate(row):
                    assert -2 <= x <= 2
                    if x:
                        fac[0, c, t] |= np.uint64(1 << e)
                    if x < 0:
                        sgn[0, c, t] |= np.uint64(1 << e)
                    if abs(x) == 2:
                        two[0, c, t] |= np.uint64(1 << e)
        ok = np.zeros(1, np.uint8)
        O.lib().fgo_validate_zb(1, m, O._ptr(np.array([n], np.int32)), O._ptr(np.array([m], np.int32)), O._ptr(fac),
                                O._ptr(sgn), O._ptr(two), O._ptr(ok))
        assert ok[0] == 1, name
    # and the converter reads them back (values of magnitude 2 kept)
    txt = os.path.join(work, "zb.txt")
    run([os.path.join(BIN, "scheme_converter"), "-i", out, "-o", txt], work)
    back = os.path.join(work, "zb_back")
    run([os.path.join(BIN, "scheme_converter"), "-i", txt, "-o", back, "--ring", "ZB"], work)
    assert (len(os.listdir(back)) if os.path.isdir(back) else 1) == len(files)


def test_flip_graph_fast_mode_runs_every_move(work):
    """flip_graph --mode fast on Z2 with the reference's default resizing (0.2) and sandwiching and
    basis-change moves: no note that a move is off, the walks resize, and every saved scheme is an
    exact Z2 scheme of its sizes."""
    import json
    import numpy as np
    from oracle import oracle as O
    out = os.path.join(work, "fast_moves")
    os.makedirs(out)
    log = run([os.path.join(BIN, "flip_graph"), "-n1", "2", "-n2", "3", "-n3", "3", "--ring", "Z2", "--mode", "fast",
               "--schemes", "256", "--max-iterations", "2000", "--plus-iterations", "500", "--sandwiching-probability",
               "20", "--basis-probability", "20", "--seed", "9", "--max-launches", "6", "--path", out], work)
    assert "not available" not in log and "treated as 0" not in log, log[-2000:]
    files = sorted(os.listdir(out))
    assert files and all(f.endswith("_Z2.json") for f in files)
    sizes = set()
    for name in files:
        d = json.load(open(os.path.join(out, name)))
        n, m = d["n"], d["m"]
        sizes.add(tuple(n))
        b = O.WalkBatch(1, max(m, 1), "z2")
        b.n[0] = n
        b.m[0] = m
        for c, key_ in enumerate("uvw"):
            for t, row in enumerate(d[key_]):
                b.fac[0, c, t] = sum(1 << e for e, x in enumerate(row) if x % 2)
        assert O.validate(b).all(), name
    assert len(sizes) > 1  # resized schemes were saved too
