"""The additions reducer's --max-flips mode on the GPU through the C ABI.

Per iteration (reduceIteration, scheme_additions_reducer.cu:172-182): from the
second on, fg_reducer_flip turns schemes 1.. into flipped copies of scheme 0
(flipSchemesKernel, :448-460), drawing from the reducers' own XORWOW streams;
then one reduction with independent=false, and the incumbent is one whole
reducer (updateBestTogether, :296-339).  Every flipped scheme, rank, reducer
count, mode, fresh-variable list and draw count equals the CPU oracle
replaying the same streams; the flipped schemes stay exact.
"""
import gzip
import os
import platform
import subprocess
import json

import numpy as np
import pytest

from helpers import golden, read_scheme_text
from oracle import oracle as O

pytestmark = pytest.mark.gpu
fg = pytest.importorskip("flipgraphgpu_gb300")


def load_zt():
    with gzip.open(golden("input_zt_333.txt.gz"), "rt") as f:
        return read_scheme_text(f.read())


def exact(n, ranks, coef):
    """Integer Brent check of coefficient rows [schemes][3][m][64]."""
    S, m = coef.shape[0], coef.shape[2]
    bits = (np.uint64(1) << np.arange(64, dtype=np.uint64))
    fac = np.where(coef != 0, bits, np.uint64(0)).sum(axis=3, dtype=np.uint64)
    sgn = np.where(coef < 0, bits, np.uint64(0)).sum(axis=3, dtype=np.uint64)
    valid = np.zeros((S, 3, m), np.uint8)
    for s in range(S):
        valid[s, :, :ranks[s]] = 1
    return O.validate_arrays("zt", np.tile(np.asarray(n, np.int32), (S, 1)), np.asarray(ranks, np.int32), fac, sgn,
                             valid)


@pytest.mark.parametrize("count,schemes,seed,max_flips", [(16, 8, 43, 20), (24, 24, 44, 60), (12, 3, 45, 1)])
def test_flip_iterations_vs_oracle(count, schemes, seed, max_flips):
    n, m, coef0 = load_zt()
    red = fg.Reducer(n, m, np.tile(coef0[None], (schemes, 1, 1, 1)), count=count, schemes=schemes, seed=seed)
    draws, unis = fg.xorwow_tape(seed, 0, count, 200000)
    tape = O.make_tape([(draws[r], unis[r]) for r in range(count)])
    used = np.zeros(count, np.int64)
    coef, ranks = np.tile(coef0[None], (schemes, 1, 1, 1)), np.full(schemes, m, np.int32)
    best_fresh, best_vars = np.zeros(3, np.int32), np.zeros((3, 500, 2), np.int32)
    reduced = None
    for it in range(1, 4):
        if it > 1:
            g_ranks, g_coef = red.flip(max_flips)
            coef, ranks, consumed, bad = O.flip_schemes(n, m, coef0, schemes, max_flips, O.tape_tail(tape, used))
            assert bad == 0
            assert np.array_equal(g_ranks, ranks), it
            assert np.array_equal(g_coef, coef), it
            assert exact(n, ranks, coef).all()
            used[:schemes] += consumed
        g = red.run(independent=False, best_fresh=best_fresh, best_vars=best_vars)
        state = O.reducer_state(best_fresh, best_vars)
        out, modes, consumed, vars_ = O.reduce_schemes(n, m, coef, ranks, count, O.tape_tail(tape, used),
                                                      independent=False, best=state)
        O.reducer_state_free(state)
        assert np.array_equal(out[:, 0::3], g["additions"]), it
        assert np.array_equal(out[:, 1::3], g["fresh"]), it
        assert np.array_equal(out[:, 2::3], g["naive"]), it
        assert np.array_equal(modes, g["mode"]), it
        assert np.array_equal(consumed, g["draws"]), it
        assert np.array_equal(vars_, g["vars"]), it  # rows past 2 * fresh are zero on both sides
        used += consumed
        # updateBestTogether: one reducer's three components, lowest total additions then fresh
        tot, fresh = g["additions"].sum(1), g["fresh"].sum(1)
        top = min(range(count), key=lambda r: (tot[r], fresh[r], r))
        if reduced is None or (tot[top], fresh[top]) < reduced:
            reduced = (tot[top], fresh[top])
            best_fresh, best_vars = g["fresh"][top].copy(), g["vars"][top].copy()
    red.close()


def test_flip_needs_streams_and_a_ternary_scheme():
    n, m, coef0 = load_zt()
    red = fg.Reducer(n, m, np.tile(coef0[None], (8, 1, 1, 1)), count=4, schemes=8, seed=3)
    with pytest.raises(fg.FlipGraphError):
        red.flip(5)  # 8 schemes, 4 streams
    red.close()
    two = coef0.copy()
    two[0, 0, 0] = 2
    red = fg.Reducer(n, m, np.tile(two[None], (2, 1, 1, 1)), count=4, schemes=2, seed=3)
    with pytest.raises(fg.FlipGraphError):
        red.flip(5)
    red.close()


def test_cli_max_flips(tmp_path):
    exe = os.path.join(os.path.dirname(fg.__file__), "_lib", platform.machine(), "additions_reducer")
    src = tmp_path / "in.txt"
    with gzip.open(golden("input_zt_333.txt.gz"), "rt") as f:
        src.write_text(f.read())
    out = tmp_path / "out"
    out.mkdir()  # the executable, like the reference's, writes into an existing directory
    r = subprocess.run([exe, "-i", str(src), "-o", str(out), "--count", "32", "--schemes-count", "8", "--max-flips", "30",
                        "--seed", "52", "--max-no-improvements", "2"], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:]
    assert "- max flips: 30" in r.stdout
    saved = sorted(os.listdir(out))
    assert saved, r.stdout[-2000:]
    # The saved reduced scheme's additions are its expressions' count: fresh + sum(|e| - 1).
    for name in saved:
        d = json.load(open(out / name))
        adds = sum(len(d[f"{c}_fresh"]) + sum(len(e) - 1 for e in d[c]) for c in "uvw")
        assert adds == d["complexity"]["reduced"], name
