"""GPU additions reducer through the C ABI.

Against the reference's own reducer kernel (tests/golden/reduce_*.bin: one
runReducersKernel launch, 12 reducers, seed 41) and against the CPU oracle
replaying the same cuRAND streams, including partial initialisation from an
incumbent and the non-independent variant.
"""
import gzip

import numpy as np
import pytest

import golden_io
from helpers import golden, read_scheme_text
from oracle import oracle as O

pytestmark = pytest.mark.gpu
fg = pytest.importorskip("flipgraphgpu_gb300")


def load_input(ring):
    with gzip.open(golden(f"input_{ring}_333.txt.gz"), "rt") as f:
        return read_scheme_text(f.read())


@pytest.mark.parametrize("ring", ["zt", "z2"])
def test_reducer_matches_reference_kernel(ring):
    n, m, coef = load_input(ring)
    d = golden_io.read_reduce(golden(f"reduce_{ring}_333.bin.gz"))
    red = fg.Reducer(n, m, coef[None], count=d["count"], schemes=1, seed=d["seed"])
    out = red.run(independent=True)
    red.close()
    for r in range(d["count"]):
        ref = d["reducers"][r]
        got = tuple(tuple(int(x) for x in (out["additions"][r, c], out["fresh"][r, c], out["naive"][r, c]))
                    for c in range(3))
        assert got == (ref["u"], ref["v"], ref["w"]), r
        names = [fg.mode_name(out["mode"][r, c], out["scale"][r, c]) for c in range(3)]
        assert names == ref["modes"], r
        if d["tapes"][r]["used"] >= 0:
            assert out["draws"][r] == d["tapes"][r]["used"], r


def oracle_run(n, m, coef, count, draws, unis, start, used, independent, best=None):
    tape = O.make_tape([(draws[r, start[r]:start[r] + used[r]], unis[r, start[r]:start[r] + used[r]])
                        for r in range(count)])
    out, modes, consumed, st = O.reduce(n, m, coef, count, tape, independent=independent, best=best)
    O.reducer_state_free(st)
    return out, modes, consumed


@pytest.mark.parametrize("ring,seed,independent", [("zt", 7, True), ("z2", 8, True), ("zt", 9, False), ("z2", 10, False)])
def test_reducer_two_iterations_vs_oracle(ring, seed, independent):
    n, m, coef = load_input(ring)
    count = 24
    red = fg.Reducer(n, m, coef[None], count=count, schemes=1, seed=seed)
    first = red.run(independent=True)
    # Incumbent: reducer 0's variables (greedy), fed back for partial initialisation.
    best_fresh = first["fresh"][0].copy()
    best_vars = first["vars"][0].copy()
    second = red.run(independent=independent, best_fresh=best_fresh, best_vars=best_vars)
    red.close()
    total = int((first["draws"] + second["draws"]).max())
    draws, unis = fg.xorwow_tape(seed, 0, count, total)
    zeros = np.zeros(count, np.int64)
    o1, _, c1 = oracle_run(n, m, coef, count, draws, unis, zeros, first["draws"], True)
    state = O.reducer_state(best_fresh, best_vars)
    o2, _, c2 = oracle_run(n, m, coef, count, draws, unis, first["draws"].astype(np.int64), second["draws"],
                           independent, best=state)
    O.reducer_state_free(state)
    for o, g, c in ((o1, first, c1), (o2, second, c2)):
        assert np.array_equal(o[:, 0::3], g["additions"])
        assert np.array_equal(o[:, 1::3], g["fresh"])
        assert np.array_equal(o[:, 2::3], g["naive"])
        assert np.array_equal(c, g["draws"])


@pytest.mark.parametrize("seed", [5, 6])
def test_reducer_matches_reference_on_444_rank47(seed):
    """32 reducers on a 4x4x4 Z2 scheme of rank 47 (the config the post-search benchmark runs):
    additions, fresh variables, naive counts and modes equal the reference kernel's, including the
    greedy-intersections reducers whose scores the GPU computes block-parallel."""
    import json
    with open(golden("scheme_444_z2_r47.txt")) as f:
        n, m, coef = read_scheme_text(f.read())
    with open(golden("reduce_444_r47.json")) as f:
        ref = json.load(f)["seeds"][str(seed)]
    red = fg.Reducer(n, m, coef[None], count=len(ref), schemes=1, seed=seed)
    out = red.run(independent=True)
    red.close()
    for r, want in enumerate(ref):
        got = [[int(out[k][r, c]) for k in ("additions", "fresh", "naive")] for c in range(3)]
        assert got == [want["u"], want["v"], want["w"]], r
        names = [fg.mode_name(out["mode"][r, c], out["scale"][r, c]) for c in range(3)]
        assert names == want["modes"], r


def test_reducer_with_tables_in_global_memory_vs_oracle():
    """Dense expressions whose pair tables exceed shared memory (the reducer then keeps them in
    global memory, blocks looping over reducers): results and draw counts equal the oracle's."""
    rng = np.random.default_rng(21)
    n, m = (4, 4, 4), 48
    coef = np.zeros((3, m, 64), np.int8)
    for c in range(3):
        coef[c, :, :16] = (rng.random((m, 16)) < 0.5).astype(np.int8)
    coef[:, :, :16][coef[:, :, :16].sum(axis=2) == 0] = 1
    count, seed = 6, 12
    red = fg.Reducer(n, m, coef[None], count=count, schemes=1, seed=seed)
    out = red.run(independent=True)
    red.close()
    draws, unis = fg.xorwow_tape(seed, 0, count, int(out["draws"].max()))
    o, _, c = oracle_run(n, m, coef, count, draws, unis, np.zeros(count, np.int64), out["draws"], True)
    assert np.array_equal(o[:, 0::3], out["additions"])
    assert np.array_equal(o[:, 1::3], out["fresh"])
    assert np.array_equal(o[:, 2::3], out["naive"])
    assert np.array_equal(c, out["draws"])
