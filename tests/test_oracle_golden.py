"""The CPU oracle against the reference's own outputs (tests/golden/).

The fixtures were recorded from the reference's unmodified CUDA kernels on a
GB300 (tests/golden/make_golden.py).  Replaying each walk's recorded XORWOW
tape, the oracle must reproduce every launch's state byte for byte: factors,
FlipSet list order, flips counter, best rank, best scheme, and the exact
number of draws the reference consumed.
"""
import glob
import gzip
import os

import numpy as np
import pytest

import golden_io
from helpers import diff_walk, golden, read_scheme_text, strassen_blocks, walk_fixtures
from oracle import oracle as O


@pytest.mark.parametrize("path", walk_fixtures(), ids=lambda p: os.path.basename(p).split(".")[0])
def test_walk_matches_reference(path):
    d = golden_io.read_walk(path)
    ring, S = d["ring"], d["walks"]
    n1, n2, n3 = d["n"]
    if d["resize_p"] > 0:
        return check_resize_walk(d)
    batch = O.WalkBatch(S, n1 * n2 * n3, ring)
    moves = dict(sandwich_p=d["sandwich_p"], basis_p=d["basis_p"])
    O.init_naive(batch, n1, n2, n3)
    for w in range(S):
        init = {"scheme": d["initial"][w], "flips": 0, "best_rank": n1 * n2 * n3, "best": d["initial"][w]}
        assert not diff_walk(batch, w, init, ring), "naive scheme differs from the reference's"
    tape = O.make_tape([(t["draws"], t["uniforms"]) for t in d["tapes"]])
    for L, block in enumerate(d["launches"]):
        cfg = batch.cfg("tape", d["iterations"], d["plus_iterations"], 1, d["expand_p"], d["reduce_p"], **moves)
        O.walk(batch, cfg, tape)
        assert not batch.status.any()
        for w in range(S):
            assert not diff_walk(batch, w, block[w], ring), f"launch {L} walk {w}"
        assert O.validate(batch).all()
    assert [int(x) for x in batch.rng_pos] == [t["used"] for t in d["tapes"]]


def check_resize_walk(d):
    """Resize dumps: the table of best ranks per size spans launches, so the oracle reruns
    launches 1..L from the naive start and compares every walk after each L (sizes, factors,
    lists, best sizes and scheme, flips counter, best rank) and the draws consumed."""
    S, ring = d["walks"], d["ring"]
    n1, n2, n3 = d["n"]
    tape = O.make_tape([(t["draws"], t["uniforms"]) for t in d["tapes"]])
    for L, block in enumerate(d["launches"]):
        batch = O.WalkBatch(S, 352, ring)
        O.init_naive(batch, n1, n2, n3)
        cfg = batch.cfg("tape", d["iterations"], d["plus_iterations"], L + 1, d["expand_p"], d["reduce_p"],
                        resize_p=d["resize_p"])
        assert O.walk(batch, cfg, tape) == 0
        for w in range(S):
            assert not diff_walk(batch, w, block[w], ring), f"launch {L} walk {w}: {diff_walk(batch, w, block[w], ring)}"
        assert O.validate(batch).all() and O.validate(batch, best=True).all()
    assert [int(x) for x in batch.rng_pos] == [t["used"] for t in d["tapes"]]


@pytest.mark.parametrize("ring", ["zt", "z2"])
def test_reducer_matches_reference(ring):
    with gzip.open(golden(f"input_{ring}_333.txt.gz"), "rt") as f:
        n, m, coef = read_scheme_text(f.read())
    d = golden_io.read_reduce(golden(f"reduce_{ring}_333.bin.gz"))
    keep = [r for r in range(d["count"]) if d["tapes"][r]["used"] >= 0]
    assert len(keep) >= 3
    tape = O.make_tape([(t["draws"], t["uniforms"]) for t in d["tapes"]])
    out, modes, consumed, state = O.reduce(n, m, coef, d["count"], tape)
    O.reducer_state_free(state)
    for r in keep:
        ref = d["reducers"][r]
        assert (tuple(out[r, 0:3]), tuple(out[r, 3:6]), tuple(out[r, 6:9])) == (ref["u"], ref["v"], ref["w"]), r
        assert consumed[r] == d["tapes"][r]["used"], r


MODE_PREFIX = {0: "g", 1: "ga", 2: "gr", 3: "gi", 4: "wr", 5: "mix", 6: "rnd"}


def test_reducer_max_flips_matches_reference():
    """The reducer's --max-flips iterations as the reference ran them (ref_harness reduce with
    MAX_FLIPS: flipSchemesKernel from the second iteration, runReducersKernel with
    independent=false, updateBestTogether): flipped ranks, every reducer's counts, modes and
    draws, and the incumbent's improvement, replayed by the oracle from the same tapes."""
    with gzip.open(golden("input_zt_333.txt.gz"), "rt") as f:
        n, m, coef0 = read_scheme_text(f.read())
    d = golden_io.read_reduce_flips(golden("flipreduce_zt_333_f20.bin.gz"))
    count, schemes, flips = d["count"], d["schemes"], d["max_flips"]
    tape = O.make_tape([(t["draws"], t["uniforms"]) for t in d["tapes"]])
    used = np.zeros(count, np.int64)
    coef, ranks = np.tile(coef0[None], (schemes, 1, 1, 1)), np.full(schemes, m, np.int32)
    best_fresh, best_vars = np.zeros(3, np.int32), np.zeros((3, 500, 2), np.int32)
    nn = [n[0] * n[1], n[1] * n[2], n[2] * n[0]]
    reduced = None
    for it, ref in enumerate(d["iterations"], start=1):
        if it > 1:
            coef, ranks, consumed, bad = O.flip_schemes(n, m, coef0, schemes, flips, O.tape_tail(tape, used))
            assert bad == 0
            used[:schemes] += consumed
        assert list(ranks) == ref["ranks"], it
        state = O.reducer_state(best_fresh, best_vars)
        out, modes, consumed, vars_ = O.reduce_schemes(n, m, coef, ranks, count, O.tape_tail(tape, used),
                                                      independent=False, best=state)
        O.reducer_state_free(state)
        used += consumed
        for r in range(count):
            rr = ref["reducers"][r]
            assert (tuple(out[r, 0:3]), tuple(out[r, 3:6]), tuple(out[r, 6:9])) == (rr["u"], rr["v"], rr["w"]), (it, r)
            assert [MODE_PREFIX[int(x)] for x in modes[r]] == [x.rstrip("0123456789") for x in rr["modes"]], (it, r)
        if reduced is None:  # SchemeAdditionsReducer::initialize: naive additions, maximal fresh counts
            reduced = (int(out[0, 2] + out[0, 5] + out[0, 8]),
                       nn[0] * (nn[0] - 1) + nn[1] * (nn[1] - 1) + m * (m - 1))
        # updateBestTogether: the reference's top reducer has the lowest (additions, fresh) total
        tot = out[:, 0] + out[:, 3] + out[:, 6]
        fresh = out[:, 1] + out[:, 4] + out[:, 7]
        top = ref["top"]
        assert (tot[top], fresh[top]) == min(zip(tot, fresh)), it
        improved = (tot[top], fresh[top]) < reduced
        assert int(improved) == ref["improved"], it
        if improved:
            reduced = (int(tot[top]), int(fresh[top]))
            best_fresh, best_vars = out[top, 1::3].astype(np.int32), vars_[top].copy()
    assert [int(x) for x in used] == [t["used"] for t in d["tapes"]]


@pytest.mark.parametrize("shape", [(2, 2, 2), (2, 3, 4), (3, 3, 3), (4, 4, 4), (3, 4, 5), (4, 5, 8)])
def test_naive_schemes_validate(shape):
    n1, n2, n3 = shape
    for ring in ("z2", "zt"):
        b = O.WalkBatch(2, n1 * n2 * n3, ring)
        O.init_naive(b, n1, n2, n3)
        assert O.validate(b).all()
        # A single flipped bit breaks the Brent equations.
        b.fac[1, 2, 0] ^= 1
        assert list(O.validate(b)) == [True, False]


def test_reference_inputs_validate():
    for ring in ("z2", "zt"):
        with gzip.open(golden(f"input_{ring}_333.txt.gz"), "rt") as f:
            (n1, n2, n3), m, coef = read_scheme_text(f.read())
        fac = np.zeros((1, 3, m), np.uint64)
        sgn = np.zeros((1, 3, m), np.uint64)
        for c in range(3):
            for t in range(m):
                for j in range(64):
                    if coef[c, t, j]:
                        fac[0, c, t] |= np.uint64(1 << j)
                        if coef[c, t, j] < 0:
                            sgn[0, c, t] |= np.uint64(1 << j)
        n = np.array([[n1, n2, n3]], np.int32)
        mm = np.array([m], np.int32)
        assert O.validate_arrays("z2", n, mm, fac)[0]  # every ZT scheme is also valid mod 2
        ok_zt = O.validate_arrays("zt", n, mm, fac, sgn, np.ones((1, 3, m), np.uint8))[0]
        assert ok_zt == (ring == "zt")


def test_philox_known_answer():
    # Random123 known-answer vector for Philox4x32-10 with zero counter and key.
    assert O.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]


def test_fast_mode_walk_is_deterministic_and_valid():
    b1 = O.WalkBatch(8, 27, "z2")
    O.init_naive(b1, 3, 3, 3)
    b2 = b1.copy()
    cfg = b1.cfg("philox", iterations=2000, plus_iterations=300, launches=2, seed=7)
    O.walk(b1, cfg)
    O.walk(b2, cfg)
    for f in ("m", "fac", "list_size", "list_pairs", "rng_pos", "best_m", "best_fac"):
        assert np.array_equal(getattr(b1, f), getattr(b2, f))
    assert O.validate(b1).all() and O.validate(b1, best=True).all()
    assert (b1.best_m < 27).any()


@pytest.mark.parametrize("shape", [(3, 3, 3), (2, 4, 8), (2, 2, 17)])
def test_fast_mode_moves_keep_schemes_exact(shape):
    """Fast mode (implicit pairs) with sandwiching, basis changes and the Gauss reduction at a
    high rate: deterministic, every scheme exact, and the moves change the trajectory."""
    n1, n2, n3 = shape
    b1 = O.WalkBatch(8, n1 * n2 * n3, "z2")
    O.init_naive(b1, n1, n2, n3)
    b2, b0 = b1.copy(), b1.copy()
    kw = dict(iterations=600, plus_iterations=200, launches=2, seed=11)
    cfg = b1.cfg("fast", sandwich_p=60.0, basis_p=60.0, gauss_p=30.0, **kw)
    O.walk(b1, cfg)
    O.walk(b2, cfg)
    O.walk(b0, b0.cfg("fast", **kw))
    for f in ("m", "fac", "rng_pos", "best_m", "best_fac"):
        assert np.array_equal(getattr(b1, f), getattr(b2, f))
    assert O.validate(b1).all() and O.validate(b1, best=True).all()
    assert (b1.rng_pos > b0.rng_pos).all()
    assert not np.array_equal(b1.fac, b0.fac)


def gauss_fixtures():
    return sorted(glob.glob(golden("gauss_z2_s*.bin.gz")))


def gauss_input():
    with gzip.open(golden("gauss_input_z2.txt.gz"), "rt") as f:
        return golden_io.read_scheme_text(f.read())


@pytest.mark.parametrize("path", gauss_fixtures(), ids=lambda p: os.path.basename(p).split(".")[0])
def test_reduce_gauss_matches_reference(path):
    """SchemeZ2::tryReduceGauss (never called by the reference's walk), one call per scheme
    with the reference's stream: same result flag, same scheme after the call (zero terms and
    all), same number of draws."""
    d = golden_io.read_gauss(path)
    schemes = gauss_input()
    assert d["count"] == len(schemes)
    b = O.WalkBatch(len(schemes), 352, "z2")
    for w, s in enumerate(schemes):
        b.n[w] = s["n"]
        b.m[w] = s["m"]
        for c in range(3):
            b.fac[w, c, :s["m"]] = s["uvw"][c]
    tape = O.make_tape([(t["draws"], t["uniforms"]) for t in d["tapes"]])
    found = O.reduce_gauss(b, b.cfg("tape"), tape)
    assert not b.status.any()
    want = np.array([r["found"] for r in d["results"]])
    assert np.array_equal(found, want)
    assert 20 < want.sum() < len(want)
    for w, r in enumerate(d["results"]):
        s = r["scheme"]
        assert list(b.n[w]) == s["n"] and b.m[w] == s["m"], w
        for c in range(3):
            assert np.array_equal(b.fac[w, c, :s["m"]], np.asarray(s["uvw"][c], np.uint64)), (w, c)
    assert [int(x) for x in b.rng_pos] == [t["used"] for t in d["tapes"]]


def test_flip_pass_properties():
    """flipSchemesKernel's restatement on synthetic streams: max_flips 0 takes one draw per
    stream and copies the scheme; with flips every scheme stays an exact ternary scheme."""
    with gzip.open(golden("input_zt_333.txt.gz"), "rt") as f:
        n, m, coef0 = read_scheme_text(f.read())
    rng = np.random.default_rng(7)
    S = 10
    tapes = []
    for _ in range(S):
        d = rng.integers(0, 2 ** 32, 60000, dtype=np.uint64).astype(np.uint32)
        tapes.append((d, ((d >> np.uint32(8)).astype(np.float32) + 1) / np.float32(16777216.0)))
    tape = O.make_tape(tapes)
    coef, ranks, consumed, bad = O.flip_schemes(n, m, coef0, S, 0, tape)
    assert bad == 0 and (coef == coef0[None]).all() and (ranks == m).all()
    assert list(consumed) == [0] + [1] * (S - 1)
    coef, ranks, consumed, bad = O.flip_schemes(n, m, coef0, S, 40, tape)
    assert bad == 0 and (coef[0] == coef0).all() and (ranks <= m).all() and (consumed[1:] >= 1).all()
    bits = np.uint64(1) << np.arange(64, dtype=np.uint64)
    fac = np.where(coef != 0, bits, np.uint64(0)).sum(axis=3, dtype=np.uint64)
    sgn = np.where(coef < 0, bits, np.uint64(0)).sum(axis=3, dtype=np.uint64)
    valid = np.zeros((S, 3, m), np.uint8)
    for s in range(S):
        valid[s, :, :ranks[s]] = 1
        assert not coef[s, :, ranks[s]:].any()
    assert O.validate_arrays("zt", np.tile(np.asarray(n, np.int32), (S, 1)), ranks, fac, sgn, valid).all()
    assert (coef[1:] != coef0[None]).any()  # the flips changed schemes


def test_ternary_factors_up_to_31_entries_stay_sign_extended():
    """The thread-per-walk ternary kernel keeps factors of 17-31 entries as 32-bit words standing
    for sext(word): the reference's random split sign-extends its second 16-bit chunk, naive
    factors leave bits 31-63 clear, and xor / and keep the property.  From a 2x2x10 scheme below
    the naive rank (so that factors of 20 entries are split), the oracle's walk keeps bits 32-63
    of every value and sign equal to bit 31 after every launch, and every scheme exact."""
    (n1, n2, n3), terms = strassen_blocks(5)
    S, cap, m = 16, 48, len(terms)
    b = O.WalkBatch(S, cap, "zt")
    b.n[:] = (n1, n2, n3)
    b.m[:] = m
    for t, tri in enumerate(terms):
        for c, d in enumerate(tri):
            for e, x in d.items():
                b.fac[:, c, t] |= np.uint64(1 << e)
                if x < 0:
                    b.sgn[:, c, t] |= np.uint64(1 << e)
    b.valid[:, :, :m] = 1
    b.best_fac[:] = b.fac
    b.best_sgn[:] = b.sgn
    b.best_valid[:] = b.valid
    b.best_rank[:] = m
    b.best_m[:] = m
    assert O.validate(b).all()
    ranks = set()
    for launch in range(4):
        O.walk(b, b.cfg("philox", iterations=500, plus_iterations=60, launches=1, expand_p=200.0, seed=5 + launch))
        assert O.validate(b).all() and not b.status.any()
        for arr in (b.fac, b.sgn, b.best_fac, b.best_sgn):
            assert np.isin(arr >> np.uint64(31), [0, (1 << 33) - 1]).all()
        ranks.update(int(x) for x in b.m)
    assert len(ranks) > 1  # the walks left the starting rank: splits and merges ran
