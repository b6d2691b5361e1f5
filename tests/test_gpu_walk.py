"""GPU walk parity through the C ABI.

* Reference stream (XORWOW): the library's kernels against the reference's
  own recorded kernel states (tests/golden), byte for byte; and against the
  CPU oracle replaying the same cuRAND stream on larger batches.
* Fast stream (Philox): the library's kernels against the oracle's fast mode.
"""
import numpy as np
import pytest

import golden_io
from helpers import diff_walk, strassen_blocks, walk_fixtures
from oracle import oracle as O

pytestmark = pytest.mark.gpu

fg = pytest.importorskip("flipgraphgpu_gb300")


def compare_records(rec, b, ctx=""):
    """Library records vs oracle batch: every field, exactly."""
    fields = ["n", "m", "fac", "list_size", "list_pairs", "flips", "best_rank", "best_m", "best_fac", "rng_pos", "status"]
    if rec.ring == "zt":
        fields += ["sgn", "valid", "best_sgn", "best_valid"]
    for f in fields:
        a, o = getattr(rec, f), getattr(b, f)
        if not np.array_equal(a, o):
            bad = np.argwhere(a != o)
            raise AssertionError(f"{ctx}: field {f} differs at {bad[:5].tolist()} (of {len(bad)})")


def test_xorwow_tape_is_the_reference_stream():
    d = golden_io.read_walk([p for p in walk_fixtures() if "z2_333" in p][0])
    n = min(len(t["draws"]) for t in d["tapes"])
    draws, unis = fg.xorwow_tape(d["seed"], 0, d["walks"], n)
    for w, t in enumerate(d["tapes"]):
        assert np.array_equal(draws[w], t["draws"][:n])
        assert np.array_equal(unis[w].view(np.uint32), t["uniforms"][:n].view(np.uint32))


def test_philox_device_matches_oracle():
    rng = np.random.default_rng(5)
    ctr = rng.integers(0, 2**32, size=(257, 4), dtype=np.uint64).astype(np.uint32)
    key = (0xDEADBEEF, 0x12345678)
    out = fg.philox_blocks(ctr, key)
    for q in range(len(ctr)):
        assert list(out[q]) == O.philox([int(x) for x in ctr[q]], list(key))


@pytest.mark.parametrize("list_kernel", ["warp", "thread"])
@pytest.mark.parametrize("path", walk_fixtures(), ids=lambda p: p.split("/")[-1].split(".")[0])
def test_walk_matches_reference_kernel(path, list_kernel):
    """Same seed, same flags: the library reproduces the reference's per-launch state, with one
    warp per walk and (without the sandwiching and basis moves) one thread per walk."""
    d = golden_io.read_walk(path)
    ring = d["ring"]
    moves = d["sandwich_p"] > 0 or d["basis_p"] > 0
    if list_kernel == "thread" and moves:
        pytest.skip("the thread-per-walk list kernel runs without sandwiching and basis moves")
    n1, n2, n3 = d["n"]
    cap = 352 if d["resize_p"] > 0 else n1 * n2 * n3
    with fg.Engine(d["walks"], cap, ring, "reference", d["seed"], d["iterations"], d["plus_iterations"],
                   d["expand_p"], d["reduce_p"], resize_p=d["resize_p"], sandwich_p=d["sandwich_p"],
                   basis_p=d["basis_p"]) as eng:
        if not moves:
            eng.set_list_kernel(list_kernel)
        eng.init_naive(n1, n2, n3)
        for L, block in enumerate(d["launches"]):
            eng.run(1)
            rec = eng.records()
            for w in range(d["walks"]):
                errs = diff_walk(rec, w, block[w], ring)
                assert not errs, f"launch {L} walk {w}: {errs}"
        assert [int(x) for x in rec.rng_pos] == [t["used"] for t in d["tapes"]]
        assert eng.validate().all()
        assert eng.validate(best=True).all()


@pytest.mark.parametrize("ring,mode,shape,S,iters,plus,resize_p,sandwich_p,basis_p,launches", [
    ("z2", "reference", (3, 3, 3), 32, 300, 100, 0.3, 0.0, 0.0, 3),
    ("z2", "reference", (2, 3, 4), 24, 200, 50, 0.9, 0.0, 0.0, 3),
    ("z2", "philox", (2, 2, 3), 24, 200, 50, 0.7, 0.0, 0.0, 4),
    ("zt", "reference", (2, 2, 3), 16, 60, 40, 0.8, 0.0, 0.0, 3),
    ("zt", "reference", (2, 3, 3), 12, 50, 30, 0.5, 0.0, 0.0, 3),
    ("z2", "reference", (3, 3, 3), 32, 300, 100, 0.0, 20.0, 20.0, 3),
    ("z2", "philox", (2, 3, 4), 32, 300, 100, 0.0, 40.0, 10.0, 3),
    ("z2", "reference", (2, 3, 3), 24, 200, 60, 0.6, 15.0, 15.0, 3),
    ("zt", "reference", (3, 3, 3), 12, 60, 40, 0.0, 10.0, 20.0, 3),
    ("zt", "philox", (2, 3, 3), 12, 60, 40, 0.5, 5.0, 20.0, 3),
])
@pytest.mark.parametrize("list_kernel", ["warp", "thread"])
def test_meta_moves_vs_oracle(ring, mode, shape, S, iters, plus, resize_p, sandwich_p, basis_p, launches, list_kernel):
    """Resize meta-operators, sandwiching and basis changes on the GPU (one warp per walk; one
    thread per walk with resizing alone) against the oracle: sizes, factors, lists, best schemes
    and sizes, best ranks and stream positions."""
    if list_kernel == "thread" and (sandwich_p > 0 or basis_p > 0):
        pytest.skip("the thread-per-walk list kernel runs without sandwiching and basis moves")
    n1, n2, n3 = shape
    seed = 500 + n1 + n2 + n3
    cap = 352 if resize_p > 0 else n1 * n2 * n3
    with fg.Engine(S, cap, ring, mode, seed, iters, plus, 0.01, 0.0, resize_p=resize_p, sandwich_p=sandwich_p,
                   basis_p=basis_p) as eng:
        eng.set_list_kernel(list_kernel)
        eng.init_naive(n1, n2, n3)
        rec0 = eng.records()
        eng.run(launches)
        rec = eng.records()
        assert eng.validate().all() and eng.validate(best=True).all()
    if resize_p > 0:
        assert len({tuple(x) for x in rec.n}) > 1, "no walk changed size"
    kw = dict(iterations=iters, plus_iterations=plus, expand_p=0.01, reduce_p=0.0, resize_p=resize_p,
              sandwich_p=sandwich_p, basis_p=basis_p, seed=seed)
    b = batch_from(rec0)
    b.best_n[:] = rec0.n
    if mode == "reference":
        used = int(rec.rng_pos.max())
        draws, unis = fg.xorwow_tape(seed, 0, S, used)
        tape = O.make_tape([(draws[w, :rec.rng_pos[w]], unis[w, :rec.rng_pos[w]]) for w in range(S)])
        O.walk(b, b.cfg("tape", launches=launches, **kw), tape)
    else:
        O.walk(b, b.cfg("philox", launches=launches, **kw))
    compare_records(rec, b, f"{ring} {mode} {shape}")
    if resize_p > 0:
        assert np.array_equal(rec.best_n, b.best_n)


def batch_from(rec0):
    """Oracle batch holding a copy of library records (including stream positions)."""
    b = O.WalkBatch(rec0.walks, rec0.cap, rec0.ring)
    fields = ["n", "m", "fac", "list_size", "list_pairs", "flips", "best_rank", "best_m", "best_fac", "rng_pos"]
    if rec0.ring == "zt":
        fields += ["sgn", "valid", "best_sgn", "best_valid"]
    for f in fields:
        getattr(b, f)[...] = getattr(rec0, f)
    return b


def run_oracle_like(rec0, cfg_kw, launches, rng, tape=None):
    b = batch_from(rec0)
    cfg = b.cfg(rng, launches=launches, **cfg_kw)
    O.walk(b, cfg, tape)
    return b


def xorwow_tape_for(rec, seed):
    used = int(rec.rng_pos.max())
    draws, unis = fg.xorwow_tape(seed, 0, rec.walks, used)
    return O.make_tape([(draws[w, :rec.rng_pos[w]], unis[w, :rec.rng_pos[w]]) for w in range(rec.walks)])


@pytest.mark.parametrize("shape,S,iters,plus,expand_p,reduce_p", [
    ((3, 3, 3), 64, 400, 100, 0.01, 0.0),
    ((2, 2, 3), 64, 600, 50, 10.0, 0.0),
    ((2, 3, 3), 32, 600, 100, 0.01, 20.0),
    ((4, 4, 4), 16, 150, 100, 0.01, 0.0),
    ((2, 4, 5), 16, 300, 100, 2.0, 0.0),   # nn = 8 x 20 x 10: factors of more than 16 entries
])
@pytest.mark.parametrize("list_kernel", ["warp", "thread"])
def test_zt_walk_reference_stream_vs_oracle(shape, S, iters, plus, expand_p, reduce_p, list_kernel):
    n1, n2, n3 = shape
    if list_kernel == "thread" and max(n1 * n2, n2 * n3, n3 * n1) > 31:
        pytest.skip("the thread-per-walk ternary kernel holds factors of at most 31 entries")
    cap = n1 * n2 * n3
    seed = 500 + n1 * 100 + n2 * 10 + n3
    kw = dict(iterations=iters, plus_iterations=plus, expand_p=expand_p, reduce_p=reduce_p)
    with fg.Engine(S, cap, "zt", "reference", seed, iters, plus, expand_p, reduce_p) as eng:
        eng.set_list_kernel(list_kernel)
        eng.init_naive(n1, n2, n3)
        rec0 = eng.records()
        eng.run(2)
        rec = eng.records()
        assert eng.validate().all() and eng.validate(best=True).all()
    b = run_oracle_like(rec0, kw, 2, "tape", xorwow_tape_for(rec, seed))
    compare_records(rec, b, f"zt {shape}")


@pytest.mark.parametrize("ring,shape", [("z2", (3, 3, 3)), ("z2", (4, 4, 4)), ("zt", (3, 3, 3)), ("zt", (2, 3, 4))])
def test_minimize_vs_oracle(ring, shape):
    """One walk launch to leave the naive scheme, then one minimizer launch (flips without reductions)."""
    n1, n2, n3 = shape
    S, cap, seed = 32, n1 * n2 * n3, 4242
    with fg.Engine(S, cap, ring, "reference", seed, 300, 100000) as eng:
        eng.init_naive(n1, n2, n3)
        eng.run(1)
        rec0 = eng.records()
        best0 = O.complexity(ring, rec0.n, rec0.m, rec0.fac)
        bc = eng.minimize(best0.copy())
        rec = eng.records()
        assert eng.validate().all() and eng.validate(best=True).all()
    # Oracle: the same launch, replaying the stream from where the walk left it.
    draws, unis = fg.xorwow_tape(seed, 0, S, int(rec.rng_pos.max()))
    tape = O.make_tape([(draws[w, :rec.rng_pos[w]], unis[w, :rec.rng_pos[w]]) for w in range(S)])
    b = batch_from(rec0)
    obc = best0.copy()
    O.minimize(b, b.cfg("tape", iterations=300, plus_iterations=100000), obc, tape)
    assert np.array_equal(bc, obc)
    assert (bc <= best0).all() and (bc < best0).any()
    compare_records(rec, b, f"minimize {ring} {shape}")
    assert np.array_equal(O.complexity(ring, rec.n, rec.best_m, rec.best_fac)[bc < best0], bc[bc < best0])


@pytest.mark.parametrize("shapes,iters,plus,expand_p,reduce_p", [
    ([(3, 3, 3)], 4000, 300, 0.01, 0.0),
    ([(2, 2, 2)], 2000, 50, 2.0, 0.0),
    ([(2, 3, 4)], 2000, 300, 0.01, 20.0),
    ([(4, 4, 4)], 2000, 800, 0.01, 0.0),
    ([(3, 4, 5)], 1500, 600, 4.0, 0.0),
    ([(2, 2, 2), (2, 2, 3), (2, 3, 4), (3, 3, 4), (3, 4, 5), (4, 4, 4)], 1500, 500, 0.01, 0.0),  # segments
    ([(2, 4, 8)], 600, 200, 0.01, 0.0),   # nn = 8 x 32 x 16: 64-bit words
    ([(4, 5, 8)], 300, 200, 0.01, 0.0),   # nn = 20 x 40 x 32, cap 160
])
@pytest.mark.parametrize("kernel,lanes", [("auto", 0), ("thread", 0), ("group", 4), ("group", 8), ("group", 16),
                                          ("warp", 0)],
                         ids=["auto", "thread", "group4", "group8", "group16", "warp"])
def test_walk_fast_mode_vs_oracle(shapes, iters, plus, expand_p, reduce_p, kernel, lanes):
    """Fast mode runs one thread, a group of lanes or one warp per walk; all follow the oracle exactly."""
    per = 40
    S = per * len(shapes)
    cap = max(a * b * c for a, b, c in shapes)
    sh = np.array([shapes[w // per] for w in range(S)], np.int32)
    seed = 9001 + len(shapes)
    kw = dict(iterations=iters, plus_iterations=plus, expand_p=expand_p, reduce_p=reduce_p, seed=seed)
    with fg.Engine(S, cap, "z2", "fast", seed, iters, plus, expand_p, reduce_p) as eng:
        eng.set_fast_kernel(kernel, lanes)
        eng.init_naive_shapes(sh)
        rec0 = eng.records()
        st = eng.run(2)
        rec = eng.records()
        assert eng.validate().all() and eng.validate(best=True).all()
    assert st["walks_valid"] == S and st["flips"] > 0
    assert not rec.list_size.any()
    b = run_oracle_like(rec0, kw, 2, "fast")
    compare_records(rec, b, f"{shapes}")


@pytest.mark.parametrize("kernel", ["split", "warp", "group"])
@pytest.mark.parametrize("shape,resize_p,launches", [((2, 3, 3), 0.5, 4), ((3, 3, 3), 0.2, 3), ((2, 2, 4), 1.0, 5)])
def test_fast_mode_resize_vs_oracle(shape, resize_p, launches, kernel):
    """The fast mode with the resize meta-operators (the reference's default --resize-probability
    0.2): each launch runs a random number of fast steps, then the resize step (reference list order,
    Philox stream) and the per-size best-rank table; field for field equal to the oracle's fast mode,
    every scheme exact, grown factors of at most 56 entries."""
    n1, n2, n3 = shape
    S, cap, seed, iters, plus = 64, 352, 71 + n1 * n2 * n3, 400, 300
    kw = dict(iterations=iters, plus_iterations=plus, expand_p=0.01, reduce_p=0.0, seed=seed, resize_p=resize_p)
    with fg.Engine(S, cap, "z2", "fast", seed, iters, plus, 0.01, 0.0, resize_p=resize_p) as eng:
        if kernel == "split":  # thread per walk up to 64 slots, a warp per walk for larger grown shapes
            eng.set_fast_split(64)
        else:
            eng.set_fast_kernel(kernel, 16 if kernel == "group" else 0)
        eng.init_naive(n1, n2, n3)
        rec0 = eng.records()
        eng.run(launches)
        rec = eng.records()
        assert eng.validate().all() and eng.validate(best=True).all()
    b = batch_from(rec0)
    b.best_n[:] = rec0.n
    O.walk(b, b.cfg("fast", launches=launches, **kw))
    compare_records(rec, b, f"fast resize {shape} {kernel}")
    assert np.array_equal(rec.best_n, b.best_n)
    assert len({tuple(x) for x in rec.n}) > 1  # the walks did resize
    nn = np.maximum.reduce([rec.n[:, 0] * rec.n[:, 1], rec.n[:, 1] * rec.n[:, 2], rec.n[:, 2] * rec.n[:, 0]])
    assert nn.max() <= 56


@pytest.mark.parametrize("kernel,lanes", [("thread", 0), ("group", 4), ("group", 16), ("warp", 0)],
                         ids=["thread", "group4", "group16", "warp"])
@pytest.mark.parametrize("shape,S,iters,plus,sandwich_p,basis_p", [
    ((3, 3, 3), 64, 600, 300, 24.0, 48.0),
    ((2, 3, 4), 64, 600, 200, 60.0, 0.0),
    ((4, 4, 4), 32, 400, 500, 0.0, 40.0),
    ((2, 4, 8), 32, 300, 200, 15.0, 30.0),   # nn = 8 x 32 x 16: 64-bit words
    ((2, 2, 17), 16, 200, 100, 20.0, 20.0),  # n > 16: sandwiching skipped (MAX_SANDWICHING_N), basis moves run
])
def test_fast_mode_sandwich_and_basis_vs_oracle(shape, S, iters, plus, sandwich_p, basis_p, kernel, lanes):
    """Sandwiching and basis-change moves in the fast mode (flip_graph.cu:560-564): gated per step on
    the walk's Philox stream after the expansion, on every fast kernel; field for field equal to the
    oracle's fast mode, every scheme exact."""
    n1, n2, n3 = shape
    cap, seed = n1 * n2 * n3, 313 + n1 * n2 * n3
    kw = dict(iterations=iters, plus_iterations=plus, expand_p=0.01, reduce_p=0.0, seed=seed,
              sandwich_p=sandwich_p, basis_p=basis_p)
    with fg.Engine(S, cap, "z2", "fast", seed, iters, plus, 0.01, 0.0, sandwich_p=sandwich_p,
                   basis_p=basis_p) as eng:
        eng.set_fast_kernel(kernel, lanes)
        eng.init_naive(n1, n2, n3)
        rec0 = eng.records()
        st = eng.run(2)
        rec = eng.records()
        assert eng.validate().all() and eng.validate(best=True).all()
    assert st["walks_valid"] == S and st["flips"] > 0
    b = run_oracle_like(rec0, kw, 2, "fast")
    compare_records(rec, b, f"fast moves {shape} {kernel}{lanes}")


@pytest.mark.parametrize("kernel", ["split", "group"])
def test_fast_mode_all_moves_with_resizing_vs_oracle(kernel):
    """The fast mode with resizing, sandwiching and basis changes together: the moves run on the
    resized shapes too; equal to the oracle's fast mode."""
    S, cap, seed, iters, plus = 64, 352, 4242, 400, 300
    kw = dict(iterations=iters, plus_iterations=plus, expand_p=0.01, reduce_p=0.0, seed=seed, resize_p=0.5,
              sandwich_p=20.0, basis_p=20.0)
    with fg.Engine(S, cap, "z2", "fast", seed, iters, plus, 0.01, 0.0, resize_p=0.5, sandwich_p=20.0,
                   basis_p=20.0) as eng:
        if kernel == "split":
            eng.set_fast_split(64)
        else:
            eng.set_fast_kernel("group", 8)
        eng.init_naive(2, 3, 3)
        rec0 = eng.records()
        eng.run(4)
        rec = eng.records()
        assert eng.validate().all() and eng.validate(best=True).all()
    b = batch_from(rec0)
    b.best_n[:] = rec0.n
    O.walk(b, b.cfg("fast", launches=4, **kw))
    compare_records(rec, b, f"fast resize + moves {kernel}")
    assert np.array_equal(rec.best_n, b.best_n)
    assert len({tuple(x) for x in rec.n}) > 1


@pytest.mark.parametrize("shape,S,iters,plus,expand_p,reduce_p,launches", [
    ((3, 3, 3), 96, 3000, 400, 0.01, 0.0, 2),
    ((2, 2, 3), 64, 2000, 100, 5.0, 0.0, 1),
    ((2, 3, 4), 64, 2000, 300, 0.01, 10.0, 1),
    ((4, 4, 4), 32, 1500, 600, 0.01, 0.0, 1),
    ((3, 4, 5), 32, 1200, 500, 3.0, 0.0, 1),
    ((2, 5, 5), 16, 800, 200, 0.01, 0.0, 1),   # nn = 25 x 25 x 10, cap 50 -> two slots per lane
    ((4, 5, 8), 8, 400, 200, 0.01, 0.0, 1),    # nn = 20 x 40 x 32, cap 160, > 32-bit factors
])
@pytest.mark.parametrize("list_kernel", ["warp", "thread"])
def test_walk_reference_stream_vs_oracle(shape, S, iters, plus, expand_p, reduce_p, launches, list_kernel):
    n1, n2, n3 = shape
    cap = n1 * n2 * n3
    seed = 1000 + n1 * 100 + n2 * 10 + n3
    kw = dict(iterations=iters, plus_iterations=plus, expand_p=expand_p, reduce_p=reduce_p)
    with fg.Engine(S, cap, "z2", "xorwow", seed, iters, plus, expand_p, reduce_p) as eng:
        eng.set_list_kernel(list_kernel)
        eng.init_naive(n1, n2, n3)
        rec0 = eng.records()
        eng.run(launches)
        rec = eng.records()
        assert eng.validate().all() and eng.validate(best=True).all()
    used = int(rec.rng_pos.max())
    draws, unis = fg.xorwow_tape(seed, 0, S, used)
    tape = O.make_tape([(draws[w, :rec.rng_pos[w]], unis[w, :rec.rng_pos[w]]) for w in range(S)])
    b = run_oracle_like(rec0, kw, launches, "tape", tape)
    compare_records(rec, b, f"{shape}")


@pytest.mark.parametrize("shape,S,iters,plus,expand_p,reduce_p", [
    ((3, 3, 3), 128, 4000, 300, 0.01, 0.0),
    ((2, 2, 2), 64, 2000, 50, 2.0, 0.0),
    ((2, 3, 4), 64, 2000, 300, 0.01, 20.0),
    ((4, 4, 4), 32, 2000, 800, 0.01, 0.0),
    ((3, 4, 5), 32, 1500, 600, 4.0, 0.0),
    ((4, 5, 8), 8, 500, 200, 0.01, 0.0),
])
@pytest.mark.parametrize("list_kernel", ["warp", "thread"])
def test_walk_fast_stream_vs_oracle(shape, S, iters, plus, expand_p, reduce_p, list_kernel):
    n1, n2, n3 = shape
    cap = n1 * n2 * n3
    seed = 77 + n1 + n2 + n3
    kw = dict(iterations=iters, plus_iterations=plus, expand_p=expand_p, reduce_p=reduce_p, seed=seed)
    with fg.Engine(S, cap, "z2", "philox", seed, iters, plus, expand_p, reduce_p) as eng:
        eng.set_list_kernel(list_kernel)
        eng.init_naive(n1, n2, n3)
        rec0 = eng.records()
        eng.run(2)
        rec = eng.records()
        assert eng.validate().all() and eng.validate(best=True).all()
    b = run_oracle_like(rec0, kw, 2, "philox")
    compare_records(rec, b, f"{shape}")


def test_validate_matches_oracle_on_corrupted_schemes():
    with fg.Engine(64, 27, "z2", "philox", 3, 500, 100) as eng:
        eng.init_naive(3, 3, 3)
        eng.run(1)
        rec = eng.records()
        rng = np.random.default_rng(0)
        for w in range(0, 64, 2):
            c, t = rng.integers(0, 3), rng.integers(0, rec.m[w])
            rec.fac[w, c, t] ^= np.uint64(1 << int(rng.integers(0, 9)))
        eng.set_records(rec)
        got = eng.validate()
    want = O.validate_arrays("z2", rec.n, rec.m, rec.fac)
    assert np.array_equal(got, want)
    assert not got[::2].any() and got[1::2].all()


@pytest.mark.parametrize("ring", ["z2", "zt"])
def test_malformed_records_are_rejected_before_any_copy(ring):
    """A record whose sizes, ranks or FlipSet pairs fall outside the scheme is refused on
    the host with a message, and the handle keeps its state: the next launch is the one
    an untouched handle makes."""
    with fg.Engine(8, 27, ring, "reference", 5, 300, 100) as eng, \
            fg.Engine(8, 27, ring, "reference", 5, 300, 100) as twin:
        for e in (eng, twin):
            e.init_naive(3, 3, 3)
            e.run(1)
        good = eng.records()
        cases = []
        r = eng.records(); r.list_pairs[3, 1, 0] = (30 << 16) | 2; r.list_size[3, 1] = max(r.list_size[3, 1], 1)
        cases.append(("pair above the rank", r))
        r = eng.records(); r.list_pairs[2, 0, 0] = (4 << 16) | 4; r.list_size[2, 0] = max(r.list_size[2, 0], 1)
        cases.append(("pair of one slot", r))
        r = eng.records(); r.list_size[0, 2] = fg.LIST_CAP + 1; cases.append(("list size", r))
        r = eng.records(); r.m[5] = 28; cases.append(("rank above cap", r))
        r = eng.records(); r.best_m[6] = -1; cases.append(("negative best rank", r))
        r = eng.records(); r.n[1] = (0, 3, 3); cases.append(("empty matrix", r))
        r = eng.records(); r.n[1] = (9, 9, 1); cases.append(("81 entries", r))
        for name, bad in cases:
            with pytest.raises(fg.FlipGraphError):
                eng.set_records(bad)
            assert fg.library().fg_last_error(), name
        for e in (eng, twin):
            e.run(1)
        a, b = eng.records(), twin.records()
        compare_records(a, b, "after rejected records")
        assert not np.array_equal(a.fac, good.fac)  # the walks did move


def planted_gauss(rec, rng):
    """Plants in every walk a zero-sum group (a, x_1, c), ..., (a, x_k, c), (a, x_1 ^ ... ^ x_k, c)
    (k = 2..4) at random positions: the scheme stays exact and the Gauss reduction has a
    combination to fold."""
    for w in range(rec.walks):
        n = [int(x) for x in rec.n[w]]
        nn = [n[0] * n[1], n[1] * n[2], n[2] * n[0]]
        m = int(rec.m[w])
        p = int(rng.integers(3))
        j, i = ((p + 1) % 3, (p + 2) % 3) if rng.integers(2) else ((p + 2) % 3, (p + 1) % 3)
        k = int(rng.integers(2, 5))
        xs = [int(rng.integers(1, 1 << nn[j])) for _ in range(k)]
        t = 0
        for x in xs:
            t ^= x
        if t == 0:
            xs[0] ^= 1
            t ^= 1
        a = int(rec.fac[w, p, int(rng.integers(m))])
        c = int(rng.integers(1, 1 << nn[i]))
        terms = [tuple(int(rec.fac[w, q, s]) for q in range(3)) for s in range(m)]
        for x in xs + [t]:
            term = [0, 0, 0]
            term[p], term[j], term[i] = a, x, c
            terms.insert(int(rng.integers(len(terms) + 1)), tuple(term))
        rec.m[w] = len(terms)
        for q in range(3):
            rec.fac[w, q, :] = 0
            rec.fac[w, q, :len(terms)] = [s[q] for s in terms]
        rec.best_fac[w] = rec.fac[w]
        rec.best_m[w] = rec.best_rank[w] = len(terms)


@pytest.mark.parametrize("mode,shape", [("reference", (3, 3, 3)), ("philox", (3, 3, 3)), ("reference", (2, 3, 4)),
                                        ("philox", (4, 4, 4))])
def test_gauss_reduction_vs_oracle(mode, shape):
    """The Gauss (XOR) reduction gated into the walk (no reference counterpart in the walk;
    the reduction itself is pinned against the reference's tryReduceGauss on the CPU) against
    the oracle, on schemes with planted combinations: every field after every launch."""
    n1, n2, n3 = shape
    S, cap, seed = 64, n1 * n2 * n3 + 8, 700 + n1 * n2 * n3
    iters, plus = 40, 100000
    with fg.Engine(S, cap, "z2", mode, seed, iters, plus, 0.01, 0.0, gauss_p=80.0) as eng:
        eng.init_naive(n1, n2, n3)
        rec = eng.records()
        planted_gauss(rec, np.random.default_rng(seed))
        eng.set_records(rec)
        eng.rebuild_lists()
        rec0 = eng.records()
        m0 = rec0.m.copy()
        assert eng.validate().all()
        eng.run(2)
        rec = eng.records()
        assert eng.validate().all() and eng.validate(best=True).all()
    kw = dict(iterations=iters, plus_iterations=plus, expand_p=0.01, reduce_p=0.0, gauss_p=80.0, seed=seed)
    b = batch_from(rec0)
    if mode == "reference":
        used = int(rec.rng_pos.max())
        draws, unis = fg.xorwow_tape(seed, 0, S, used)
        tape = O.make_tape([(draws[w, :rec.rng_pos[w]], unis[w, :rec.rng_pos[w]]) for w in range(S)])
        O.walk(b, b.cfg("tape", launches=2, **kw), tape)
    else:
        O.walk(b, b.cfg("philox", launches=2, **kw))
    compare_records(rec, b, f"gauss {mode} {shape}")
    assert (rec.m < m0).mean() > 0.5


@pytest.mark.parametrize("kernel,lanes", [("thread", 0), ("group", 8), ("warp", 0)], ids=["thread", "group8", "warp"])
@pytest.mark.parametrize("shape", [(3, 3, 3), (2, 3, 4), (4, 4, 4)])
def test_fast_mode_gauss_reduction_vs_oracle(shape, kernel, lanes):
    """The Gauss (XOR) reduction in the fast mode (gated after the reduction gate, Philox stream,
    partner counts kept through the fold and the compaction) on schemes with planted
    combinations, on every fast kernel: field for field equal to the oracle's fast mode."""
    n1, n2, n3 = shape
    S, cap, seed = 64, n1 * n2 * n3 + 8, 900 + n1 * n2 * n3
    iters, plus = 60, 100000
    with fg.Engine(S, cap, "z2", "philox", seed, iters, plus, 0.01, 0.0) as src:
        src.init_naive(n1, n2, n3)
        rec = src.records()
    planted_gauss(rec, np.random.default_rng(seed))
    fast = fg.Records(S, cap, "z2", lists=False)
    for f in ("n", "m", "fac", "best_fac", "best_rank", "best_m"):
        getattr(fast, f)[...] = getattr(rec, f)
    with fg.Engine(S, cap, "z2", "fast", seed, iters, plus, 0.01, 0.0, gauss_p=60.0, sandwich_p=10.0) as eng:
        eng.set_fast_kernel(kernel, lanes)
        eng.set_records(fast)
        rec0 = eng.records()
        m0 = rec0.m.copy()
        assert eng.validate().all()
        eng.run(2)
        out = eng.records()
        assert eng.validate().all() and eng.validate(best=True).all()
    kw = dict(iterations=iters, plus_iterations=plus, expand_p=0.01, reduce_p=0.0, gauss_p=60.0, sandwich_p=10.0,
              seed=seed)
    b = run_oracle_like(rec0, kw, 2, "fast")
    compare_records(out, b, f"fast gauss {shape} {kernel}")
    assert (out.m < m0).mean() > 0.5


@pytest.mark.parametrize("mode,shape,resize_p", [("reference", (3, 3, 3), 0.0), ("philox", (2, 3, 3), 0.0),
                                                 ("reference", (2, 2, 3), 0.6)])
def test_ternary_sandwiching_vs_oracle(mode, shape, resize_p):
    """Opt-in ternary sandwiching (signed permutations; the reference's move is empty) against
    the oracle, with the basis changes on: every field after the launches, schemes exact."""
    n1, n2, n3 = shape
    S, iters, plus, launches = 16, 80, 40, 3
    seed = 800 + n1 + n2 + n3
    cap = 352 if resize_p > 0 else n1 * n2 * n3
    kw = dict(resize_p=resize_p, sandwich_p=20.0, basis_p=10.0)
    with fg.Engine(S, cap, "zt", mode, seed, iters, plus, 0.01, 0.0, zt_sandwich=True, **kw) as eng:
        eng.init_naive(n1, n2, n3)
        rec0 = eng.records()
        eng.run(launches)
        rec = eng.records()
        assert eng.validate().all() and eng.validate(best=True).all()
    b = batch_from(rec0)
    b.best_n[:] = rec0.n
    cfg = dict(iterations=iters, plus_iterations=plus, expand_p=0.01, reduce_p=0.0, seed=seed, zt_sandwich=1, **kw)
    if mode == "reference":
        used = int(rec.rng_pos.max())
        draws, unis = fg.xorwow_tape(seed, 0, S, used)
        tape = O.make_tape([(draws[w, :rec.rng_pos[w]], unis[w, :rec.rng_pos[w]]) for w in range(S)])
        O.walk(b, b.cfg("tape", launches=launches, **cfg), tape)
    else:
        O.walk(b, b.cfg("philox", launches=launches, **cfg))
    compare_records(rec, b, f"ternary sandwiching {mode} {shape}")


def test_autotune_and_graph_replay_keep_trajectories():
    """fg_autotune times the kernels on a snapshot it puts back, and the later launches replay a
    captured CUDA graph: the records after four launches equal those of an untuned run."""
    shapes = [(2, 2, 3), (3, 3, 3), (3, 4, 5), (4, 4, 4), (5, 5, 5)]
    per = 640
    S = per * len(shapes)
    sh = np.array([shapes[w // per] for w in range(S)], np.int32)
    out = []
    for tune in (False, True):
        with fg.Engine(S, 125, "z2", "fast", 31, 400, 2000, 0.5, 0.0) as eng:
            eng.init_naive_shapes(sh)
            if tune:
                choice = eng.autotune(100)
                assert len(choice) == len(shapes)
                assert all(k in (0, 1, 2) and (w in (1, 2, 4, 6, 8) if k == 0 else w == 0) for k, _, w in choice)
            for _ in range(4):
                eng.run(1)
            out.append(eng.records())
            assert eng.validate().all()
    for f in ("n", "m", "fac", "flips", "best_rank", "best_m", "best_fac", "rng_pos", "status"):
        assert np.array_equal(getattr(out[0], f), getattr(out[1], f)), f


@pytest.mark.parametrize("ring", ["z2", "zt"])
def test_list_autotune_keeps_bit_exact_trajectories(ring):
    """In the reference mode fg_autotune picks each segment's warps per block for the thread-per-walk
    list kernel on a snapshot of records, lists and cuRAND states that it puts back: the tuned run
    equals the untuned one field for field, lists and stream positions included."""
    shapes = [(2, 2, 2), (2, 3, 3), (3, 3, 3), (2, 4, 4)]
    per = 1536
    S = per * len(shapes)
    sh = np.array([shapes[w // per] for w in range(S)], np.int32)
    out = []
    for tune in (False, True):
        with fg.Engine(S, 32, ring, "reference", 17, 300, 2000, 0.5, 0.0) as eng:
            eng.set_list_kernel("thread")
            eng.init_naive_shapes(sh)
            if tune:
                choice = eng.autotune(50)
                assert len(choice) == len(shapes)
                assert all(k == 0 and l == 0 and w in (2, 4, 6, 8) for k, l, w in choice)
            for _ in range(3):
                eng.run(1)
            out.append(eng.records())
            assert eng.validate().all()
    for f in ("n", "m", "fac", "sgn", "flips", "best_rank", "best_m", "best_fac", "rng_pos", "status",
              "list_size", "list_pairs"):
        a, o = getattr(out[0], f, None), getattr(out[1], f, None)
        if a is not None:
            assert np.array_equal(a, o), f


@pytest.mark.parametrize("shape,S", [((3, 3, 3), 256), ((4, 4, 4), 256), ((2, 4, 8), 256), ((3, 3, 3), 10240)])
def test_fast_minimize_vs_oracle(shape, S):
    """The fast-mode minimizer (warp per walk for few walks, thread per walk for many; Philox,
    implicit pairs) against the oracle's fast-mode minimizeKernel: best complexities, schemes
    and stream positions."""
    n1, n2, n3 = shape
    cap, seed = n1 * n2 * n3, 515
    with fg.Engine(S, cap, "z2", "fast", seed, 600, 100000) as eng:
        eng.init_naive(n1, n2, n3)
        eng.run(1)
        rec0 = eng.records()
        best0 = O.complexity("z2", rec0.n, rec0.m, rec0.fac)
        bc = eng.minimize(best0.copy())
        rec = eng.records()
        assert eng.validate().all() and eng.validate(best=True).all()
    b = batch_from(rec0)
    obc = best0.copy()
    O.minimize(b, b.cfg("fast", iterations=600, plus_iterations=100000, seed=seed), obc)
    assert np.array_equal(bc, obc)
    assert (bc <= best0).all() and (bc < best0).any()
    for f in ("m", "fac", "best_m", "best_fac", "rng_pos", "status"):
        a, o = getattr(rec, f), getattr(b, f)
        assert np.array_equal(a, o), f


@pytest.mark.parametrize("ring,mode", [("z2", "reference"), ("z2", "philox"), ("zt", "reference"), ("zt", "philox")])
def test_list_kernels_agree_on_a_large_mixed_batch(ring, mode):
    """20,480 walks over several shapes: the automatic choice takes the thread-per-walk list
    kernel (enough walks to fill the GPU); it equals the warp-per-walk kernel field for field."""
    shapes = [(2, 2, 2), (2, 2, 3), (2, 3, 4), (3, 3, 4), (3, 4, 5), (4, 4, 4)]
    S = 20480
    sh = np.array([shapes[w * len(shapes) // S] for w in range(S)], np.int32)
    out = {}
    for kernel in ("warp", "thread", "auto"):
        with fg.Engine(S, 64, ring, mode, 5, 300 if ring == "zt" else 600, 300, 2.0, 0.0) as eng:
            eng.set_list_kernel(kernel)
            eng.init_naive_shapes(sh)
            eng.run(2)
            out[kernel] = eng.records()
            assert eng.validate().all() and eng.validate(best=True).all()
    compare_records(out["thread"], out["warp"], f"{ring} {mode} thread vs warp")
    compare_records(out["auto"], out["warp"], f"{ring} {mode} auto vs warp")


@pytest.mark.parametrize("shape", [(3, 4, 5), (4, 4, 5), (5, 5, 5), (2, 3, 10)])
def test_zt_thread_list_kernel_on_wide_factors_vs_oracle(shape):
    """Ternary factors of 17-31 entries in the thread-per-walk list kernel (32-bit words standing
    for the reference's sign-extended 64-bit factors): random splits draw two chunks, the records
    come back sign-extended; field for field equal to the oracle replaying the cuRAND stream."""
    n1, n2, n3 = shape
    S, iters, plus, expand_p = 64, 300, 60, 3.0
    cap = n1 * n2 * n3 + 8
    seed = 900 + n1 * 100 + n2 * 10 + n3
    kw = dict(iterations=iters, plus_iterations=plus, expand_p=expand_p, reduce_p=0.0)
    with fg.Engine(S, cap, "zt", "reference", seed, iters, plus, expand_p, 0.0) as eng:
        eng.set_list_kernel("thread")
        eng.init_naive(n1, n2, n3)
        rec0 = eng.records()
        eng.run(2)
        rec = eng.records()
        assert eng.validate().all() and eng.validate(best=True).all()
    b = run_oracle_like(rec0, kw, 2, "tape", xorwow_tape_for(rec, seed))
    compare_records(rec, b, f"zt wide {shape}")
    hi = rec.fac >> np.uint64(31)  # bits 31-63: all zero or all one
    assert np.isin(hi, [0, (1 << 33) - 1]).all()


@pytest.mark.parametrize("mode", ["philox", "reference"])
def test_zt_thread_list_kernel_splits_wide_factors_vs_oracle(mode):
    """From a scheme below the naive rank the ternary walks split factors of 20 entries (two
    16-bit chunks, the second sign-extended in the reference); the thread-per-walk kernel's
    32-bit words follow the oracle field for field, records written back sign-extended."""
    (n1, n2, n3), terms = strassen_blocks(5)
    S, cap, seed, iters, plus = 64, 48, 97, 1500, 60
    m = len(terms)
    rec = fg.Records(S, cap, "zt")
    rec.n[:] = (n1, n2, n3)
    rec.m[:] = m
    for t, tri in enumerate(terms):
        for c, d in enumerate(tri):
            for e, x in d.items():
                rec.fac[:, c, t] |= np.uint64(1 << e)
                if x < 0:
                    rec.sgn[:, c, t] |= np.uint64(1 << e)
    rec.valid[:, :, :m] = 1
    rec.best_fac[:] = rec.fac
    rec.best_sgn[:] = rec.sgn
    rec.best_valid[:] = rec.valid
    rec.best_rank[:] = m
    rec.best_m[:] = m
    kw = dict(iterations=iters, plus_iterations=plus, expand_p=200.0, reduce_p=0.0, seed=seed)
    with fg.Engine(S, cap, "zt", mode, seed, iters, plus, 200.0, 0.0) as eng:
        eng.set_list_kernel("thread")
        eng.set_records(rec)
        eng.rebuild_lists()
        rec0 = eng.records()
        assert eng.validate().all()
        eng.run(2)
        out = eng.records()
        assert eng.validate().all() and eng.validate(best=True).all()
    tape = xorwow_tape_for(out, seed) if mode == "reference" else None
    b = run_oracle_like(rec0, kw, 2, "tape" if mode == "reference" else "philox", tape)
    compare_records(out, b, f"zt splits {mode}")
    assert (out.m != m).any()


def test_zt_factors_of_32_entries_take_the_warp_kernel():
    """A naive factor of 32 entries sets bit 31 without copying it into bits 32-63, which the
    thread kernel's 32-bit words cannot stand for: the thread kernel is refused, the automatic
    choice runs the warp kernel."""
    with fg.Engine(64, 72, "zt", "reference", 5, 100, 60, 0.01, 0.0) as eng:
        eng.set_list_kernel("thread")
        eng.init_naive(2, 4, 8)
        with pytest.raises(fg.FlipGraphError):
            eng.run(1)
    with fg.Engine(64, 72, "zt", "reference", 5, 100, 60, 0.01, 0.0) as eng:
        eng.init_naive(2, 4, 8)
        st = eng.run(1)
        assert st["walks_valid"] == 64


def test_zt_wide_records_with_an_invalid_factor_take_the_warp_kernel():
    """An input factor marked invalid (valid = 0) has no place in the 32-bit words of factors of
    > 16 entries: the thread kernel is refused for such records, the automatic choice takes the
    warp kernel, and the walk still follows the oracle."""
    S, n, seed, iters = 64, (3, 4, 5), 77, 200
    with fg.Engine(S, 68, "zt", "reference", seed, iters, 60, 0.01, 0.0) as eng:
        eng.init_naive(*n)
        rec0 = eng.records()
    rec0.valid[5, 0, 3] = 0
    rec0.best_valid[5, 0, 3] = 0
    with fg.Engine(S, 68, "zt", "reference", seed, iters, 60, 0.01, 0.0) as eng:
        eng.set_records(rec0)
        eng.set_list_kernel("thread")
        with pytest.raises(fg.FlipGraphError):
            eng.run(1)
    with fg.Engine(S, 68, "zt", "reference", seed, iters, 60, 0.01, 0.0) as eng:
        eng.set_records(rec0)
        eng.run(1)
        rec = eng.records()
    b = run_oracle_like(rec0, dict(iterations=iters, plus_iterations=60, expand_p=0.01, reduce_p=0.0), 1, "tape",
                        xorwow_tape_for(rec, seed))
    compare_records(rec, b, "zt wide, one invalid factor")


def test_thread_list_kernel_is_refused_where_it_does_not_apply():
    with fg.Engine(32, 27, "zt", "reference", 1, 10, 100, sandwich_p=1.0) as eng:
        with pytest.raises(fg.FlipGraphError):
            eng.set_list_kernel("thread")
    with fg.Engine(32, 27, "z2", "reference", 1, 10, 100, gauss_p=1.0) as eng:
        with pytest.raises(fg.FlipGraphError):
            eng.set_list_kernel("thread")


@pytest.mark.parametrize("kernel,lanes", [("thread", 0), ("group", 8), ("warp", 0)])
@pytest.mark.parametrize("m", [5, 6, 7, 8])
def test_fast_mode_flip_of_a_zero_factor_vs_oracle(kernel, lanes, m):
    """A term with a zero factor (the reference's random split can leave one) flipped on its
    equal partner: the flip's old factor is zero, which also matches the empty slots past the
    rank.  Every fast kernel must leave those slots alone and follow the oracle."""
    S, cap, seed = 64, 8, 321
    terms = [(1, 1, 1), (1, 0, 2), (2, 4, 4), (4, 8, 8), (8, 2, 4), (3, 5, 6), (5, 6, 3), (6, 3, 5)][:m]
    rec0 = fg.Records(S, cap, "z2")
    rec0.n[:] = (2, 2, 2)
    rec0.m[:] = m
    rec0.fac[:] = 0
    for t, uvw in enumerate(terms):
        for c in range(3):
            rec0.fac[:, c, t] = uvw[c]
    rec0.best_fac[:] = rec0.fac
    rec0.best_rank[:] = m
    rec0.best_m[:] = m
    kw = dict(iterations=60, plus_iterations=10**6, expand_p=0.0, reduce_p=0.0, seed=seed)
    with fg.Engine(S, cap, "z2", "fast", seed, 60, 10**6, 0.0, 0.0) as eng:
        eng.set_fast_kernel(kernel, lanes)
        eng.set_records(rec0)
        rec0 = eng.records()
        eng.run(1)
        rec = eng.records()
    assert not rec.status.any()
    b = run_oracle_like(rec0, kw, 1, "fast")
    compare_records(rec, b, f"zero factor {kernel} m={m}")
