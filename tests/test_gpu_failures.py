"""Failure paths on the GPU, made on purpose and bounded: no test here faults,
traps or hangs a GPU.

* A retry bound that runs out.  The reference leaves tryPlus's pair rejection
  unbounded (scheme_z2.cu:1036-1039, scheme_integer.cu:984-987): on a scheme
  where every pair of terms shares a factor it would spin forever.  Here the
  loop stops after `retry_cap` redraws, the walk's status gets FG_WALK_RETRY,
  fg_run returns FG_ERR_WALK, and the stopped state equals the oracle's, which
  bounds the same loop the same way.
* A slot overflow: a handle whose slots are fewer than n1*n2*n3 lets a plus
  transition reach the last slot; the walk stops with FG_WALK_OVERFLOW, again
  equal to the oracle.
* The learned proposal's entropy fallback (uniform choice among the candidates
  when the score distribution's entropy is below the threshold) taken on every
  step.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

fg = pytest.importorskip("flipgraphgpu_gb300")

FG_ERR_WALK = 5
WALK_RETRY, WALK_OVERFLOW = 2, 4


def compare_records(rec, b, ctx=""):
    fields = ["n", "m", "fac", "list_size", "list_pairs", "flips", "best_rank", "best_m", "best_fac", "rng_pos",
              "status"]
    if rec.ring == "zt":
        fields += ["sgn", "valid", "best_sgn", "best_valid"]
    for f in fields:
        a, o = getattr(rec, f), getattr(b, f)
        if not np.array_equal(a, o):
            bad = np.argwhere(a != o)
            raise AssertionError(f"{ctx}: field {f} differs at {bad[:5].tolist()} (of {len(bad)})")


def put_scheme(rec, ring, shape, terms):
    """Writes the same scheme (terms = [(u, v, w)] of nonnegative bit masks) into every walk."""
    m = len(terms)
    rec.n[:] = shape
    rec.m[:] = m
    rec.fac[:] = 0
    for t, uvw in enumerate(terms):
        for c in range(3):
            rec.fac[:, c, t] = uvw[c]
    if ring == "zt":
        rec.sgn[:] = 0
        rec.valid[:] = 0
        rec.valid[:, :, :m] = 1
    rec.best_fac[:] = rec.fac
    if ring == "zt":
        rec.best_sgn[:] = rec.sgn
        rec.best_valid[:] = rec.valid
    rec.best_rank[:] = m
    rec.best_m[:] = m
    rec.flips[:] = 0
    rec.list_size[:] = 0
    rec.list_pairs[:] = 0


def oracle_twin(rec0, cfg_kw, rng, tape=None):
    b = O.WalkBatch(rec0.walks, rec0.cap, rec0.ring)
    fields = ["n", "m", "fac", "list_size", "list_pairs", "flips", "best_rank", "best_m", "best_fac", "rng_pos"]
    if rec0.ring == "zt":
        fields += ["sgn", "valid", "best_sgn", "best_valid"]
    for f in fields:
        getattr(b, f)[...] = getattr(rec0, f)
    O.walk(b, b.cfg(rng, launches=1, **cfg_kw), tape)
    return b


def run_stopped(eng):
    """One launch that must end with some walk stopped: fg_run returns FG_ERR_WALK."""
    with pytest.raises(fg.FlipGraphError) as e:
        eng.run(1)
    assert e.value.status == FG_ERR_WALK
    return eng.records()


# Two terms sharing their first factor: every pair shares a factor, so tryPlus can never
# find its two terms; flips keep the other factors distinct and nonzero, so the rank
# stays 2.  Plus after every flip.
STUCK = [(1, 1, 1), (1, 2, 2)]


@pytest.mark.parametrize("ring,mode,kernel", [("z2", "reference", None), ("z2", "philox", None),
                                              ("z2", "fast", "thread"), ("z2", "fast", "warp"),
                                              ("zt", "reference", None), ("zt", "philox", None)])
def test_retry_bound_runs_out_like_the_oracle(ring, mode, kernel):
    S, cap, seed, cap_retry = 64, 8, 4242, 50
    iters, plus = 40, 1
    with fg.Engine(S, cap, ring, mode, seed, iters, plus, 0.0, 0.0, retry_cap=cap_retry) as eng:
        if kernel:
            eng.set_fast_kernel(kernel)
        rec0 = fg.Records(S, cap, ring)
        put_scheme(rec0, ring, (2, 2, 2), STUCK)
        eng.set_records(rec0)
        if mode != "fast":
            eng.rebuild_lists()
        rec0 = eng.records()
        rec = run_stopped(eng)
    assert (rec.status & WALK_RETRY).all(), rec.status
    # every walk stopped at its first plus transition, right after one accepted flip
    assert (rec.m == 2).all()
    assert (rec.rng_pos > 2 * cap_retry).all()
    kw = dict(iterations=iters, plus_iterations=plus, expand_p=0.0, reduce_p=0.0, seed=seed, retry_cap=cap_retry)
    tape = None
    if mode == "reference":
        used = int(rec.rng_pos.max())
        draws, unis = fg.xorwow_tape(seed, 0, S, used)
        tape = O.make_tape([(draws[w, :rec.rng_pos[w]], unis[w, :rec.rng_pos[w]]) for w in range(S)])
    b = oracle_twin(rec0, kw, {"reference": "tape", "philox": "philox", "fast": "fast"}[mode], tape)
    compare_records(rec, b, f"{ring} {mode}")


def test_default_bound_lets_the_same_walks_run():
    """With the default bound a feasible scheme never stops: the naive 2x2x2 scheme with plus
    after every flip runs the whole launch and every walk stays valid."""
    with fg.Engine(64, 8, "z2", "fast", 7, 500, 1, 0.0, 0.0) as eng:
        eng.init_naive(2, 2, 2)
        st = eng.run(1)
        assert st["walks_failed"] == 0 and st["walks_valid"] == 64
        assert not eng.records().status.any()


@pytest.mark.parametrize("mode", ["reference", "fast"])
def test_slot_overflow_stops_the_walk_like_the_oracle(mode):
    """Four slots for a 2x2x2 scheme of rank 4: the first plus transition needs a fifth slot."""
    S, cap, seed, iters, plus = 64, 4, 99, 40, 1
    terms = [(1, 1, 1), (1, 2, 2), (2, 4, 4), (4, 8, 8)]
    with fg.Engine(S, cap, "z2", mode, seed, iters, plus, 0.0, 0.0) as eng:
        rec0 = fg.Records(S, cap, "z2")
        put_scheme(rec0, "z2", (2, 2, 2), terms)
        eng.set_records(rec0)
        if mode != "fast":
            eng.rebuild_lists()
        rec0 = eng.records()
        rec = run_stopped(eng)
    assert (rec.status & WALK_OVERFLOW).all(), rec.status
    kw = dict(iterations=iters, plus_iterations=plus, expand_p=0.0, reduce_p=0.0, seed=seed)
    tape = None
    if mode == "reference":
        used = int(rec.rng_pos.max())
        draws, unis = fg.xorwow_tape(seed, 0, S, used)
        tape = O.make_tape([(draws[w, :rec.rng_pos[w]], unis[w, :rec.rng_pos[w]]) for w in range(S)])
    b = oracle_twin(rec0, kw, "tape" if mode == "reference" else "fast", tape)
    compare_records(rec, b, f"overflow {mode}")


def test_flip_graph_reports_walks_stopped_at_the_retry_bound(tmp_path):
    """The executable keeps running the other walks and says how many stopped."""
    import os
    import subprocess
    exe = os.path.join(os.path.dirname(fg.LIB_PATH), "flip_graph")
    inp = tmp_path / "stuck.txt"
    # flip_graph's text input: a count, then "n1 n2 n3 m" and U, V, W rows (entries of each factor)
    rows = []
    for c in range(3):
        for u in STUCK:
            rows.append(" ".join(str((u[c] >> q) & 1) for q in range(4)))
    inp.write_text("1\n2 2 2 2\n" + "\n".join(rows) + "\n")
    r = subprocess.run([exe, "-n1", "2", "-n2", "2", "-n3", "2", "--ring", "Z2", "--input-path", str(inp),
                        "--schemes", "32", "--max-iterations", "20", "--plus-iterations", "1",
                        "--expand-probability", "0", "--resize-probability", "0", "--retry-cap", "50",
                        "--max-launches", "2", "--seed", "5", "--path", str(tmp_path / "out")],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=120)
    assert r.returncode == 0, r.stdout
    assert "32 walk(s) stopped at a retry bound or a slot overflow" in r.stdout, r.stdout


def test_learned_entropy_fallback_is_taken_on_every_step():
    """min_entropy above log K: every choice among the K candidates is the uniform fallback, so the
    walk equals the one with no network at all, whatever the network; with the threshold at 0 the
    network's scores choose and the walk differs."""
    S, K, seed, iters = 256, 8, 31, 300

    def walk(net, min_entropy):
        with fg.Engine(S, 27, "z2", "learned", seed, iters, 50000, 0.01, 0.0) as eng:
            eng.set_proposal(net, candidates=K, temperature=1.0, min_entropy=min_entropy)
            eng.init_naive(3, 3, 3)
            eng.run(1)
            rec = eng.records()
            assert eng.validate().all()
            return rec

    with fg.Mlp(seed=3) as net_a, fg.Mlp(seed=4) as net_b:
        uniform = walk(None, 0.0)
        fall_a = walk(net_a, 100.0)
        fall_b = walk(net_b, 100.0)
        scored = walk(net_a, 0.0)
    for f in ("m", "fac", "flips", "best_rank", "best_fac", "rng_pos"):
        assert np.array_equal(getattr(fall_a, f), getattr(uniform, f)), f
        assert np.array_equal(getattr(fall_b, f), getattr(uniform, f)), f
    assert not np.array_equal(scored.fac, uniform.fac)
