"""ctypes binding of the CPU oracle (oracle/fg_oracle.cpp) -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg import
this module, and only as the checker / the CPU baseline; the product never
does.  The walk-record arrays here have the same layout as the CUDA
library's exported records (include/flipgraph.h), so results compare with
numpy equality.
"""
import ctypes
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MAX_PAIRS = 500
RING = {"z2": 0, "zt": 1, "zb": 2}
RNG = {"tape": 0, "philox": 1, "fast": 2}


def lib_path():
    return os.path.join(HERE, "build", platform.machine(), "libfg_oracle.so")


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return lib_path()


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            build()
        _lib = ctypes.CDLL(path)
        _lib.fgo_walk.restype = ctypes.c_int
        _lib.fgo_init_naive.restype = ctypes.c_int
        _lib.fgo_minimize.restype = ctypes.c_int
        _lib.fgo_validate.restype = ctypes.c_int
        _lib.fgo_reduce.restype = ctypes.c_int
        _lib.fgo_reduce_schemes.restype = ctypes.c_int
        _lib.fgo_flip_schemes.restype = ctypes.c_int
        _lib.fgo_reduce_gauss.restype = ctypes.c_int
        _lib.fgo_validate_zb.restype = ctypes.c_int
        _lib.fgo_lookahead_ttr.restype = ctypes.c_int
    return _lib


class WalkCfg(ctypes.Structure):
    _fields_ = [("ring", ctypes.c_int32), ("rng", ctypes.c_int32), ("cap", ctypes.c_int32),
                ("iterations", ctypes.c_int32), ("plus_iterations", ctypes.c_int32),
                ("launches", ctypes.c_int32), ("expand_p", ctypes.c_double),
                ("reduce_p", ctypes.c_double), ("seed", ctypes.c_uint64), ("resize_p", ctypes.c_double),
                ("sandwich_p", ctypes.c_double), ("basis_p", ctypes.c_double), ("gauss_p", ctypes.c_double),
                ("zt_sandwich", ctypes.c_int32), ("retry_cap", ctypes.c_int32)]


class _Batch(ctypes.Structure):
    _fields_ = [(name, ctypes.c_void_p) for name in
                ("n", "m", "fac", "sgn", "valid", "list_size", "list_pairs", "flips", "best_rank",
                 "best_m", "best_fac", "best_sgn", "best_valid", "rng_pos", "status", "accepted", "best_n",
                 "fac2", "best_fac2")]


class _Tape(ctypes.Structure):
    _fields_ = [("draws", ctypes.c_void_p), ("uniforms", ctypes.c_void_p), ("offsets", ctypes.c_void_p)]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class WalkBatch:
    """S walk records with `cap` factor slots each (numpy, C-contiguous)."""

    FIELDS = ("n", "m", "fac", "sgn", "valid", "list_size", "list_pairs", "flips", "best_rank",
              "best_m", "best_fac", "best_sgn", "best_valid", "rng_pos", "status", "accepted", "best_n",
              "fac2", "best_fac2")

    def __init__(self, S, cap, ring="z2"):
        self.S, self.cap, self.ring = S, cap, ring
        zt = ring == "zt"
        zb = ring == "zb"
        signed = zt or zb
        self.n = np.zeros((S, 3), np.int32)
        self.m = np.zeros(S, np.int32)
        self.fac = np.zeros((S, 3, cap), np.uint64)
        self.sgn = np.zeros((S, 3, cap), np.uint64) if signed else None
        self.valid = np.zeros((S, 3, cap), np.uint8) if zt else None
        self.list_size = np.zeros((S, 3), np.int32)
        self.list_pairs = np.zeros((S, 3, MAX_PAIRS), np.uint32)
        self.flips = np.zeros(S, np.int32)
        self.best_rank = np.zeros(S, np.int32)
        self.best_m = np.zeros(S, np.int32)
        self.best_fac = np.zeros((S, 3, cap), np.uint64)
        self.best_sgn = np.zeros((S, 3, cap), np.uint64) if signed else None
        self.best_valid = np.zeros((S, 3, cap), np.uint8) if zt else None
        self.rng_pos = np.zeros(S, np.int64)
        self.status = np.zeros(S, np.int32)
        self.accepted = np.zeros(S, np.int64)
        self.best_n = np.zeros((S, 3), np.int32)
        self.fac2 = np.zeros((S, 3, cap), np.uint64) if zb else None
        self.best_fac2 = np.zeros((S, 3, cap), np.uint64) if zb else None

    def copy(self):
        b = WalkBatch.__new__(WalkBatch)
        b.S, b.cap, b.ring = self.S, self.cap, self.ring
        for f in self.FIELDS:
            v = getattr(self, f)
            setattr(b, f, None if v is None else v.copy())
        return b

    def _c(self):
        return _Batch(*[_ptr(getattr(self, f)) for f in self.FIELDS])

    def cfg(self, rng="tape", iterations=1000, plus_iterations=8000, launches=1, expand_p=0.01,
            reduce_p=0.0, seed=0, resize_p=0.0, sandwich_p=0.0, basis_p=0.0, gauss_p=0.0, zt_sandwich=0,
            retry_cap=0):
        return WalkCfg(RING[self.ring], RNG[rng], self.cap, iterations, plus_iterations, launches,
                       expand_p, reduce_p, seed, resize_p, sandwich_p, basis_p, gauss_p, zt_sandwich, retry_cap)


def make_tape(tapes):
    """tapes: list of (draws uint32 array, uniforms float32 array) per walk."""
    offs = np.zeros(len(tapes) + 1, np.int64)
    for i, (d, _) in enumerate(tapes):
        offs[i + 1] = offs[i] + len(d)
    draws = np.concatenate([np.asarray(d, np.uint32) for d, _ in tapes]) if tapes else np.zeros(0, np.uint32)
    unis = np.concatenate([np.asarray(u, np.float32) for _, u in tapes]) if tapes else np.zeros(0, np.float32)
    draws = np.ascontiguousarray(draws)
    unis = np.ascontiguousarray(unis)
    return (draws, unis, offs)


def _tape_c(tape):
    if tape is None:
        return None, None
    draws, unis, offs = tape
    return _Tape(_ptr(draws), _ptr(unis), _ptr(offs)), (draws, unis, offs)


def init_naive(batch, n1, n2, n3):
    cfg = batch.cfg()
    cb = batch._c()
    return lib().fgo_init_naive(ctypes.byref(cfg), batch.S, n1, n2, n3, ctypes.byref(cb))


def walk(batch, cfg, tape=None):
    cb = batch._c()
    t, _keep = _tape_c(tape)
    return lib().fgo_walk(ctypes.byref(cfg), batch.S, ctypes.byref(cb), ctypes.byref(t) if t else None)


def lookahead_ttr(shape, walks, target, max_steps, plus_iterations=50000, expand_p=0.01, iterations=1000,
                  seed=1, greedy=False):
    """Steps from the naive scheme to rank `target` per fast-mode Z2 walk under the uniform
    proposal or (greedy) an exact one-step lookahead that takes a rank-lowering flip
    whenever one exists; -1 for a walk that did not get there within max_steps."""
    n1, n2, n3 = shape
    steps = np.zeros(walks, np.int64)
    rc = lib().fgo_lookahead_ttr(n1, n2, n3, walks, target, ctypes.c_int64(max_steps), plus_iterations,
                                 ctypes.c_double(expand_p), iterations, ctypes.c_uint64(seed), int(greedy),
                                 steps.ctypes.data_as(ctypes.c_void_p))
    if rc < 0:
        raise ValueError("unsupported shape")
    return steps


def reduce_gauss(batch, cfg, tape=None):
    """One SchemeZ2::tryReduceGauss call per walk, as the reference makes it; returns the
    per-walk found flags."""
    cb = batch._c()
    t, _keep = _tape_c(tape)
    found = np.zeros(batch.S, np.int32)
    rc = lib().fgo_reduce_gauss(ctypes.byref(cfg), batch.S, ctypes.byref(cb), ctypes.byref(t) if t else None,
                                _ptr(found))
    assert rc == 0
    return found


def minimize(batch, cfg, best_complexity, tape=None):
    cb = batch._c()
    t, _keep = _tape_c(tape)
    return lib().fgo_minimize(ctypes.byref(cfg), batch.S, ctypes.byref(cb), ctypes.byref(t) if t else None,
                              _ptr(best_complexity))


def validate(batch, best=False):
    out = np.zeros(batch.S, np.uint8)
    m = batch.best_m if best else batch.m
    n = batch.best_n if best and batch.best_n.any() else batch.n
    fac = batch.best_fac if best else batch.fac
    sgn = batch.best_sgn if best else batch.sgn
    val = batch.best_valid if best else batch.valid
    if batch.ring == "zb":
        fac2 = batch.best_fac2 if best else batch.fac2
        lib().fgo_validate_zb(batch.S, batch.cap, _ptr(np.ascontiguousarray(n)), _ptr(m), _ptr(fac), _ptr(sgn),
                              _ptr(fac2), _ptr(out))
        return out.astype(bool)
    lib().fgo_validate(RING[batch.ring], batch.S, batch.cap, _ptr(np.ascontiguousarray(n)), _ptr(m), _ptr(fac),
                       _ptr(sgn), _ptr(val), _ptr(out))
    return out.astype(bool)


def zb_coefficients(fac, sgn, fac2):
    """int8 coefficient arrays [..., 64] from ZB sign-magnitude masks."""
    bits = np.arange(64, dtype=np.uint64)
    nz = (fac[..., None] >> bits) & np.uint64(1)
    neg = (sgn[..., None] >> bits) & np.uint64(1)
    two = (fac2[..., None] >> bits) & np.uint64(1)
    mag = nz.astype(np.int8) * (1 + two.astype(np.int8))
    return np.where(neg.astype(bool), -mag, mag).astype(np.int8)


def validate_arrays(ring, n, m, fac, sgn=None, valid=None):
    n = np.ascontiguousarray(n, np.int32)
    m = np.ascontiguousarray(m, np.int32)
    fac = np.ascontiguousarray(fac, np.uint64)
    S, _, cap = fac.shape
    out = np.zeros(S, np.uint8)
    lib().fgo_validate(RING[ring], S, cap, _ptr(n), _ptr(m), _ptr(fac),
                       _ptr(None if sgn is None else np.ascontiguousarray(sgn, np.uint64)),
                       _ptr(None if valid is None else np.ascontiguousarray(valid, np.uint8)), _ptr(out))
    return out.astype(bool)


def complexity(ring, n, m, fac):
    n = np.ascontiguousarray(n, np.int32)
    m = np.ascontiguousarray(m, np.int32)
    fac = np.ascontiguousarray(fac, np.uint64)
    S, _, cap = fac.shape
    out = np.zeros(S, np.int32)
    lib().fgo_complexity(RING[ring], S, cap, _ptr(n), _ptr(m), _ptr(fac), _ptr(out))
    return out


def set_fma(fuse_float, fuse_double):
    lib().fgo_set_fma(int(fuse_float), int(fuse_double))


def reduce(n, m, coef, count, tape=None, independent=True, rng="tape", seed=0, best=None):
    """One additions-reducer launch; returns (out[count,9], modes[count,3], consumed[count], state)."""
    coef = np.ascontiguousarray(coef, np.int8)
    assert coef.shape == (3, m, 64)
    out = np.zeros((count, 9), np.int32)
    modes = np.zeros((count, 3), np.int32)
    consumed = np.zeros(count, np.int64)
    t, _keep = _tape_c(tape)
    state = ctypes.c_void_p()
    lib().fgo_reduce(n[0], n[1], n[2], m, _ptr(coef), count, int(independent),
                     ctypes.byref(t) if t else None, RNG[rng], ctypes.c_uint64(seed), _ptr(out), _ptr(modes),
                     _ptr(consumed), best, ctypes.byref(state))
    # out columns per component: additions, fresh, naive
    return out, modes, consumed, state


def tape_tail(tape, used):
    """The tape with the first used[w] draws of every walk consumed (a stream continued)."""
    draws, unis, offs = tape
    parts = [(draws[offs[w] + used[w]:offs[w + 1]], unis[offs[w] + used[w]:offs[w + 1]]) for w in range(len(offs) - 1)]
    return make_tape(parts)


def flip_schemes(n, m, coef0, schemes, max_flips, tape):
    """flipSchemesKernel: schemes 1.. := scheme 0 after up to max_flips ZT flips (stream s = tape walk s).
    Returns (coef [schemes,3,m,64], ranks [schemes], consumed [schemes], status count)."""
    coef0 = np.ascontiguousarray(coef0, np.int8)
    assert coef0.shape == (3, m, 64)
    coef = np.zeros((schemes, 3, m, 64), np.int8)
    ranks = np.zeros(schemes, np.int32)
    consumed = np.zeros(schemes, np.int64)
    t, _keep = _tape_c(tape)
    bad = lib().fgo_flip_schemes(n[0], n[1], n[2], m, _ptr(coef0), schemes, max_flips, ctypes.byref(t), _ptr(coef),
                                 _ptr(ranks), _ptr(consumed))
    return coef, ranks, consumed, bad


def reduce_schemes(n, m, coef, ranks, count, tape, independent=False, best=None):
    """One reducer launch over several schemes (reducer r: scheme r % schemes at rank ranks[s]).
    Returns (out[count,9], modes[count,3], consumed[count], vars[count,3,500,2])."""
    coef = np.ascontiguousarray(coef, np.int8)
    schemes = coef.shape[0]
    assert coef.shape == (schemes, 3, m, 64)
    ranks = np.ascontiguousarray(ranks, np.int32)
    out = np.zeros((count, 9), np.int32)
    modes = np.zeros((count, 3), np.int32)
    consumed = np.zeros(count, np.int64)
    vars_ = np.zeros((count, 3, 500, 2), np.int32)
    t, _keep = _tape_c(tape)
    lib().fgo_reduce_schemes(n[0], n[1], n[2], m, _ptr(coef), _ptr(ranks), schemes, count, int(independent),
                             ctypes.byref(t), _ptr(out), _ptr(modes), _ptr(consumed), best, _ptr(vars_))
    return out, modes, consumed, vars_


def reducer_state_free(state):
    lib().fgo_reducer_state_free(state)


def reducer_state(fresh, vars_):
    """Incumbent state from fresh counts [3] and variables [3][500][2]."""
    f = np.ascontiguousarray(fresh, np.int32)
    v = np.ascontiguousarray(vars_, np.int32)
    lib().fgo_reducer_state_make.restype = ctypes.c_void_p
    return ctypes.c_void_p(lib().fgo_reducer_state_make(_ptr(f), _ptr(v)))


def philox(ctr, key):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib().fgo_philox4x32_10(c, k, o)
    return list(o)
