"""flipgraphgpu_gb300 -- GB300-native flip-graph search for matrix multiplication schemes.

Python view of libflipgraph.so's C ABI (include/flipgraph.h).  The search
itself runs in hand-written sm_103a CUDA kernels; this module only moves
records and calls the library.  There is no CPU fallback: if the CUDA
library cannot be loaded every entry point raises.

    from flipgraphgpu_gb300 import Engine
    eng = Engine(walks=1024, cap=27, seed=1, iterations=10000, plus_iterations=50000)
    eng.init_naive(3, 3, 3)
    stats = eng.run(launches=1)
    rec = eng.records()
"""
import ctypes
import os
import platform

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_lib", platform.machine(), "libflipgraph.so")
LIST_CAP = 500
MAX_RANK = 350
RINGS = {"z2": 0, "zt": 1, "zb": 2}
MODES = {"reference": 0, "philox": 1, "fast": 2, "xorwow": 0, "learned": 3}
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "capacity", 4: "state", 5: "walk failure"}


class FlipGraphError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [("ring", ctypes.c_int32), ("mode", ctypes.c_int32), ("walks", ctypes.c_int32),
                ("cap", ctypes.c_int32), ("seed", ctypes.c_uint64), ("iterations", ctypes.c_int32),
                ("plus_iterations", ctypes.c_int32), ("expand_p", ctypes.c_double), ("reduce_p", ctypes.c_double),
                ("device", ctypes.c_int32), ("walks_per_block", ctypes.c_int32), ("resize_p", ctypes.c_double),
                ("sandwich_p", ctypes.c_double), ("basis_p", ctypes.c_double), ("gauss_p", ctypes.c_double),
                ("zt_sandwich", ctypes.c_int32), ("retry_cap", ctypes.c_int32)]


class _Records(ctypes.Structure):
    _fields_ = [(name, ctypes.c_void_p) for name in
                ("n", "m", "fac", "sgn", "valid", "list_size", "list_pairs", "flips", "best_rank",
                 "best_m", "best_fac", "best_sgn", "best_valid", "rng_pos", "status", "best_n",
                 "fac2", "best_fac2")]


# Element type and per-walk shape of every records field ("cap": the handle's slot count).
_FIELD_LAYOUT = {
    "n": (np.int32, (3,)), "m": (np.int32, ()), "fac": (np.uint64, (3, "cap")), "sgn": (np.uint64, (3, "cap")),
    "valid": (np.uint8, (3, "cap")), "list_size": (np.int32, (3,)), "list_pairs": (np.uint32, (3, LIST_CAP)),
    "flips": (np.int32, ()), "best_rank": (np.int32, ()), "best_m": (np.int32, ()),
    "best_fac": (np.uint64, (3, "cap")), "best_sgn": (np.uint64, (3, "cap")), "best_valid": (np.uint8, (3, "cap")),
    "rng_pos": (np.int64, ()), "status": (np.int32, ()), "best_n": (np.int32, (3,)),
    "fac2": (np.uint64, (3, "cap")), "best_fac2": (np.uint64, (3, "cap")),
}


class Stats(ctypes.Structure):
    _fields_ = [("flips", ctypes.c_uint64), ("verified_flips", ctypes.c_uint64), ("walks_valid", ctypes.c_int32),
                ("walks_failed", ctypes.c_int32), ("min_rank", ctypes.c_int32), ("min_best_rank", ctypes.c_int32),
                ("kernel_ms", ctypes.c_float), ("verify_ms", ctypes.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def library():
    """Loads libflipgraph.so (building it first when only sources are present)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _build
        _build.build()
    lib = ctypes.CDLL(LIB_PATH)
    lib.fg_last_error.restype = ctypes.c_char_p
    lib.fg_version.restype = ctypes.c_char_p
    for name in ("fg_create", "fg_destroy", "fg_init_naive", "fg_set_records", "fg_get_records", "fg_run",
                 "fg_minimize", "fg_validate", "fg_xorwow_tape", "fg_philox_blocks", "fg_init_naive_shapes",
                 "fg_get_counters", "fg_host_alloc", "fg_host_free", "fg_reducer_create", "fg_reducer_run",
                 "fg_reducer_destroy", "fg_set_fast_split", "fg_get_scheme"):
        getattr(lib, name).restype = ctypes.c_int
    _lib = lib
    return lib


def _check(status):
    if status != 0:
        raise FlipGraphError(status, library().fg_last_error().decode())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class PinnedBuffer:
    """Page-locked host memory (fg_host_alloc) viewed as a numpy array."""

    def __init__(self, shape, dtype):
        self.nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self.p = ctypes.c_void_p()
        _check(library().fg_host_alloc(ctypes.c_uint64(self.nbytes), ctypes.byref(self.p)))
        buf = (ctypes.c_uint8 * self.nbytes).from_address(self.p.value)
        self.array = np.frombuffer(buf, dtype=dtype).reshape(shape)

    def __del__(self):
        try:
            if self.p:
                library().fg_host_free(self.p)
        except Exception:
            pass


class Records:
    """Host walk records (the C ABI's fg_records), numpy arrays.

    With pinned=True every array lives in page-locked memory (fast DMA)."""

    FIELDS = _Records._fields_

    def __init__(self, walks, cap, ring="z2", pinned=False, lists=True):
        """lists=False leaves out the FlipSet pairs (the fast and learned modes keep none)."""
        zt = ring == "zt"
        zb = ring == "zb"
        self.walks, self.cap, self.ring = walks, cap, ring
        self._pins = []
        if pinned:
            self._alloc_pinned(walks, cap, zt, zb, lists)
            return
        self.n = np.zeros((walks, 3), np.int32)
        self.m = np.zeros(walks, np.int32)
        self.fac = np.zeros((walks, 3, cap), np.uint64)
        self.sgn = np.zeros((walks, 3, cap), np.uint64) if zt or zb else None
        self.valid = np.zeros((walks, 3, cap), np.uint8) if zt else None
        self.list_size = np.zeros((walks, 3), np.int32)
        self.list_pairs = np.zeros((walks, 3, LIST_CAP), np.uint32) if lists else None
        self.flips = np.zeros(walks, np.int32)
        self.best_rank = np.zeros(walks, np.int32)
        self.best_m = np.zeros(walks, np.int32)
        self.best_fac = np.zeros((walks, 3, cap), np.uint64)
        self.best_sgn = np.zeros((walks, 3, cap), np.uint64) if zt or zb else None
        self.best_valid = np.zeros((walks, 3, cap), np.uint8) if zt else None
        self.rng_pos = np.zeros(walks, np.int64)
        self.status = np.zeros(walks, np.int32)
        self.best_n = np.zeros((walks, 3), np.int32)
        self.fac2 = np.zeros((walks, 3, cap), np.uint64) if zb else None
        self.best_fac2 = np.zeros((walks, 3, cap), np.uint64) if zb else None

    def coefficients(self, best=False):
        """ZB: int8 coefficients [walks][3][cap][64] from the sign-magnitude masks."""
        fac, sgn, two = (self.best_fac, self.best_sgn, self.best_fac2) if best else (self.fac, self.sgn, self.fac2)
        bits = np.arange(64, dtype=np.uint64)
        nz = ((fac[..., None] >> bits) & np.uint64(1)).astype(np.int8)
        mag = nz * (1 + ((two[..., None] >> bits) & np.uint64(1)).astype(np.int8))
        return np.where(((sgn[..., None] >> bits) & np.uint64(1)).astype(bool), -mag, mag).astype(np.int8)

    def _alloc_pinned(self, walks, cap, zt, zb=False, lists=True):
        def pin(shape, dtype):
            b = PinnedBuffer(shape, dtype)
            self._pins.append(b)
            b.array[...] = 0
            return b.array
        self.n = pin((walks, 3), np.int32)
        self.m = pin((walks,), np.int32)
        self.fac = pin((walks, 3, cap), np.uint64)
        self.sgn = pin((walks, 3, cap), np.uint64) if zt or zb else None
        self.valid = pin((walks, 3, cap), np.uint8) if zt else None
        self.list_size = pin((walks, 3), np.int32)
        self.list_pairs = pin((walks, 3, LIST_CAP), np.uint32) if lists else None
        self.flips = pin((walks,), np.int32)
        self.best_rank = pin((walks,), np.int32)
        self.best_m = pin((walks,), np.int32)
        self.best_fac = pin((walks, 3, cap), np.uint64)
        self.best_sgn = pin((walks, 3, cap), np.uint64) if zt or zb else None
        self.best_valid = pin((walks, 3, cap), np.uint8) if zt else None
        self.rng_pos = pin((walks,), np.int64)
        self.status = pin((walks,), np.int32)
        self.best_n = pin((walks, 3), np.int32)
        self.fac2 = pin((walks, 3, cap), np.uint64) if zb else None
        self.best_fac2 = pin((walks, 3, cap), np.uint64) if zb else None

    def nbytes(self):
        return sum(getattr(self, f).nbytes for f, _ in self.FIELDS if getattr(self, f) is not None)

    def _c(self):
        return _Records(*[_ptr(getattr(self, f)) for f, _ in self.FIELDS])


class Engine:
    """One fg_handle: `walks` independent walks on one GPU."""

    def __init__(self, walks, cap, ring="z2", mode="reference", seed=1, iterations=10000, plus_iterations=8000,
                 expand_p=0.01, reduce_p=0.0, device=0, walks_per_block=0, resize_p=0.0, sandwich_p=0.0,
                 basis_p=0.0, gauss_p=0.0, zt_sandwich=False, retry_cap=0):
        """mode: "reference" (XORWOW, reference lists, bit-exact), "philox" (Philox, lists) or
        "fast" (Philox, implicit pair enumeration, thread-per-walk kernel).  retry_cap bounds the
        loops the reference leaves unbounded (0 = the library default, 2^20)."""
        self.lib = library()
        self.cfg = Config(RINGS[ring], MODES[mode], walks, cap, seed, iterations, plus_iterations, expand_p,
                          reduce_p, device, walks_per_block, resize_p, sandwich_p, basis_p, gauss_p,
                          int(zt_sandwich), retry_cap)
        self.walks, self.cap, self.ring = walks, cap, ring
        self.h = ctypes.c_void_p()
        _check(self.lib.fg_create(ctypes.byref(self.cfg), ctypes.byref(self.h)))

    def close(self):
        if self.h:
            self.lib.fg_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def init_naive(self, n1, n2, n3):
        _check(self.lib.fg_init_naive(self.h, n1, n2, n3))

    def set_proposal(self, mlp=None, candidates=1, temperature=1.0, min_entropy=0.0):
        """Learned mode: score `candidates` uniform candidate flips per step with `mlp` (an Mlp,
        or None for a uniform choice) and sample from softmax(score / temperature)."""
        self.lib.fg_set_proposal.restype = ctypes.c_int
        _check(self.lib.fg_set_proposal(self.h, mlp.h if mlp is not None else None, int(candidates),
                                        ctypes.c_float(temperature), ctypes.c_float(min_entropy)))
        self._mlp = mlp  # keep the network alive while it is in use

    def collect_records(self, every=16, horizon=1000, launches=1, capacity=1 << 20):
        """Learned mode, one candidate: run plain walks and return (features [n][3] uint64,
        labels [n] float32) -- label 1 if the rank dropped within `horizon` flips."""
        f = np.zeros((capacity, 3), np.uint64)
        y = np.zeros(capacity, np.float32)
        n = ctypes.c_int64()
        self.lib.fg_collect_records.restype = ctypes.c_int
        _check(self.lib.fg_collect_records(self.h, int(every), int(horizon), int(launches), ctypes.c_int64(capacity),
                                           _ptr(f), _ptr(y), ctypes.byref(n)))
        return f[:n.value].copy(), y[:n.value].copy()

    def rebuild_lists(self):
        """List modes: rebuild the FlipSet lists from the current factors (initFlips order)."""
        self.lib.fg_rebuild_lists.restype = ctypes.c_int
        _check(self.lib.fg_rebuild_lists(self.h))

    def set_list_kernel(self, kernel):
        """List modes: 'thread' (one thread per walk; no sandwiching, basis changes or Gauss
        reduction), 'warp' (one warp per walk) or 'auto'.  Results are identical."""
        kinds = {"auto": -1, "warp": 0, "thread": 1}
        self.lib.fg_set_list_kernel.restype = ctypes.c_int
        _check(self.lib.fg_set_list_kernel(self.h, kinds[kernel]))

    def set_fast_kernel(self, kernel, lanes=0):
        """Fast mode kernel for every segment: 'thread', 'group' (lanes 4/8/16, 0 = auto),
        'warp', or 'auto'.  Results are identical; only speed changes."""
        kinds = {"auto": -1, "thread": 0, "group": 1, "warp": 2}
        self.lib.fg_set_fast_kernel.restype = ctypes.c_int
        _check(self.lib.fg_set_fast_kernel(self.h, kinds[kernel], int(lanes)))

    def autotune(self, iterations=200):
        """Z2 fast mode: per shape segment, the fastest kernel over `iterations` steps; list modes on
        the thread-per-walk list kernel: per segment, the fastest warps per block (trajectories
        unchanged).  Returns [(kind, lanes, warps_per_block)] per segment, kind 0 thread, 1 group,
        2 warp per walk."""
        n = self.lib.fg_segment_count(self.h)
        kinds = np.zeros(max(n, 1), np.int32)
        lanes = np.zeros(max(n, 1), np.int32)
        warps = np.zeros(max(n, 1), np.int32)
        _check(self.lib.fg_autotune(self.h, iterations, _ptr(kinds), _ptr(lanes), _ptr(warps)))
        return [(int(k), int(l), int(w)) for k, l, w in zip(kinds[:n], lanes[:n], warps[:n])]

    def set_fast_split(self, simt_max_cap):
        """Fast mode kernel choice (same results): -1 automatic, else one thread per walk up to
        this slot count and one warp per walk above."""
        _check(self.lib.fg_set_fast_split(self.h, int(simt_max_cap)))

    def init_naive_shapes(self, shapes):
        """Walk w starts from the naive shapes[w] scheme (many shapes in one batch)."""
        sh = np.ascontiguousarray(shapes, np.int32).reshape(self.walks, 3)
        _check(self.lib.fg_init_naive_shapes(self.h, _ptr(sh)))

    def counters(self):
        """Per-walk m, best_rank, best_m, flips since the last rank drop, flips of the last launch, validity."""
        m = np.zeros(self.walks, np.int32)
        best = np.zeros(self.walks, np.int32)
        best_m = np.zeros(self.walks, np.int32)
        since = np.zeros(self.walks, np.int32)
        flips = np.zeros(self.walks, np.uint64)
        valid = np.zeros(self.walks, np.uint8)
        _check(self.lib.fg_get_counters(self.h, _ptr(m), _ptr(best), _ptr(best_m), _ptr(since), _ptr(flips),
                                        _ptr(valid)))
        return {"m": m, "best_rank": best, "best_m": best_m, "flips_since_drop": since, "flips": flips,
                "valid": valid.astype(bool)}

    def _match(self, rec):
        """The library reads and writes every array of `rec` at this handle's sizes."""
        if (rec.walks, rec.cap, rec.ring) != (self.walks, self.cap, self.ring):
            raise ValueError(f"records for {rec.walks} walks, cap {rec.cap}, ring {rec.ring}; "
                             f"the engine has {self.walks}, {self.cap}, {self.ring}")
        for f, _ in Records.FIELDS:
            a = getattr(rec, f)
            if a is None:
                continue
            dtype, per_walk = _FIELD_LAYOUT[f]
            shape = (self.walks,) + tuple(self.cap if d == "cap" else d for d in per_walk)
            if not (a.flags.c_contiguous and a.dtype == dtype and a.shape == shape):
                raise ValueError(f"records field {f}: contiguous {np.dtype(dtype).name} {list(shape)} expected, "
                                 f"got {a.dtype.name} {list(a.shape)}")

    def set_records(self, rec):
        self._match(rec)
        c = rec._c()
        _check(self.lib.fg_set_records(self.h, ctypes.byref(c)))

    def records(self, into=None):
        rec = into if into is not None else Records(self.walks, self.cap, self.ring)
        self._match(rec)
        c = rec._c()
        _check(self.lib.fg_get_records(self.h, ctypes.byref(c)))
        return rec

    def run(self, launches=1):
        st = Stats()
        _check(self.lib.fg_run(self.h, launches, ctypes.byref(st)))
        return st.as_dict()

    def minimize(self, best_complexity):
        bc = np.ascontiguousarray(best_complexity, np.int32)
        _check(self.lib.fg_minimize(self.h, _ptr(bc)))
        return bc

    def validate(self, best=False):
        out = np.zeros(self.walks, np.uint8)
        _check(self.lib.fg_validate(self.h, int(best), _ptr(out)))
        return out.astype(bool)


class ReducerConfig(ctypes.Structure):
    _fields_ = [("count", ctypes.c_int32), ("schemes", ctypes.c_int32), ("seed", ctypes.c_uint64),
                ("device", ctypes.c_int32), ("threads", ctypes.c_int32)]


MODE_NAMES = {0: "g", 1: "ga", 2: "gr", 3: "gi", 4: "wr", 5: "mix", 6: "rnd"}


def mode_name(mode, scale):
    """AdditionsReducer::getMode (additions_reducer.cuh:183-204)."""
    name = MODE_NAMES[int(mode)]
    if name in ("gr", "gi"):
        name += str(int(np.float32(scale) * np.float32(100)))
    return name


class Reducer:
    """Additions reducers on the GPU: `count` reducers over `schemes` schemes.

    coef: int8 [schemes][3][m][64] coefficients (U rows, V rows, W rows)."""

    def __init__(self, n, m, coef, count=32, schemes=1, seed=1, device=0, threads=0):
        self.lib = library()
        self.count, self.m, self.n = count, m, tuple(n)
        self.coef = np.ascontiguousarray(coef, np.int8).reshape(schemes, 3, m, 64)
        self.cfg = ReducerConfig(count, schemes, seed, device, threads)
        self.h = ctypes.c_void_p()
        _check(self.lib.fg_reducer_create(ctypes.byref(self.cfg), n[0], n[1], n[2], m, _ptr(self.coef),
                                          ctypes.byref(self.h)))

    def run(self, independent=True, best_fresh=None, best_vars=None, want_vars=True):
        """One runReducersKernel launch; want_vars=False skips copying the fresh variables back
        (out["vars"] is then None)."""
        counts = np.zeros((self.count, 13), np.int32)
        scale = np.zeros((self.count, 3), np.float32)
        vars_ = np.zeros((self.count, 3, 500, 2), np.int32) if want_vars else None
        bf = np.ascontiguousarray(best_fresh if best_fresh is not None else np.zeros(3), np.int32)
        bv = np.ascontiguousarray(best_vars if best_vars is not None else np.zeros((3, 500, 2)), np.int32)
        _check(self.lib.fg_reducer_run(self.h, int(independent), _ptr(bf), _ptr(bv), _ptr(counts), _ptr(scale),
                                       _ptr(vars_) if vars_ is not None else None))
        per = counts[:, :12].reshape(self.count, 3, 4)
        return {"additions": per[:, :, 0].copy(), "fresh": per[:, :, 1].copy(), "naive": per[:, :, 2].copy(),
                "mode": per[:, :, 3].copy(), "draws": counts[:, 12].copy(), "scale": scale, "vars": vars_}

    def flip(self, max_flips):
        """--max-flips pass (fg_reducer_flip): schemes 1.. become scheme 0 after up to max_flips ternary
        flips from their reducers' streams.  Returns (ranks [schemes], coef [schemes][3][m][64])."""
        schemes = self.cfg.schemes
        ranks = np.zeros(schemes, np.int32)
        coef = np.zeros((schemes, 3, self.m, 64), np.int8)
        _check(self.lib.fg_reducer_flip(self.h, int(max_flips), _ptr(ranks), _ptr(coef)))
        return ranks, coef

    def close(self):
        if self.h:
            self.lib.fg_reducer_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def reducer_run_noalloc(n, m, coef, count=32, schemes=1, seed=1, device=0, independent=True, best_fresh=None,
                        best_vars=None):
    """One reducer pass with no device allocation (fg_reducer_run_noalloc): the same counts as
    Reducer(...).run() on a fresh Reducer.  Calls share one static scratch array in the library
    and must not overlap."""
    lib = library()
    fn = lib.fg_reducer_run_noalloc
    fn.restype = ctypes.c_int
    coef = np.ascontiguousarray(coef, np.int8).reshape(schemes, 3, m, 64)
    cfg = ReducerConfig(count, schemes, seed, device)
    counts = np.zeros((count, 13), np.int32)
    scale = np.zeros((count, 3), np.float32)
    bf = np.ascontiguousarray(best_fresh if best_fresh is not None else np.zeros(3), np.int32)
    bv = np.ascontiguousarray(best_vars if best_vars is not None else np.zeros((3, 500, 2)), np.int32)
    _check(fn(ctypes.byref(cfg), n[0], n[1], n[2], m, _ptr(coef), int(independent), _ptr(bf), _ptr(bv),
              _ptr(counts), _ptr(scale)))
    per = counts[:, :12].reshape(count, 3, 4)
    return {"additions": per[:, :, 0].copy(), "fresh": per[:, :, 1].copy(), "naive": per[:, :, 2].copy(),
            "mode": per[:, :, 3].copy(), "draws": counts[:, 12].copy(), "scale": scale}


def gemm_bf16(a_bits, b_bits, mode=0, bias=None, mask=None, accumulate=None, device=0):
    """Tensor-core GEMM D = A B^T on bf16 bit patterns (uint16): mode 0 -> fp32 D (plus
    `accumulate` when given), 1 -> bf16 relu(D + bias), 2 -> bf16 D masked where mask > 0."""
    lib = library()
    fn = lib.fg_gemm_bf16
    fn.restype = ctypes.c_int
    a = np.ascontiguousarray(a_bits, np.uint16)
    b = np.ascontiguousarray(b_bits, np.uint16)
    (m, k), (n, k2) = a.shape, b.shape
    if k != k2:
        raise ValueError("inner dimensions differ")
    bias = None if bias is None else np.ascontiguousarray(bias, np.float32)
    mask = None if mask is None else np.ascontiguousarray(mask, np.uint16)
    if mode == 0:
        out = np.zeros((m, n), np.float32) if accumulate is None else np.ascontiguousarray(accumulate, np.float32)
        _check(fn(_ptr(a), _ptr(b), _ptr(bias), _ptr(mask), m, n, k, 0, int(accumulate is not None), _ptr(out), None,
                  device))
    else:
        out = np.zeros((m, n), np.uint16)
        _check(fn(_ptr(a), _ptr(b), _ptr(bias), _ptr(mask), m, n, k, mode, 0, None, _ptr(out), device))
    return out


class Mlp:
    """The learned proposal's scoring network on the GPU (fg_mlp_*).  Features are
    [rows][3] uint64 words (192 binary features); params one fp32 vector."""

    def __init__(self, seed=1, device=0):
        self.lib = library()
        for name in ("fg_mlp_create", "fg_mlp_destroy", "fg_mlp_set_params", "fg_mlp_get_params",
                     "fg_mlp_gradients", "fg_mlp_score", "fg_mlp_train", "fg_mlp_param_count"):
            getattr(self.lib, name).restype = ctypes.c_int
        self.n_params = int(self.lib.fg_mlp_param_count())
        self.h = ctypes.c_void_p()
        _check(self.lib.fg_mlp_create(device, ctypes.c_uint64(seed), ctypes.byref(self.h)))

    def params(self):
        p = np.zeros(self.n_params, np.float32)
        _check(self.lib.fg_mlp_get_params(self.h, _ptr(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n_params
        _check(self.lib.fg_mlp_set_params(self.h, _ptr(p)))

    def gradients(self, features, labels):
        f = np.ascontiguousarray(features, np.uint64)
        y = np.ascontiguousarray(labels, np.float32)
        g = np.zeros(self.n_params, np.float32)
        loss = ctypes.c_float()
        _check(self.lib.fg_mlp_gradients(self.h, _ptr(f), _ptr(y), len(y), ctypes.byref(loss), _ptr(g)))
        return float(loss.value), g

    def score(self, features):
        f = np.ascontiguousarray(features, np.uint64)
        out = np.zeros(len(f), np.float32)
        _check(self.lib.fg_mlp_score(self.h, _ptr(f), len(f), _ptr(out)))
        return out

    def train(self, features, labels, batch=4096, epochs=1, lr=1e-3, seed=1):
        f = np.ascontiguousarray(features, np.uint64)
        y = np.ascontiguousarray(labels, np.float32)
        loss = ctypes.c_float()
        _check(self.lib.fg_mlp_train(self.h, _ptr(f), _ptr(y), ctypes.c_int64(len(y)), batch, epochs,
                                     ctypes.c_float(lr), ctypes.c_uint64(seed), ctypes.byref(loss)))
        return float(loss.value)

    def close(self):
        if self.h:
            self.lib.fg_mlp_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def xorwow_tape(seed, first_walk, count, draws, device=0):
    """The reference's per-walk cuRAND XORWOW stream, recorded on the GPU."""
    d = np.zeros((count, draws), np.uint32)
    u = np.zeros((count, draws), np.float32)
    _check(library().fg_xorwow_tape(ctypes.c_uint64(seed), first_walk, count, draws, device, _ptr(d), _ptr(u)))
    return d, u


def philox_blocks(ctr, key, device=0):
    ctr = np.ascontiguousarray(ctr, np.uint32).reshape(-1, 4)
    out = np.zeros_like(ctr)
    _check(library().fg_philox_blocks(_ptr(ctr), len(ctr), key[0], key[1], device, _ptr(out)))
    return out


def version():
    return library().fg_version().decode()
