"""Readers for the golden fixture files written by oracle/ref_harness.cu.

All records are little-endian.  A *scheme* record is
    n[3] int32, m int32,
    for c in (u, v, w): m factors
        Z2 factor: uint64 bitmask
        ZT factor: uint64 values, uint64 signs, int32 valid
    [only when the record carries FlipSet lists]
    for c in (u, v, w): size int32, size x uint32 packed pairs (i << 16) | j

A walk file ("FGW1") holds a header, the initial schemes, one block per launch
(flips counter, best rank, scheme with lists, best scheme without lists,
validity) and one XORWOW tape per walk: consumed draw count followed by the
curand() values and the curand_uniform() values of those draws.

A reduce file ("FGR1") holds per-reducer (U, V, W) x (additions, fresh
variables, naive additions), the mode strings, and the per-reducer tapes.

A Gauss file ("FGG1") holds the scheme count and seed, per scheme the
result of one SchemeZ2::tryReduceGauss call and the Z2 scheme after it
(without lists), and the per-scheme tapes.
"""
import gzip
import struct

import numpy as np


class _Reader:
    def __init__(self, data):
        self.b = data
        self.o = 0

    def i32(self, n=None):
        if n is None:
            v = struct.unpack_from("<i", self.b, self.o)[0]
            self.o += 4
            return v
        v = np.frombuffer(self.b, dtype="<i4", count=n, offset=self.o).copy()
        self.o += 4 * n
        return v

    def u32(self, n):
        v = np.frombuffer(self.b, dtype="<u4", count=n, offset=self.o).copy()
        self.o += 4 * n
        return v

    def f32(self, n):
        v = np.frombuffer(self.b, dtype="<f4", count=n, offset=self.o).copy()
        self.o += 4 * n
        return v

    def u64(self):
        v = struct.unpack_from("<Q", self.b, self.o)[0]
        self.o += 8
        return v

    def f64(self):
        v = struct.unpack_from("<d", self.b, self.o)[0]
        self.o += 8
        return v


def _open(path):
    if path.endswith(".gz"):
        with gzip.open(path, "rb") as f:
            return f.read()
    with open(path, "rb") as f:
        return f.read()


def _scheme(r, zt, with_flips):
    n = [r.i32() for _ in range(3)]
    m = r.i32()
    s = {"n": n, "m": m}
    if zt:
        vals = np.zeros((3, m), dtype=np.uint64)
        sgns = np.zeros((3, m), dtype=np.uint64)
        valid = np.zeros((3, m), dtype=np.int32)
        for c in range(3):
            for t in range(m):
                vals[c, t] = r.u64()
                sgns[c, t] = r.u64()
                valid[c, t] = r.i32()
        s["values"], s["signs"], s["valid"] = vals, sgns, valid
    else:
        uvw = np.zeros((3, m), dtype=np.uint64)
        for c in range(3):
            for t in range(m):
                uvw[c, t] = r.u64()
        s["uvw"] = uvw
    if with_flips:
        s["flips"] = []
        for c in range(3):
            size = r.i32()
            s["flips"].append(r.u32(size))
    return s


def _tapes(r, count):
    tapes = []
    for _ in range(count):
        used = r.i32()
        n = max(used, 0)
        tapes.append({"used": used, "draws": r.u32(n), "uniforms": r.f32(n)})
    return tapes


def read_walk(path):
    r = _Reader(_open(path))
    magic = r.i32()
    assert magic in (0x46475731, 0x46475732, 0x46475733), "not a walk dump"
    zt = r.i32() == 1
    d = {"ring": "zt" if zt else "z2"}
    d["n"] = [r.i32() for _ in range(3)]
    d["walks"] = S = r.i32()
    d["iterations"] = r.i32()
    d["plus_iterations"] = r.i32()
    d["expand_p"] = r.f64()
    d["reduce_p"] = r.f64()
    d["resize_p"] = r.f64() if magic in (0x46475732, 0x46475733) else 0.0
    d["sandwich_p"] = r.f64() if magic == 0x46475733 else 0.0
    d["basis_p"] = r.f64() if magic == 0x46475733 else 0.0
    d["seed"] = r.i32()
    d["n_launches"] = L = r.i32()
    d["initial"] = [_scheme(r, zt, True) for _ in range(S)]
    d["launches"] = []
    for _ in range(L):
        block = []
        for _ in range(S):
            e = {"flips": r.i32(), "best_rank": r.i32()}
            e["scheme"] = _scheme(r, zt, True)
            e["best"] = _scheme(r, zt, False)
            e["valid"] = r.i32()
            block.append(e)
        d["launches"].append(block)
    d["tapes"] = _tapes(r, S)
    assert r.o == len(r.b), "trailing bytes in walk dump"
    return d


def read_reduce(path):
    r = _Reader(_open(path))
    assert r.i32() == 0x46475231, "not a reduce dump"
    count = r.i32()
    d = {"count": count, "seed": r.i32(), "reducers": []}
    for _ in range(count + 1):
        v = r.i32(9)
        ln = r.i32()
        modes = bytes(r.b[r.o:r.o + ln]).decode()
        r.o += ln
        d["reducers"].append({"u": tuple(int(x) for x in v[0:3]), "v": tuple(int(x) for x in v[3:6]),
                              "w": tuple(int(x) for x in v[6:9]), "modes": modes.split(",")})
    d["tapes"] = _tapes(r, count)
    assert r.o == len(r.b), "trailing bytes in reduce dump"
    return d


def read_reduce_flips(path):
    """ref_harness reduce with MAX_FLIPS > 0: per iteration the schemes' ranks, every reducer's
    counts and modes, and the top reducer of updateBestTogether; then the reducer tapes."""
    r = _Reader(_open(path))
    assert r.i32() == 0x46475232, "not a flip-reduce dump"
    count, seed, schemes, max_flips, iterations = (r.i32() for _ in range(5))
    d = {"count": count, "seed": seed, "schemes": schemes, "max_flips": max_flips, "iterations": []}
    for _ in range(iterations):
        it = {"ranks": [int(x) for x in r.i32(schemes)], "reducers": []}
        for _ in range(count):
            v = r.i32(9)
            ln = r.i32()
            modes = bytes(r.b[r.o:r.o + ln]).decode()
            r.o += ln
            it["reducers"].append({"u": tuple(int(x) for x in v[0:3]), "v": tuple(int(x) for x in v[3:6]),
                                   "w": tuple(int(x) for x in v[6:9]), "modes": modes.split(",")})
        it["top"] = r.i32()
        it["improved"] = r.i32()
        d["iterations"].append(it)
    d["tapes"] = _tapes(r, count)
    assert r.o == len(r.b), "trailing bytes in flip-reduce dump"
    return d


def read_gauss(path):
    r = _Reader(_open(path))
    assert r.i32() == 0x46474731, "not a Gauss dump"
    count = r.i32()
    d = {"count": count, "seed": r.i32(), "results": []}
    for _ in range(count):
        found = r.i32()
        d["results"].append({"found": found, "scheme": _scheme(r, False, False)})
    d["tapes"] = _tapes(r, count)
    assert r.o == len(r.b), "trailing bytes in Gauss dump"
    return d


def read_scheme_text(text):
    """Schemes of flip_graph's text layout (count, then sized Z2 schemes) as
    {"n", "m", "uvw"} with uvw[c] a uint64 array of bitmasks (|value| mod 2)."""
    tok = text.split()
    p = 1
    out = []
    for _ in range(int(tok[0])):
        n = [int(x) for x in tok[p:p + 3]]
        m = int(tok[p + 3])
        p += 4
        nn = [n[0] * n[1], n[1] * n[2], n[2] * n[0]]
        uvw = []
        for c in range(3):
            vals = np.array(tok[p:p + m * nn[c]], dtype=np.int64).reshape(m, nn[c]) % 2
            p += m * nn[c]
            uvw.append((vals.astype(np.uint64) << np.arange(nn[c], dtype=np.uint64)).sum(axis=1).astype(np.uint64))
        out.append({"n": n, "m": m, "uvw": uvw})
    return out


def factor_values(s, ring, c, t, nn):
    """Coefficient list of factor c of term t (length nn)."""
    if ring == "z2":
        x = int(s["uvw"][c, t])
        return [(x >> j) & 1 for j in range(nn)]
    v = int(s["values"][c, t])
    g = int(s["signs"][c, t])
    return [((v >> j) & 1) * (-1 if (g >> j) & 1 else 1) for j in range(nn)]


def scheme_to_text(s, ring, header=True):
    """The reference's whitespace-integer body format (scheme_z2.cu:72-96)."""
    n = s["n"]
    nn = [n[0] * n[1], n[1] * n[2], n[2] * n[0]]
    lines = []
    if header:
        lines.append(f"{n[0]} {n[1]} {n[2]} {s['m']}")
    for c in range(3):
        for t in range(s["m"]):
            lines.append(" ".join(str(x) for x in factor_values(s, ring, c, t, nn[c])))
    return "\n".join(lines) + "\n"
