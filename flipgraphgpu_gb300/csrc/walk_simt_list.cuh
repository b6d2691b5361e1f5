// List-mode Z2 walk, one THREAD per walk: the reference's walk step for step
// (src/entities/flip_graph.cu:520-573, src/schemes/scheme_z2.cu,
// src/entities/flip_set.cu) with its FlipSet lists, so with the cuRAND XORWOW
// stream it reproduces the reference's trajectories bit for bit, like the
// warp-per-walk Z2Walk, at a fraction of the instructions per flip: a warp
// advances 32 walks at once instead of one.
//
// Layout.  Factors live in shared memory, 32 walks interleaved by lane: word
// (c, t) of the lane's walk at x[(c * ld + t) * 32], so every access a thread
// makes to its own walk hits bank `lane`.  The three FlipSet lists live in a
// global scratch buffer as 16-bit pairs (a << 8 | b; slots <= 256), eight to a
// 16-byte vector, the vectors of a group of 32 walks interleaved by lane:
// vector (c, v) of the lane's walk at V[(c * kListVecs + v) * 32].  A list scan
// loads 8 entries per thread per load (a warp reads 512 contiguous bytes) and
// tests them with byte-wise SIMD compares.  The lists' live part stays in L2.
#pragma once
#include "fg_device.cuh"
#include "walk_simt.cuh"

namespace fg {

// Per-thread XORWOW (the reference's stream), one cuRAND state per walk.
using ThreadXorwow = XorwowDraws;

// 16-bit list entries: eight per 16-byte vector, ceil(500 / 8) vectors per component.
constexpr int kListVecs = (kListCap + 7) / 8;

__device__ __forceinline__ uint32_t pack16(int a, int b) { return ((uint32_t)a << 8) | (uint32_t)b; }

// Bit e (0..7) set when entry e of the vector holds index idx (< 256) in either half.
__device__ __forceinline__ unsigned vec_touch_mask(const uint4 &v, uint32_t idx) {
    const uint32_t rep = idx * 0x01010101u;
    const uint32_t w[4] = {__vcmpeq4(v.x, rep), __vcmpeq4(v.y, rep), __vcmpeq4(v.z, rep), __vcmpeq4(v.w, rep)};
    unsigned m = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) m |= (((w[q] & 0xFFFFu) ? 1u : 0u) | ((w[q] >> 16) ? 2u : 0u)) << (2 * q);
    return m;
}

// The three FlipSet lists of one walk (flip_set.cu) in the scratch layout above, with
// the reference's append and swap-with-last removal order.
struct SimtLists {
    uint4 *V;  // this walk's list column in the global scratch (16-bit entries)
    int sz0, sz1, sz2;

    __device__ __forceinline__ uint4 vec(int c, int v) const { return V[(size_t)(c * kListVecs + v) << 5]; }
    __device__ __forceinline__ uint16_t *entry(int c, int q) const {
        return reinterpret_cast<uint16_t *>(V + ((size_t)(c * kListVecs + (q >> 3)) << 5)) + (q & 7);
    }
    __device__ __forceinline__ uint32_t Lq(int c, int q) const { return *entry(c, q); }
    __device__ __forceinline__ void setLq(int c, int q, uint32_t v) { *entry(c, q) = (uint16_t)v; }
    __device__ __forceinline__ int sz(int c) const { return c == 0 ? sz0 : (c == 1 ? sz1 : sz2); }
    __device__ __forceinline__ void setSz(int c, int v) { if (c == 0) sz0 = v; else if (c == 1) sz1 = v; else sz2 = v; }

    // FlipSet::add (flip_set.cu:7-13): appended, silently dropped past the capacity.
    __device__ __forceinline__ void listAdd(int c, int a, int b) {
        const int s = sz(c);
        if (s >= kListCap) return;
        setLq(c, s, pack16(a, b));
        setSz(c, s + 1);
    }

    // FlipSet::remove(index) (flip_set.cu:27-31): every pair touching idx is
    // replaced by the last pair, which is then tested at the same position.  The
    // scan reads two vectors (16 entries) per step and skips them whole when no
    // live entry from position q on matches.
    __device__ void listRemoveIndex(int c, uint32_t idx) {
        int s = sz(c), q = 0;
        while (q < s) {
            const int v = q >> 3;
            const uint4 a = vec(c, v);
            const bool two = (v + 1) * 8 < s;
            const uint4 b = two ? vec(c, v + 1) : make_uint4(0u, 0u, 0u, 0u);
            unsigned hit = vec_touch_mask(a, idx) | (two ? vec_touch_mask(b, idx) << 8 : 0u);
            hit &= ~0u << (q & 7);                                          // from position q on
            const int live = s - v * 8;                                      // entries below s
            if (live < 16) hit &= (1u << live) - 1u;
            if (!hit) { q = (v + 2) * 8; continue; }
            q = v * 8 + __ffs(hit) - 1;
            s--;
            setLq(c, q, Lq(c, s));  // position q is tested again
        }
        setSz(c, s);
    }
};

template <class W, class R>
struct SimtListZ2 : SimtLists {
    W *x;      // this walk's factor column in shared memory
    int ld;    // slots per component in shared memory (<= 256)
    int cap;   // slots a rank may reach (addTriplet beyond it overflows)
    int n0, n1, n2, nn0, nn1, nn2, full;
    int m;
    int status;
    R &r;

    __device__ SimtListZ2(R &rr) : r(rr) {}

    __device__ __forceinline__ W X(int c, int t) const { return x[(size_t)(c * ld + t) << 5]; }
    __device__ __forceinline__ void setX(int c, int t, W v) { x[(size_t)(c * ld + t) << 5] = v; }
    __device__ __forceinline__ int nn(int c) const { return c == 0 ? nn0 : (c == 1 ? nn1 : nn2); }
    __device__ __forceinline__ bool nonzero(int t) const { return X(0, t) && X(1, t) && X(2, t); }

    // initFlips (scheme_z2.cu:141-150): all equal pairs, lexicographic, capped.
    __device__ void rebuild() {
        for (int c = 0; c < 3; c++) {
            int s = 0;
            for (int a = 0; a < m; a++) {
                const W v = X(c, a);
                for (int b = a + 1; b < m; b++)
                    if (X(c, b) == v) {
                        if (s < kListCap) setLq(c, s, pack16(a, b));
                        s++;
                    }
            }
            setSz(c, s < kListCap ? s : kListCap);
        }
    }

    __device__ __forceinline__ void moveTerm(int dst, int src) {
        for (int c = 0; c < 3; c++) setX(c, dst, X(c, src));
    }

    // removeZeroes (scheme_z2.cu:152-164); the moved term is not re-checked.
    __device__ void removeZeroes() {
        while (m > 0 && !nonzero(m - 1)) m--;
        for (int t = 0; t < m; t++)
            if (!nonzero(t)) { m--; moveTerm(t, m); }
    }

    __device__ __forceinline__ void removeAt(int t) {  // scheme_z2.cu:166-175
        m--;
        if (t != m) moveTerm(t, m);
    }

    __device__ __forceinline__ void addTriplet(int i, int j, int k, W a, W b, W c) {  // scheme_z2.cu:177-182
        if (m >= cap) { status |= ST_OVERFLOW; return; }
        setX(i, m, a); setX(j, m, b); setX(k, m, c);
        m++;
    }

    __device__ void reduce(int i, int a, int b) {  // scheme_z2.cu:631-641
        const W v = X(i, a) ^ X(i, b);
        setX(i, a, v);
        removeAt(b);
        if (!v) removeZeroes();
        rebuild();
    }

    // flip (scheme_z2.cu:531-577).
    __device__ void flip(int i, int j, int k, int a, int b, bool checkReduce) {
        const W xja = X(j, a) ^ X(j, b);
        const W xkb = X(k, b) ^ X(k, a);
        setX(j, a, xja);
        setX(k, b, xkb);
        listRemoveIndex(j, (uint32_t)a);
        listRemoveIndex(k, (uint32_t)b);
        if (!xja || !xkb) {
            removeZeroes();
            rebuild();
            return;
        }
        const W xia = X(i, a), xka = X(k, a), xib = X(i, b), xjb = X(j, b);
        for (int t = 0; t < m; t++) {
            const W vj = X(j, t), vk = X(k, t);
            if (t != a && vj == xja) {
                if (checkReduce) {
                    const W vi = X(i, t);
                    if (vi == xia) { reduce(k, t, a); return; }
                    if (vk == xka) { reduce(i, t, a); return; }
                }
                listAdd(j, a, t);
            }
            if (t != b && vk == xkb) {
                if (checkReduce) {
                    const W vi = X(i, t);
                    if (vi == xib) { reduce(j, t, b); return; }
                    if (vj == xjb) { reduce(i, t, b); return; }
                }
                listAdd(k, b, t);
            }
        }
    }

    __device__ bool tryFlip(bool checkReduce) {  // scheme_z2.cu:982-1027
        const int size = sz0 + sz1 + sz2;
        if (!size) return false;
        int idx = (int)r.below((uint32_t)size);
        int i, j, k;
        uint32_t pr;
        if (idx < sz0) { i = 0; j = 1; k = 2; pr = Lq(0, idx); }
        else if (idx < sz0 + sz1) { i = 1; j = 0; k = 2; pr = Lq(1, idx - sz0); }
        else { i = 2; j = 0; k = 1; pr = Lq(2, idx - sz0 - sz1); }
        int a = (int)(pr >> 8), b = (int)(pr & 0xFFu);
        if (r.coin()) { int tmp = j; j = k; k = tmp; }
        if (r.coin()) { int tmp = a; a = b; b = tmp; }
        flip(i, j, k, a, b, checkReduce);
        return true;
    }

    __device__ void plus(int i, int j, int k, int p, int q, int variant) {  // scheme_z2.cu:579-612
        const W a1 = X(i, p), b1 = X(j, p), c1 = X(k, p);
        const W a2 = X(i, q), b2 = X(j, q), c2 = X(k, q);
        const W a = a1 ^ a2, b = b1 ^ b2, c = c1 ^ c2;
        if (variant == 0) { setX(j, p, b); setX(i, q, a); addTriplet(i, j, k, a1, b2, c); }
        else if (variant == 1) { setX(k, p, c); setX(j, q, b); addTriplet(i, j, k, a, b1, c2); }
        else { setX(i, p, a); setX(k, q, c); addTriplet(i, j, k, a2, b, c1); }
        if (!a || !b || !c) removeZeroes();
        rebuild();
    }

    __device__ void split(int i, int j, int k, int t, W a1) {  // scheme_z2.cu:614-619
        const W a2 = X(i, t) ^ a1, bj = X(j, t), bk = X(k, t);
        setX(i, t, a1);
        addTriplet(i, j, k, a2, bj, bk);
        rebuild();
    }

    __device__ __forceinline__ void perm3(int &i, int &j, int &k) {  // randomPermutation(p, 3)
        int p0 = 0, p1 = 1, p2 = 2;
        int q = (int)r.below(3);
        if (q == 0) { int t = p2; p2 = p0; p0 = t; } else if (q == 1) { int t = p2; p2 = p1; p1 = t; }
        q = (int)r.below(2);
        if (q == 0) { int t = p1; p1 = p0; p0 = t; }
        i = p0; j = p1; k = p2;
    }

    __device__ bool tryPlus() {  // scheme_z2.cu:1029-1050
        if (m >= kMaxRank || m >= full) return false;
        int a = (int)r.below((uint32_t)m), b = (int)r.below((uint32_t)m);
        int guard = 0;
        while (a == b || X(0, a) == X(0, b) || X(1, a) == X(1, b) || X(2, a) == X(2, b)) {
            if (++guard > retry_cap_of(r.P)) { status |= ST_RETRY; return false; }
            a = (int)r.below((uint32_t)m);
            b = (int)r.below((uint32_t)m);
        }
        int i, j, k;
        perm3(i, j, k);
        int variant = (int)r.below(3);
        plus(i, j, k, a, b, variant);
        return true;
    }

    __device__ bool trySplit() {  // scheme_z2.cu:1052-1078
        if (m >= kMaxRank || m >= full) return false;
        int t = (int)r.below((uint32_t)m);
        int i, j, k;
        perm3(i, j, k);
        W a1 = (W)r.mask(nn(i));
        const W a2 = X(i, t);
        int loop = 0;
        while (loop < 5 && a1 == a2) { a1 = (W)r.mask(nn(i)); loop++; }
        if (loop == 5) return false;
        split(i, j, k, t, a1);
        return true;
    }

    __device__ bool trySplitExisted() {  // scheme_z2.cu:1080-1104
        if (m >= kMaxRank || m >= full) return false;
        int i, j, k;
        perm3(i, j, k);
        int a = (int)r.below((uint32_t)m), b = (int)r.below((uint32_t)m);
        int loop = 0;
        while (loop < 5 && (a == b || X(i, a) == X(i, b))) { b = (int)r.below((uint32_t)m); loop++; }
        if (loop == 5) return false;
        split(i, j, k, a, X(i, b));
        return true;
    }

    __device__ bool tryExpand(int count) {  // scheme_z2.cu:1106-1125
        bool result = false;
        for (int q = 0; q < count && m < full; q++) {
            int v = (int)r.below(3);
            if (v == 0) result |= tryPlus();
            else if (v == 1) result |= trySplit();
            else result |= trySplitExisted();
        }
        return result;
    }

    // tryReduce (scheme_z2.cu:1127-1154): the first list-0 pair sharing a second
    // factor, else the first list-1 pair sharing the third.
    __device__ bool tryReduce() {
        for (int q = 0; q < sz0; q++) {
            const uint32_t pr = Lq(0, q);
            const int a = (int)(pr >> 8), b = (int)(pr & 0xFFu);
            if (X(1, a) == X(1, b)) { reduce(2, a, b); return true; }
            if (X(2, a) == X(2, b)) { reduce(1, a, b); return true; }
        }
        for (int q = 0; q < sz1; q++) {
            const uint32_t pr = Lq(1, q);
            const int a = (int)(pr >> 8), b = (int)(pr & 0xFFu);
            if (X(2, a) == X(2, b)) { reduce(0, a, b); return true; }
        }
        return false;
    }
};

}  // namespace fg
