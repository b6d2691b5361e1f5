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
// global scratch buffer, interleaved the same way per group of 32 walks:
// entry (c, q) at L[(c * kListCap + q) * 32]; a warp scanning entry q of its 32
// walks reads one 128-byte line.  The lists' live part (a few hundred entries
// per walk) stays in L2.
#pragma once
#include "fg_device.cuh"
#include "walk_simt.cuh"

namespace fg {

// Per-thread XORWOW (the reference's stream), one cuRAND state per walk.
using ThreadXorwow = XorwowDraws;

template <class W, class R>
struct SimtListZ2 {
    W *x;         // this walk's factor column in shared memory
    uint32_t *L;  // this walk's list column in the global scratch
    int ld;       // slots per component in shared memory
    int cap;      // slots a rank may reach (addTriplet beyond it overflows)
    int n0, n1, n2, nn0, nn1, nn2, full;
    int m;
    int sz0, sz1, sz2;
    int status;
    R &r;

    __device__ SimtListZ2(R &rr) : r(rr) {}

    __device__ __forceinline__ W X(int c, int t) const { return x[(size_t)(c * ld + t) << 5]; }
    __device__ __forceinline__ void setX(int c, int t, W v) { x[(size_t)(c * ld + t) << 5] = v; }
    __device__ __forceinline__ uint32_t Lq(int c, int q) const { return L[(size_t)(c * kListCap + q) << 5]; }
    __device__ __forceinline__ void setLq(int c, int q, uint32_t v) { L[(size_t)(c * kListCap + q) << 5] = v; }
    __device__ __forceinline__ int sz(int c) const { return c == 0 ? sz0 : (c == 1 ? sz1 : sz2); }
    __device__ __forceinline__ void setSz(int c, int v) { if (c == 0) sz0 = v; else if (c == 1) sz1 = v; else sz2 = v; }
    __device__ __forceinline__ int nn(int c) const { return c == 0 ? nn0 : (c == 1 ? nn1 : nn2); }
    __device__ __forceinline__ bool nonzero(int t) const { return X(0, t) && X(1, t) && X(2, t); }

    // FlipSet::add (flip_set.cu:7-13): appended, silently dropped past the capacity.
    __device__ __forceinline__ void listAdd(int c, int a, int b) {
        const int s = sz(c);
        if (s >= kListCap) return;
        setLq(c, s, ((uint32_t)a << 16) | (uint32_t)b);
        setSz(c, s + 1);
    }

    // FlipSet::remove(index) (flip_set.cu:27-31): every pair touching idx is
    // replaced by the last pair, which is then tested at the same position.  Four
    // entries are loaded at a time; a group without a match is skipped whole.
    __device__ void listRemoveIndex(int c, uint32_t idx) {
        int s = sz(c), q = 0;
        while (q + 4 <= s) {
            const uint32_t v0 = Lq(c, q), v1 = Lq(c, q + 1), v2 = Lq(c, q + 2), v3 = Lq(c, q + 3);
            const bool h0 = touches(v0, idx), h1 = touches(v1, idx), h2 = touches(v2, idx), h3 = touches(v3, idx);
            if (!(h0 | h1 | h2 | h3)) { q += 4; continue; }
            q += h0 ? 0 : (h1 ? 1 : (h2 ? 2 : 3));
            s--;
            setLq(c, q, Lq(c, s));  // position q is tested again
        }
        while (q < s) {
            if (touches(Lq(c, q), idx)) { s--; setLq(c, q, Lq(c, s)); }
            else q++;
        }
        setSz(c, s);
    }

    // initFlips (scheme_z2.cu:141-150): all equal pairs, lexicographic, capped.
    __device__ void rebuild() {
        for (int c = 0; c < 3; c++) {
            int s = 0;
            for (int a = 0; a < m; a++) {
                const W v = X(c, a);
                for (int b = a + 1; b < m; b++)
                    if (X(c, b) == v) {
                        if (s < kListCap) setLq(c, s, ((uint32_t)a << 16) | (uint32_t)b);
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
        int a = (int)(pr >> 16), b = (int)(pr & 0xFFFFu);
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
            const int a = (int)(pr >> 16), b = (int)(pr & 0xFFFFu);
            if (X(1, a) == X(1, b)) { reduce(2, a, b); return true; }
            if (X(2, a) == X(2, b)) { reduce(1, a, b); return true; }
        }
        for (int q = 0; q < sz1; q++) {
            const uint32_t pr = Lq(1, q);
            const int a = (int)(pr >> 16), b = (int)(pr & 0xFFFFu);
            if (X(2, a) == X(2, b)) { reduce(0, a, b); return true; }
        }
        return false;
    }
};

}  // namespace fg
