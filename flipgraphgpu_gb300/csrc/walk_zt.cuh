// Ternary ("ZT") walk: coefficients in {-1, 0, 1}, one warp per walk, scheme
// and FlipSet lists in shared memory.  Semantics follow the reference's
// SchemeInteger (src/schemes/scheme_integer.cu) and Addition
// (src/entities/addition.cu) exactly: overflow-checked sums, the sign
// canonicalisation (first nonzero of u and v positive), the candidate order of
// tryFlip (a uniformly random permutation of all listed pairs, two orientation
// draws per candidate), and the compaction orders.
#pragma once
#include "fg_device.cuh"

namespace fg {

// A ternary vector as the reference's Addition: bit r of v = entry r nonzero,
// bit r of s = entry r negative; ok = no overflow happened.
struct Tern {
    uint64_t v, s;
    bool ok;
};

__device__ __forceinline__ bool teq(const Tern &a, const Tern &b) { return a.v == b.v && a.s == b.s; }
__device__ __forceinline__ bool firstPositive(uint64_t v, uint64_t s) { return v == 0 || (v & ~(v & (v - 1)) & ~s); }
__device__ __forceinline__ Tern tadd(const Tern &a, const Tern &b) {  // addition.cu:112-119
    Tern r;
    r.v = a.v ^ b.v;
    r.s = ((a.s & a.v) | (b.s & b.v)) & r.v;
    r.ok = !(a.v & b.v & ~(a.s ^ b.s));
    return r;
}
__device__ __forceinline__ Tern tsub(const Tern &a, const Tern &b) {  // addition.cu:121-128
    Tern r;
    r.v = a.v ^ b.v;
    r.s = ((a.s & a.v) | (~b.s & b.v)) & r.v;
    r.ok = !(a.v & b.v & (a.s ^ b.s));
    return r;
}
__device__ __forceinline__ int tcompare(const Tern &a, const Tern &b) {  // addition.cu:82-93
    if (a.v != b.v) return 0;
    if (a.s == b.s) return 1;
    if (a.s == (~b.s & b.v)) return -1;
    return 0;
}
__device__ __forceinline__ bool tlimit(const Tern &a, bool fp) { return a.ok && (!fp || firstPositive(a.v, a.s)); }
__device__ __forceinline__ bool tlimitSum(const Tern &a, const Tern &b, bool fp) {  // addition.cu:172-186
    if (a.v & b.v & ~(a.s ^ b.s)) return false;
    if (!fp) return true;
    uint64_t sv = a.v ^ b.v;
    return firstPositive(sv, ((a.s & a.v) | (b.s & b.v)) & sv);
}
__device__ __forceinline__ bool tlimitSub(const Tern &a, const Tern &b, bool fp) {  // addition.cu:188-202
    if (a.v & b.v & (a.s ^ b.s)) return false;
    if (!fp) return true;
    uint64_t sv = a.v ^ b.v;
    return firstPositive(sv, ((a.s & a.v) | (~b.s & b.v)) & sv);
}
__device__ __forceinline__ bool tposSub(const Tern &a, const Tern &b) {  // positiveFirstNonZeroSub
    uint64_t sv = a.v ^ b.v;
    return firstPositive(sv, ((a.s & a.v) | (~b.s & b.v)) & sv);
}

// Shared-memory footprint of a ZT walk: values + signs [3][cap] u64, valid [3][cap]
// bytes (padded to 8), lists [3][500] u32, permutation draws [3*500] u16.
__host__ __device__ inline size_t zt_smem_bytes(int cap) {
    size_t okb = ((size_t)3 * cap + 7) / 8 * 8;
    return (size_t)6 * cap * 8 + okb + (size_t)3 * kListCap * 4 + (size_t)3 * kListCap * 2;
}

template <class R, int S>
struct ZTWalk {
    uint64_t *xv, *xs;  // [3][cap]
    uint8_t *xo;        // [3][cap]
    uint32_t *L;        // [3][kListCap]
    uint16_t *J;        // [3*kListCap] permutation draws
    int cap;
    int n0, n1, n2, nn0, nn1, nn2, full;
    int m;
    int sz0, sz1, sz2;
    int status;
    R &r;

    __device__ ZTWalk(R &rr) : r(rr) {}

    __device__ __forceinline__ Tern X(int c, int t) const {
        int q = c * cap + t;
        return Tern{xv[q], xs[q], xo[q] != 0};
    }
    __device__ __forceinline__ void setX(int c, int t, const Tern &a) {  // lane 0 only
        int q = c * cap + t;
        xv[q] = a.v; xs[q] = a.s; xo[q] = a.ok;
    }
    __device__ __forceinline__ uint32_t *list(int c) { return L + c * kListCap; }
    __device__ __forceinline__ int sz(int c) const { return c == 0 ? sz0 : (c == 1 ? sz1 : sz2); }
    __device__ __forceinline__ void setSz(int c, int v) { if (c == 0) sz0 = v; else if (c == 1) sz1 = v; else sz2 = v; }
    __device__ __forceinline__ int nn(int c) const { return c == 0 ? nn0 : (c == 1 ? nn1 : nn2); }
    __device__ __forceinline__ bool nonzero(int t) const { return xv[t] && xv[cap + t] && xv[2 * cap + t]; }

    // initFlips (scheme_integer.cu:229-238): pairs with identical values and signs.
    __device__ __noinline__ void rebuild() {
        __syncwarp();
        for (int c = 0; c < 3; c++) {
            uint32_t *Lc = list(c);
            int total = 0;
#pragma unroll
            for (int s = 0; s < S; s++) {
                int t = 32 * s + lane_id();
                int cnt = 0;
                uint64_t v = 0, g = 0;
                if (t < m) {
                    v = xv[c * cap + t]; g = xs[c * cap + t];
                    for (int u = t + 1; u < m; u++) cnt += xv[c * cap + u] == v && xs[c * cap + u] == g;
                }
                int incl = warp_inclusive_sum(cnt);
                int pos = total + incl - cnt;
                if (t < m && cnt)
                    for (int u = t + 1; u < m; u++)
                        if (xv[c * cap + u] == v && xs[c * cap + u] == g) {
                            if (pos < kListCap) Lc[pos] = ((uint32_t)t << 16) | (uint32_t)u;
                            pos++;
                        }
                total += __shfl_sync(kFull, incl, 31);
            }
            setSz(c, total < kListCap ? total : kListCap);
        }
        __syncwarp();
    }

    __device__ __forceinline__ void moveTerm(int dst, int src) {  // lane 0
        for (int c = 0; c < 3; c++) setX(c, dst, X(c, src));
    }

    // removeZeroes (scheme_integer.cu:240-251): the moved term is re-checked.
    __device__ __noinline__ void removeZeroes() {
        __syncwarp();
        int mm = m;
        if (lane_id() == 0)
            for (int t = 0; t < mm; t++) {
                if (nonzero(t)) continue;
                mm--;
                moveTerm(t, mm);
                t--;
            }
        m = __shfl_sync(kFull, mm, 0);
        __syncwarp();
    }

    __device__ void removeAt(int t) {
        __syncwarp();
        m--;
        if (t != m && lane_id() == 0) moveTerm(t, m);
        __syncwarp();
    }

    __device__ void addTriplet(int i, int j, int k, const Tern &a, const Tern &b, const Tern &c) {
        if (m >= cap) { status |= ST_OVERFLOW; return; }
        if (lane_id() == 0) { setX(i, m, a); setX(j, m, b); setX(k, m, c); }
        m++;
        __syncwarp();
    }

    // fixSigns (scheme_integer.cu:398-425); terms are independent, so lanes fix their own.
    __device__ __noinline__ bool fixSigns() {
        __syncwarp();
        bool changed = false;
        for (int t = lane_id(); t < m; t += 32) {
            const bool pi = firstPositive(xv[t], xs[t]), pj = firstPositive(xv[cap + t], xs[cap + t]);
            if (pi && pj) continue;
            int c0 = (!pi && !pj) ? 0 : (!pi ? 0 : 1);
            int c1 = (!pi && !pj) ? 1 : 2;
            xs[c0 * cap + t] = ~xs[c0 * cap + t] & xv[c0 * cap + t];
            xs[c1 * cap + t] = ~xs[c1 * cap + t] & xv[c1 * cap + t];
            changed = true;
        }
        __syncwarp();
        return __any_sync(kFull, changed);
    }

    __device__ __noinline__ void reduceAdd(int i, int a, int b) {  // scheme_integer.cu:549-559
        Tern x = tadd(X(i, a), X(i, b));
        __syncwarp();
        if (lane_id() == 0) setX(i, a, x);
        __syncwarp();
        removeAt(b);
        if (!x.v) removeZeroes();
        rebuild();
    }

    __device__ __noinline__ void reduceSub(int i, int a, int b) {  // scheme_integer.cu:561-571
        Tern x = tsub(X(i, a), X(i, b));
        __syncwarp();
        if (lane_id() == 0) setX(i, a, x);
        __syncwarp();
        removeAt(b);
        if (!x.v) removeZeroes();
        rebuild();
    }

    __device__ bool tryReduceGauss() { return false; }  // Z2 only (scheme_z2.cu:1156-1163)

    // tryReduce (scheme_integer.cu:1062-1101): first listed pair (list order) that can merge.
    __device__ __noinline__ bool tryReduce() {
        for (int base = 0; base < sz0; base += 32) {
            int p = base + lane_id(), act = 0;
            if (p < sz0) {
                uint32_t pr = list(0)[p];
                int a = (int)(pr >> 16), b = (int)(pr & 0xFFFFu);
                const Tern u1 = X(1, a), u2 = X(1, b), w1 = X(2, a), w2 = X(2, b);
                if (teq(u1, u2) && tlimitSum(w1, w2, false)) act = 1;
                else {
                    int cmp2 = tcompare(w1, w2);
                    if (cmp2 == 1 && tlimitSum(u1, u2, true)) act = 2;
                    else if (cmp2 == -1 && tlimitSub(u1, u2, true)) act = 3;
                }
            }
            unsigned bm = __ballot_sync(kFull, act != 0);
            if (bm) {
                int src = __ffs(bm) - 1;
                int ac = __shfl_sync(kFull, act, src);
                uint32_t pr = list(0)[base + src];
                int a = (int)(pr >> 16), b = (int)(pr & 0xFFFFu);
                if (ac == 1) reduceAdd(2, a, b);
                else if (ac == 2) reduceAdd(1, a, b);
                else reduceSub(1, a, b);
                return true;
            }
        }
        for (int base = 0; base < sz1; base += 32) {
            int p = base + lane_id(), act = 0;
            if (p < sz1) {
                uint32_t pr = list(1)[p];
                int a = (int)(pr >> 16), b = (int)(pr & 0xFFFFu);
                int cmp2 = tcompare(X(2, a), X(2, b));
                if (cmp2 == 1 && tlimitSum(X(0, a), X(0, b), true)) act = 1;
                else if (cmp2 == -1 && tlimitSub(X(0, a), X(0, b), true)) act = 2;
            }
            unsigned bm = __ballot_sync(kFull, act != 0);
            if (bm) {
                int src = __ffs(bm) - 1;
                int ac = __shfl_sync(kFull, act, src);
                uint32_t pr = list(1)[base + src];
                int a = (int)(pr >> 16), b = (int)(pr & 0xFFFFu);
                if (ac == 1) reduceAdd(0, a, b);
                else reduceSub(0, a, b);
                return true;
            }
        }
        return false;
    }

    // j-part action at term t (scheme_integer.cu:445-469): 0 none, 1..4 the four reductions.
    __device__ __forceinline__ int actionJ(int i, int j, int k, int t, int a) const {
        const Tern it = X(i, t), ia = X(i, a), kt = X(k, t), ka = X(k, a);
        int cmpI = tcompare(it, ia);
        if (cmpI == 1 && tlimitSum(kt, ka, k != 2)) return 1;
        if (i == 2 && cmpI == -1 && tlimitSub(kt, ka, true)) return 2;
        int cmpK = tcompare(kt, ka);
        if (cmpK == 1 && tlimitSum(it, ia, i != 2)) return 3;
        if (k == 2 && cmpK == -1 && tlimitSub(it, ia, true)) return 4;
        return 0;
    }

    // flip (scheme_integer.cu:428-501).
    __device__ __noinline__ void flip(int i, int j, int k, int a, int b, bool checkReduce) {
        Tern ja = X(j, a), jb = X(j, b), kb = X(k, b), ka = X(k, a);
        Tern nja = tadd(ja, jb);  // uvw[j][a] += uvw[j][b]
        Tern nkb = tsub(kb, ka);  // uvw[k][b] -= uvw[k][a]
        __syncwarp();
        if (lane_id() == 0) { setX(j, a, nja); setX(k, b, nkb); }
        __syncwarp();
        setSz(j, list_remove_index(list(j), sz(j), (uint32_t)a));
        setSz(k, list_remove_index(list(k), sz(k), (uint32_t)b));
        if (!nja.v || !nkb.v) {
            removeZeroes();
            rebuild();
            int guard = 0;
            while (tryReduce())
                if (++guard > retry_cap_of(r.P)) { status |= ST_RETRY; break; }
            return;
        }
        unsigned eqJ[S], eqK[S];
        int found = -1;
#pragma unroll
        for (int s = 0; s < S; s++) {
            int t = 32 * s + lane_id();
            bool eJ = false, eK = false;
            int aJ = 0, aK = 0;
            if (t < m) {
                eJ = t != a && teq(X(j, t), nja);
                eK = t != b && teq(X(k, t), nkb);
                if (checkReduce && eJ) aJ = actionJ(i, j, k, t, a);
                if (checkReduce && eK) aK = actionJ(i, k, j, t, b);
            }
            unsigned bR = __ballot_sync(kFull, aJ != 0 || aK != 0);
            eqJ[s] = __ballot_sync(kFull, eJ);
            eqK[s] = __ballot_sync(kFull, eK);
            if (found < 0 && bR) found = 32 * s + __ffs(bR) - 1;
        }
        if (found >= 0) {
            const int t = found;
            const bool eJ = t != a && teq(X(j, t), nja);
            const int aJ = eJ ? actionJ(i, j, k, t, a) : 0;
            if (aJ) {
                if (aJ == 1) reduceAdd(k, t, a);
                else if (aJ == 2) reduceSub(k, t, a);
                else if (aJ == 3) reduceAdd(i, t, a);
                else reduceSub(i, t, a);
            } else {
                // k-part (scheme_integer.cu:473-497): the same tests with j and k exchanged.
                const int aK = actionJ(i, k, j, t, b);
                if (aK == 1) reduceAdd(j, t, b);
                else if (aK == 2) reduceSub(j, t, b);
                else if (aK == 3) reduceAdd(i, t, b);
                else reduceSub(i, t, b);
            }
            return;
        }
        setSz(j, list_append<S>(list(j), sz(j), (uint32_t)a, eqJ));
        setSz(k, list_append<S>(list(k), sz(k), (uint32_t)b, eqK));
    }

    // plus (scheme_integer.cu:503-539).
    __device__ __noinline__ void plus(int i, int j, int k, int p, int q, int variant) {
        const Tern a1 = X(i, p), b1 = X(j, p), c1 = X(k, p);
        const Tern a2 = X(i, q), b2 = X(j, q), c2 = X(k, q);
        const Tern aAdd = tadd(a1, a2), bAdd = tadd(b1, b2), cAdd = tadd(c1, c2);
        const Tern aSub = tsub(a2, a1), bSub = tsub(b2, b1), cSub = tsub(c2, c1);
        __syncwarp();
        if (variant == 0 && tlimit(aSub, i != 2) && tlimit(bAdd, j != 2) && tlimit(cSub, k != 2)) {
            if (lane_id() == 0) { setX(j, p, bAdd); setX(i, q, aSub); }
            addTriplet(i, j, k, a1, b2, cSub);
        } else if (variant == 1 && tlimit(aSub, i != 2) && tlimit(bSub, j != 2) && tlimit(cAdd, k != 2)) {
            if (lane_id() == 0) { setX(k, p, cAdd); setX(j, q, bSub); }
            addTriplet(i, j, k, aSub, b1, c2);
        } else if (tlimit(aAdd, i != 2) && tlimit(bSub, j != 2) && tlimit(cSub, k != 2)) {
            if (lane_id() == 0) { setX(i, p, aAdd); setX(k, q, cSub); }
            addTriplet(i, j, k, a2, bSub, c1);
        }
        __syncwarp();
        removeZeroes();
        fixSigns();
        rebuild();
    }

    __device__ __noinline__ void split(int i, int j, int k, int t, const Tern &a) {  // scheme_integer.cu:541-547
        const Tern rest = tsub(X(i, t), a), bj = X(j, t), bk = X(k, t);
        addTriplet(i, j, k, rest, bj, bk);
        __syncwarp();
        if (lane_id() == 0) setX(i, t, a);
        __syncwarp();
        fixSigns();
        rebuild();
    }

    // Position p of the random permutation of [0, n) drawn by randomPermutation
    // (random.cuh:9-22) from the draws J[i] = curand() % (i + 1), i = n-1..1: the
    // swaps are traced backwards, so 32 lanes evaluate 32 positions at once.
    __device__ __forceinline__ int permAt(int p, int n) const {
        int pos = p;
        for (int i = 1; i < n; i++) {
            int j = J[i];
            pos = pos == i ? j : (pos == j ? i : pos);
        }
        return pos;
    }

    // tryFlip (scheme_integer.cu:907-975).
    __device__ __noinline__ bool tryFlip(bool checkReduce) {
        const int size = sz0 + sz1 + sz2;
        // randomPermutation(indices, size): draws for i = size-1 .. 1.
        for (int i = size - 1; i >= 1; i--) {
            uint32_t x = r.below((uint32_t)(i + 1));
            if (lane_id() == 0) J[i] = (uint16_t)x;
        }
        __syncwarp();
        for (int p0 = 0; p0 < size; p0 += 32) {
            int mine = p0 + lane_id() < size ? permAt(p0 + lane_id(), size) : 0;
            const int lim = size - p0 < 32 ? size - p0 : 32;
            for (int q = 0; q < lim; q++) {
                int idx = __shfl_sync(kFull, mine, q);
                int i, j, k;
                uint32_t pr;
                if (idx < sz0) { i = 0; j = 1; k = 2; pr = list(0)[idx]; }
                else if (idx < sz0 + sz1) { i = 1; j = 0; k = 2; pr = list(1)[idx - sz0]; }
                else { i = 2; j = 0; k = 1; pr = list(2)[idx - sz0 - sz1]; }
                int a = (int)(pr >> 16), b = (int)(pr & 0xFFFFu);
                if (r.coin()) { int tmp = j; j = k; k = tmp; }
                if (r.coin()) { int tmp = a; a = b; b = tmp; }
                const Tern ja = X(j, a), jb = X(j, b), ka = X(k, a), kb = X(k, b);
                int fj = -1, fk = 0, fa = 0, fb = 0;
                if (tlimitSum(ja, jb, j != 2) && tlimitSub(kb, ka, false)) {
                    fj = j; fk = k;
                    const bool keep = k == 2 || tposSub(kb, ka);
                    fa = keep ? a : b; fb = keep ? b : a;
                } else if (tlimitSum(ka, kb, k != 2) && tlimitSub(jb, ja, false)) {
                    fj = k; fk = j;
                    const bool keep = j == 2 || tposSub(jb, ja);
                    fa = keep ? a : b; fb = keep ? b : a;
                }
                if (fj >= 0) {
                    flip(i, fj, fk, fa, fb, checkReduce);
                    return true;
                }
            }
        }
        return false;
    }

    __device__ __forceinline__ void perm3(int &i, int &j, int &k) {
        int p0 = 0, p1 = 1, p2 = 2;
        int q = (int)r.below(3);
        if (q == 0) { int t = p2; p2 = p0; p0 = t; } else if (q == 1) { int t = p2; p2 = p1; p1 = t; }
        q = (int)r.below(2);
        if (q == 0) { int t = p1; p1 = p0; p0 = t; }
        i = p0; j = p1; k = p2;
    }

    __device__ __noinline__ bool tryPlus() {  // scheme_integer.cu:977-998
        if (m >= kMaxRank || m >= full) return false;
        int a = (int)r.below((uint32_t)m), b = (int)r.below((uint32_t)m);
        int guard = 0;
        while (a == b || teq(X(0, a), X(0, b)) || teq(X(1, a), X(1, b)) || teq(X(2, a), X(2, b))) {
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

    // Addition::random (addition.cu:66-80): chunk 16 is sign-extended (uint16
    // promoted to int before the shift) and chunks >= 32 shift out to zero.
    __device__ Tern randomTern(int n) {
        Tern a{0, 0, true};
        for (int i = 0; i < n; i += 16) {
            uint32_t sb = r.raw() & 0xFFFFu;
            uint32_t vb = r.raw() & 0xFFFFu;
            int32_t vs = i >= 32 ? 0 : (int32_t)(vb << i);
            int32_t ss = i >= 32 ? 0 : (int32_t)(sb << i);
            a.v |= (uint64_t)(int64_t)vs;
            a.s |= (uint64_t)(int64_t)ss;
        }
        a.s &= a.v;
        return a;
    }

    __device__ __noinline__ bool trySplit() {  // scheme_integer.cu:1000-1020
        if (m >= kMaxRank || m >= full) return false;
        int t = (int)r.below((uint32_t)m);
        int i, j, k;
        perm3(i, j, k);
        Tern a = randomTern(nn(i));
        if (!tlimitSub(X(i, t), a, i != 2)) return false;
        split(i, j, k, t, a);
        return true;
    }

    __device__ __noinline__ bool trySplitExisted() {  // scheme_integer.cu:1022-1043
        if (m >= kMaxRank || m >= full) return false;
        int a, b, i;
        int guard = 0;
        do {
            if (++guard > retry_cap_of(r.P)) { status |= ST_RETRY; return false; }
            a = (int)r.below((uint32_t)m);
            b = (int)r.below((uint32_t)m);
            i = (int)r.below(3);
        } while (a == b || teq(X(i, a), X(i, b)));
        if (!tlimitSub(X(i, a), X(i, b), i != 2)) return false;
        const Tern xb = X(i, b);
        split(i, (i + 1) % 3, (i + 2) % 3, a, xb);
        return true;
    }

    __device__ bool tryExpand(int count) {  // scheme_integer.cu:1045-1060
        bool result = false;
        for (int q = 0; q < count && m < kMaxRank; q++) {
            int v = (int)r.below(3);
            if (v == 0) result |= tryPlus();
            else if (v == 1) result |= trySplit();
            else result |= trySplitExisted();
            if (status) break;
        }
        return result;
    }
};

}  // namespace fg
