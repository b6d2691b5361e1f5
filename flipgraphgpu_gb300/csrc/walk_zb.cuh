// Bounded-integer ("ZB") walk: coefficients in [-2, 2], fast mode (Philox
// stream, implicit enumeration of ordered pairs of factors equal up to sign,
// in canonical order), one warp per walk.  No reference counterpart: the
// reference's integer ring is {-1, 0, 1}; the rules restate SchemeInteger's
// walk for the wider bound (oracle/fg_oracle.cpp, struct ZB, is the same
// algorithm on the CPU):
//   flip (a, b) with x_b = e x_a in component i, (j, k) the other two in a
//     coin-chosen order, s = +-1 by a second coin: y_a += s e y_b,
//     z_b -= s z_a; a proposal leaving [-2, 2] is rejected (the step is spent);
//   signs canonical: first nonzero entry of u and of v positive (fixSigns,
//     scheme_integer.cu:398-425); negating a factor keeps it equal up to sign,
//     so partner counts do not change;
//   a term with a zero factor is removed; after a flip, term a then term b is
//     absorbed by the first term (ascending) sharing two factors with it up to
//     sign whose merged third factor stays in bounds;
//   plus / split / split-existed as SchemeInteger with the bound checked.
//
// Layout: coefficient vectors are three two's-complement bit planes (value =
// b0 + 2 b1 - 4 b2, entry e at bit e), so sums, negations, the bound check
// and sign tests are a few word operations.  Walk state in shared memory:
// planes [3 components][3 planes][cap] u64 and partner counts [3][cap] u16.
// Lane l owns terms t = 32 q + l (slot q), so ascending term order is slot
// by slot and a warp access to one slot touches 32 consecutive words.
// Rare structural edits (plus, split, merges, compaction) are computed by all
// lanes from shared memory with the replicated stream and written by lane 0,
// followed by a count rebuild.  Records use sign-magnitude masks (fac =
// nonzero, sgn = negative, fac2 = |c| = 2).
#pragma once
#include "fg_device.cuh"

namespace fg {

struct Vec3 {
    uint64_t b0, b1, b2;
};

__device__ __forceinline__ bool v3eq(const Vec3 &a, const Vec3 &b) { return a.b0 == b.b0 && a.b1 == b.b1 && a.b2 == b.b2; }
__device__ __forceinline__ bool v3zero(const Vec3 &a) { return !(a.b0 | a.b1 | a.b2); }
// -b on the entries of mask L (two's complement: invert, add one).
__device__ __forceinline__ Vec3 v3neg(const Vec3 &b, uint64_t L) {
    const uint64_t x0 = ~b.b0 & L, x1 = ~b.b1 & L, x2 = ~b.b2 & L;
    Vec3 n;
    n.b0 = b.b0;
    uint64_t c = x0;
    n.b1 = x1 ^ c;
    c &= x1;
    n.b2 = x2 ^ c;
    return n;
}
// out = a + b; false when an entry leaves [-2, 2] (4-plane sum checked).
__device__ __forceinline__ bool v3add(const Vec3 &a, const Vec3 &b, Vec3 &out) {
    const uint64_t s0 = a.b0 ^ b.b0, c1 = a.b0 & b.b0;
    const uint64_t t1 = a.b1 ^ b.b1, s1 = t1 ^ c1, c2 = (a.b1 & b.b1) | (c1 & t1);
    const uint64_t t2 = a.b2 ^ b.b2, s2 = t2 ^ c2, c3 = (a.b2 & b.b2) | (c2 & t2);
    const uint64_t s3 = t2 ^ c3;  // sign extension: plane 3 of each operand is its plane 2
    const uint64_t bad = (~s3 & (s2 | (s1 & s0))) | (s3 & ~(s2 & s1));
    out.b0 = s0; out.b1 = s1; out.b2 = s2;
    return bad == 0;
}
__device__ __forceinline__ bool v3sub(const Vec3 &a, const Vec3 &b, uint64_t L, Vec3 &out) { return v3add(a, v3neg(b, L), out); }
__device__ __forceinline__ bool v3firstPositive(const Vec3 &a) {
    const uint64_t nz = a.b0 | a.b1 | a.b2;
    return !(a.b2 & nz & (~nz + 1));
}
// 1 equal, -1 negated, 0 otherwise (nb = -b)
__device__ __forceinline__ int v3rel(const Vec3 &a, const Vec3 &b, const Vec3 &nb) {
    return v3eq(a, b) ? 1 : (v3eq(a, nb) ? -1 : 0);
}
// sign-magnitude masks <-> planes
__device__ __forceinline__ Vec3 v3fromMasks(uint64_t nz, uint64_t neg, uint64_t two) {
    return Vec3{nz & ~two, (two | neg) & nz, neg & nz};
}
__device__ __forceinline__ void v3toMasks(const Vec3 &v, uint64_t &nz, uint64_t &neg, uint64_t &two) {
    nz = v.b0 | v.b1;
    neg = v.b2;
    two = v.b1 & ~v.b0;
}

// Shared-memory words of one walk: planes [9][cap] u64 + counts [3][cap] u16, padded.
__host__ __device__ inline int zb_words(int cap) { return 9 * cap + (6 * cap + 7) / 8 + 1; }

struct ZBWalk {
    uint64_t *X;  // [3][3][cap]
    uint16_t *H;  // [3][cap]
    int cap, nslot;
    int n0, n1, n2, full;
    int nnc[3];
    uint64_t Lc[3];
    int m, P0, P1, P2, status;
    PhiloxDraws &r;

    __device__ ZBWalk(PhiloxDraws &rr) : r(rr) {}

    __device__ __forceinline__ Vec3 get(int c, int t) const {
        const uint64_t *p = X + (size_t)c * 3 * cap + t;
        return Vec3{p[0], p[cap], p[2 * cap]};
    }
    __device__ __forceinline__ void put(int c, int t, const Vec3 &v) {  // one writer
        uint64_t *p = X + (size_t)c * 3 * cap + t;
        p[0] = v.b0; p[cap] = v.b1; p[2 * cap] = v.b2;
    }
    __device__ __forceinline__ uint16_t &cnt(int c, int t) const { return H[c * cap + t]; }
    __device__ __forceinline__ void addP(int c, int d) { if (c == 0) P0 += d; else if (c == 1) P1 += d; else P2 += d; }
    __device__ __forceinline__ bool sim(const Vec3 &a, const Vec3 &b, const Vec3 &nb) const { return v3eq(a, b) || v3eq(a, nb); }
    __device__ __forceinline__ bool zeroTerm(int t) const { return v3zero(get(0, t)) || v3zero(get(1, t)) || v3zero(get(2, t)); }

    // ------------------------------------------------------------ counts
    __device__ void rebuildCounts() {
        __syncwarp();
        int tot[3] = {0, 0, 0};
        for (int c = 0; c < 3; c++) {
            int loc = 0;
            for (int q = 0; q < nslot; q++) {
                const int t = 32 * q + lane_id();
                if (t >= m) break;
                const Vec3 v = get(c, t), nv = v3neg(v, Lc[c]);
                int h = 0;
                for (int u = 0; u < m; u++) h += (u != t) && sim(get(c, u), v, nv);
                cnt(c, t) = (uint16_t)h;
                loc += h;
            }
            tot[c] = (int)__reduce_add_sync(kFull, (unsigned)loc);
        }
        P0 = tot[0]; P1 = tot[1]; P2 = tot[2];
        __syncwarp();
    }

    // Word (c, t) := nw with incremental partner counts (warp).
    __device__ void setWord(int c, int t, const Vec3 &nw) {
        const Vec3 old = get(c, t), nold = v3neg(old, Lc[c]), nnew = v3neg(nw, Lc[c]);
        const int ho = cnt(c, t);
        __syncwarp();
        int hn = 0;
        for (int q = 0; q < nslot; q++) {
            const int u = 32 * q + lane_id();
            if (u >= m) break;
            if (u == t) continue;
            const Vec3 w = get(c, u);
            const int dec = sim(w, old, nold), inc = sim(w, nw, nnew);
            if (dec != inc) cnt(c, u) = (uint16_t)(cnt(c, u) + inc - dec);
            hn += inc;
        }
        hn = (int)__reduce_add_sync(kFull, (unsigned)hn);
        __syncwarp();
        if (lane_id() == 0) {
            put(c, t, nw);
            cnt(c, t) = (uint16_t)hn;
        }
        addP(c, 2 * (hn - ho));
        __syncwarp();
    }

    // ------------------------------------------------------------ structure
    __device__ void fixSigns(int t) {  // scheme_integer.cu:398-425 for one term; counts unchanged
        __syncwarp();
        const bool pi = v3firstPositive(get(0, t)), pj = v3firstPositive(get(1, t));
        if (!(pi && pj) && lane_id() == 0) {
            const int c0 = (!pi && !pj) ? 0 : (!pi ? 0 : 1);
            const int c1 = (!pi && !pj) ? 1 : 2;
            put(c0, t, v3neg(get(c0, t), Lc[c0]));
            put(c1, t, v3neg(get(c1, t), Lc[c1]));
        }
        __syncwarp();
    }
    __device__ void moveTerm(int dst, int src) {  // lane 0
        for (int c = 0; c < 3; c++) put(c, dst, get(c, src));
    }
    __device__ void removeAt(int t) {  // counts are rebuilt by the caller
        __syncwarp();
        m--;
        if (t != m && lane_id() == 0) moveTerm(t, m);
        __syncwarp();
    }
    __device__ void removeZeroes() {  // re-checks the moved term
        __syncwarp();
        int mm = m;
        if (lane_id() == 0)
            for (int t = 0; t < mm; t++)
                if (zeroTerm(t)) {
                    mm--;
                    if (t != mm) moveTerm(t, mm);
                    t--;
                }
        m = __shfl_sync(kFull, mm, 0);
        __syncwarp();
    }
    __device__ void append(const Vec3 &a, const Vec3 &b, const Vec3 &c) {
        if (m >= cap || m >= kMaxRank) { status |= ST_OVERFLOW; return; }
        __syncwarp();
        if (lane_id() == 0) { put(0, m, a); put(1, m, b); put(2, m, c); }
        m++;
        __syncwarp();
    }

    // Term a's factors and their negations, for the merge tests against it.
    struct Term {
        Vec3 f[3], nf[3];
    };
    __device__ Term term(int a) const {
        Term T;
        for (int c = 0; c < 3; c++) {
            T.f[c] = get(c, a);
            T.nf[c] = v3neg(T.f[c], Lc[c]);
        }
        return T;
    }
    // Term t shares two factors with term A up to sign, third merged within bounds.
    __device__ bool mergeable(const Term &A, int t, int &rr, Vec3 &merged) const {
        int e[3];
        for (int c = 0; c < 3; c++) e[c] = v3rel(get(c, t), A.f[c], A.nf[c]);
        if ((e[0] != 0) + (e[1] != 0) + (e[2] != 0) < 2) return false;
        const int p0s[3] = {0, 0, 1}, p1s[3] = {1, 2, 2};
        for (int q = 0; q < 3; q++) {
            const int p0 = p0s[q], p1 = p1s[q];
            if (!e[p0] || !e[p1]) continue;
            const int k = 3 - p0 - p1;
            if (v3add(get(k, t), e[p0] * e[p1] > 0 ? A.f[k] : A.nf[k], merged)) {
                rr = k;
                return true;
            }
        }
        return false;
    }
    // keep absorbs drop: x_r[keep] = merged, drop removed, keep removed too when merged is zero.
    __device__ void merge(int keep, int drop, int rc, const Vec3 &merged) {
        __syncwarp();
        if (lane_id() == 0) put(rc, keep, merged);
        __syncwarp();
        const bool zero = v3zero(merged);
        removeAt(drop);
        if (keep == m) keep = drop;
        if (zero) removeAt(keep);
        else fixSigns(keep);
        rebuildCounts();
    }
    // First term t != a (ascending) that absorbs a.
    __device__ bool reduceWith(int a) {
        const Term A = term(a);
        for (int q = 0; q < nslot; q++) {
            const int t = 32 * q + lane_id();
            int rr = 0;
            Vec3 mg;
            const bool ok = t < m && t != a && mergeable(A, t, rr, mg);
            const unsigned bm = __ballot_sync(kFull, ok);
            if (bm) {
                const int src = __ffs(bm) - 1;
                const int rc = __shfl_sync(kFull, rr, src);
                const Vec3 merged{__shfl_sync(kFull, mg.b0, src), __shfl_sync(kFull, mg.b1, src),
                                  __shfl_sync(kFull, mg.b2, src)};
                merge(32 * q + src, a, rc, merged);
                return true;
            }
        }
        return false;
    }
    __device__ bool tryReduce() {  // first pair (a < b), b absorbed by a
        for (int a = 0; a < m; a++) {
            for (int q = (a + 1) / 32; q < nslot; q++) {
                const int b = 32 * q + lane_id();
                int rr = 0;
                Vec3 mg;
                // b absorbed by a: merged = x_r[a] + e x_r[b], the relation being symmetric
                bool ok = false;
                if (b > a && b < m) {
                    const Term B = term(b);
                    ok = mergeable(B, a, rr, mg);
                }
                const unsigned bm = __ballot_sync(kFull, ok);
                if (bm) {
                    const int src = __ffs(bm) - 1;
                    const int rc = __shfl_sync(kFull, rr, src);
                    const Vec3 merged{__shfl_sync(kFull, mg.b0, src), __shfl_sync(kFull, mg.b1, src),
                                      __shfl_sync(kFull, mg.b2, src)};
                    merge(a, 32 * q + src, rc, merged);
                    return true;
                }
            }
        }
        return false;
    }

    // ------------------------------------------------------------ flip
    // 1 accepted, 0 no pair, -1 rejected by the bound.
    __device__ int tryFlip() {
        const int Ptot = P0 + P1 + P2;
        if (Ptot <= 0) return 0;
        int q = (int)r.below((uint32_t)Ptot);
        int c;
        if (q < P0) c = 0;
        else if (q < P0 + P1) { c = 1; q -= P0; }
        else { c = 2; q -= P0 + P1; }
        // term a: slot totals, then the lane inside the slot
        int xs = -1, hv = 0;
        for (int x = 0; x < nslot; x++) {
            const int t = 32 * x + lane_id();
            const int hx = t < m ? (int)cnt(c, t) : 0;
            const int tx = (int)__reduce_add_sync(kFull, (unsigned)hx);
            if (xs < 0) {
                if (q < tx) { xs = x; hv = hx; }
                else q -= tx;
            }
        }
        if (xs < 0) { status |= ST_INTERNAL; return 0; }
        const int incl = warp_inclusive_sum(hv);
        const unsigned over = __ballot_sync(kFull, incl > q);
        if (!over) { status |= ST_INTERNAL; return 0; }
        const int owner = __ffs(over) - 1;
        int k = q - __shfl_sync(kFull, incl - hv, owner);
        const int a = 32 * xs + owner;
        const Vec3 va = get(c, a), nva = v3neg(va, Lc[c]);
        // partner b: the k-th other term (ascending) equal to a's factor up to sign
        int b = -1;
        for (int x = 0; x < nslot && b < 0; x++) {
            const int t = 32 * x + lane_id();
            unsigned bits = __ballot_sync(kFull, t < m && t != a && sim(get(c, t), va, nva));
            const int cnt_ = __popc(bits);
            if (k < cnt_) {
                for (int z = 0; z < k; z++) bits &= bits - 1;
                b = 32 * x + __ffs(bits) - 1;
            } else {
                k -= cnt_;
            }
        }
        if (b < 0) { status |= ST_INTERNAL; return 0; }
        const int e = v3eq(get(c, b), va) ? 1 : -1;
        int j = c == 0 ? 1 : 0, kk = c == 2 ? 1 : 2;
        if (r.coin()) { const int tmp = j; j = kk; kk = tmp; }
        const int sg = r.coin() ? -1 : 1;
        const Vec3 yb = get(j, b), za = get(kk, a);
        Vec3 na, nb;
        if (!v3add(get(j, a), sg * e > 0 ? yb : v3neg(yb, Lc[j]), na)) return -1;
        if (!v3add(get(kk, b), sg > 0 ? v3neg(za, Lc[kk]) : za, nb)) return -1;
        setWord(j, a, na);
        setWord(kk, b, nb);
        fixSigns(a);
        fixSigns(b);
        if (v3zero(na) || v3zero(nb)) {
            removeZeroes();
            rebuildCounts();
            return 1;
        }
        if (!reduceWith(a)) reduceWith(b);
        return 1;
    }

    // ------------------------------------------------------------ expansions
    __device__ __forceinline__ void perm3(int &i, int &j, int &k) {  // randomPermutation(p, 3)
        int p0 = 0, p1 = 1, p2 = 2;
        int q = (int)r.below(3);
        if (q == 0) { int t = p2; p2 = p0; p0 = t; } else if (q == 1) { int t = p2; p2 = p1; p1 = t; }
        q = (int)r.below(2);
        if (q == 0) { int t = p1; p1 = p0; p0 = t; }
        i = p0; j = p1; k = p2;
    }
    __device__ bool tryPlus() {
        if (m >= kMaxRank || m >= full) return false;
        int a = (int)r.below((uint32_t)m), b = (int)r.below((uint32_t)m);
        int guard = 0;
        auto same = [&](int c) {
            const Vec3 B = get(c, b);
            return sim(get(c, a), B, v3neg(B, Lc[c]));
        };
        while (a == b || same(0) || same(1) || same(2)) {
            if (++guard > retry_cap_of(r.P)) { status |= ST_RETRY; return false; }
            a = (int)r.below((uint32_t)m);
            b = (int)r.below((uint32_t)m);
        }
        int i, j, k;
        perm3(i, j, k);
        Vec3 ti, tj, tk;
        if (!v3sub(get(i, a), get(i, b), Lc[i], ti) || !v3sub(get(j, a), get(j, b), Lc[j], tj) ||
            !v3add(get(k, a), get(k, b), tk))
            return false;
        const Vec3 Bi = get(i, b), Bj = get(j, b), Ak = get(k, a);
        __syncwarp();
        if (lane_id() == 0) {
            put(i, a, ti);
            put(j, b, tj);
            put(k, b, Ak);
        }
        __syncwarp();
        fixSigns(a);
        fixSigns(b);
        if (!v3zero(tk)) {
            Vec3 t3[3];
            t3[i] = Bi; t3[j] = Bj; t3[k] = tk;
            append(t3[0], t3[1], t3[2]);
            fixSigns(m - 1);
        }
        rebuildCounts();
        return true;
    }
    __device__ __forceinline__ uint64_t mask64(int bits) {
        const uint64_t low = bits >= 64 ? ~0ull : ((1ull << bits) - 1);
        if (bits <= 32) return (uint64_t)r.raw() & low;
        const uint64_t lo = r.raw();
        return (lo | ((uint64_t)r.raw() << 32)) & low;
    }
    __device__ __forceinline__ Vec3 randomTernary(int bits) {
        const uint64_t nz = mask64(bits);
        const uint64_t neg = mask64(bits) & nz;
        return v3fromMasks(nz, neg, 0);
    }
    __device__ void split(int i, int t, const Vec3 &v, const Vec3 &rest) {
        Vec3 nt[3] = {get(0, t), get(1, t), get(2, t)};
        nt[i] = rest;
        __syncwarp();
        if (lane_id() == 0) put(i, t, v);
        __syncwarp();
        fixSigns(t);
        append(nt[0], nt[1], nt[2]);
        fixSigns(m - 1);
        rebuildCounts();
    }
    __device__ bool trySplit() {
        if (m >= kMaxRank || m >= full) return false;
        const int t = (int)r.below((uint32_t)m);
        int i, j, k;
        perm3(i, j, k);
        Vec3 v = randomTernary(nnc[i]), rest;
        const Vec3 x = get(i, t);
        auto bad = [&]() { return v3zero(v) || v3eq(v, x) || !v3sub(x, v, Lc[i], rest); };
        int loop = 0;
        while (loop < 5 && bad()) { v = randomTernary(nnc[i]); loop++; }
        if (loop == 5) return false;
        split(i, t, v, rest);
        return true;
    }
    __device__ bool trySplitExisted() {
        if (m >= kMaxRank || m >= full) return false;
        int i, j, k;
        perm3(i, j, k);
        const int a = (int)r.below((uint32_t)m);
        int b = (int)r.below((uint32_t)m);
        Vec3 rest;
        auto bad = [&]() { return a == b || v3eq(get(i, a), get(i, b)) || !v3sub(get(i, a), get(i, b), Lc[i], rest); };
        int loop = 0;
        while (loop < 5 && bad()) { b = (int)r.below((uint32_t)m); loop++; }
        if (loop == 5) return false;
        split(i, a, get(i, b), rest);
        return true;
    }
    __device__ bool tryExpand(int count) {
        bool result = false;
        for (int q = 0; q < count && m < full; q++) {
            const int v = (int)r.below(3);
            if (v == 0) result |= tryPlus();
            else if (v == 1) result |= trySplit();
            else result |= trySplitExisted();
        }
        return result;
    }
};

}  // namespace fg
