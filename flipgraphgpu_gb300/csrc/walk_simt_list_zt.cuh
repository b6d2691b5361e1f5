// List-mode ternary (ZT) walk, one THREAD per walk: the reference's SchemeInteger
// walk (src/schemes/scheme_integer.cu, src/entities/addition.cu) step for step,
// so with the cuRAND XORWOW stream it reproduces the reference's trajectories
// bit for bit, like the warp-per-walk ZTWalk.
//
// The reference's tryFlip visits the listed pairs in a random permutation of all
// of them (randomPermutation, random.cuh:9-22: one draw per pair), so its cost
// per flip is dominated by those draws.  The warp walker computes every draw in
// every lane; here each thread draws for its own walk.  The draws
// j_i = curand() % (i + 1), i = size-1 .. 1, are written eight to a 16-byte
// vector into the walk's column of the global scratch; position p of the
// permutation is then traced back through the swaps (pos = j_i when pos = i,
// i when pos = j_i), several positions per pass over the draws.
//
// Layout: values and signs of the factors in shared memory, 32 walks interleaved
// by lane (word (c, t) at [(c * ld + t) * 32]), as 32-bit words: factors of at
// most 31 entries.  The reference's random split (Addition::random, 16 bits per
// chunk) shifts its second chunk as an int, so bits 32-63 of such a factor copy
// bit 31, and the naive factors of at most 31 entries leave bits 31-63 clear; a
// 32-bit word w stands for the 64-bit factor sext(w), and every operation of the
// walk (xor, and, equality, lowest set bit) commutes with that extension.  (A
// naive factor of 32 entries sets bit 31 alone: such shapes take the warp kernel.)  A factor that overflowed (the reference's Addition::valid false,
// only possible for input coefficients outside {-1, 0, 1}; the walk's own moves
// test their limits first) is marked by bit 31 of its sign word in walks whose
// factors hold at most 16 entries (mk = that bit); walks with wider factors need
// every input factor valid (the host checks) and use all 32 bits (mk = 0).
// Lists as in walk_simt_list.cuh.
#pragma once
#include <type_traits>
#include "walk_simt_list.cuh"
#include "walk_zt.cuh"

namespace fg {

// 16-byte vectors of permutation draws per walk: positions up to 3 * kListCap.
constexpr int kPermVecs = (3 * kListCap + 7) / 8;
constexpr uint32_t kInvalidMark = 0x80000000u;

// x % d for 2 <= d <= 3 * kListCap + 1 by multiplication with the divisor's magic number
// (Granlund and Montgomery, "Division by invariant integers using multiplication", PLDI
// 1994, unsigned N = 32): mg = (m, l) with l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1;
// q = (t + ((x - t) >> 1)) >> (l - 1) with t = mulhi(m, x).  Exact for every 32-bit x.
constexpr int kRemTableSize = 3 * kListCap + 2;

__device__ __forceinline__ uint32_t rem_magic(uint32_t x, uint32_t d, uint2 mg) {
    const uint32_t t = __umulhi(mg.x, x);
    const uint32_t q = (t + ((x - t) >> 1)) >> (mg.y - 1);
    return x - q * d;
}

template <class R>
struct SimtListZT : SimtLists {
    uint32_t *xv, *xs;  // this walk's value and sign columns in shared memory
    uint4 *J;           // this walk's permutation-draw column in the global scratch
    const uint2 *mg;    // remainder magic numbers, indexed by divisor
    uint32_t mk;        // the invalid mark of a sign word: kInvalidMark, or 0 for factors of > 16 entries
    int ld;             // slots per component in shared memory (<= 256)
    int cap;            // slots a rank may reach
    int n0, n1, n2, nn0, nn1, nn2, full;
    int m;
    int status;
    R &r;

    __device__ SimtListZT(R &rr) : r(rr) {}

    __device__ __forceinline__ size_t at(int c, int t) const { return (size_t)(c * ld + t) << 5; }
    __device__ __forceinline__ Tern X(int c, int t) const {
        const uint32_t s = xs[at(c, t)];
        return Tern{(uint64_t)xv[at(c, t)], (uint64_t)(s & ~mk), !(s & mk)};
    }
    __device__ __forceinline__ void setX(int c, int t, const Tern &a) {
        xv[at(c, t)] = (uint32_t)a.v;
        if (!a.ok && !mk) status |= ST_INTERNAL;  // no mark for factors of > 16 entries
        xs[at(c, t)] = (uint32_t)a.s | (a.ok ? 0u : mk);
    }
    __device__ __forceinline__ bool sameX(int c, int t, const Tern &a) const {  // values and signs
        return xv[at(c, t)] == (uint32_t)a.v && (xs[at(c, t)] & ~mk) == (uint32_t)a.s;
    }
    __device__ __forceinline__ int nn(int c) const { return c == 0 ? nn0 : (c == 1 ? nn1 : nn2); }
    __device__ __forceinline__ bool nonzero(int t) const { return xv[at(0, t)] && xv[at(1, t)] && xv[at(2, t)]; }

    // initFlips (scheme_integer.cu:229-238): pairs with identical values and signs.
    __device__ __forceinline__ void rebuild() {
        for (int c = 0; c < 3; c++) {
            int s = 0;
            for (int a = 0; a < m; a++) {
                const Tern v = X(c, a);
                for (int b = a + 1; b < m; b++)
                    if (sameX(c, b, v)) {
                        if (s < kListCap) setLq(c, s, pack16(a, b));
                        s++;
                    }
            }
            setSz(c, s < kListCap ? s : kListCap);
        }
    }

    __device__ __forceinline__ void moveTerm(int dst, int src) {
        for (int c = 0; c < 3; c++) { xv[at(c, dst)] = xv[at(c, src)]; xs[at(c, dst)] = xs[at(c, src)]; }
    }

    // removeZeroes (scheme_integer.cu:240-251): the moved term is re-checked.
    __device__ __forceinline__ void removeZeroes() {
        for (int t = 0; t < m; t++) {
            if (nonzero(t)) continue;
            m--;
            moveTerm(t, m);
            t--;
        }
    }

    __device__ __forceinline__ void removeAt(int t) {
        m--;
        if (t != m) moveTerm(t, m);
    }

    __device__ __forceinline__ void addTriplet(int i, int j, int k, const Tern &a, const Tern &b, const Tern &c) {
        if (m >= cap) { status |= ST_OVERFLOW; return; }
        setX(i, m, a); setX(j, m, b); setX(k, m, c);
        m++;
    }

    // fixSigns (scheme_integer.cu:398-425): first nonzero of u and v positive.
    __device__ __forceinline__ void fixSigns() {
        for (int t = 0; t < m; t++) {
            const uint32_t v0 = xv[at(0, t)], v1 = xv[at(1, t)];
            const uint32_t s0 = xs[at(0, t)] & ~mk, s1 = xs[at(1, t)] & ~mk;
            const bool pi = firstPositive(v0, s0), pj = firstPositive(v1, s1);
            if (pi && pj) continue;
            const int c0 = (!pi && !pj) ? 0 : (!pi ? 0 : 1);
            const int c1 = (!pi && !pj) ? 1 : 2;
            xs[at(c0, t)] = (~xs[at(c0, t)] & xv[at(c0, t)] & ~mk) | (xs[at(c0, t)] & mk);
            xs[at(c1, t)] = (~xs[at(c1, t)] & xv[at(c1, t)] & ~mk) | (xs[at(c1, t)] & mk);
        }
    }

    __device__ __forceinline__ void reduceAdd(int i, int a, int b) {  // scheme_integer.cu:549-559
        const Tern x = tadd(X(i, a), X(i, b));
        setX(i, a, x);
        removeAt(b);
        if (!x.v) removeZeroes();
        rebuild();
    }

    __device__ __forceinline__ void reduceSub(int i, int a, int b) {  // scheme_integer.cu:561-571
        const Tern x = tsub(X(i, a), X(i, b));
        setX(i, a, x);
        removeAt(b);
        if (!x.v) removeZeroes();
        rebuild();
    }

    // tryReduce (scheme_integer.cu:1062-1101): the first listed pair (list order) that can merge.
    __device__ __forceinline__ bool tryReduce() {
        for (int q = 0; q < sz0; q++) {
            const uint32_t pr = Lq(0, q);
            const int a = (int)(pr >> 8), b = (int)(pr & 0xFFu);
            const Tern u1 = X(1, a), u2 = X(1, b), w1 = X(2, a), w2 = X(2, b);
            if (teq(u1, u2) && tlimitSum(w1, w2, false)) { reduceAdd(2, a, b); return true; }
            const int cmp2 = tcompare(w1, w2);
            if (cmp2 == 1 && tlimitSum(u1, u2, true)) { reduceAdd(1, a, b); return true; }
            if (cmp2 == -1 && tlimitSub(u1, u2, true)) { reduceSub(1, a, b); return true; }
        }
        for (int q = 0; q < sz1; q++) {
            const uint32_t pr = Lq(1, q);
            const int a = (int)(pr >> 8), b = (int)(pr & 0xFFu);
            const int cmp2 = tcompare(X(2, a), X(2, b));
            if (cmp2 == 1 && tlimitSum(X(0, a), X(0, b), true)) { reduceAdd(0, a, b); return true; }
            if (cmp2 == -1 && tlimitSub(X(0, a), X(0, b), true)) { reduceSub(0, a, b); return true; }
        }
        return false;
    }

    // The reduction a new partner t of term a in component j triggers (scheme_integer.cu:
    // 445-469): 0 none, 1..4 = reduceAdd(k), reduceSub(k), reduceAdd(i), reduceSub(i).
    __device__ __forceinline__ int action(int i, int j, int k, int t, int a) const {
        const Tern it = X(i, t), ia = X(i, a), kt = X(k, t), ka = X(k, a);
        const int cmpI = tcompare(it, ia);
        if (cmpI == 1 && tlimitSum(kt, ka, k != 2)) return 1;
        if (i == 2 && cmpI == -1 && tlimitSub(kt, ka, true)) return 2;
        const int cmpK = tcompare(kt, ka);
        if (cmpK == 1 && tlimitSum(it, ia, i != 2)) return 3;
        if (k == 2 && cmpK == -1 && tlimitSub(it, ia, true)) return 4;
        return 0;
    }

    __device__ __forceinline__ void apply(int act, int i, int k, int t, int a) {
        if (act == 1) reduceAdd(k, t, a);
        else if (act == 2) reduceSub(k, t, a);
        else if (act == 3) reduceAdd(i, t, a);
        else reduceSub(i, t, a);
    }

    // flip (scheme_integer.cu:428-501).
    __device__ __forceinline__ void flip(int i, int j, int k, int a, int b, bool checkReduce) {
        const Tern nja = tadd(X(j, a), X(j, b));  // uvw[j][a] += uvw[j][b]
        const Tern nkb = tsub(X(k, b), X(k, a));  // uvw[k][b] -= uvw[k][a]
        setX(j, a, nja);
        setX(k, b, nkb);
        listRemoveIndex(j, (uint32_t)a);
        listRemoveIndex(k, (uint32_t)b);
        if (!nja.v || !nkb.v) {
            removeZeroes();
            rebuild();
            int guard = 0;
            while (tryReduce())
                if (++guard > retry_cap_of(r.P)) { status |= ST_RETRY; break; }
            return;
        }
        for (int t = 0; t < m; t++) {
            if (t != a && sameX(j, t, nja)) {
                if (checkReduce) {
                    const int act = action(i, j, k, t, a);
                    if (act) { apply(act, i, k, t, a); return; }
                }
                listAdd(j, a, t);
            }
            if (t != b && sameX(k, t, nkb)) {
                if (checkReduce) {
                    const int act = action(i, k, j, t, b);
                    if (act) { apply(act, i, j, t, b); return; }
                }
                listAdd(k, b, t);
            }
        }
    }

    // The permutation draws of randomPermutation(indices, size): j_i for i = size-1 .. 1,
    // stored eight to a vector (element i % 8 of vector i / 8).  Descending i, each draw
    // is shifted in at the bottom of a 128-bit accumulator, so element e ends at bits 16e.
    __device__ __forceinline__ void drawPermutation(int size) {
        uint64_t lo = 0, hi = 0;
        for (int i = size - 1; i >= 1; i--) {
            uint64_t x;
            if constexpr (std::is_same<R, XorwowDraws>::value)  // curand() % (i + 1), exactly
                x = rem_magic(r.raw(), (uint32_t)(i + 1), __ldg(mg + i + 1));
            else
                x = r.below((uint32_t)(i + 1));
            hi = (hi << 16) | (lo >> 48);
            lo = (lo << 16) | x;
            if ((i & 7) == 0 || i == 1) {
                if (i == 1) {  // there is no draw for i = 0: element 0 of the first vector stays empty
                    hi = (hi << 16) | (lo >> 48);
                    lo <<= 16;
                }
                J[(size_t)(i >> 3) << 5] = make_uint4((uint32_t)lo, (uint32_t)(lo >> 32), (uint32_t)hi,
                                                      (uint32_t)(hi >> 32));
            }
        }
    }

    // Positions p .. p+N-1 of the permutation, traced back through the swaps.
    template <int N>
    __device__ __forceinline__ void tracePositions(int p, int size, int (&pos)[N]) const {
#pragma unroll
        for (int q = 0; q < N; q++) pos[q] = p + q;
        for (int v = 0; v <= (size - 1) >> 3; v++) {
            const uint4 buf = J[(size_t)v << 5];
            const uint32_t wv[4] = {buf.x, buf.y, buf.z, buf.w};
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int i = v * 8 + u;
                if (i < 1 || i >= size) continue;
                const int j = (int)((wv[u >> 1] >> (16 * (u & 1))) & 0xFFFFu);
#pragma unroll
                for (int q = 0; q < N; q++) pos[q] = pos[q] == i ? j : (pos[q] == j ? i : pos[q]);
            }
        }
    }

    // Candidate `idx` of the listed pairs with its two orientation draws and the reference's
    // bound tests; on success the flip's (j, k, a, b) in fj, fk, fa, fb and fi = i.
    __device__ __forceinline__ bool tryCandidate(int idx, int &fi, int &fj, int &fk, int &fa, int &fb) {
        int i, j, k;
        uint32_t pr;
        if (idx < sz0) { i = 0; j = 1; k = 2; pr = Lq(0, idx); }
        else if (idx < sz0 + sz1) { i = 1; j = 0; k = 2; pr = Lq(1, idx - sz0); }
        else { i = 2; j = 0; k = 1; pr = Lq(2, idx - sz0 - sz1); }
        int a = (int)(pr >> 8), b = (int)(pr & 0xFFu);
        if (r.coin()) { int tmp = j; j = k; k = tmp; }
        if (r.coin()) { int tmp = a; a = b; b = tmp; }
        const Tern ja = X(j, a), jb = X(j, b), ka = X(k, a), kb = X(k, b);
        if (tlimitSum(ja, jb, j != 2) && tlimitSub(kb, ka, false)) {
            const bool keep = k == 2 || tposSub(kb, ka);
            fi = i; fj = j; fk = k; fa = keep ? a : b; fb = keep ? b : a;
            return true;
        }
        if (tlimitSum(ka, kb, k != 2) && tlimitSub(jb, ja, false)) {
            const bool keep = j == 2 || tposSub(jb, ja);
            fi = i; fj = k; fk = j; fa = keep ? a : b; fb = keep ? b : a;
            return true;
        }
        return false;
    }

    // tryFlip (scheme_integer.cu:907-975).  The candidates are searched first and the flip is
    // applied once after the search, so the 32 walks of a warp apply their flips together
    // whichever candidate each accepted.  Nearly every flip accepts its first candidate, so
    // the first pass traces two positions, later passes eight.
    __device__ __forceinline__ bool tryFlip(bool checkReduce) {
        const int size = sz0 + sz1 + sz2;
        drawPermutation(size);
        int fi = -1, fj = 0, fk = 0, fa = 0, fb = 0;
        {
            int pos[2];
            tracePositions<2>(0, size, pos);
            if (size > 0 && tryCandidate(pos[0], fi, fj, fk, fa, fb)) {}
            else if (size > 1 && tryCandidate(pos[1], fi, fj, fk, fa, fb)) {}
        }
        for (int p0 = 2; fi < 0 && p0 < size; p0 += 8) {
            int pos[8];
            tracePositions<8>(p0, size, pos);
            const int lim = size - p0 < 8 ? size - p0 : 8;
#pragma unroll
            for (int q = 0; q < 8; q++)
                if (q < lim && fi < 0) tryCandidate(pos[q], fi, fj, fk, fa, fb);
        }
        if (fi < 0) return false;
        flip(fi, fj, fk, fa, fb, checkReduce);
        return true;
    }

    // plus (scheme_integer.cu:503-539).
    __device__ __forceinline__ void plus(int i, int j, int k, int p, int q, int variant) {
        const Tern a1 = X(i, p), b1 = X(j, p), c1 = X(k, p);
        const Tern a2 = X(i, q), b2 = X(j, q), c2 = X(k, q);
        const Tern aAdd = tadd(a1, a2), bAdd = tadd(b1, b2), cAdd = tadd(c1, c2);
        const Tern aSub = tsub(a2, a1), bSub = tsub(b2, b1), cSub = tsub(c2, c1);
        if (variant == 0 && tlimit(aSub, i != 2) && tlimit(bAdd, j != 2) && tlimit(cSub, k != 2)) {
            setX(j, p, bAdd); setX(i, q, aSub);
            addTriplet(i, j, k, a1, b2, cSub);
        } else if (variant == 1 && tlimit(aSub, i != 2) && tlimit(bSub, j != 2) && tlimit(cAdd, k != 2)) {
            setX(k, p, cAdd); setX(j, q, bSub);
            addTriplet(i, j, k, aSub, b1, c2);
        } else if (tlimit(aAdd, i != 2) && tlimit(bSub, j != 2) && tlimit(cSub, k != 2)) {
            setX(i, p, aAdd); setX(k, q, cSub);
            addTriplet(i, j, k, a2, bSub, c1);
        }
        removeZeroes();
        fixSigns();
        rebuild();
    }

    __device__ __forceinline__ void split(int i, int j, int k, int t, const Tern &a) {  // scheme_integer.cu:541-547
        const Tern rest = tsub(X(i, t), a), bj = X(j, t), bk = X(k, t);
        addTriplet(i, j, k, rest, bj, bk);
        setX(i, t, a);
        fixSigns();
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

    __device__ __forceinline__ bool tryPlus() {  // scheme_integer.cu:977-998
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
        const int variant = (int)r.below(3);
        plus(i, j, k, a, b, variant);
        return true;
    }

    // Addition::random (addition.cu:66-80): a sign chunk then a value chunk of 16 bits per 16
    // entries; the second chunk lands in bits 16-31 (its sign extension is implicit).
    __device__ __forceinline__ Tern randomTern(int n) {
        uint32_t sb = r.raw() & 0xFFFFu;
        uint32_t vb = r.raw() & 0xFFFFu;
        if (n > 16) {
            sb |= (r.raw() & 0xFFFFu) << 16;
            vb |= (r.raw() & 0xFFFFu) << 16;
        }
        return Tern{(uint64_t)vb, (uint64_t)(sb & vb), true};
    }

    __device__ __forceinline__ bool trySplit() {  // scheme_integer.cu:1000-1020
        if (m >= kMaxRank || m >= full) return false;
        const int t = (int)r.below((uint32_t)m);
        int i, j, k;
        perm3(i, j, k);
        const Tern a = randomTern(nn(i));
        if (!tlimitSub(X(i, t), a, i != 2)) return false;
        split(i, j, k, t, a);
        return true;
    }

    __device__ __forceinline__ bool trySplitExisted() {  // scheme_integer.cu:1022-1043
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

    __device__ __forceinline__ bool tryExpand(int count) {  // scheme_integer.cu:1045-1060
        bool result = false;
        for (int q = 0; q < count && m < kMaxRank; q++) {
            const int v = (int)r.below(3);
            if (v == 0) result |= tryPlus();
            else if (v == 1) result |= trySplit();
            else result |= trySplitExisted();
            if (status) break;
        }
        return result;
    }
};

}  // namespace fg
