// Fast-mode Z2 walk: one THREAD per walk (SIMT across walks).
//
// Each warp holds 32 walks in shared memory, interleaved by lane:
// word (c, t, lane) = factor c of term t of the lane's walk, so every access
// a thread makes to its own walk hits bank (lane) -- conflict free for any
// per-thread index.  The top byte of each word counts the term's equal
// partners in that component (how many other terms carry the same factor);
// the factor itself uses the low bits (<= 24 bits in a 32-bit word, <= 56 in
// a 64-bit word).  With these counts a uniformly random ordered equal pair is
// located by a prefix walk over the counts, and after a flip the counts are
// updated in the same O(m) scan that looks for reductions -- no FlipSet lists.
//
// Semantics: the reference's walk (flip_graph.cu:520-573, scheme_z2.cu) with
// the Philox stream and implicit pair enumeration: the flip proposal is
// uniform over equal-factor pairs with a uniform orientation, exactly the
// reference's distribution; ranks drop, plus transitions, splits and
// compaction orders follow the reference.
#pragma once
#include "fg_device.cuh"
#include "gf2.cuh"

namespace fg {

// Per-thread Philox stream: the same word sequence as PhiloxDraws (word q of
// walk w = Philox(ctr = (q/4 lo, q/4 hi, w, 0), key)[q % 4]).
struct ThreadPhilox {
    uint32_t k0, k1, walk;
    uint64_t count;
    int64_t blk;
    uint4 buf;
    const WalkParams *P;
    __device__ __forceinline__ uint32_t raw() {
        int64_t b = (int64_t)(count >> 2);
        if (b != blk) {
            buf = philox4x32_10(make_uint4((uint32_t)b, (uint32_t)((uint64_t)b >> 32), walk, 0u), k0, k1);
            blk = b;
        }
        uint32_t e = (uint32_t)count & 3u;
        count++;
        return e == 0 ? buf.x : e == 1 ? buf.y : e == 2 ? buf.z : buf.w;
    }
    __device__ __forceinline__ uint32_t below(uint32_t k) { return __umulhi(raw(), k); }
    __device__ __forceinline__ bool coin() { return raw() >> 31; }
    __device__ __forceinline__ bool gate(uint64_t T) { return T != kGateOff && (uint64_t)raw() < T; }
    __device__ __forceinline__ bool gate_reduce() { return gate(P->reduce_T); }
    __device__ __forceinline__ bool gate_expand() { return gate(P->expand_T); }
    __device__ __forceinline__ bool gate_sandwich() { return gate(P->sandwich_T); }
    __device__ __forceinline__ bool gate_basis() { return gate(P->basis_T); }
    __device__ __forceinline__ bool gate_gauss() { return gate(P->gauss_T); }
    __device__ __forceinline__ bool tie() { return raw() < 42949672u; }
    __device__ __forceinline__ uint64_t mask(int nn) { return nn >= 32 ? (uint64_t)raw() : (uint64_t)(raw() & ((1u << nn) - 1u)); }
};

// SH = log2 of the word stride: 5 for the thread-per-walk layout (32 walks
// interleaved by lane), 0 for one walk stored compactly (the warp-per-walk
// kernel runs its rare structural edits through this code on lane 0), -1 for
// a stride chosen at run time (the learned walk's global-memory layout, all
// walks interleaved).
template <class W, int SH = 5>
struct SimtZ2 {
    static constexpr int HS = (int)sizeof(W) * 8 - 8;  // partner count lives in bits [HS, HS+8)
    static constexpr W FM = ((W)1 << HS) - 1;
    static constexpr W ONE = (W)1 << HS;

    W *s;  // this walk: word (c, t) at s[(c * ld + t) << SH] (SH < 0: shift rsh, set at run time)
    int rsh = 0;
    int cap;  // term slots (capacity)
    int ld;   // words between components (>= cap; set by every user)
    int n0, n1, n2, nn0, nn1, nn2, full;
    int m;
    int P0, P1, P2;  // ordered equal pairs per component
    int status;
    ThreadPhilox &r;

    __device__ SimtZ2(ThreadPhilox &rr) : r(rr) {}

    __device__ __forceinline__ int sh() const { return SH >= 0 ? SH : rsh; }
    __device__ __forceinline__ W &A(int c, int t) const { return s[(size_t)(c * ld + t) << sh()]; }
    __device__ __forceinline__ W F(int c, int t) const { return A(c, t) & FM; }
    __device__ __forceinline__ int nn(int c) const { return c == 0 ? nn0 : (c == 1 ? nn1 : nn2); }
    __device__ __forceinline__ bool nonzero(int t) const { return F(0, t) && F(1, t) && F(2, t); }
    __device__ __forceinline__ void addP(int c, int d) { if (c == 0) P0 += d; else if (c == 1) P1 += d; else P2 += d; }

    // Partner counts of every term from scratch (once per launch; every edit
    // below keeps them exact incrementally, in O(m) per changed word).
    __device__ void rebuild() {
        int tot[3] = {0, 0, 0};
#pragma unroll
        for (int c = 0; c < 3; c++) {
            for (int t = 0; t < m; t++) {
                const W v = F(c, t);
                int h = 0;
                for (int u = 0; u < m; u++) h += (u != t) & (F(c, u) == v);
                A(c, t) = v | ((W)h << HS);
                tot[c] += h;
            }
        }
        P0 = tot[0]; P1 = tot[1]; P2 = tot[2];
    }

    // Word (c, t) becomes v; the partner counts of t and of the terms that
    // shared its old or share its new factor follow.
    __device__ void setWord(int c, int t, W v) {
        const W w0 = A(c, t), old = w0 & FM;
        if (old == v) return;
        W *p = &A(c, 0);
        int h = 0;
        for (int u = 0; u < m; u++) {
            const W w = p[(size_t)u << sh()], f = w & FM;
            if (u == t) continue;
            if (f == old) p[(size_t)u << sh()] = w - ONE;
            else if (f == v) { p[(size_t)u << sh()] = w + ONE; h++; }
        }
        A(c, t) = v | ((W)h << HS);
        addP(c, 2 * (h - (int)(w0 >> HS)));
    }

    // Term t leaves the partner sets of the other terms [0, m).
    __device__ void dropCounts(int t) {
#pragma unroll 1
        for (int c = 0; c < 3; c++) {
            const W w0 = A(c, t), v = w0 & FM;
            const int h = (int)(w0 >> HS);
            if (!h) continue;
            W *p = &A(c, 0);
            for (int u = 0; u < m; u++)
                if (u != t && (p[(size_t)u << sh()] & FM) == v) p[(size_t)u << sh()] -= ONE;
            addP(c, -2 * h);
        }
    }

    // Term t (holding bare factors) joins the partner sets of the terms [0, m).
    __device__ void addCounts(int t) {
#pragma unroll 1
        for (int c = 0; c < 3; c++) {
            const W v = F(c, t);
            W *p = &A(c, 0);
            int h = 0;
            for (int u = 0; u < m; u++)
                if (u != t && (p[(size_t)u << sh()] & FM) == v) { p[(size_t)u << sh()] += ONE; h++; }
            A(c, t) = v | ((W)h << HS);
            addP(c, 2 * h);
        }
    }

    __device__ __forceinline__ void moveTerm(int dst, int src) {  // words keep their counts
#pragma unroll
        for (int c = 0; c < 3; c++) A(c, dst) = A(c, src);
    }

    __device__ __forceinline__ void clearTerm(int t) {  // words past the rank read as zero
#pragma unroll
        for (int c = 0; c < 3; c++) A(c, t) = 0;
    }

    __device__ void removeZeroes() {  // scheme_z2.cu:152-164 (no re-check of the moved term)
        while (m > 0 && !nonzero(m - 1)) { dropCounts(m - 1); m--; clearTerm(m); }
        for (int t = 0; t < m; t++)
            if (!nonzero(t)) { dropCounts(t); m--; moveTerm(t, m); clearTerm(m); }
    }

    __device__ void removeAt(int t) {
        dropCounts(t);
        m--;
        if (t != m) moveTerm(t, m);
        clearTerm(m);
    }

    __device__ void addTriplet(int i, int j, int k, W a, W b, W c) {
        if (m >= cap) { status |= ST_OVERFLOW; return; }
        A(i, m) = a; A(j, m) = b; A(k, m) = c;
        addCounts(m);
        m++;
    }

    __device__ void reduce(int i, int a, int b) {  // scheme_z2.cu:631-641
        const W v = F(i, a) ^ F(i, b);
        setWord(i, a, v);
        removeAt(b);
        if (!v) removeZeroes();
    }

    // flip (scheme_z2.cu:531-577) with the count update fused into the reduction scan.
    __device__ void flip(int i, int j, int k, int a, int b, bool checkReduce) {
        const W wja = A(j, a), wjb = A(j, b), wka = A(k, a), wkb = A(k, b);
        const W oldA = wja & FM, newA = oldA ^ (wjb & FM);
        const W oldB = wkb & FM, newB = oldB ^ (wka & FM);
        const int oldHa = (int)(wja >> HS), oldHb = (int)(wkb >> HS);
        if (!newA || !newB) {
            setWord(j, a, newA);
            setWord(k, b, newB);
            removeZeroes();
            return;
        }
        A(j, a) = newA;
        A(k, b) = newB;
        const W xia = F(i, a), xka = wka & FM, xib = F(i, b), xjb = wjb & FM;
        int cntA = 0, cntB = 0, red = -1, part = 0;
        // One pass: count updates over all terms, and at the (rare) new partners the
        // reduction test; the first term (ascending) that triggers one wins, its
        // j-part tested before its k-part.  Factor bits do not change in the pass.
        W *pj = &A(j, 0), *pk = &A(k, 0);
        // SH = 5: words past the rank are zero and never match (factors are nonzero), so
        // the pass runs over whole groups of 4 without a remainder loop (3-7 % faster).
        const int mEnd = SH == 5 ? (m + 3) & ~3 : m;
#pragma unroll 4
        for (int t = 0; t < mEnd; t++) {
            const W wj = pj[(size_t)t << sh()], wk = pk[(size_t)t << sh()];
            const W vj = wj & FM, vk = wk & FM;
            const bool oj = (vj == oldA) & (t != a), nj = (vj == newA) & (t != a);
            const bool ok = (vk == oldB) & (t != b), nk = (vk == newB) & (t != b);
            cntA += nj;
            cntB += nk;
            // Unconditional write-back: the 32 lanes hold 32 different walks, so a
            // conditional store diverges; storing every word is 16 % faster (4x4x4).
            pj[(size_t)t << sh()] = wj + (nj ? ONE : (W)0) - (oj ? ONE : (W)0);
            pk[(size_t)t << sh()] = wk + (nk ? ONE : (W)0) - (ok ? ONE : (W)0);
            if (checkReduce && (nj | nk) && red < 0) {
                const W vi = F(i, t);
                if (nj && (vi == xia || vk == xka)) { red = t; part = 0; }
                else if (nk && (vi == xib || vj == xjb)) { red = t; part = 1; }
            }
        }
        A(j, a) = newA | ((W)cntA << HS);
        A(k, b) = newB | ((W)cntB << HS);
        addP(j, 2 * (cntA - oldHa));
        addP(k, 2 * (cntB - oldHb));
        if (red >= 0) {
            // The reference tests, at the first such term, the j-part before the k-part.
            const int t = red;
            if (part == 0) {
                if (F(i, t) == xia) reduce(k, t, a);
                else reduce(i, t, a);
            } else {
                if (F(i, t) == xib) reduce(j, t, b);
                else reduce(i, t, b);
            }
        }
    }

    // Uniform ordered equal pair in canonical order (component, term, partner), then
    // a uniform orientation and the flip.
    __device__ __forceinline__ bool tryFlip(bool checkReduce) {
        int c, a, b;
        if (!pickPair(c, a, b)) return false;
        int i = c, j = c == 0 ? 1 : 0, k = c == 2 ? 1 : 2;
        if (r.coin()) { int tmp = j; j = k; k = tmp; }
        flip(i, j, k, a, b, checkReduce);
        return true;
    }

    // One draw: the q-th ordered equal pair in canonical order.
    __device__ __forceinline__ bool pickPair(int &c, int &a, int &b) {
        const int Ptot = P0 + P1 + P2;
        if (Ptot <= 0) return false;
        int q = (int)r.below((uint32_t)Ptot);
        if (q < P0) c = 0;
        else if (q < P0 + P1) { c = 1; q -= P0; }
        else { c = 2; q -= P0 + P1; }
        // Term a: prefix walk over the partner counts, four terms per step
        // (loads past the last term read 0).
        const W *pc = &A(c, 0);
        // The thread-per-walk layout (SH = 5) keeps the words past the rank zero and
        // its component stride a multiple of 4, so its scans need no bounds tests (6 % faster).
        auto word = [&](int t) -> W { return (SH == 5 || t < m) ? pc[(size_t)t << sh()] : (W)0; };
        a = 0;
        for (; a < m; a += 4) {
            const int h0 = (int)(word(a) >> HS);
            const int h1 = (int)(word(a + 1) >> HS);
            const int h2 = (int)(word(a + 2) >> HS);
            const int h3 = (int)(word(a + 3) >> HS);
            const int s4 = h0 + h1 + h2 + h3;
            if (q < s4) {
                if (q < h0) break;
                q -= h0;
                if (q < h1) { a += 1; break; }
                q -= h1;
                if (q < h2) { a += 2; break; }
                q -= h2;
                a += 3;
                break;
            }
            q -= s4;
        }
        if (a >= m) { status |= ST_INTERNAL; return false; }
        // Partner b: the q-th other term (ascending) with the same factor.
        const W va = pc[(size_t)a << sh()] & FM;
        b = 0;
        for (; b < m; b += 4) {
            const bool e0 = ((word(b) & FM) == va) & (b != a);
            const bool e1 = ((word(b + 1) & FM) == va) & (b + 1 != a);
            const bool e2 = ((word(b + 2) & FM) == va) & (b + 2 != a);
            const bool e3 = ((word(b + 3) & FM) == va) & (b + 3 != a);
            const int s4 = (int)e0 + (int)e1 + (int)e2 + (int)e3;
            if (q < s4) {
                if (e0) { if (q == 0) break; q--; }
                if (e1) { if (q == 0) { b += 1; break; } q--; }
                if (e2) { if (q == 0) { b += 2; break; } q--; }
                b += 3;
                break;
            }
            q -= s4;
        }
        if (b >= m) { status |= ST_INTERNAL; return false; }
        return true;
    }

    __device__ void plus(int i, int j, int k, int p, int q, int variant) {  // scheme_z2.cu:579-612
        const W a1 = F(i, p), b1 = F(j, p), c1 = F(k, p);
        const W a2 = F(i, q), b2 = F(j, q), c2 = F(k, q);
        const W a = a1 ^ a2, b = b1 ^ b2, c = c1 ^ c2;
        if (variant == 0) { setWord(j, p, b); setWord(i, q, a); addTriplet(i, j, k, a1, b2, c); }
        else if (variant == 1) { setWord(k, p, c); setWord(j, q, b); addTriplet(i, j, k, a, b1, c2); }
        else { setWord(i, p, a); setWord(k, q, c); addTriplet(i, j, k, a2, b, c1); }
        if (!a || !b || !c) removeZeroes();
    }

    __device__ void split(int i, int j, int k, int t, W a1) {  // scheme_z2.cu:614-619
        const W a2 = F(i, t) ^ a1, bj = F(j, t), bk = F(k, t);
        setWord(i, t, a1);
        addTriplet(i, j, k, a2, bj, bk);
    }

    __device__ __forceinline__ void perm3(int &i, int &j, int &k) {
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
        while (a == b || F(0, a) == F(0, b) || F(1, a) == F(1, b) || F(2, a) == F(2, b)) {
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
        const W a2 = F(i, t);
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
        while (loop < 5 && (a == b || F(i, a) == F(i, b))) { b = (int)r.below((uint32_t)m); loop++; }
        if (loop == 5) return false;
        split(i, j, k, a, F(i, b));
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

    // tryReduce (scheme_z2.cu:1127-1154) over the equal pairs in canonical order.
    __device__ bool tryReduce() {
        for (int a = 0; a < m; a++)
            for (int b = a + 1; b < m; b++)
                if (F(0, a) == F(0, b)) {
                    if (F(1, a) == F(1, b)) { reduce(2, a, b); return true; }
                    if (F(2, a) == F(2, b)) { reduce(1, a, b); return true; }
                }
        for (int a = 0; a < m; a++)
            for (int b = a + 1; b < m; b++)
                if (F(1, a) == F(1, b) && F(2, a) == F(2, b)) { reduce(0, a, b); return true; }
        return false;
    }

    // sandwiching (scheme_z2.cu:1277-1300): every term conjugated by random invertible
    // matrices.  Conjugation is a bijection on each component, so equal factors stay equal
    // and the partner counts in the top bytes stand.
    __device__ __noinline__ void sandwich() {
        if (n0 > 16 || n1 > 16 || n2 > 16) return;  // MAX_SANDWICHING_N, config.cuh:40
        uint32_t u[16], u1[16], v[16], v1[16], w[16], w1[16];
        if (!invertible_gf2(n0, u, u1, r, status) || !invertible_gf2(n1, v, v1, r, status) ||
            !invertible_gf2(n2, w, w1, r, status))
            return;
        for (int t = 0; t < m; t++) {
            W &x0 = A(0, t), &x1 = A(1, t), &x2 = A(2, t);
            x0 = (x0 & ~FM) | (W)conj_gf2((uint64_t)(x0 & FM), u, v1, n0, n1);
            x1 = (x1 & ~FM) | (W)conj_gf2((uint64_t)(x1 & FM), v, w1, n1, n2);
            x2 = (x2 & ~FM) | (W)conj_gf2((uint64_t)(x2 & FM), w, u1, n2, n0);
        }
    }

    // swapBasis (scheme_z2.cu:1302-1313, swapBasisRows / swapBasisColumns 864-914): two
    // basis vectors trade places in U and W (rows) or V and W (columns).  A permutation of
    // entries keeps equal factors equal, so the partner counts stand.
    __device__ __noinline__ void swapBasis() {
        const bool rows = r.raw() % 2;
        const int nb = rows ? n0 : n2;
        const int a = (int)(r.raw() % (uint32_t)nb), b = (int)(r.raw() % (uint32_t)nb);
        if (a == b) return;
        // entries (i, j) of an n x k matrix sit at bit i * k + j; swapping index a and b of
        // the rows (or columns) swaps the bits of two rows (or two columns)
        auto swapRows = [](uint64_t x, int k, int p, int q) {
            const uint64_t mk = k >= 64 ? ~0ull : ((1ull << k) - 1);
            const uint64_t rp = (x >> (p * k)) & mk, rq = (x >> (q * k)) & mk;
            return (x & ~((mk << (p * k)) | (mk << (q * k)))) | (rp << (q * k)) | (rq << (p * k));
        };
        auto swapCols = [](uint64_t x, int n, int k, int p, int q) {
            for (int i = 0; i < n; i++) {
                const uint64_t bp = (x >> (i * k + p)) & 1ull, bq = (x >> (i * k + q)) & 1ull;
                x ^= (bp ^ bq) * ((1ull << (i * k + p)) | (1ull << (i * k + q)));
            }
            return x;
        };
        for (int t = 0; t < m; t++) {
            if (rows) {  // rows of U (n0 x n1) and columns of W (n2 x n0)
                W &x0 = A(0, t), &x2 = A(2, t);
                x0 = (x0 & ~FM) | (W)swapRows((uint64_t)(x0 & FM), n1, a, b);
                x2 = (x2 & ~FM) | (W)swapCols((uint64_t)(x2 & FM), n2, n0, a, b);
            } else {  // columns of V (n1 x n2) and rows of W (n2 x n0)
                W &x1 = A(1, t), &x2 = A(2, t);
                x1 = (x1 & ~FM) | (W)swapCols((uint64_t)(x1 & FM), n1, n2, a, b);
                x2 = (x2 & ~FM) | (W)swapRows((uint64_t)(x2 & FM), n0, a, b);
            }
        }
    }

    // First XOR combination inside a run of terms (findXorCombination's search order): target
    // member t, then members a < b < c < d of the run skipping t; a 4-term sum is tested before
    // the 3-term sum of its prefix, which is tested before the 2-term sum.  comb receives the
    // members then the target; returns their number (0: none).
    __device__ int gaussXor(int j, const uint16_t *run, int size, int *comb) const {
        if (size < 3) return 0;
        for (int t = 0; t < size; t++) {
            const W target = F(j, run[t]);
            for (int a = 0; a < size; a++) {
                if (a == t) continue;
                const W va = F(j, run[a]);
                for (int b = a + 1; b < size; b++) {
                    if (b == t) continue;
                    const W vb = F(j, run[b]);
                    for (int c = b + 1; c < size; c++) {
                        if (c == t) continue;
                        const W vc = F(j, run[c]);
                        for (int d = c + 1; d < size; d++) {
                            if (d == t) continue;
                            if ((va ^ vb ^ vc ^ F(j, run[d])) == target) {
                                comb[0] = run[a]; comb[1] = run[b]; comb[2] = run[c]; comb[3] = run[d]; comb[4] = run[t];
                                return 5;
                            }
                        }
                        if ((va ^ vb ^ vc) == target) {
                            comb[0] = run[a]; comb[1] = run[b]; comb[2] = run[c]; comb[3] = run[t];
                            return 4;
                        }
                    }
                    if ((va ^ vb) == target) {
                        comb[0] = run[a]; comb[1] = run[b]; comb[2] = run[t];
                        return 3;
                    }
                }
            }
        }
        return 0;
    }

    // tryReduceGauss (scheme_z2.cu:312-442,621-629,1156-1163; defined by the reference, not
    // called by its walk): for the components p in a random order (randomPermutation of 3),
    // the terms sorted by their p-factor with the reference's Shell sort (gaps 701, 301, 132,
    // 57, 23, 10, 4, 1; each sort starts from the previous order), and in each run of equal
    // p-factors a member whose factor in component p+1 (then p+2) is the XOR of 2-4 other
    // members' factors there is folded into them: its third factor is added to theirs and
    // the term removed, then zero terms are compacted.  Partner counts follow every edit.
    __device__ __noinline__ bool tryReduceGauss() {
        int perm[3] = {0, 1, 2};
        for (int q = 2; q > 0; q--) {
            const int j = (int)r.below((uint32_t)(q + 1));
            const int t = perm[q]; perm[q] = perm[j]; perm[j] = t;
        }
        uint16_t idx[kMaxRank + 2];
        for (int t = 0; t < m; t++) idx[t] = (uint16_t)t;
        int comb[5], size = 0, i = -1;
        for (int q = 0; q < 3 && i < 0; q++) {
            const int p = perm[q];
            constexpr int gaps[8] = {701, 301, 132, 57, 23, 10, 4, 1};
            for (int g = 0; g < 8; g++) {
                const int gap = gaps[g];
                if (gap > m) continue;
                for (int a = gap; a < m; a++) {
                    const uint16_t tmp = idx[a];
                    const W key = F(p, tmp);
                    int b = a;
                    while (b >= gap && F(p, idx[b - gap]) > key) {
                        idx[b] = idx[b - gap];
                        b -= gap;
                    }
                    idx[b] = tmp;
                }
            }
            int start = 0;
            for (int e = 1; e <= m && i < 0; e++) {
                if (e != m && F(p, idx[e]) == F(p, idx[start])) continue;
                if ((size = gaussXor((p + 1) % 3, idx + start, e - start, comb)) > 0) i = (p + 2) % 3;
                else if ((size = gaussXor((p + 2) % 3, idx + start, e - start, comb)) > 0) i = (p + 1) % 3;
                start = e;
            }
        }
        if (i < 0) return false;
        const int last = comb[size - 1];
        for (int q = 0; q < size - 1; q++) setWord(i, comb[q], F(i, comb[q]) ^ F(i, last));  // reduceGauss
        removeAt(last);
        removeZeroes();
        return true;
    }

    __device__ int complexity() const {
        int c = 0;
        for (int t = 0; t < m; t++) c += __popcll((uint64_t)F(0, t)) + __popcll((uint64_t)F(1, t)) + __popcll((uint64_t)F(2, t));
        return c - 2 * m - nn2;
    }
};

}  // namespace fg
