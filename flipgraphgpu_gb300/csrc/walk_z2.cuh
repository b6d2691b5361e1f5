// Z2 walk: one warp per walk, scheme and FlipSet lists in shared memory.
//
// Semantics follow the reference exactly (dronperminov/FlipGraphGPU,
// src/schemes/scheme_z2.cu and src/entities/flip_graph.cu:520-573): the same
// list order, the same compaction order, the same draw sites.  The work is
// spread over the warp: candidate scans, reduction detection, list edits and
// list rebuilds use ballots over terms (t = lane + 32*s) and list chunks.
#pragma once
#include "fg_device.cuh"

namespace fg {

template <class R, int S>
struct Z2Walk {
    uint64_t *x;  // [3][cap] shared
    uint32_t *L;  // [3][kListCap] shared
    int cap;
    int n0, n1, n2, nn0, nn1, nn2, full;  // full = n0*n1*n2
    int m;
    int sz0, sz1, sz2;
    int status;
    R &r;

    __device__ Z2Walk(R &rr) : r(rr) {}

    __device__ __forceinline__ uint64_t X(int c, int t) const { return x[c * cap + t]; }
    __device__ __forceinline__ void setX(int c, int t, uint64_t v) { x[c * cap + t] = v; }  // lane 0 only
    __device__ __forceinline__ uint32_t *list(int c) { return L + c * kListCap; }
    __device__ __forceinline__ int sz(int c) const { return c == 0 ? sz0 : (c == 1 ? sz1 : sz2); }
    __device__ __forceinline__ void setSz(int c, int v) { if (c == 0) sz0 = v; else if (c == 1) sz1 = v; else sz2 = v; }
    __device__ __forceinline__ int nn(int c) const { return c == 0 ? nn0 : (c == 1 ? nn1 : nn2); }
    __device__ __forceinline__ bool nonzero(int t) const { return X(0, t) && X(1, t) && X(2, t); }

    // ------------------------------------------------------------ structure
    // initFlips (scheme_z2.cu:141-150): all equal pairs, lexicographic, capped.
    __device__ __noinline__ void rebuild() {
        __syncwarp();
        for (int c = 0; c < 3; c++) {
            uint32_t *Lc = list(c);
            int total = 0;
#pragma unroll
            for (int s = 0; s < S; s++) {
                int t = 32 * s + lane_id();
                int cnt = 0;
                uint64_t v = t < m ? X(c, t) : 0;
                if (t < m)
                    for (int u = t + 1; u < m; u++) cnt += X(c, u) == v;
                int incl = warp_inclusive_sum(cnt);
                int pos = total + incl - cnt;
                if (t < m && cnt)
                    for (int u = t + 1; u < m; u++)
                        if (X(c, u) == v) {
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

    // removeZeroes (scheme_z2.cu:152-164); the moved term is not re-checked.
    __device__ __noinline__ void removeZeroes() {
        __syncwarp();
        int mm = m;
        if (lane_id() == 0) {
            while (mm > 0 && !nonzero(mm - 1)) mm--;
            for (int t = 0; t < mm; t++)
                if (!nonzero(t)) { mm--; moveTerm(t, mm); }
        }
        m = __shfl_sync(kFull, mm, 0);
        __syncwarp();
    }

    __device__ void removeAt(int t) {  // scheme_z2.cu:166-175
        __syncwarp();
        m--;
        if (t != m && lane_id() == 0) moveTerm(t, m);
        __syncwarp();
    }

    __device__ void addTriplet(int i, int j, int k, uint64_t a, uint64_t b, uint64_t c) {
        if (m >= cap) { status |= ST_OVERFLOW; return; }
        if (lane_id() == 0) { setX(i, m, a); setX(j, m, b); setX(k, m, c); }
        m++;
        __syncwarp();
    }

    __device__ __noinline__ void reduce(int i, int a, int b) {  // scheme_z2.cu:631-641
        uint64_t v = X(i, a) ^ X(i, b);
        __syncwarp();
        if (lane_id() == 0) setX(i, a, v);
        __syncwarp();
        removeAt(b);
        if (!v) removeZeroes();
        rebuild();
    }

    // ------------------------------------------------------------ flip
    // scheme_z2.cu:531-577.
    __device__ void flip(int i, int j, int k, int a, int b, bool checkReduce) {
        const uint64_t xja = X(j, a) ^ X(j, b);
        const uint64_t xkb = X(k, b) ^ X(k, a);
        __syncwarp();
        if (lane_id() == 0) { setX(j, a, xja); setX(k, b, xkb); }
        __syncwarp();
        setSz(j, list_remove_index(list(j), sz(j), (uint32_t)a));
        setSz(k, list_remove_index(list(k), sz(k), (uint32_t)b));
        if (!xja || !xkb) {
            removeZeroes();
            rebuild();
            return;
        }
        const uint64_t xia = X(i, a), xka = X(k, a), xib = X(i, b), xjb = X(j, b);
        unsigned eqJ[S], eqK[S];
        int found = -1;
#pragma unroll
        for (int s = 0; s < S; s++) {
            int t = 32 * s + lane_id();
            bool in = t < m;
            uint64_t vi = in ? X(i, t) : 0, vj = in ? X(j, t) : 0, vk = in ? X(k, t) : 0;
            bool eJ = in && t != a && vj == xja;
            bool eK = in && t != b && vk == xkb;
            bool red = checkReduce && ((eJ && (vi == xia || vk == xka)) || (eK && (vi == xib || vj == xjb)));
            unsigned bR = __ballot_sync(kFull, red);
            eqJ[s] = __ballot_sync(kFull, eJ);
            eqK[s] = __ballot_sync(kFull, eK);
            if (found < 0 && bR) found = 32 * s + __ffs(bR) - 1;
        }
        if (found >= 0) {
            // The first term (ascending) that triggers a reduction; at that term the
            // reference tests the j-part before the k-part.
            const int t = found;
            const uint64_t vi = X(i, t), vj = X(j, t), vk = X(k, t);
            const bool eJ = t != a && vj == xja;
            if (eJ && vi == xia) reduce(k, t, a);
            else if (eJ && vk == xka) reduce(i, t, a);
            else if (vi == xib) reduce(j, t, b);
            else reduce(i, t, b);
            return;
        }
        setSz(j, list_append<S>(list(j), sz(j), (uint32_t)a, eqJ));
        setSz(k, list_append<S>(list(k), sz(k), (uint32_t)b, eqK));
    }

    // plus (scheme_z2.cu:579-612).
    __device__ __noinline__ void plus(int i, int j, int k, int p, int q, int variant) {
        const uint64_t a1 = X(i, p), b1 = X(j, p), c1 = X(k, p);
        const uint64_t a2 = X(i, q), b2 = X(j, q), c2 = X(k, q);
        const uint64_t a = a1 ^ a2, b = b1 ^ b2, c = c1 ^ c2;
        __syncwarp();
        if (variant == 0) {
            if (lane_id() == 0) { setX(j, p, b); setX(i, q, a); }
            addTriplet(i, j, k, a1, b2, c);
        } else if (variant == 1) {
            if (lane_id() == 0) { setX(k, p, c); setX(j, q, b); }
            addTriplet(i, j, k, a, b1, c2);
        } else {
            if (lane_id() == 0) { setX(i, p, a); setX(k, q, c); }
            addTriplet(i, j, k, a2, b, c1);
        }
        __syncwarp();
        if (!a || !b || !c) removeZeroes();
        rebuild();
    }

    __device__ __noinline__ void split(int i, int j, int k, int t, uint64_t a1) {  // scheme_z2.cu:614-619
        const uint64_t a2 = X(i, t) ^ a1, bj = X(j, t), bk = X(k, t);
        __syncwarp();
        if (lane_id() == 0) setX(i, t, a1);
        addTriplet(i, j, k, a2, bj, bk);
        rebuild();
    }

    // ------------------------------------------------------------ random moves
    __device__ bool tryFlip(bool checkReduce) {  // scheme_z2.cu:982-1027
        const int size = sz0 + sz1 + sz2;
        if (!size) return false;
        int idx = (int)r.below((uint32_t)size);
        int i, j, k;
        uint32_t pr;
        if (idx < sz0) { i = 0; j = 1; k = 2; pr = list(0)[idx]; }
        else if (idx < sz0 + sz1) { i = 1; j = 0; k = 2; pr = list(1)[idx - sz0]; }
        else { i = 2; j = 0; k = 1; pr = list(2)[idx - sz0 - sz1]; }
        int a = (int)(pr >> 16), b = (int)(pr & 0xFFFFu);
        if (r.coin()) { int tmp = j; j = k; k = tmp; }
        if (r.coin()) { int tmp = a; a = b; b = tmp; }
        flip(i, j, k, a, b, checkReduce);
        return true;
    }

    __device__ __forceinline__ void perm3(int &i, int &j, int &k) {  // randomPermutation(p, 3)
        int p0 = 0, p1 = 1, p2 = 2;
        int q = (int)r.below(3);  // i = 2
        if (q == 0) { int t = p2; p2 = p0; p0 = t; } else if (q == 1) { int t = p2; p2 = p1; p1 = t; }
        q = (int)r.below(2);      // i = 1
        if (q == 0) { int t = p1; p1 = p0; p0 = t; }
        i = p0; j = p1; k = p2;
    }

    __device__ __noinline__ bool tryPlus() {  // scheme_z2.cu:1029-1050
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

    __device__ __noinline__ bool trySplit() {  // scheme_z2.cu:1052-1078
        if (m >= kMaxRank || m >= full) return false;
        int t = (int)r.below((uint32_t)m);
        int i, j, k;
        perm3(i, j, k);
        uint64_t a1 = r.mask(nn(i));
        const uint64_t a2 = X(i, t);
        int loop = 0;
        while (loop < 5 && a1 == a2) { a1 = r.mask(nn(i)); loop++; }
        if (loop == 5) return false;
        split(i, j, k, t, a1);
        return true;
    }

    __device__ __noinline__ bool trySplitExisted() {  // scheme_z2.cu:1080-1104
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

    // tryReduce (scheme_z2.cu:1127-1154): first list-0 pair sharing a second
    // factor, else first list-1 pair sharing the third; ballots over list chunks.
    __device__ __noinline__ bool tryReduce() {
        for (int base = 0; base < sz0; base += 32) {
            int p = base + lane_id();
            int hit = 0;
            if (p < sz0) {
                uint32_t pr = list(0)[p];
                int a = (int)(pr >> 16), b = (int)(pr & 0xFFFFu);
                hit = X(1, a) == X(1, b) ? 1 : (X(2, a) == X(2, b) ? 2 : 0);
            }
            unsigned bm = __ballot_sync(kFull, hit != 0);
            if (bm) {
                int src = __ffs(bm) - 1;
                int h = __shfl_sync(kFull, hit, src);
                uint32_t pr = list(0)[base + src];
                reduce(h == 1 ? 2 : 1, (int)(pr >> 16), (int)(pr & 0xFFFFu));
                return true;
            }
        }
        for (int base = 0; base < sz1; base += 32) {
            int p = base + lane_id();
            bool hit = false;
            if (p < sz1) {
                uint32_t pr = list(1)[p];
                hit = X(2, pr >> 16) == X(2, pr & 0xFFFFu);
            }
            unsigned bm = __ballot_sync(kFull, hit);
            if (bm) {
                uint32_t pr = list(1)[base + __ffs(bm) - 1];
                reduce(0, (int)(pr >> 16), (int)(pr & 0xFFFFu));
                return true;
            }
        }
        return false;
    }

    // ------------------------------------------------------------ Gauss (XOR) reduction
    // tryReduceGauss (scheme_z2.cu:312-442,621-629,1156-1163), which the reference defines
    // but never calls.  For the components p in a random order, the term indices are
    // sorted by their p-factor with the reference's Shell sort (gaps 701 ... 1; not
    // stable, and each sort starts from the previous order, so the order inside a run of
    // equal factors is the reference's); in each run, a member whose factor in component
    // p+1 (then p+2) is the XOR of 2, 3 or 4 other members' factors there is folded into
    // them (its third factor is added to theirs) and removed.  The search is serial on
    // lane 0 (a rare move); the draws are the lanes' replicated stream.  Unlike the
    // reference, zero terms are then removed and the lists rebuilt, as a walk needs.
    __device__ int gaussXor(int j, const int *run, int size, int *comb) const {
        if (size < 3) return 0;
        for (int t = 0; t < size; t++) {
            const uint64_t target = X(j, run[t]);
            for (int a = 0; a < size; a++) {
                if (a == t) continue;
                const uint64_t va = X(j, run[a]);
                for (int b = a + 1; b < size; b++) {
                    if (b == t) continue;
                    const uint64_t vb = X(j, run[b]);
                    for (int c = b + 1; c < size; c++) {
                        if (c == t) continue;
                        const uint64_t vc = X(j, run[c]);
                        for (int d = c + 1; d < size; d++) {
                            if (d == t) continue;
                            if ((va ^ vb ^ vc ^ X(j, run[d])) == target) {
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

    __device__ __noinline__ bool tryReduceGauss() {
        int perm[3];
        perm3(perm[0], perm[1], perm[2]);
        int comp = -1, size = 0, comb[5] = {0, 0, 0, 0, 0};
        if (lane_id() == 0) {
            constexpr int gaps[8] = {701, 301, 132, 57, 23, 10, 4, 1};
            int idx[kMaxRank + 2];
            const int mm = m < kMaxRank + 2 ? m : kMaxRank + 2;
            for (int t = 0; t < mm; t++) idx[t] = t;
            for (int q = 0; q < 3 && comp < 0; q++) {
                const int p = perm[q];
                for (int g = 0; g < 8; g++) {
                    const int gap = gaps[g];
                    if (gap > mm) continue;
                    for (int i = gap; i < mm; i++) {
                        const int tmp = idx[i];
                        const uint64_t v = X(p, tmp);
                        int k = i;
                        while (k >= gap && X(p, idx[k - gap]) > v) {
                            idx[k] = idx[k - gap];
                            k -= gap;
                        }
                        idx[k] = tmp;
                    }
                }
                int start = 0;
                for (int e = 1; e <= mm && comp < 0; e++) {
                    if (e != mm && X(p, idx[e]) == X(p, idx[start])) continue;
                    if ((size = gaussXor((p + 1) % 3, idx + start, e - start, comb)) > 0) comp = (p + 2) % 3;
                    else if ((size = gaussXor((p + 2) % 3, idx + start, e - start, comb)) > 0) comp = (p + 1) % 3;
                    start = e;
                }
            }
        }
        comp = __shfl_sync(kFull, comp, 0);
        if (comp < 0) return false;
        size = __shfl_sync(kFull, size, 0);
        const int last = __shfl_sync(kFull, comb[size - 1 < 0 ? 0 : size - 1], 0);
        __syncwarp();
        if (lane_id() == 0)
            for (int q = 0; q < size - 1; q++) setX(comp, comb[q], X(comp, comb[q]) ^ X(comp, last));
        __syncwarp();
        removeAt(last);
        removeZeroes();
        rebuild();
        return true;
    }
};

}  // namespace fg
