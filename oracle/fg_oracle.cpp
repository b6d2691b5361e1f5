// CPU oracle for the flip-graph hot path -- TEST INFRASTRUCTURE ONLY.
//
// Restates, operation for operation, the reference's search-path algorithms
// (dronperminov/FlipGraphGPU; citations are path:line in that project):
//   FlipSet                      src/entities/flip_set.cu:1-43
//   SchemeZ2 walk algebra        src/schemes/scheme_z2.cu:3-182,531-641,982-1154
//   Addition (ternary vector)    src/entities/addition.cu:1-232
//   SchemeInteger walk algebra   src/schemes/scheme_integer.cu:3-147,229-269,398-571,907-1101
//   randint / randomPermutation  src/utils/random.cuh:5-22
//   randomWalkKernel             src/entities/flip_graph.cu:520-573
//   minimizeKernel               src/entities/complexity_minimizer.cu:190-214
//   AdditionsReducer / PairsCounter / runReducersKernel
//                                src/entities/additions_reducer.cuh, pairs_counter.cuh,
//                                src/entities/scheme_additions_reducer.cu:463-540
// It is the checker of the CUDA library, never the thing measured or shipped.
//
// Draws come from a policy object: RefDraws replays a recorded cuRAND XORWOW
// tape (curand() words and curand_uniform() floats recorded on the GPU), and
// reproduces the reference's stream; FastDraws is the library's fast-mode
// stream (Philox4x32-10, Salmon et al. SC'11) with cheaper draw sites:
// multiply-high instead of modulo, integer thresholds instead of float gates,
// and no draw for a gate whose probability is zero.  Control flow is the
// same for both, so one implementation serves both modes.
//
// The reference's unbounded retry loops (scheme_z2.cu:1036, scheme_integer.cu:984,1029)
// are bounded by kRetryCap; hitting it sets status bit 2 (the reference would hang).
#include "fg_oracle.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

namespace {

constexpr int kMaxRank = 350;   // config.cuh:10
constexpr int kMaxPairs = 500;  // config.cuh:14
constexpr int kRetryCap = 1 << 20;
inline int retry_cap(const fgo_walk_cfg *cfg) { return cfg->retry_cap > 0 ? cfg->retry_cap : kRetryCap; }
constexpr int kMaxMatrix = 64;      // config.cuh:11 (64-bit factors)
constexpr int kMaxExtensionN = 16;  // config.cuh:37
enum { ST_TAPE = 1, ST_RETRY = 2, ST_OVERFLOW = 4 };

// Ternary sandwiching on (fgo_walk_cfg::zt_sandwich): set for the duration of one fgo_walk call.
int g_ternarySandwich = 0;

inline int popc64(uint64_t x) { return __builtin_popcountll(x); }

// ------------------------------------------------------------ Philox4x32-10
void philox(const uint32_t c_in[4], const uint32_t k_in[2], uint32_t out[4]) {
    uint32_t c0 = c_in[0], c1 = c_in[1], c2 = c_in[2], c3 = c_in[3];
    uint32_t k0 = k_in[0], k1 = k_in[1];
    for (int r = 0; r < 10; r++) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// ------------------------------------------------------------ draw policies
struct RefDraws {
    const uint32_t *d = nullptr;
    const float *u = nullptr;
    int64_t n = 0, pos = 0;
    int32_t *status = nullptr;
    uint32_t raw() {
        if (pos >= n) { *status |= ST_TAPE; return 0; }
        return d[pos++];
    }
    float uniform() {
        if (pos >= n) { *status |= ST_TAPE; return 1.0f; }
        return u[pos++];
    }
    uint32_t below(uint32_t k) { return raw() % k; }             // curand() % k
    bool coin() { return raw() % 2; }                              // curand() % 2
    // curand_uniform(&state) * maxIterations < p   (flip_graph.cu:550-562)
    bool gate(double p, int iters) { float x = uniform(); return (double)(x * (float)iters) < p; }
    bool tie() { return (double)uniform() < 0.01; }              // flip_graph.cu:545
    uint64_t mask(int nn) { return (uint64_t)raw() % ((uint64_t)1 << nn); }  // scheme_z2.cu:1064
};

// Fast-mode stream: word q of walk w is Philox(ctr = (q/4 lo, q/4 hi, w, 0), key = seed)[q%4].
struct FastDraws {
    uint32_t key[2] = {0, 0};
    uint32_t walk = 0;
    int64_t pos = 0;
    int64_t cached = -1;
    uint32_t block[4];
    int32_t *status = nullptr;
    uint32_t raw() {
        int64_t b = pos >> 2;
        if (b != cached) {
            uint32_t c[4] = {(uint32_t)b, (uint32_t)((uint64_t)b >> 32), walk, 0u};
            philox(c, key, block);
            cached = b;
        }
        return block[pos++ & 3];
    }
    float uniform() { return (float)(raw() >> 8) * (1.0f / 16777216.0f); }
    uint32_t below(uint32_t k) { return (uint32_t)(((uint64_t)raw() * k) >> 32); }
    bool coin() { return raw() >> 31; }
    bool gate(double p, int iters) {
        if (!(p > 0)) return false;  // can never fire: no draw
        double q = p / (double)iters;
        uint64_t t = q >= 1.0 ? ((uint64_t)1 << 32) : (uint64_t)(q * 4294967296.0);
        return (uint64_t)raw() < t;
    }
    bool tie() { return raw() < 42949672u; }  // floor(0.01 * 2^32)
    uint64_t mask(int nn) { return nn >= 32 ? (uint64_t)raw() : (uint64_t)(raw() & ((1u << nn) - 1u)); }
};

template <class R> inline int randint(int a, int b, R &r) { return a + (int)r.below((uint32_t)(b - a + 1)); }

template <class R> inline void permutation(int *p, int n, R &r) {  // random.cuh:9-22
    for (int i = 0; i < n; i++) p[i] = i;
    for (int i = n - 1; i > 0; i--) {
        int j = (int)r.below((uint32_t)(i + 1));
        std::swap(p[i], p[j]);
    }
}

// ------------------------------------------------------------ FlipSet
struct FlipList {
    int size = 0;
    uint32_t pairs[kMaxPairs];
    void clear() { size = 0; }
    void add(uint32_t a, uint32_t b) {  // flip_set.cu:7-13: silently full at 500
        if (size >= kMaxPairs) return;
        pairs[size++] = (a << 16) | b;
    }
    void removeIndex(uint32_t idx) {  // flip_set.cu:27-31
        for (int p = 0; p < size; p++)
            if ((pairs[p] >> 16) == idx || (pairs[p] & 0xFFFFu) == idx) {
                pairs[p] = pairs[--size];
                p--;
            }
    }
    int first(int p) const { return (int)(pairs[p] >> 16); }
    int second(int p) const { return (int)(pairs[p] & 0xFFFFu); }
};

// ------------------------------------------------------------ Z2 scheme
struct Z2 {
    int n[3], nn[3], m;
    uint64_t x[3][kMaxRank];
    FlipList lists[3];
    int32_t *status;
    int retryCap = kRetryCap;  // fgo_walk_cfg::retry_cap (0 there = kRetryCap)
    int slotCap = kMaxRank;    // the records' slots per walk (fgo_walk_cfg::cap)
    int maxMatrix = kMaxMatrix;  // resizing: most entries of a grown factor (56 in the fast mode)
    // Implicit pair enumeration (the library's fast mode): no FlipSet lists;
    // a flip samples an ordered equal-factor pair uniformly in the canonical
    // order (component c, term t ascending, partner t' ascending).
    bool implicit = false;

    bool nonzero(int t) const { return x[0][t] && x[1][t] && x[2][t]; }

    void initNaive(int n1, int n2, int n3) {  // scheme_z2.cu:32-55
        n[0] = n1; n[1] = n2; n[2] = n3;
        nn[0] = n1 * n2; nn[1] = n2 * n3; nn[2] = n3 * n1;
        m = n1 * n2 * n3;
        for (int i = 0; i < n1; i++)
            for (int j = 0; j < n3; j++)
                for (int k = 0; k < n2; k++) {
                    int t = (i * n3 + j) * n2 + k;
                    x[0][t] = (uint64_t)1 << (i * n2 + k);
                    x[1][t] = (uint64_t)1 << (k * n3 + j);
                    x[2][t] = (uint64_t)1 << (j * n1 + i);
                }
        rebuildLists();
    }

    void rebuildLists() {  // initFlips, scheme_z2.cu:141-150
        for (int c = 0; c < 3; c++) {
            lists[c].clear();
            if (implicit) continue;
            for (int a = 0; a < m; a++)
                for (int b = a + 1; b < m; b++)
                    if (x[c][a] == x[c][b]) lists[c].add(a, b);
        }
    }

    int partners(int c, int t) const {
        int k = 0;
        for (int u = 0; u < m; u++) k += u != t && x[c][u] == x[c][t];
        return k;
    }

    // Fast-mode flip proposal: q uniform over the ordered equal pairs, located in
    // canonical order; the orientation of the pair comes from the ordering, one
    // coin orients (j, k) as in the reference.
    template <class R> bool tryFlipImplicit(R &r, bool checkReduce) {
        int total[3] = {0, 0, 0};
        for (int c = 0; c < 3; c++)
            for (int t = 0; t < m; t++) total[c] += partners(c, t);
        uint32_t P = (uint32_t)(total[0] + total[1] + total[2]);
        if (!P) return false;
        uint32_t q = r.below(P);
        int c = 0;
        while (q >= (uint32_t)total[c]) { q -= total[c]; c++; }
        int a = 0;
        for (;; a++) {
            uint32_t h = (uint32_t)partners(c, a);
            if (q < h) break;
            q -= h;
        }
        int b = 0;
        for (;; b++)
            if (b != a && x[c][b] == x[c][a]) {
                if (q == 0) break;
                q--;
            }
        int i = c, j = c == 0 ? 1 : 0, k = c == 2 ? 1 : 2;
        if (r.coin()) std::swap(j, k);
        flip(i, j, k, a, b, checkReduce);
        return true;
    }

    void moveTerm(int dst, int src) { for (int c = 0; c < 3; c++) x[c][dst] = x[c][src]; }

    void removeZeroes() {  // scheme_z2.cu:152-164 (no re-check of the moved term)
        while (m > 0 && !nonzero(m - 1)) m--;
        for (int t = 0; t < m; t++)
            if (!nonzero(t)) { m--; moveTerm(t, m); }
    }

    void removeAt(int t) {  // scheme_z2.cu:166-175
        m--;
        if (t == m) return;
        moveTerm(t, m);
    }

    void addTriplet(int i, int j, int k, uint64_t a, uint64_t b, uint64_t c) {  // scheme_z2.cu:177-182
        if (m >= kMaxRank || m >= slotCap) { *status |= ST_OVERFLOW; return; }
        x[i][m] = a; x[j][m] = b; x[k][m] = c;
        m++;
    }

    void reduce(int i, int a, int b) {  // scheme_z2.cu:631-641
        x[i][a] ^= x[i][b];
        bool zero = !x[i][a];
        removeAt(b);
        if (zero) removeZeroes();
        rebuildLists();
    }

    void flip(int i, int j, int k, int a, int b, bool checkReduce) {  // scheme_z2.cu:531-577
        x[j][a] ^= x[j][b];
        x[k][b] ^= x[k][a];
        lists[j].removeIndex(a);
        lists[k].removeIndex(b);
        if (!x[j][a] || !x[k][b]) {
            removeZeroes();
            rebuildLists();
            return;
        }
        for (int t = 0; t < m; t++) {
            if (t != a && x[j][t] == x[j][a]) {
                if (checkReduce) {
                    if (x[i][t] == x[i][a]) { reduce(k, t, a); return; }
                    if (x[k][t] == x[k][a]) { reduce(i, t, a); return; }
                }
                if (!implicit) lists[j].add(a, t);
            }
            if (t != b && x[k][t] == x[k][b]) {
                if (checkReduce) {
                    if (x[i][t] == x[i][b]) { reduce(j, t, b); return; }
                    if (x[j][t] == x[j][b]) { reduce(i, t, b); return; }
                }
                if (!implicit) lists[k].add(b, t);
            }
        }
    }

    void plus(int i, int j, int k, int p, int q, int variant) {  // scheme_z2.cu:579-612
        const uint64_t a1 = x[i][p], b1 = x[j][p], c1 = x[k][p];
        const uint64_t a2 = x[i][q], b2 = x[j][q], c2 = x[k][q];
        const uint64_t a = a1 ^ a2, b = b1 ^ b2, c = c1 ^ c2;
        if (variant == 0) { x[j][p] = b; x[i][q] = a; addTriplet(i, j, k, a1, b2, c); }
        else if (variant == 1) { x[k][p] = c; x[j][q] = b; addTriplet(i, j, k, a, b1, c2); }
        else { x[i][p] = a; x[k][q] = c; addTriplet(i, j, k, a2, b, c1); }
        if (!a || !b || !c) removeZeroes();
        rebuildLists();
    }

    void split(int i, int j, int k, int t, uint64_t a1) {  // scheme_z2.cu:614-619
        uint64_t a2 = x[i][t] ^ a1;
        x[i][t] = a1;
        addTriplet(i, j, k, a2, x[j][t], x[k][t]);
        rebuildLists();
    }

    template <class R> bool tryFlip(R &r, bool checkReduce) {  // scheme_z2.cu:982-1027
        if (implicit) return tryFlipImplicit(r, checkReduce);
        int size = lists[0].size + lists[1].size + lists[2].size;
        if (!size) return false;
        int idx = (int)r.below((uint32_t)size);
        int i, j, k, a, b;
        if (idx < lists[0].size) { i = 0; j = 1; k = 2; a = lists[0].first(idx); b = lists[0].second(idx); }
        else if (idx < lists[0].size + lists[1].size) {
            idx -= lists[0].size; i = 1; j = 0; k = 2; a = lists[1].first(idx); b = lists[1].second(idx);
        } else {
            idx -= lists[0].size + lists[1].size; i = 2; j = 0; k = 1; a = lists[2].first(idx); b = lists[2].second(idx);
        }
        if (r.coin()) std::swap(j, k);
        if (r.coin()) std::swap(a, b);
        flip(i, j, k, a, b, checkReduce);
        return true;
    }

    template <class R> bool tryPlus(R &r) {  // scheme_z2.cu:1029-1050
        if (m >= kMaxRank || m >= n[0] * n[1] * n[2]) return false;
        int a = (int)r.below(m), b = (int)r.below(m);
        int guard = 0;
        while (a == b || x[0][a] == x[0][b] || x[1][a] == x[1][b] || x[2][a] == x[2][b]) {
            if (++guard > retryCap) { *status |= ST_RETRY; return false; }
            a = (int)r.below(m);
            b = (int)r.below(m);
        }
        int perm[3];
        permutation(perm, 3, r);
        int variant = (int)r.below(3);
        plus(perm[0], perm[1], perm[2], a, b, variant);
        return true;
    }

    template <class R> bool trySplit(R &r) {  // scheme_z2.cu:1052-1078
        if (m >= kMaxRank || m >= n[0] * n[1] * n[2]) return false;
        int t = (int)r.below(m);
        int perm[3];
        permutation(perm, 3, r);
        int i = perm[0], j = perm[1], k = perm[2];
        uint64_t a1 = r.mask(nn[i]);
        const uint64_t a2 = x[i][t];
        int loop = 0;
        while (loop < 5 && a1 == a2) { a1 = r.mask(nn[i]); loop++; }
        if (loop == 5) return false;
        split(i, j, k, t, a1);
        return true;
    }

    template <class R> bool trySplitExisted(R &r) {  // scheme_z2.cu:1080-1104
        if (m >= kMaxRank || m >= n[0] * n[1] * n[2]) return false;
        int perm[3];
        permutation(perm, 3, r);
        int i = perm[0], j = perm[1], k = perm[2];
        int a = (int)r.below(m), b = (int)r.below(m);
        int loop = 0;
        while (loop < 5 && (a == b || x[i][a] == x[i][b])) { b = (int)r.below(m); loop++; }
        if (loop == 5) return false;
        split(i, j, k, a, x[i][b]);
        return true;
    }

    template <class R> bool tryExpand(int count, R &r) {  // scheme_z2.cu:1106-1125
        int maxRank = n[0] * n[1] * n[2];
        bool result = false;
        for (int q = 0; q < count && m < maxRank; q++) {
            int v = (int)r.below(3);
            if (v == 0) result |= tryPlus(r);
            else if (v == 1) result |= trySplit(r);
            else result |= trySplitExisted(r);
        }
        return result;
    }

    bool tryReduce() {  // scheme_z2.cu:1127-1154
        if (implicit) {  // same tests over the equal pairs in canonical order
            for (int a = 0; a < m; a++)
                for (int b = a + 1; b < m; b++)
                    if (x[0][a] == x[0][b]) {
                        if (x[1][a] == x[1][b]) { reduce(2, a, b); return true; }
                        if (x[2][a] == x[2][b]) { reduce(1, a, b); return true; }
                    }
            for (int a = 0; a < m; a++)
                for (int b = a + 1; b < m; b++)
                    if (x[1][a] == x[1][b] && x[2][a] == x[2][b]) { reduce(0, a, b); return true; }
            return false;
        }
        for (int p = 0; p < lists[0].size; p++) {
            int a = lists[0].first(p), b = lists[0].second(p);
            if (x[1][a] == x[1][b]) { reduce(2, a, b); return true; }
            if (x[2][a] == x[2][b]) { reduce(1, a, b); return true; }
        }
        for (int p = 0; p < lists[1].size; p++) {
            int a = lists[1].first(p), b = lists[1].second(p);
            if (x[2][a] == x[2][b]) { reduce(0, a, b); return true; }
        }
        return false;
    }

    // ---------------------------------------------------------------- Gauss (XOR) reduction
    // tryReduceGauss (scheme_z2.cu:312-442,621-629,1156-1163), defined but never called by the
    // reference.  For components p in a random order, the terms are sorted by their p-factor
    // with the reference's Shell sort (gaps 701, 301, 132, 57, 23, 10, 4, 1; not stable, so the
    // order inside a run of equal factors follows it exactly); in each run, a member whose
    // factor in component j = p+1 (then p+2) is the XOR of 2, 3 or 4 other members' factors
    // there is folded into them: its third factor (component i) is added to theirs and the
    // term is removed, one rank less.  The reference leaves zero factors and the FlipSets as
    // they are; `cleanup` (the walk's use) removes zero terms and rebuilds the lists.
    static void shellSort(int *idx, const uint64_t *v, int count) {
        static const int gaps[8] = {701, 301, 132, 57, 23, 10, 4, 1};
        for (int g = 0; g < 8; g++) {
            const int gap = gaps[g];
            if (gap > count) continue;
            for (int i = gap; i < count; i++) {
                const int tmp = idx[i];
                int j = i;
                while (j >= gap && v[idx[j - gap]] > v[tmp]) {
                    idx[j] = idx[j - gap];
                    j -= gap;
                }
                idx[j] = tmp;
            }
        }
    }
    // First combination (search order of findXorCombination): target member t, then members
    // a < b < c < d (indices into the run) skipping t; 4-term sums are tested before the
    // 3-term sum of the same prefix, which is tested before the 2-term sum.
    int findXor(int j, const int *run, int size, int *comb) const {
        if (size < 3) return 0;
        for (int t = 0; t < size; t++) {
            const uint64_t target = x[j][run[t]];
            for (int a = 0; a < size; a++) {
                if (a == t) continue;
                const uint64_t va = x[j][run[a]];
                for (int b = a + 1; b < size; b++) {
                    if (b == t) continue;
                    const uint64_t vb = x[j][run[b]];
                    for (int c = b + 1; c < size; c++) {
                        if (c == t) continue;
                        const uint64_t vc = x[j][run[c]];
                        for (int d = c + 1; d < size; d++) {
                            if (d == t) continue;
                            if ((va ^ vb ^ vc ^ x[j][run[d]]) == target) {
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
    template <class R> bool tryReduceGauss(R &r, bool cleanup) {
        int perm[3];
        permutation(perm, 3, r);
        int idx[kMaxRank], comb[5];
        int i = -1, size = 0;
        for (int t = 0; t < m; t++) idx[t] = t;  // once: each sort starts from the previous order
        for (int q = 0; q < 3 && i < 0; q++) {
            const int p = perm[q];
            shellSort(idx, x[p], m);
            int start = 0;
            for (int e = 1; e <= m && i < 0; e++) {
                if (e != m && x[p][idx[e]] == x[p][idx[start]]) continue;
                if ((size = findXor((p + 1) % 3, idx + start, e - start, comb)) > 0) i = (p + 2) % 3;
                else if ((size = findXor((p + 2) % 3, idx + start, e - start, comb)) > 0) i = (p + 1) % 3;
                start = e;
            }
        }
        if (i < 0) return false;
        const int last = comb[size - 1];
        for (int q = 0; q < size - 1; q++) x[i][comb[q]] ^= x[i][last];  // reduceGauss, scheme_z2.cu:621-629
        removeAt(last);
        if (cleanup) {
            removeZeroes();
            rebuildLists();
        }
        return true;
    }

    int complexity() const {  // scheme_z2.cu:127-139
        int count = 0;
        for (int t = 0; t < m; t++)
            for (int c = 0; c < 3; c++) count += popc64(x[c][t]);
        return count - 2 * m - nn[2];
    }

    // ---------------------------------------------------------------- basis moves
    // Random invertible n x n matrix over GF(2) and its inverse (scheme_z2.cu:444-492,
    // random.cuh:24-32): row i = the low n bits of one draw, redrawn until Gauss-Jordan
    // elimination of [M | I] finds every pivot.  Rows are bit masks (entry (i, j) = bit j).
    template <class R> bool invertibleMatrix(int n_, uint32_t *mrow, uint32_t *inv, R &r) {
        const uint32_t low = n_ >= 32 ? 0xFFFFFFFFu : ((1u << n_) - 1u);
        for (int guard = 0; guard <= retryCap; guard++) {
            for (int i = 0; i < n_; i++) mrow[i] = r.raw() & low;
            uint64_t aug[16];
            for (int i = 0; i < n_; i++) aug[i] = (uint64_t)mrow[i] | ((uint64_t)1 << (n_ + i));
            bool ok = true;
            for (int col = 0; col < n_ && ok; col++) {
                int piv = -1;
                for (int row = col; row < n_; row++)
                    if ((aug[row] >> col) & 1) { piv = row; break; }
                if (piv < 0) { ok = false; break; }
                std::swap(aug[col], aug[piv]);
                for (int row = 0; row < n_; row++)
                    if (row != col && ((aug[row] >> col) & 1)) aug[row] ^= aug[col];
            }
            if (!ok) continue;
            for (int i = 0; i < n_; i++) inv[i] = (uint32_t)(aug[i] >> n_) & low;
            return true;
        }
        *status |= ST_RETRY;
        return false;
    }
    // left (n1 x n1) * X (n1 x n2, bit i*n2+j) * right (n2 x n2), over GF(2) (scheme_z2.cu:494-529)
    static uint64_t conj(uint64_t x, const uint32_t *left, const uint32_t *right, int n1, int n2) {
        const uint64_t rowMask = n2 >= 64 ? ~0ull : ((1ull << n2) - 1);
        uint64_t out = 0;
        for (int i = 0; i < n1; i++) {
            uint64_t r1 = 0;  // row i of left * X
            for (int k = 0; k < n1; k++)
                if ((left[i] >> k) & 1) r1 ^= (x >> (k * n2)) & rowMask;
            uint64_t r2 = 0;  // row i of (left * X) * right
            for (int k = 0; k < n2; k++)
                if ((r1 >> k) & 1) r2 ^= right[k];
            out |= (r2 & rowMask) << (i * n2);
        }
        return out;
    }
    template <class R> void sandwiching(R &r) {  // scheme_z2.cu:1277-1300
        // The reference sizes its matrices for n <= 16 (config.cuh:40, MAX_SANDWICHING_N);
        // larger sizes overrun them there and are skipped here.
        if (n[0] > 16 || n[1] > 16 || n[2] > 16) return;
        uint32_t u[16], u1[16], v[16], v1[16], w[16], w1[16];
        if (!invertibleMatrix(n[0], u, u1, r) || !invertibleMatrix(n[1], v, v1, r) || !invertibleMatrix(n[2], w, w1, r))
            return;
        for (int t = 0; t < m; t++) {
            x[0][t] = conj(x[0][t], u, v1, n[0], n[1]);
            x[1][t] = conj(x[1][t], v, w1, n[1], n[2]);
            x[2][t] = conj(x[2][t], w, u1, n[2], n[0]);
        }
        rebuildLists();
    }
    // swapBasisRows / swapBasisColumns (scheme_z2.cu:864-914): two basis vectors trade places.
    void swapBasisRows(int i1, int i2) {
        int rows[64];
        for (int q = 0; q < n[0]; q++) rows[q] = q;
        rows[i1] = i2;
        rows[i2] = i1;
        for (int t = 0; t < m; t++) {
            uint64_t u = 0, w = 0;
            for (int i = 0; i < n[0]; i++)
                for (int j = 0; j < n[1]; j++) u |= ((x[0][t] >> (rows[i] * n[1] + j)) & 1ull) << (i * n[1] + j);
            for (int i = 0; i < n[2]; i++)
                for (int j = 0; j < n[0]; j++) w |= ((x[2][t] >> (i * n[0] + rows[j])) & 1ull) << (i * n[0] + j);
            x[0][t] = u;
            x[2][t] = w;
        }
    }
    void swapBasisColumns(int j1, int j2) {
        int cols[64];
        for (int q = 0; q < n[2]; q++) cols[q] = q;
        cols[j1] = j2;
        cols[j2] = j1;
        for (int t = 0; t < m; t++) {
            uint64_t v = 0, w = 0;
            for (int i = 0; i < n[1]; i++)
                for (int j = 0; j < n[2]; j++) v |= ((x[1][t] >> (i * n[2] + cols[j])) & 1ull) << (i * n[2] + j);
            for (int i = 0; i < n[2]; i++)
                for (int j = 0; j < n[0]; j++) w |= ((x[2][t] >> (cols[i] * n[0] + j)) & 1ull) << (i * n[0] + j);
            x[1][t] = v;
            x[2][t] = w;
        }
    }
    template <class R> void swapBasis(R &r) {  // scheme_z2.cu:1302-1313 (lists stay valid)
        if (r.raw() % 2) {
            const int i1 = (int)(r.raw() % (uint32_t)n[0]), i2 = (int)(r.raw() % (uint32_t)n[0]);
            swapBasisRows(i1, i2);
        } else {
            const int j1 = (int)(r.raw() % (uint32_t)n[2]), j2 = (int)(r.raw() % (uint32_t)n[2]);
            swapBasisColumns(j1, j2);
        }
    }

    // ---------------------------------------------------------------- resize
    // Meta-operators that change the matrix sizes (scheme_z2.cu:184-310,
    // 643-979, 1165-1275).  Matrix c is n[c] x n[c+1] (W transposed), entry
    // (i, j) at bit i * n[c+1] + j.
    void setN(int a, int b, int c) {
        n[0] = a; n[1] = b; n[2] = c;
        for (int q = 0; q < 3; q++) nn[q] = n[q] * n[(q + 1) % 3];
    }
    static uint64_t bit(uint64_t v, int k) { return (v >> k) & 1ull; }

    void excludeRow(int c, int row) {  // scheme_z2.cu:205-224
        const int r = n[c], cols = n[(c + 1) % 3];
        for (int t = 0; t < m; t++) {
            uint64_t v = 0;
            for (int i = 0, i2 = 0; i < r; i++) {
                if (i == row) continue;
                for (int j = 0; j < cols; j++) v |= bit(x[c][t], i * cols + j) << (i2 * cols + j);
                i2++;
            }
            x[c][t] = v;
        }
    }
    void excludeColumn(int c, int col) {  // scheme_z2.cu:184-203
        const int r = n[c], cols = n[(c + 1) % 3];
        for (int t = 0; t < m; t++) {
            uint64_t v = 0;
            for (int i = 0; i < r; i++)
                for (int j = 0, j2 = 0; j < cols; j++) {
                    if (j == col) continue;
                    v |= bit(x[c][t], i * cols + j) << (i * (cols - 1) + j2);
                    j2++;
                }
            x[c][t] = v;
        }
    }
    void addColumn(int c) {  // scheme_z2.cu:226-239 (addRow, 241-254, leaves the bits in place)
        const int r = n[c], cols = n[(c + 1) % 3];
        for (int t = 0; t < m; t++) {
            uint64_t v = 0;
            for (int i = 0; i < r; i++)
                for (int j = 0; j < cols; j++) v |= bit(x[c][t], i * cols + j) << (i * (cols + 1) + j);
            x[c][t] = v;
        }
    }

    bool isValidProject(int i, int minN) const {  // scheme_z2.cu:256-258
        return n[i] - 1 >= minN && n[(i + 1) % 3] >= minN && n[(i + 2) % 3] >= minN;
    }
    bool isValidGrown(const int g[3], int extraRank, int maxN) const {  // scheme_z2.cu:260-294
        if (extraRank > kMaxRank) return false;
        for (int q = 0; q < 3; q++)
            if (g[q] * g[(q + 1) % 3] > maxMatrix || g[q] > maxN) return false;
        return true;
    }
    bool isValidExtension(int i, int maxN) const {
        int g[3] = {n[0], n[1], n[2]};
        g[i] += 1;
        return isValidGrown(g, m + g[(i + 1) % 3] * g[(i + 2) % 3], maxN);
    }
    bool isValidProduct(int i, int maxN) const {
        int g[3] = {n[0], n[1], n[2]};
        g[i] *= 2;
        return isValidGrown(g, m * 2, maxN);
    }

    void project(int p, int q) {  // scheme_z2.cu:643-653
        excludeRow(p, q);
        excludeColumn((p + 2) % 3, q);
        int g[3] = {n[0], n[1], n[2]};
        g[p]--;
        setN(g[0], g[1], g[2]);
        removeZeroes();
        rebuildLists();
    }

    void extend(int p) {  // scheme_z2.cu:655-687 (terms added with the old sizes)
        const int a = n[0], b = n[1], c = n[2];
        if (p == 0) {
            addColumn(2);
            for (int i = 0; i < c; i++)
                for (int j = 0; j < b; j++)
                    addTriplet(0, 1, 2, 1ull << (a * b + j), 1ull << (j * c + i), 1ull << (i * (a + 1) + a));
        } else if (p == 1) {
            addColumn(0);
            for (int i = 0; i < a; i++)
                for (int j = 0; j < c; j++)
                    addTriplet(0, 1, 2, 1ull << (i * (b + 1) + b), 1ull << (b * c + j), 1ull << (j * a + i));
        } else {
            addColumn(1);
            for (int i = 0; i < a; i++)
                for (int j = 0; j < b; j++)
                    addTriplet(0, 1, 2, 1ull << (i * b + j), 1ull << (j * (c + 1) + c), 1ull << (c * a + i));
        }
        int g[3] = {a, b, c};
        g[p]++;
        setN(g[0], g[1], g[2]);
        rebuildLists();
    }

    // Copies of a term's three matrices placed at block offsets (d0, d1, d2) of
    // new sizes g: matrix c entry (i, j) -> (i + d[c], j + d[c+1]).
    static uint64_t place(uint64_t v, int rows, int cols, int newCols, int di, int dj) {
        uint64_t o = 0;
        for (int i = 0; i < rows; i++)
            for (int j = 0; j < cols; j++) o |= bit(v, i * cols + j) << ((i + di) * newCols + j + dj);
        return o;
    }

    void product(int p) {  // scheme_z2.cu:689-747: block-diagonal doubling of size p
        int g[3] = {n[0], n[1], n[2]}, d[3];
        g[p] *= 2;
        for (int q = 0; q < 3; q++) d[q] = q == p ? n[q] : 0;
        for (int t = 0; t < m; t++)
            for (int c = 0; c < 3; c++) {
                const int c1 = (c + 1) % 3;
                const uint64_t v = x[c][t];
                x[c][t] = place(v, n[c], n[c1], g[c1], 0, 0);
                x[c][t + m] = place(v, n[c], n[c1], g[c1], d[c], d[c1]);
            }
        m *= 2;
        setN(g[0], g[1], g[2]);
        rebuildLists();
    }

    void merge(const Z2 &o, int p) {  // scheme_z2.cu:749-817: o's terms in the new block of size p
        int g[3] = {n[0], n[1], n[2]}, d[3];
        for (int q = 0; q < 3; q++) {
            g[q] = q == p ? n[q] + o.n[q] : n[q];
            d[q] = q == p ? n[q] : 0;
        }
        for (int t = 0; t < m; t++)
            for (int c = 0; c < 3; c++) x[c][t] = place(x[c][t], n[c], n[(c + 1) % 3], g[(c + 1) % 3], 0, 0);
        for (int t = 0; t < o.m; t++)
            for (int c = 0; c < 3; c++) {
                const int c1 = (c + 1) % 3;
                x[c][m + t] = place(o.x[c][t], o.n[c], o.n[c1], g[c1], d[c], d[c1]);
            }
        m += o.m;
        setN(g[0], g[1], g[2]);
        rebuildLists();
    }

    void productWith(const Z2 &o) {  // scheme_z2.cu:819-862: tensor product, terms (t1, t2) row-major
        Z2 *a = new Z2(*this);
        setN(a->n[0] * o.n[0], a->n[1] * o.n[1], a->n[2] * o.n[2]);
        m = a->m * o.m;
        for (int t1 = 0; t1 < a->m; t1++)
            for (int t2 = 0; t2 < o.m; t2++) {
                const int t = t1 * o.m + t2;
                for (int c = 0; c < 3; c++) {
                    const int c1 = (c + 1) % 3;
                    uint64_t v = 0;
                    for (int e1 = 0; e1 < a->nn[c]; e1++) {
                        if (!bit(a->x[c][t1], e1)) continue;
                        const int r1 = e1 / a->n[c1], q1 = e1 % a->n[c1];
                        for (int e2 = 0; e2 < o.nn[c]; e2++) {
                            if (!bit(o.x[c][t2], e2)) continue;
                            const int r2 = e2 / o.n[c1], q2 = e2 % o.n[c1];
                            v |= 1ull << ((r1 * o.n[c] + r2) * n[c1] + q1 * o.n[c1] + q2);
                        }
                    }
                    x[c][t] = v;
                }
            }
        delete a;
        rebuildLists();
    }

    void swapSize(int p1, int p2) {  // scheme_z2.cu:916-979
        if (p1 == p2) return;
        if (p1 > p2) std::swap(p1, p2);
        int idx[3];
        if (p1 == 0 && p2 == 1) { idx[0] = 0; idx[1] = 2; idx[2] = 1; }
        else if (p1 == 0 && p2 == 2) { idx[0] = 1; idx[1] = 0; idx[2] = 2; }
        else { idx[0] = 2; idx[1] = 1; idx[2] = 0; }
        int g[3];
        for (int q = 0; q < 3; q++) g[q] = n[(idx[q] + 1) % 3];
        for (int t = 0; t < m; t++) {
            uint64_t v[3];
            for (int c = 0; c < 3; c++) {
                // new matrix c (g[c] x g[c+1]) is the transpose of old matrix idx[c]
                const int rows = g[c], cols = g[(c + 1) % 3];
                uint64_t o = 0;
                for (int i = 0; i < rows; i++)
                    for (int j = 0; j < cols; j++) o |= bit(x[idx[c]][t], j * rows + i) << (i * cols + j);
                v[c] = o;
            }
            for (int c = 0; c < 3; c++) x[c][t] = v[c];
        }
        setN(g[0], g[1], g[2]);
        rebuildLists();
    }

    void reduceAll() {  // while (tryReduce()) ; (bounded)
        for (int guard = 0; tryReduce(); guard++)
            if (guard > retryCap) { *status |= ST_RETRY; return; }
    }

    template <class R> bool tryProject(R &r, int minN = 2) {  // scheme_z2.cu:1165-1185
        int idx[3], size = 0;
        for (int i = 0; i < 3; i++)
            if (isValidProject(i, minN)) idx[size++] = i;
        if (!size) return false;
        const int p = idx[r.raw() % (uint32_t)size];
        const int q = (int)(r.raw() % (uint32_t)n[p]);
        project(p, q);
        reduceAll();
        return true;
    }
    template <class R> bool tryExtend(R &r, int maxN = 16) {  // scheme_z2.cu:1187-1206
        int idx[3], size = 0;
        for (int i = 0; i < 3; i++)
            if (isValidExtension(i, maxN)) idx[size++] = i;
        if (!size) return false;
        extend(idx[r.raw() % (uint32_t)size]);
        reduceAll();
        return true;
    }
    template <class R> bool tryProduct(R &r, int maxN = 16) {  // scheme_z2.cu:1208-1223
        int idx[3], size = 0;
        for (int i = 0; i < 3; i++)
            if (isValidProduct(i, maxN)) idx[size++] = i;
        if (!size) return false;
        product(idx[r.raw() % (uint32_t)size]);
        return true;
    }
    template <class R> bool tryMerge(const Z2 &o, R &r) {  // scheme_z2.cu:1225-1254
        if (m + o.m > kMaxRank) return false;
        const bool eq0 = n[0] == o.n[0], eq1 = n[1] == o.n[1], eq2 = n[2] == o.n[2];
        const int s0 = n[0] + o.n[0], s1 = n[1] + o.n[1], s2 = n[2] + o.n[2];
        int p[3], size = 0;
        if (s0 <= kMaxExtensionN && s0 * n[1] <= maxMatrix && s0 * n[2] <= maxMatrix && eq1 && eq2) p[size++] = 0;
        if (eq0 && s1 <= kMaxExtensionN && n[0] * s1 <= maxMatrix && n[2] * s1 <= maxMatrix && eq2) p[size++] = 1;
        if (eq0 && eq1 && s2 <= kMaxExtensionN && n[0] * s2 <= maxMatrix && n[1] * s2 <= maxMatrix) p[size++] = 2;
        if (!size) return false;
        merge(o, p[r.raw() % (uint32_t)size]);
        return true;
    }
    bool tryProductWith(const Z2 &o) {  // scheme_z2.cu:1256-1275
        if (m * o.m > kMaxRank) return false;
        int g[3];
        for (int q = 0; q < 3; q++) g[q] = n[q] * o.n[q];
        for (int q = 0; q < 3; q++)
            if (g[q] > kMaxExtensionN || g[q] * g[(q + 1) % 3] > maxMatrix) return false;
        productWith(o);
        return true;
    }
    template <class R> void swapSizeRandom(R &r) {  // scheme_z2.cu:1315-1323
        int p1, p2;
        do {
            p1 = (int)(r.raw() % 3u);
            p2 = (int)(r.raw() % 3u);
        } while (p1 == p2);
        swapSize(p1, p2);
    }
};

// ------------------------------------------------------------ ternary vector
struct Tern {  // addition.cuh:8-13 (n is implied by the slot)
    uint64_t v = 0, s = 0;
    bool ok = true;
    bool operator==(const Tern &o) const { return v == o.v && s == o.s; }
    explicit operator bool() const { return v != 0; }
    int at(int idx) const { int r = (int)((v >> idx) & 1); return ((s >> idx) & 1) ? -r : r; }
    Tern add(const Tern &o) const {  // addition.cu:112-119
        Tern r;
        r.v = v ^ o.v;
        r.s = ((s & v) | (o.s & o.v)) & r.v;
        r.ok = !(v & o.v & ~(s ^ o.s));
        return r;
    }
    Tern sub(const Tern &o) const {  // addition.cu:121-128
        Tern r;
        r.v = v ^ o.v;
        r.s = ((s & v) | (~o.s & o.v)) & r.v;
        r.ok = !(v & o.v & (s ^ o.s));
        return r;
    }
    void addIn(const Tern &o) {  // addition.cu:138-146
        uint64_t sv1 = s & v, sv2 = o.s & o.v;
        ok = !(v & o.v & ~(s ^ o.s));
        v ^= o.v;
        s = (sv1 | sv2) & v;
    }
    void subIn(const Tern &o) {  // addition.cu:148-156
        uint64_t sv1 = s & v, sv2 = ~o.s & o.v;
        ok = !(v & o.v & (s ^ o.s));
        v ^= o.v;
        s = (sv1 | sv2) & v;
    }
    void negate() { s = ~s & v; }  // inverse(), addition.cu:62-64
    int compare(const Tern &o) const {  // addition.cu:82-93
        if (v != o.v) return 0;
        if (s == o.s) return 1;
        if (s == (~o.s & o.v)) return -1;
        return 0;
    }
    static bool firstPositive(uint64_t vv, uint64_t ss) { return vv == 0 || (vv & ~(vv & (vv - 1)) & ~ss); }
    bool positiveFirstNonZero() const { return firstPositive(v, s); }
    bool limit(bool fp) const { if (!ok) return false; return fp ? firstPositive(v, s) : true; }
    bool limitSum(const Tern &o, bool fp) const {  // addition.cu:172-186
        if (v & o.v & ~(s ^ o.s)) return false;
        if (fp) { uint64_t sv = v ^ o.v; return firstPositive(sv, ((s & v) | (o.s & o.v)) & sv); }
        return true;
    }
    bool limitSub(const Tern &o, bool fp) const {  // addition.cu:188-202
        if (v & o.v & (s ^ o.s)) return false;
        if (fp) { uint64_t sv = v ^ o.v; return firstPositive(sv, ((s & v) | (~o.s & o.v)) & sv); }
        return true;
    }
    bool positiveFirstNonZeroSub(const Tern &o) const {
        uint64_t sv = v ^ o.v;
        return firstPositive(sv, ((s & v) | (~o.s & o.v)) & sv);
    }
};

// Addition::random (addition.cu:66-80): the reference shifts a uint16 promoted
// to int, so chunk 16 is sign-extended into bits 32..63 and chunks >= 32 shift
// out to zero (PTX shl.b32 clamps its shift amount); both are reproduced.
template <class R> Tern randomTern(int n, R &r) {
    Tern a;
    for (int i = 0; i < n; i += 16) {
        uint32_t sb = r.raw() & 0xFFFF;
        uint32_t vb = r.raw() & 0xFFFF;
        int32_t vs = i >= 32 ? 0 : (int32_t)(vb << i);
        int32_t ss = i >= 32 ? 0 : (int32_t)(sb << i);
        a.v |= (uint64_t)(int64_t)vs;
        a.s |= (uint64_t)(int64_t)ss;
    }
    a.s &= a.v;
    a.ok = true;
    return a;
}

// ------------------------------------------------------------ ZT scheme
struct ZT {
    int n[3], nn[3], m;
    Tern x[3][kMaxRank];
    FlipList lists[3];
    int32_t *status;
    int retryCap = kRetryCap;  // fgo_walk_cfg::retry_cap (0 there = kRetryCap)
    int slotCap = kMaxRank;    // the records' slots per walk (fgo_walk_cfg::cap)

    bool nonzero(int t) const { return x[0][t].v && x[1][t].v && x[2][t].v; }

    void initNaive(int n1, int n2, int n3) {  // scheme_integer.cu:41-64
        n[0] = n1; n[1] = n2; n[2] = n3;
        nn[0] = n1 * n2; nn[1] = n2 * n3; nn[2] = n3 * n1;
        m = n1 * n2 * n3;
        for (int i = 0; i < n1; i++)
            for (int j = 0; j < n3; j++)
                for (int k = 0; k < n2; k++) {
                    int t = (i * n3 + j) * n2 + k;
                    x[0][t] = Tern{(uint64_t)1 << (i * n2 + k), 0, true};
                    x[1][t] = Tern{(uint64_t)1 << (k * n3 + j), 0, true};
                    x[2][t] = Tern{(uint64_t)1 << (j * n1 + i), 0, true};
                }
        rebuildLists();
    }

    void rebuildLists() {  // scheme_integer.cu:229-238
        for (int c = 0; c < 3; c++) {
            lists[c].clear();
            for (int a = 0; a < m; a++)
                for (int b = a + 1; b < m; b++)
                    if (x[c][a] == x[c][b]) lists[c].add(a, b);
        }
    }

    void moveTerm(int dst, int src) { for (int c = 0; c < 3; c++) x[c][dst] = x[c][src]; }

    void removeZeroes() {  // scheme_integer.cu:240-251 (re-checks the moved term)
        for (int t = 0; t < m; t++) {
            if (nonzero(t)) continue;
            m--;
            moveTerm(t, m);
            t--;
        }
    }

    void removeAt(int t) {
        m--;
        if (t == m) return;
        moveTerm(t, m);
    }

    void addTriplet(int i, int j, int k, const Tern &a, const Tern &b, const Tern &c) {
        if (m >= kMaxRank || m >= slotCap) { *status |= ST_OVERFLOW; return; }
        x[i][m] = a; x[j][m] = b; x[k][m] = c;
        m++;
    }

    bool fixSigns() {  // scheme_integer.cu:398-425
        bool changed = false;
        for (int t = 0; t < m; t++) {
            bool pi = x[0][t].positiveFirstNonZero(), pj = x[1][t].positiveFirstNonZero();
            if (pi && pj) continue;
            if (!pi && !pj) { x[0][t].negate(); x[1][t].negate(); }
            else if (!pi) { x[0][t].negate(); x[2][t].negate(); }
            else { x[1][t].negate(); x[2][t].negate(); }
            changed = true;
        }
        return changed;
    }

    void reduceAdd(int i, int a, int b) {  // scheme_integer.cu:549-559
        x[i][a].addIn(x[i][b]);
        bool zero = !x[i][a].v;
        removeAt(b);
        if (zero) removeZeroes();
        rebuildLists();
    }

    void reduceSub(int i, int a, int b) {  // scheme_integer.cu:561-571
        x[i][a].subIn(x[i][b]);
        bool zero = !x[i][a].v;
        removeAt(b);
        if (zero) removeZeroes();
        rebuildLists();
    }

    bool tryReduce() {  // scheme_integer.cu:1062-1101
        for (int p = 0; p < lists[0].size; p++) {
            int a = lists[0].first(p), b = lists[0].second(p);
            if (x[1][a] == x[1][b] && x[2][a].limitSum(x[2][b], false)) { reduceAdd(2, a, b); return true; }
            int cmp2 = x[2][a].compare(x[2][b]);
            if (cmp2 == 1 && x[1][a].limitSum(x[1][b], true)) { reduceAdd(1, a, b); return true; }
            if (cmp2 == -1 && x[1][a].limitSub(x[1][b], true)) { reduceSub(1, a, b); return true; }
        }
        for (int p = 0; p < lists[1].size; p++) {
            int a = lists[1].first(p), b = lists[1].second(p);
            int cmp2 = x[2][a].compare(x[2][b]);
            if (cmp2 == 1 && x[0][a].limitSum(x[0][b], true)) { reduceAdd(0, a, b); return true; }
            if (cmp2 == -1 && x[0][a].limitSub(x[0][b], true)) { reduceSub(0, a, b); return true; }
        }
        return false;
    }

    void flip(int i, int j, int k, int a, int b, bool checkReduce) {  // scheme_integer.cu:428-501
        x[j][a].addIn(x[j][b]);
        x[k][b].subIn(x[k][a]);
        lists[j].removeIndex(a);
        lists[k].removeIndex(b);
        if (!x[j][a].v || !x[k][b].v) {
            removeZeroes();
            rebuildLists();
            int guard = 0;
            while (tryReduce())
                if (++guard > retryCap) { *status |= ST_RETRY; break; }
            return;
        }
        for (int t = 0; t < m; t++) {
            if (t != a && x[j][t] == x[j][a]) {
                if (checkReduce) {
                    int cmpI = x[i][t].compare(x[i][a]);
                    if (cmpI == 1 && x[k][t].limitSum(x[k][a], k != 2)) { reduceAdd(k, t, a); return; }
                    if (i == 2 && cmpI == -1 && x[k][t].limitSub(x[k][a], true)) { reduceSub(k, t, a); return; }
                    int cmpK = x[k][t].compare(x[k][a]);
                    if (cmpK == 1 && x[i][t].limitSum(x[i][a], i != 2)) { reduceAdd(i, t, a); return; }
                    if (k == 2 && cmpK == -1 && x[i][t].limitSub(x[i][a], true)) { reduceSub(i, t, a); return; }
                }
                lists[j].add(a, t);
            }
            if (t != b && x[k][t] == x[k][b]) {
                if (checkReduce) {
                    int cmpI = x[i][t].compare(x[i][b]);
                    if (cmpI == 1 && x[j][t].limitSum(x[j][b], j != 2)) { reduceAdd(j, t, b); return; }
                    if (i == 2 && cmpI == -1 && x[j][t].limitSub(x[j][b], true)) { reduceSub(j, t, b); return; }
                    int cmpJ = x[j][t].compare(x[j][b]);
                    if (cmpJ == 1 && x[i][t].limitSum(x[i][b], i != 2)) { reduceAdd(i, t, b); return; }
                    if (j == 2 && cmpJ == -1 && x[i][t].limitSub(x[i][b], true)) { reduceSub(i, t, b); return; }
                }
                lists[k].add(b, t);
            }
        }
    }

    void plus(int i, int j, int k, int p, int q, int variant) {  // scheme_integer.cu:503-539
        const Tern a1 = x[i][p], b1 = x[j][p], c1 = x[k][p];
        const Tern a2 = x[i][q], b2 = x[j][q], c2 = x[k][q];
        const Tern aAdd = a1.add(a2), bAdd = b1.add(b2), cAdd = c1.add(c2);
        const Tern aSub = a2.sub(a1), bSub = b2.sub(b1), cSub = c2.sub(c1);
        if (variant == 0 && aSub.limit(i != 2) && bAdd.limit(j != 2) && cSub.limit(k != 2)) {
            x[j][p] = bAdd; x[i][q] = aSub; addTriplet(i, j, k, a1, b2, cSub);
        } else if (variant == 1 && aSub.limit(i != 2) && bSub.limit(j != 2) && cAdd.limit(k != 2)) {
            x[k][p] = cAdd; x[j][q] = bSub; addTriplet(i, j, k, aSub, b1, c2);
        } else if (aAdd.limit(i != 2) && bSub.limit(j != 2) && cSub.limit(k != 2)) {
            x[i][p] = aAdd; x[k][q] = cSub; addTriplet(i, j, k, a2, bSub, c1);
        }
        removeZeroes();
        fixSigns();
        rebuildLists();
    }

    void split(int i, int j, int k, int t, const Tern &a) {  // scheme_integer.cu:541-547
        Tern rest = x[i][t].sub(a);
        Tern bj = x[j][t], bk = x[k][t];
        addTriplet(i, j, k, rest, bj, bk);
        x[i][t] = a;
        fixSigns();
        rebuildLists();
    }

    template <class R> bool tryFlip(R &r, bool checkReduce) {  // scheme_integer.cu:907-975
        int size = lists[0].size + lists[1].size + lists[2].size;
        std::vector<int> order(size > 0 ? size : 1);
        permutation(order.data(), size, r);
        for (int p = 0; p < size; p++) {
            int idx = order[p];
            int i, j, k, a, b;
            if (idx < lists[0].size) { i = 0; j = 1; k = 2; a = lists[0].first(idx); b = lists[0].second(idx); }
            else if (idx < lists[0].size + lists[1].size) {
                idx -= lists[0].size; i = 1; j = 0; k = 2; a = lists[1].first(idx); b = lists[1].second(idx);
            } else {
                idx -= lists[0].size + lists[1].size; i = 2; j = 0; k = 1; a = lists[2].first(idx); b = lists[2].second(idx);
            }
            if (r.coin()) std::swap(j, k);
            if (r.coin()) std::swap(a, b);
            if (x[j][a].limitSum(x[j][b], j != 2) && x[k][b].limitSub(x[k][a], false)) {
                if (k == 2 || x[k][b].positiveFirstNonZeroSub(x[k][a])) flip(i, j, k, a, b, checkReduce);
                else flip(i, j, k, b, a, checkReduce);
                return true;
            }
            if (x[k][a].limitSum(x[k][b], k != 2) && x[j][b].limitSub(x[j][a], false)) {
                if (j == 2 || x[j][b].positiveFirstNonZeroSub(x[j][a])) flip(i, k, j, a, b, checkReduce);
                else flip(i, k, j, b, a, checkReduce);
                return true;
            }
        }
        return false;
    }

    template <class R> bool tryPlus(R &r) {  // scheme_integer.cu:977-998
        if (m >= kMaxRank || m >= n[0] * n[1] * n[2]) return false;
        int a = (int)r.below(m), b = (int)r.below(m);
        int guard = 0;
        while (a == b || x[0][a] == x[0][b] || x[1][a] == x[1][b] || x[2][a] == x[2][b]) {
            if (++guard > retryCap) { *status |= ST_RETRY; return false; }
            a = (int)r.below(m);
            b = (int)r.below(m);
        }
        int perm[3];
        permutation(perm, 3, r);
        int variant = (int)r.below(3);
        plus(perm[0], perm[1], perm[2], a, b, variant);
        return true;
    }

    template <class R> bool trySplit(R &r) {  // scheme_integer.cu:1000-1020
        if (m >= kMaxRank || m >= n[0] * n[1] * n[2]) return false;
        int t = (int)r.below(m);
        int perm[3];
        permutation(perm, 3, r);
        int i = perm[0], j = perm[1], k = perm[2];
        Tern a = randomTern(nn[i], r);
        if (!x[i][t].limitSub(a, i != 2)) return false;
        split(i, j, k, t, a);
        return true;
    }

    template <class R> bool trySplitExisted(R &r) {  // scheme_integer.cu:1022-1043
        if (m >= kMaxRank || m >= n[0] * n[1] * n[2]) return false;
        int a, b, i;
        int guard = 0;
        do {
            if (++guard > retryCap) { *status |= ST_RETRY; return false; }
            a = (int)r.below(m);
            b = (int)r.below(m);
            i = (int)r.below(3);
        } while (a == b || x[i][a] == x[i][b]);
        if (!x[i][a].limitSub(x[i][b], i != 2)) return false;
        Tern xb = x[i][b];
        split(i, (i + 1) % 3, (i + 2) % 3, a, xb);
        return true;
    }

    template <class R> bool tryExpand(int count, R &r) {  // scheme_integer.cu:1045-1060
        bool result = false;
        for (int q = 0; q < count && m < kMaxRank; q++) {
            int v = (int)r.below(3);
            if (v == 0) result |= tryPlus(r);
            else if (v == 1) result |= trySplit(r);
            else result |= trySplitExisted(r);
        }
        return result;
    }

    int complexity() const {  // scheme_integer.cu:139-147
        int count = 0;
        for (int t = 0; t < m; t++)
            for (int c = 0; c < 3; c++) count += popc64(x[c][t].v);
        return count - 2 * m - nn[2];
    }

    // ---------------------------------------------------------------- basis moves
    template <class R> bool tryReduceGauss(R &, bool) { return false; }  // Z2 only in the reference
    // scheme_integer.cu:1215-1217 leaves the ternary move empty (only its gate draw is taken).
    // Opt-in (zt_sandwich, no reference counterpart): conjugation by random signed permutation
    // matrices, the integer matrices whose conjugation keeps every coefficient in {-1, 0, 1}:
    // U' = u U v^-1, V' = v V w^-1, W' = w W u^-1 as the Z2 move, entry (i, j) of the result =
    // sign_l(i) sign_r(j) X(p_l(i), p_r(j)); then signs are canonicalised and the lists rebuilt.
    template <class R> void signedPermutation(int n_, int *p, uint32_t &signs, R &r) {
        permutation(p, n_, r);
        signs = r.raw() & (n_ >= 32 ? 0xFFFFFFFFu : ((1u << n_) - 1u));
    }
    static Tern conjSigned(const Tern &x, const int *pl, uint32_t sl, const int *pr, uint32_t sr, int n1, int n2) {
        uint64_t v = 0, sg = 0;
        for (int i = 0; i < n1; i++)
            for (int j = 0; j < n2; j++) {
                const int src = pl[i] * n2 + pr[j], dst = i * n2 + j;
                if (!((x.v >> src) & 1)) continue;
                v |= 1ull << dst;
                if ((((x.s >> src) & 1) ^ ((sl >> i) & 1) ^ ((sr >> j) & 1)) != 0) sg |= 1ull << dst;
            }
        return mk(v, sg);
    }
    template <class R> void sandwiching(R &r) {
        if (!g_ternarySandwich || n[0] > 16 || n[1] > 16 || n[2] > 16) return;
        int pu[16], pv[16], pw[16];
        uint32_t su, sv, sw;
        signedPermutation(n[0], pu, su, r);
        signedPermutation(n[1], pv, sv, r);
        signedPermutation(n[2], pw, sw, r);
        for (int t = 0; t < m; t++) {
            x[0][t] = conjSigned(x[0][t], pu, su, pv, sv, n[0], n[1]);
            x[1][t] = conjSigned(x[1][t], pv, sv, pw, sw, n[1], n[2]);
            x[2][t] = conjSigned(x[2][t], pw, sw, pu, su, n[2], n[0]);
        }
        fixSigns();
        rebuildLists();
    }
    void swapBasisRows(int i1, int i2) {  // scheme_integer.cu:791-815
        int rows[64];
        for (int q = 0; q < n[0]; q++) rows[q] = q;
        rows[i1] = i2;
        rows[i2] = i1;
        for (int t = 0; t < m; t++) {
            uint64_t uv = 0, us = 0, wv = 0, ws = 0;
            for (int i = 0; i < n[0]; i++)
                for (int j = 0; j < n[1]; j++) moveBit(x[0][t], rows[i] * n[1] + j, i * n[1] + j, uv, us);
            for (int i = 0; i < n[2]; i++)
                for (int j = 0; j < n[0]; j++) moveBit(x[2][t], i * n[0] + rows[j], i * n[0] + j, wv, ws);
            x[0][t] = mk(uv, us);
            x[2][t] = mk(wv, ws);
        }
    }
    void swapBasisColumns(int j1, int j2) {  // scheme_integer.cu:817-841
        int cols[64];
        for (int q = 0; q < n[2]; q++) cols[q] = q;
        cols[j1] = j2;
        cols[j2] = j1;
        for (int t = 0; t < m; t++) {
            uint64_t vv = 0, vs = 0, wv = 0, ws = 0;
            for (int i = 0; i < n[1]; i++)
                for (int j = 0; j < n[2]; j++) moveBit(x[1][t], i * n[2] + cols[j], i * n[2] + j, vv, vs);
            for (int i = 0; i < n[2]; i++)
                for (int j = 0; j < n[0]; j++) moveBit(x[2][t], cols[i] * n[0] + j, i * n[0] + j, wv, ws);
            x[1][t] = mk(vv, vs);
            x[2][t] = mk(wv, ws);
        }
    }
    template <class R> void swapBasis(R &r) {  // scheme_integer.cu:1219-1233
        if (r.raw() % 2) {
            const int i1 = (int)(r.raw() % (uint32_t)n[0]), i2 = (int)(r.raw() % (uint32_t)n[0]);
            swapBasisRows(i1, i2);
        } else {
            const int j1 = (int)(r.raw() % (uint32_t)n[2]), j2 = (int)(r.raw() % (uint32_t)n[2]);
            swapBasisColumns(j1, j2);
        }
        if (fixSigns()) rebuildLists();
    }

    // ---------------------------------------------------------------- resize
    // The Z2 operators on both masks of each coefficient vector (entry (i, j)
    // of matrix c at bit i * n[c+1] + j; a negative entry's sign bit moves
    // with its value bit): scheme_integer.cu:271-340, 573-905, 1103-1240.
    void setN(int a, int b, int c) {
        n[0] = a; n[1] = b; n[2] = c;
        for (int q = 0; q < 3; q++) nn[q] = n[q] * n[(q + 1) % 3];
    }
    static uint64_t bit(uint64_t v, int k) { return (v >> k) & 1ull; }
    // moves bit `from` of both masks to bit `to` of (ov, os)
    static void moveBit(const Tern &a, int from, int to, uint64_t &ov, uint64_t &os) {
        ov |= bit(a.v, from) << to;
        os |= bit(a.s, from) << to;
    }
    static Tern mk(uint64_t v, uint64_t s) { Tern t; t.v = v; t.s = s & v; t.ok = true; return t; }
    static Tern place(const Tern &a, int rows, int cols, int newCols, int di, int dj) {
        uint64_t v = 0, sg = 0;
        for (int i = 0; i < rows; i++)
            for (int j = 0; j < cols; j++) moveBit(a, i * cols + j, (i + di) * newCols + j + dj, v, sg);
        return mk(v, sg);
    }

    bool isValidProject(int i, int minN) const {
        return n[i] - 1 >= minN && n[(i + 1) % 3] >= minN && n[(i + 2) % 3] >= minN;
    }
    bool isValidGrown(const int g[3], int rank, int maxN) const {
        if (rank > kMaxRank) return false;
        for (int q = 0; q < 3; q++)
            if (g[q] * g[(q + 1) % 3] > kMaxMatrix || g[q] > maxN) return false;
        return true;
    }
    bool isValidExtension(int i, int maxN) const {
        int g[3] = {n[0], n[1], n[2]};
        g[i] += 1;
        return isValidGrown(g, m + g[(i + 1) % 3] * g[(i + 2) % 3], maxN);
    }
    bool isValidProduct(int i, int maxN) const {
        int g[3] = {n[0], n[1], n[2]};
        g[i] *= 2;
        return isValidGrown(g, m * 2, maxN);
    }

    void project(int p, int q) {  // scheme_integer.cu:573-584
        const int rc = (p + 2) % 3;
        for (int t = 0; t < m; t++) {
            {
                const int rows = n[p], cols = n[(p + 1) % 3];
                uint64_t v = 0, sg = 0;
                for (int i = 0, i2 = 0; i < rows; i++) {
                    if (i == q) continue;
                    for (int j = 0; j < cols; j++) moveBit(x[p][t], i * cols + j, i2 * cols + j, v, sg);
                    i2++;
                }
                x[p][t] = mk(v, sg);
            }
            {
                const int rows = n[rc], cols = n[(rc + 1) % 3];
                uint64_t v = 0, sg = 0;
                for (int i = 0; i < rows; i++)
                    for (int j = 0, j2 = 0; j < cols; j++) {
                        if (j == q) continue;
                        moveBit(x[rc][t], i * cols + j, i * (cols - 1) + j2, v, sg);
                        j2++;
                    }
                x[rc][t] = mk(v, sg);
            }
        }
        int g[3] = {n[0], n[1], n[2]};
        g[p]--;
        setN(g[0], g[1], g[2]);
        removeZeroes();
        fixSigns();
        rebuildLists();
    }

    void extend(int p) {  // scheme_integer.cu:586-618
        const int a = n[0], b = n[1], c = n[2];
        const int col = p == 0 ? 2 : (p == 1 ? 0 : 1);
        const int cr = col == 0 ? a : (col == 1 ? b : c), cc = col == 0 ? b : (col == 1 ? c : a);
        for (int t = 0; t < m; t++) x[col][t] = place(x[col][t], cr, cc, cc + 1, 0, 0);
        const int outer = p == 0 ? c : a, inner = p == 0 ? b : (p == 1 ? c : b);
        for (int i = 0; i < outer; i++)
            for (int j = 0; j < inner; j++) {
                uint64_t u, v, w;
                if (p == 0) { u = 1ull << (a * b + j); v = 1ull << (j * c + i); w = 1ull << (i * (a + 1) + a); }
                else if (p == 1) { u = 1ull << (i * (b + 1) + b); v = 1ull << (b * c + j); w = 1ull << (j * a + i); }
                else { u = 1ull << (i * b + j); v = 1ull << (j * (c + 1) + c); w = 1ull << (c * a + i); }
                addTriplet(0, 1, 2, mk(u, 0), mk(v, 0), mk(w, 0));
            }
        int g[3] = {a, b, c};
        g[p]++;
        setN(g[0], g[1], g[2]);
        rebuildLists();
    }

    void product(int p) {  // scheme_integer.cu:620-678
        int g[3] = {n[0], n[1], n[2]}, d[3];
        g[p] *= 2;
        for (int q = 0; q < 3; q++) d[q] = q == p ? n[q] : 0;
        for (int t = 0; t < m; t++)
            for (int c = 0; c < 3; c++) {
                const int c1 = (c + 1) % 3;
                const Tern v = x[c][t];
                x[c][t] = place(v, n[c], n[c1], g[c1], 0, 0);
                x[c][t + m] = place(v, n[c], n[c1], g[c1], d[c], d[c1]);
            }
        m *= 2;
        setN(g[0], g[1], g[2]);
        rebuildLists();
    }

    void merge(const ZT &o, int p) {  // scheme_integer.cu:680-745
        int g[3], d[3];
        for (int q = 0; q < 3; q++) {
            g[q] = q == p ? n[q] + o.n[q] : n[q];
            d[q] = q == p ? n[q] : 0;
        }
        for (int t = 0; t < m; t++)
            for (int c = 0; c < 3; c++) x[c][t] = place(x[c][t], n[c], n[(c + 1) % 3], g[(c + 1) % 3], 0, 0);
        for (int t = 0; t < o.m; t++)
            for (int c = 0; c < 3; c++) {
                const int c1 = (c + 1) % 3;
                x[c][m + t] = place(o.x[c][t], o.n[c], o.n[c1], g[c1], d[c], d[c1]);
            }
        m += o.m;
        setN(g[0], g[1], g[2]);
        rebuildLists();
    }

    void productWith(const ZT &o) {  // scheme_integer.cu:747-841: coefficients multiply
        ZT *a = new ZT(*this);
        setN(a->n[0] * o.n[0], a->n[1] * o.n[1], a->n[2] * o.n[2]);
        m = a->m * o.m;
        for (int t1 = 0; t1 < a->m; t1++)
            for (int t2 = 0; t2 < o.m; t2++) {
                const int t = t1 * o.m + t2;
                for (int c = 0; c < 3; c++) {
                    const int c1 = (c + 1) % 3;
                    uint64_t v = 0, sg = 0;
                    const Tern &p1 = a->x[c][t1], &p2 = o.x[c][t2];
                    for (int e1 = 0; e1 < a->nn[c]; e1++) {
                        if (!bit(p1.v, e1)) continue;
                        const int r1 = e1 / a->n[c1], q1 = e1 % a->n[c1];
                        for (int e2 = 0; e2 < o.nn[c]; e2++) {
                            if (!bit(p2.v, e2)) continue;
                            const int r2 = e2 / o.n[c1], q2 = e2 % o.n[c1];
                            const int to = (r1 * o.n[c] + r2) * n[c1] + q1 * o.n[c1] + q2;
                            v |= 1ull << to;
                            sg |= (bit(p1.s, e1) ^ bit(p2.s, e2)) << to;
                        }
                    }
                    x[c][t] = mk(v, sg);
                }
            }
        delete a;
        rebuildLists();
    }

    void swapSize(int p1, int p2) {  // scheme_integer.cu:843-905
        if (p1 == p2) return;
        if (p1 > p2) std::swap(p1, p2);
        int idx[3];
        if (p1 == 0 && p2 == 1) { idx[0] = 0; idx[1] = 2; idx[2] = 1; }
        else if (p1 == 0 && p2 == 2) { idx[0] = 1; idx[1] = 0; idx[2] = 2; }
        else { idx[0] = 2; idx[1] = 1; idx[2] = 0; }
        int g[3];
        for (int q = 0; q < 3; q++) g[q] = n[(idx[q] + 1) % 3];
        for (int t = 0; t < m; t++) {
            Tern v[3];
            for (int c = 0; c < 3; c++) {
                const int rows = g[c], cols = g[(c + 1) % 3];
                uint64_t ov = 0, os = 0;
                for (int i = 0; i < rows; i++)
                    for (int j = 0; j < cols; j++) moveBit(x[idx[c]][t], j * rows + i, i * cols + j, ov, os);
                v[c] = mk(ov, os);
            }
            for (int c = 0; c < 3; c++) x[c][t] = v[c];
        }
        setN(g[0], g[1], g[2]);
        fixSigns();
        rebuildLists();
    }

    void reduceAll() {
        for (int guard = 0; tryReduce(); guard++)
            if (guard > retryCap) { *status |= ST_RETRY; return; }
    }
    template <class R> bool tryProject(R &r, int minN = 2) {  // scheme_integer.cu:1103-1123
        int idx[3], size = 0;
        for (int i = 0; i < 3; i++)
            if (isValidProject(i, minN)) idx[size++] = i;
        if (!size) return false;
        const int p = idx[r.raw() % (uint32_t)size];
        const int q = (int)(r.raw() % (uint32_t)n[p]);
        project(p, q);
        reduceAll();
        return true;
    }
    template <class R> bool tryExtend(R &r, int maxN = 16) {  // scheme_integer.cu:1125-1144
        int idx[3], size = 0;
        for (int i = 0; i < 3; i++)
            if (isValidExtension(i, maxN)) idx[size++] = i;
        if (!size) return false;
        extend(idx[r.raw() % (uint32_t)size]);
        reduceAll();
        return true;
    }
    template <class R> bool tryProduct(R &r, int maxN = 16) {  // scheme_integer.cu:1146-1161
        int idx[3], size = 0;
        for (int i = 0; i < 3; i++)
            if (isValidProduct(i, maxN)) idx[size++] = i;
        if (!size) return false;
        product(idx[r.raw() % (uint32_t)size]);
        return true;
    }
    template <class R> bool tryMerge(const ZT &o, R &r) {  // scheme_integer.cu:1163-1192
        if (m + o.m > kMaxRank) return false;
        const bool eq0 = n[0] == o.n[0], eq1 = n[1] == o.n[1], eq2 = n[2] == o.n[2];
        const int s0 = n[0] + o.n[0], s1 = n[1] + o.n[1], s2 = n[2] + o.n[2];
        int p[3], size = 0;
        if (s0 <= kMaxExtensionN && s0 * n[1] <= kMaxMatrix && s0 * n[2] <= kMaxMatrix && eq1 && eq2) p[size++] = 0;
        if (eq0 && s1 <= kMaxExtensionN && n[0] * s1 <= kMaxMatrix && n[2] * s1 <= kMaxMatrix && eq2) p[size++] = 1;
        if (eq0 && eq1 && s2 <= kMaxExtensionN && n[0] * s2 <= kMaxMatrix && n[1] * s2 <= kMaxMatrix) p[size++] = 2;
        if (!size) return false;
        merge(o, p[r.raw() % (uint32_t)size]);
        return true;
    }
    bool tryProductWith(const ZT &o) {  // scheme_integer.cu:1194-1213
        if (m * o.m > kMaxRank) return false;
        int g[3];
        for (int q = 0; q < 3; q++) g[q] = n[q] * o.n[q];
        for (int q = 0; q < 3; q++)
            if (g[q] > kMaxExtensionN || g[q] * g[(q + 1) % 3] > kMaxMatrix) return false;
        productWith(o);
        return true;
    }
    template <class R> void swapSizeRandom(R &r) {  // scheme_integer.cu:1235-1243
        int p1, p2;
        do {
            p1 = (int)(r.raw() % 3u);
            p2 = (int)(r.raw() % 3u);
        } while (p1 == p2);
        swapSize(p1, p2);
    }
};

// ------------------------------------------------------------ record <-> scheme
inline size_t facIndex(int w, int c, int t, int cap) { return ((size_t)w * 3 + c) * cap + t; }

void loadZ2(Z2 &s, const fgo_batch *b, int w, int cap) {
    for (int c = 0; c < 3; c++) s.n[c] = b->n[w * 3 + c];
    for (int c = 0; c < 3; c++) s.nn[c] = s.n[c] * s.n[(c + 1) % 3];
    s.m = b->m[w];
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < s.m; t++) s.x[c][t] = b->fac[facIndex(w, c, t, cap)];
    for (int c = 0; c < 3; c++) {
        s.lists[c].size = b->list_size[w * 3 + c];
        std::memcpy(s.lists[c].pairs, b->list_pairs + ((size_t)w * 3 + c) * kMaxPairs, sizeof(uint32_t) * s.lists[c].size);
    }
}

void storeZ2(const Z2 &s, fgo_batch *b, int w, int cap) {
    if (s.m > cap) { b->status[w] |= ST_OVERFLOW; return; }
    b->m[w] = s.m;
    for (int c = 0; c < 3; c++) b->n[w * 3 + c] = s.n[c];
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < cap; t++) b->fac[facIndex(w, c, t, cap)] = t < s.m ? s.x[c][t] : 0;
    for (int c = 0; c < 3; c++) {
        b->list_size[w * 3 + c] = s.lists[c].size;
        uint32_t *dst = b->list_pairs + ((size_t)w * 3 + c) * kMaxPairs;
        std::memset(dst, 0, sizeof(uint32_t) * kMaxPairs);
        std::memcpy(dst, s.lists[c].pairs, sizeof(uint32_t) * s.lists[c].size);
    }
}

void loadZT(ZT &s, const fgo_batch *b, int w, int cap) {
    for (int c = 0; c < 3; c++) s.n[c] = b->n[w * 3 + c];
    for (int c = 0; c < 3; c++) s.nn[c] = s.n[c] * s.n[(c + 1) % 3];
    s.m = b->m[w];
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < s.m; t++) {
            size_t q = facIndex(w, c, t, cap);
            s.x[c][t] = Tern{b->fac[q], b->sgn[q], b->valid[q] != 0};
        }
    for (int c = 0; c < 3; c++) {
        s.lists[c].size = b->list_size[w * 3 + c];
        std::memcpy(s.lists[c].pairs, b->list_pairs + ((size_t)w * 3 + c) * kMaxPairs, sizeof(uint32_t) * s.lists[c].size);
    }
}

void storeZT(const ZT &s, fgo_batch *b, int w, int cap) {
    if (s.m > cap) { b->status[w] |= ST_OVERFLOW; return; }
    b->m[w] = s.m;
    for (int c = 0; c < 3; c++) b->n[w * 3 + c] = s.n[c];
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < cap; t++) {
            size_t q = facIndex(w, c, t, cap);
            b->fac[q] = t < s.m ? s.x[c][t].v : 0;
            b->sgn[q] = t < s.m ? s.x[c][t].s : 0;
            b->valid[q] = t < s.m ? (uint8_t)s.x[c][t].ok : 0;
        }
    for (int c = 0; c < 3; c++) {
        b->list_size[w * 3 + c] = s.lists[c].size;
        uint32_t *dst = b->list_pairs + ((size_t)w * 3 + c) * kMaxPairs;
        std::memset(dst, 0, sizeof(uint32_t) * kMaxPairs);
        std::memcpy(dst, s.lists[c].pairs, sizeof(uint32_t) * s.lists[c].size);
    }
}

// best := current without lists (copyTo(target, false))
void storeBestZ2(const Z2 &s, fgo_batch *b, int w, int cap) {
    if (s.m > cap) { b->status[w] |= ST_OVERFLOW; return; }
    b->best_m[w] = s.m;
    if (b->best_n)
        for (int c = 0; c < 3; c++) b->best_n[w * 3 + c] = s.n[c];
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < cap; t++) b->best_fac[facIndex(w, c, t, cap)] = t < s.m ? s.x[c][t] : 0;
}

void storeBestZT(const ZT &s, fgo_batch *b, int w, int cap) {
    if (s.m > cap) { b->status[w] |= ST_OVERFLOW; return; }
    b->best_m[w] = s.m;
    if (b->best_n)
        for (int c = 0; c < 3; c++) b->best_n[w * 3 + c] = s.n[c];
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < cap; t++) {
            size_t q = facIndex(w, c, t, cap);
            b->best_fac[q] = t < s.m ? s.x[c][t].v : 0;
            b->best_sgn[q] = t < s.m ? s.x[c][t].s : 0;
            b->best_valid[q] = t < s.m ? (uint8_t)s.x[c][t].ok : 0;
        }
}

inline void storeBest(const Z2 &s, fgo_batch *b, int w, int cap) { storeBestZ2(s, b, w, cap); }
inline void storeBest(const ZT &s, fgo_batch *b, int w, int cap) { storeBestZT(s, b, w, cap); }

// randomWalkKernel body (flip_graph.cu:526-569) with randomIterations=false and
// sandwiching / basis probabilities 0: their gate draws are still consumed
// (RefDraws) exactly as the reference does.
template <class Scheme, class R>
void walkLaunch(Scheme &s, R &r, const fgo_walk_cfg *cfg, fgo_batch *b, int w) {
    int cap = cfg->cap;
    int flipsCount = b->flips[w];
    int bestRank = b->best_rank[w];
    int bestM = b->best_m[w];
    // randomIterations (flip_graph.cu:531): with resizing on, a launch runs randint(1, iterations) steps
    const int iters = cfg->resize_p > 0 ? randint(1, cfg->iterations, r) : cfg->iterations;
    for (int it = 0; it < iters; it++) {
        int rank = s.m;
        if (!s.tryFlip(r, true)) {
            s.tryExpand(randint(1, 2, r), r);
            if (b->status[w]) break;  // a retry bound or overflow stops the walk, as on the GPU
            continue;
        }
        if (b->accepted) b->accepted[w]++;
        if (s.m < rank) flipsCount = 0;
        flipsCount++;
        if (s.m < bestRank || (s.m == bestRank && r.tie())) {
            bestRank = s.m;
            storeBest(s, b, w, cap);
            bestM = s.m;
        }
        if (r.gate(cfg->reduce_p, cfg->iterations)) s.tryReduce();
        // Gauss reduction: not in the reference's walk; no draw at probability 0
        if (cfg->gauss_p > 0 && r.gate(cfg->gauss_p, cfg->iterations)) s.tryReduceGauss(r, true);
        if (r.gate(cfg->expand_p, cfg->iterations) && s.m <= bestM + 2) {
            if (s.tryExpand(randint(1, 2, r), r)) flipsCount = 0;
        }
        if (r.gate(cfg->sandwich_p, cfg->iterations)) s.sandwiching(r);  // flip_graph.cu:560-561
        if (r.gate(cfg->basis_p, cfg->iterations)) s.swapBasis(r);       // flip_graph.cu:563-564
        if (flipsCount >= cfg->plus_iterations && s.tryPlus(r)) flipsCount = 0;
        if (b->status[w]) break;
    }
    b->flips[w] = flipsCount;
    b->best_rank[w] = bestRank;
}

template <class Scheme> void loadScheme(Scheme &s, const fgo_batch *b, int w, int cap);
template <> void loadScheme<Z2>(Z2 &s, const fgo_batch *b, int w, int cap) { loadZ2(s, b, w, cap); }
template <> void loadScheme<ZT>(ZT &s, const fgo_batch *b, int w, int cap) { loadZT(s, b, w, cap); }
inline void storeScheme(const Z2 &s, fgo_batch *b, int w, int cap) { storeZ2(s, b, w, cap); }
inline void storeScheme(const ZT &s, fgo_batch *b, int w, int cap) { storeZT(s, b, w, cap); }

inline void setImplicit(Z2 &s, bool on) { s.implicit = on; }
inline void setImplicit(ZT &, bool) {}
// The fast mode's words keep the partner count in their top byte: grown factors of at most 56 entries.
inline void setMaxMatrix(Z2 &s, int v) { s.maxMatrix = v; }
inline void setMaxMatrix(ZT &, int) {}
inline void rebuildIfList(Z2 &s) { s.rebuildLists(); }  // implicit: clears the lists
inline void rebuildIfList(ZT &) {}

template <class Scheme>
void runWalks(const fgo_walk_cfg *cfg, int S, fgo_batch *b, const fgo_tape *tape) {
    Scheme *s = new Scheme;
    for (int w = 0; w < S; w++) {
        loadScheme(*s, b, w, cfg->cap);
        setImplicit(*s, cfg->rng == FGO_RNG_FAST);
        s->status = &b->status[w];
        s->retryCap = retry_cap(cfg);
        s->slotCap = cfg->cap;
        if (cfg->rng == FGO_RNG_TAPE) {
            RefDraws r;
            r.d = tape->draws + tape->offsets[w];
            r.u = tape->uniforms + tape->offsets[w];
            r.n = tape->offsets[w + 1] - tape->offsets[w];
            r.pos = b->rng_pos[w];
            r.status = &b->status[w];
            for (int L = 0; L < cfg->launches && !b->status[w]; L++) walkLaunch(*s, r, cfg, b, w);
            b->rng_pos[w] = r.pos;
        } else {
            FastDraws r;
            r.key[0] = (uint32_t)cfg->seed;
            r.key[1] = (uint32_t)(cfg->seed >> 32);
            r.walk = (uint32_t)w;
            r.pos = b->rng_pos[w];
            r.status = &b->status[w];
            for (int L = 0; L < cfg->launches && !b->status[w]; L++) walkLaunch(*s, r, cfg, b, w);
            b->rng_pos[w] = r.pos;
        }
        storeScheme(*s, b, w, cfg->cap);
    }
    delete s;
}

// minimizeKernel body (complexity_minimizer.cu:245-263).
template <class Scheme, class R>
void minimizeLaunch(Scheme &s, R &r, const fgo_walk_cfg *cfg, fgo_batch *b, int w, int32_t *bestC) {
    int best = bestC[w];
    for (int it = 0; it < cfg->iterations; it++) {
        if (!s.tryFlip(r, false)) break;
        int c = s.complexity();
        if (c < best) {
            best = c;
            storeBest(s, b, w, cfg->cap);
        }
        if (b->status[w]) break;
    }
    bestC[w] = best;
}

template <class Scheme>
void runMinimize(const fgo_walk_cfg *cfg, int S, fgo_batch *b, const fgo_tape *tape, int32_t *bestC) {
    Scheme *s = new Scheme;
    for (int w = 0; w < S; w++) {
        loadScheme(*s, b, w, cfg->cap);  // lists keep their persisted order
        setImplicit(*s, cfg->rng == FGO_RNG_FAST);
        s->status = &b->status[w];
        s->retryCap = retry_cap(cfg);
        s->slotCap = cfg->cap;
        if (cfg->rng == FGO_RNG_TAPE) {
            RefDraws r;
            r.d = tape->draws + tape->offsets[w];
            r.u = tape->uniforms + tape->offsets[w];
            r.n = tape->offsets[w + 1] - tape->offsets[w];
            r.pos = b->rng_pos[w];
            r.status = &b->status[w];
            minimizeLaunch(*s, r, cfg, b, w, bestC);
            b->rng_pos[w] = r.pos;
        } else {
            FastDraws r;
            r.key[0] = (uint32_t)cfg->seed;
            r.key[1] = (uint32_t)(cfg->seed >> 32);
            r.walk = (uint32_t)w;
            r.pos = b->rng_pos[w];
            r.status = &b->status[w];
            minimizeLaunch(*s, r, cfg, b, w, bestC);
            b->rng_pos[w] = r.pos;
        }
        storeScheme(*s, b, w, cfg->cap);
    }
    delete s;
}

// ============================================================ bounded integer ring (ZB)
// Coefficients in [-2, 2] (integer-coefficient search with |c| <= 2).  No
// reference counterpart: the reference's integer ring is {-1, 0, 1}
// (SchemeInteger).  The walk follows SchemeInteger's structure with the
// library's fast-mode proposal (implicit enumeration of ordered pairs of
// exactly equal factors in canonical order, Philox stream) and these rules:
//   pairs are factors equal up to sign (x_b = e x_a, e = +-1: the sign moves
//     to another slot of the term, so the pair shares the factor);
//   flip (a, b) sharing factor i, (j, k) = the other two in a coin-chosen
//     order, s = +-1 by a second coin: y_a += s e y_b, z_b -= s z_a (both
//     signs are flips, so every flip has its inverse and the walk does not
//     drift to large coefficients); a proposal whose result leaves [-2, 2]
//     is rejected (the step is spent);
//   signs: first nonzero entry of u and of v positive (SchemeInteger::fixSigns,
//     scheme_integer.cu:398-425), applied to every changed term;
//   a term with a zero factor is removed (compaction re-checks moved terms);
//   after a flip, term a then term b: the first term t (ascending) that
//     shares two factors with it up to sign (component pairs (0,1), (0,2),
//     (1,2); equal before negated) and whose merged third factor stays in
//     bounds absorbs it: x_r[t] += e * x_r[a], e = product of the two signs;
//   plus (a, b with all factors distinct, components permuted i, j, k):
//     (A_i - B_i, A_j, A_k), (B_i, A_j - B_j, A_k), (B_i, B_j, A_k + B_k),
//     the third dropped when zero; any bound violation rejects it;
//   split of factor x by r: (r, y, z) and (x - r, y, z); trySplit draws r
//     with entries in {-1, 0, 1} (nonzero mask, sign mask), trySplitExisted
//     takes another term's factor; five redraws at most, as SchemeZ2.
constexpr int kZBBound = 2;

struct ZBVec {
    int8_t c[kMaxMatrix];
};
inline bool zbEq(const ZBVec &a, const ZBVec &b) { return std::memcmp(a.c, b.c, kMaxMatrix) == 0; }
inline bool zbNegEq(const ZBVec &a, const ZBVec &b) {
    for (int e = 0; e < kMaxMatrix; e++)
        if (a.c[e] != -b.c[e]) return false;
    return true;
}
inline bool zbSim(const ZBVec &a, const ZBVec &b) { return zbEq(a, b) || zbNegEq(a, b); }
inline bool zbZero(const ZBVec &a) {
    for (int e = 0; e < kMaxMatrix; e++)
        if (a.c[e]) return false;
    return true;
}
inline bool zbFirstPositive(const ZBVec &a) {
    for (int e = 0; e < kMaxMatrix; e++)
        if (a.c[e]) return a.c[e] > 0;
    return true;
}
inline void zbNegate(ZBVec &a) {
    for (int e = 0; e < kMaxMatrix; e++) a.c[e] = (int8_t)-a.c[e];
}
// a + s*b; false when an entry leaves [-2, 2]
inline bool zbAdd(const ZBVec &a, const ZBVec &b, int s, ZBVec &out) {
    bool ok = true;
    for (int e = 0; e < kMaxMatrix; e++) {
        const int v = a.c[e] + s * b.c[e];
        ok &= v >= -kZBBound && v <= kZBBound;
        out.c[e] = (int8_t)v;
    }
    return ok;
}

struct ZB {
    int n[3], nn[3], m;
    ZBVec x[3][kMaxRank];
    int32_t *status;
    int retryCap = kRetryCap;  // fgo_walk_cfg::retry_cap (0 there = kRetryCap)
    int slotCap = kMaxRank;    // the records' slots per walk (fgo_walk_cfg::cap)

    int full() const { return n[0] * n[1] * n[2]; }
    bool zeroTerm(int t) const { return zbZero(x[0][t]) || zbZero(x[1][t]) || zbZero(x[2][t]); }

    void initNaive(int n1, int n2, int n3) {  // the standard scheme, as scheme_z2.cu:32-55
        n[0] = n1; n[1] = n2; n[2] = n3;
        nn[0] = n1 * n2; nn[1] = n2 * n3; nn[2] = n3 * n1;
        m = n1 * n2 * n3;
        std::memset(x, 0, sizeof(x));
        for (int i = 0; i < n1; i++)
            for (int j = 0; j < n3; j++)
                for (int k = 0; k < n2; k++) {
                    int t = (i * n3 + j) * n2 + k;
                    x[0][t].c[i * n2 + k] = 1;
                    x[1][t].c[k * n3 + j] = 1;
                    x[2][t].c[j * n1 + i] = 1;
                }
    }

    void fixSigns(int t) {
        const bool pi = zbFirstPositive(x[0][t]), pj = zbFirstPositive(x[1][t]);
        if (pi && pj) return;
        if (!pi && !pj) { zbNegate(x[0][t]); zbNegate(x[1][t]); }
        else if (!pi) { zbNegate(x[0][t]); zbNegate(x[2][t]); }
        else { zbNegate(x[1][t]); zbNegate(x[2][t]); }
    }
    void moveTerm(int dst, int src) { for (int c = 0; c < 3; c++) x[c][dst] = x[c][src]; }
    void removeAt(int t) { m--; if (t != m) moveTerm(t, m); }
    void removeZeroes() {
        for (int t = 0; t < m; t++)
            if (zeroTerm(t)) { removeAt(t); t--; }
    }
    void append(const ZBVec &a, const ZBVec &b, const ZBVec &c) {
        if (m >= kMaxRank || m >= slotCap) { *status |= ST_OVERFLOW; return; }
        x[0][m] = a; x[1][m] = b; x[2][m] = c;
        m++;
    }
    int partners(int c, int t) const {
        int k = 0;
        for (int u = 0; u < m; u++) k += u != t && zbSim(x[c][u], x[c][t]);
        return k;
    }

    // Two factors of term t equal term a's up to sign, third merged within bounds.
    bool mergeable(int a, int t, int &r, ZBVec &merged) const {
        static const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
        for (int q = 0; q < 3; q++) {
            const int p0 = pairs[q][0], p1 = pairs[q][1];
            const int e0 = zbEq(x[p0][t], x[p0][a]) ? 1 : (zbNegEq(x[p0][t], x[p0][a]) ? -1 : 0);
            if (!e0) continue;
            const int e1 = zbEq(x[p1][t], x[p1][a]) ? 1 : (zbNegEq(x[p1][t], x[p1][a]) ? -1 : 0);
            if (!e1) continue;
            r = 3 - p0 - p1;
            if (zbAdd(x[r][t], x[r][a], e0 * e1, merged)) return true;
        }
        return false;
    }
    // keep absorbs drop: x_r[keep] = merged, drop removed, keep removed too when merged is zero.
    void merge(int keep, int drop, int r, const ZBVec &merged) {
        x[r][keep] = merged;
        const bool zero = zbZero(merged);
        removeAt(drop);
        if (keep == m) keep = drop;  // the last term moved into drop's slot
        if (zero) removeAt(keep);
        else fixSigns(keep);
    }
    bool reduceWith(int a) {
        for (int t = 0; t < m; t++) {
            if (t == a) continue;
            int r;
            ZBVec merged;
            if (mergeable(a, t, r, merged)) { merge(t, a, r, merged); return true; }
        }
        return false;
    }
    bool tryReduce() {
        for (int a = 0; a < m; a++)
            for (int b = a + 1; b < m; b++) {
                int r;
                ZBVec merged;
                if (mergeable(b, a, r, merged)) { merge(a, b, r, merged); return true; }
            }
        return false;
    }

    // 1 accepted, 0 no candidate pair, -1 proposal rejected (bound).
    template <class R> int tryFlip(R &r) {
        int total[3] = {0, 0, 0};
        for (int c = 0; c < 3; c++)
            for (int t = 0; t < m; t++) total[c] += partners(c, t);
        const uint32_t P = (uint32_t)(total[0] + total[1] + total[2]);
        if (!P) return 0;
        uint32_t q = r.below(P);
        int c = 0;
        while (q >= (uint32_t)total[c]) { q -= total[c]; c++; }
        int a = 0;
        for (;; a++) {
            const uint32_t h = (uint32_t)partners(c, a);
            if (q < h) break;
            q -= h;
        }
        int b = 0;
        for (;; b++)
            if (b != a && zbSim(x[c][b], x[c][a])) {
                if (q == 0) break;
                q--;
            }
        const int e = zbEq(x[c][b], x[c][a]) ? 1 : -1;
        int j = c == 0 ? 1 : 0, k = c == 2 ? 1 : 2;
        if (r.coin()) std::swap(j, k);
        const int sg = r.coin() ? -1 : 1;
        ZBVec na, nb;
        if (!zbAdd(x[j][a], x[j][b], sg * e, na) || !zbAdd(x[k][b], x[k][a], -sg, nb)) return -1;
        x[j][a] = na;
        x[k][b] = nb;
        fixSigns(a);
        fixSigns(b);
        if (zeroTerm(a) || zeroTerm(b)) {
            removeZeroes();
            return 1;
        }
        if (!reduceWith(a)) reduceWith(b);
        return 1;
    }

    template <class R> bool tryPlus(R &r) {
        if (m >= kMaxRank || m >= full()) return false;
        int a = (int)r.below((uint32_t)m), b = (int)r.below((uint32_t)m);
        int guard = 0;
        while (a == b || zbSim(x[0][a], x[0][b]) || zbSim(x[1][a], x[1][b]) || zbSim(x[2][a], x[2][b])) {
            if (++guard > retryCap) { *status |= ST_RETRY; return false; }
            a = (int)r.below((uint32_t)m);
            b = (int)r.below((uint32_t)m);
        }
        int perm[3];
        permutation(perm, 3, r);
        const int i = perm[0], j = perm[1], k = perm[2];
        ZBVec ti, tj, tk;
        if (!zbAdd(x[i][a], x[i][b], -1, ti) || !zbAdd(x[j][a], x[j][b], -1, tj) || !zbAdd(x[k][a], x[k][b], 1, tk))
            return false;
        const ZBVec Bi = x[i][b], Bj = x[j][b], Ak = x[k][a];
        x[i][a] = ti;
        x[j][b] = tj;
        x[k][b] = Ak;
        fixSigns(a);
        fixSigns(b);
        if (!zbZero(tk)) {
            ZBVec t3[3];
            t3[i] = Bi; t3[j] = Bj; t3[k] = tk;
            append(t3[0], t3[1], t3[2]);
            fixSigns(m - 1);
        }
        return true;
    }

    template <class R> uint64_t mask64(int bits, R &r) {
        const uint64_t low = bits >= 64 ? ~0ull : ((1ull << bits) - 1);
        if (bits <= 32) return (uint64_t)r.raw() & low;
        const uint64_t lo = r.raw();
        return (lo | ((uint64_t)r.raw() << 32)) & low;
    }
    template <class R> ZBVec randomTernary(int bits, R &r) {
        const uint64_t nz = mask64(bits, r);
        const uint64_t neg = mask64(bits, r) & nz;
        ZBVec v;
        std::memset(v.c, 0, sizeof v.c);
        for (int e = 0; e < bits; e++)
            if ((nz >> e) & 1) v.c[e] = ((neg >> e) & 1) ? -1 : 1;
        return v;
    }
    // term t -> (v, y, z) and (x_i - v, y, z)
    void split(int i, int t, const ZBVec &v, const ZBVec &rest) {
        ZBVec nt[3] = {x[0][t], x[1][t], x[2][t]};
        nt[i] = rest;
        x[i][t] = v;
        fixSigns(t);
        append(nt[0], nt[1], nt[2]);
        fixSigns(m - 1);
    }
    template <class R> bool trySplit(R &r) {
        if (m >= kMaxRank || m >= full()) return false;
        const int t = (int)r.below((uint32_t)m);
        int perm[3];
        permutation(perm, 3, r);
        const int i = perm[0];
        ZBVec v = randomTernary(nn[i], r), rest;
        auto bad = [&]() { return zbZero(v) || zbEq(v, x[i][t]) || !zbAdd(x[i][t], v, -1, rest); };
        int loop = 0;
        while (loop < 5 && bad()) { v = randomTernary(nn[i], r); loop++; }
        if (loop == 5) return false;
        split(i, t, v, rest);
        return true;
    }
    template <class R> bool trySplitExisted(R &r) {
        if (m >= kMaxRank || m >= full()) return false;
        int perm[3];
        permutation(perm, 3, r);
        const int i = perm[0];
        const int a = (int)r.below((uint32_t)m);
        int b = (int)r.below((uint32_t)m);
        ZBVec rest;
        auto bad = [&]() { return a == b || zbEq(x[i][a], x[i][b]) || !zbAdd(x[i][a], x[i][b], -1, rest); };
        int loop = 0;
        while (loop < 5 && bad()) { b = (int)r.below((uint32_t)m); loop++; }
        if (loop == 5) return false;
        split(i, a, x[i][b], rest);
        return true;
    }
    template <class R> bool tryExpand(int count, R &r) {
        bool result = false;
        for (int q = 0; q < count && m < full(); q++) {
            const int v = (int)r.below(3);
            if (v == 0) result |= tryPlus(r);
            else if (v == 1) result |= trySplit(r);
            else result |= trySplitExisted(r);
        }
        return result;
    }
};

// Host records of ZB factors: sign-magnitude masks, fac = nonzero, sgn = negative, fac2 = |c| = 2.
inline void zbToMasks(const ZBVec &v, uint64_t &nz, uint64_t &neg, uint64_t &two) {
    nz = neg = two = 0;
    for (int e = 0; e < kMaxMatrix; e++) {
        if (!v.c[e]) continue;
        nz |= 1ull << e;
        if (v.c[e] < 0) neg |= 1ull << e;
        if (v.c[e] == 2 || v.c[e] == -2) two |= 1ull << e;
    }
}
inline ZBVec zbFromMasks(uint64_t nz, uint64_t neg, uint64_t two) {
    ZBVec v;
    for (int e = 0; e < kMaxMatrix; e++) {
        int c = (nz >> e) & 1 ? (((two >> e) & 1) ? 2 : 1) : 0;
        v.c[e] = (int8_t)(((neg >> e) & 1) ? -c : c);
    }
    return v;
}

void loadZB(ZB &s, const fgo_batch *b, int w, int cap) {
    for (int c = 0; c < 3; c++) s.n[c] = b->n[w * 3 + c];
    for (int c = 0; c < 3; c++) s.nn[c] = s.n[c] * s.n[(c + 1) % 3];
    s.m = b->m[w];
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < s.m; t++) {
            const size_t q = facIndex(w, c, t, cap);
            s.x[c][t] = zbFromMasks(b->fac[q], b->sgn[q], b->fac2[q]);
        }
}

void storeZBInto(const ZB &s, uint64_t *fac, uint64_t *sgn, uint64_t *fac2, int w, int cap) {
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < cap; t++) {
            const size_t q = facIndex(w, c, t, cap);
            uint64_t nz = 0, neg = 0, two = 0;
            if (t < s.m) zbToMasks(s.x[c][t], nz, neg, two);
            fac[q] = nz; sgn[q] = neg; fac2[q] = two;
        }
}

void storeZB(const ZB &s, fgo_batch *b, int w, int cap) {
    if (s.m > cap) { b->status[w] |= ST_OVERFLOW; return; }
    b->m[w] = s.m;
    for (int c = 0; c < 3; c++) b->n[w * 3 + c] = s.n[c];
    storeZBInto(s, b->fac, b->sgn, b->fac2, w, cap);
}

void storeBestZB(const ZB &s, fgo_batch *b, int w, int cap) {
    if (s.m > cap) { b->status[w] |= ST_OVERFLOW; return; }
    b->best_m[w] = s.m;
    storeZBInto(s, b->best_fac, b->best_sgn, b->best_fac2, w, cap);
}

// The fast-mode walk launch over ZB (the Z2 fast walk's loop, flip_graph.cu:526-569
// shape, with the bound's rejected proposals spending their step).
template <class R>
void walkLaunchZB(ZB &s, R &r, const fgo_walk_cfg *cfg, fgo_batch *b, int w) {
    const int cap = cfg->cap;
    int flipsCount = b->flips[w];
    int bestRank = b->best_rank[w];
    int bestM = b->best_m[w];
    for (int it = 0; it < cfg->iterations; it++) {
        const int rank = s.m;
        const int f = s.tryFlip(r);
        if (f == 0) {
            s.tryExpand(randint(1, 2, r), r);
            if (*s.status) break;
            continue;
        }
        if (f < 0) continue;
        if (b->accepted) b->accepted[w]++;
        if (s.m < rank) flipsCount = 0;
        flipsCount++;
        if (s.m < bestRank || (s.m == bestRank && r.tie())) {
            bestRank = s.m;
            storeBestZB(s, b, w, cap);
            bestM = s.m;
        }
        if (r.gate(cfg->reduce_p, cfg->iterations)) s.tryReduce();
        if (r.gate(cfg->expand_p, cfg->iterations) && s.m <= bestM + 2) {
            if (s.tryExpand(randint(1, 2, r), r)) flipsCount = 0;
        }
        if (flipsCount >= cfg->plus_iterations && s.tryPlus(r)) flipsCount = 0;
        if (*s.status) break;
    }
    b->flips[w] = flipsCount;
    b->best_rank[w] = bestRank;
}

void runWalksZB(const fgo_walk_cfg *cfg, int S, fgo_batch *b) {
    ZB *s = new ZB;
    for (int w = 0; w < S; w++) {
        std::memset(s->x, 0, sizeof(s->x));
        loadZB(*s, b, w, cfg->cap);
        s->status = &b->status[w];
        s->retryCap = retry_cap(cfg);
        s->slotCap = cfg->cap;
        FastDraws r;
        r.key[0] = (uint32_t)cfg->seed;
        r.key[1] = (uint32_t)(cfg->seed >> 32);
        r.walk = (uint32_t)w;
        r.pos = b->rng_pos[w];
        r.status = &b->status[w];
        for (int L = 0; L < cfg->launches && !b->status[w]; L++) walkLaunchZB(*s, r, cfg, b, w);
        b->rng_pos[w] = r.pos;
        storeZB(*s, b, w, cfg->cap);
    }
    delete s;
}

}  // namespace

// ============================================================ additions reducer
namespace {

enum { GREEDY = 0, GREEDY_ALT = 1, GREEDY_RANDOM = 2, GREEDY_INTER = 3, WEIGHTED_RANDOM = 4, MIX = 5, RANDOM = 6 };

struct Pair { int i, j, count; };

// PairsCounter (pairs_counter.cuh): pairs kept in first-insertion order with
// counts; the open-addressing table only locates them, so an ordinary map
// gives the same order.  Pairs beyond maxPairs are dropped (pairs_counter.cuh:242).
struct PairCounter {
    int maxPairs;
    std::vector<Pair> pairs;
    int topSize = 0, maxCount = 0;
    std::unordered_map<uint64_t, int> where;
    void clear() { pairs.clear(); where.clear(); topSize = 0; maxCount = 0; }
    void insert(int i, int j) {
        if (std::abs(i) > std::abs(j)) std::swap(i, j);  // canonizePair
        if (i < 0) { i = -i; j = -j; }
        uint64_t key = ((uint64_t)(uint32_t)i << 32) | (uint32_t)j;
        auto it = where.find(key);
        int idx;
        if (it == where.end()) {
            if ((int)pairs.size() >= maxPairs) return;
            idx = (int)pairs.size();
            pairs.push_back({i, j, 0});
            where[key] = idx;
        } else {
            idx = it->second;
        }
        if (++pairs[idx].count > maxCount) maxCount = pairs[idx].count;
    }
    void sort() {  // pairs_counter.cuh:73-101
        int size = (int)pairs.size();
        if (maxCount < 2) { topSize = size; return; }
        topSize = 0;
        for (int i = 0; i < size; i++) {
            if (pairs[i].count != maxCount) continue;
            if (i != topSize) std::swap(pairs[i], pairs[topSize]);
            topSize++;
        }
        int j = topSize;
        for (int i = topSize; i < size; i++)
            if (pairs[i].count > 1) pairs[j++] = pairs[i];
        pairs.resize(j);
    }
    bool any() const { return !pairs.empty() && maxCount > 1; }
};

bool intersects(const Pair &a, const Pair &b) {
    return a.i == b.i || a.i == std::abs(b.j) || std::abs(a.j) == b.i || std::abs(a.j) == std::abs(b.j);
}

// Whether nvcc's default floating-point contraction (--fmad=true) fused the
// multiply-adds of getGreedyIntersections (pairs_counter.cuh:163,167) in the
// reference build; pinned by the golden reducer fixtures.
int g_fuse_float = 1;
int g_fuse_double = 1;

struct Reducer {  // AdditionsReducer<maxExpr, maxFresh, maxLen, maxSub>
    int maxFresh, maxLen;
    std::vector<std::vector<int>> expr;
    std::vector<std::pair<int, int>> vars;
    PairCounter sub;
    int realVariables = 0, freshVariables = 0, naiveAdditions = 0, mode = GREEDY;
    float scale = -1;

    void clear() { expr.clear(); vars.clear(); realVariables = freshVariables = naiveAdditions = 0; }
    void setMode(int md) { mode = md; scale = -1; }

    bool addExpression(const int *values, int count) {  // additions_reducer.cuh:67-86
        std::vector<int> e;
        for (int i = 0; i < count; i++) {
            if (values[i] == 1) e.push_back(i + 1);
            else if (values[i] == -1) e.push_back(-(i + 1));
            else if (values[i] != 0) return false;
        }
        if (count > realVariables) realVariables = count;
        naiveAdditions += (int)e.size() - 1;
        expr.push_back(e);
        return true;
    }

    int additions() const {
        int a = freshVariables;
        for (auto &e : expr) a += (int)e.size() - 1;
        return a;
    }

    static int search(const std::vector<int> &e, int value, int start) {  // additions_reducer.cuh:247-269
        int lo = start, hi = (int)e.size() - 1, va = std::abs(value);
        while (lo <= hi) {
            int mid = lo + (hi - lo) / 2;
            int ma = std::abs(e[mid]);
            if (ma < va) lo = mid + 1;
            else if (ma > va) hi = mid - 1;
            else return mid;
        }
        return -1;
    }

    void replace(int pi, int pj) {  // additions_reducer.cuh:218-245,291-301
        int var = realVariables + freshVariables + 1;
        for (auto &e : expr) {
            if (e.size() < 2) continue;
            int i = search(e, pi, 0);
            if (i == -1) continue;
            int j = search(e, pj, i + 1);
            if (j == -1) continue;
            int v;
            if (e[i] == pi && e[j] == pj) v = var;
            else if (e[i] == -pi && e[j] == -pj) v = -var;
            else continue;
            std::vector<int> out;
            for (int q = 0; q < (int)e.size(); q++)
                if (q != i && q != j) out.push_back(e[q]);
            out.push_back(v);
            e.swap(out);
        }
        vars.push_back({pi, pj});
        freshVariables++;
    }

    void update() {  // additions_reducer.cuh:207-216
        sub.clear();
        for (auto &e : expr)
            for (size_t i = 0; i < e.size(); i++)
                for (size_t j = i + 1; j < e.size(); j++) sub.insert(e[i], e[j]);
        sub.sort();
    }

    template <class R> Pair select(int md, R &r) {  // additions_reducer.cuh:272-289
        auto &p = sub.pairs;
        int size = (int)p.size();
        if (md == GREEDY) return p[0];
        if (md == GREEDY_ALT) return p[r.raw() % (uint32_t)sub.topSize];
        if (md == GREEDY_RANDOM) {
            if (r.uniform() < scale) return p[r.raw() % (uint32_t)size];
            return p[r.raw() % (uint32_t)sub.topSize];
        }
        if (md == GREEDY_INTER) {  // pairs_counter.cuh:148-176
            int imax = 0;
            float maxScore = 0;
            for (int i = 0; i < size; i++) {
                float inter = 0;
                for (int j = 0; j < size; j++) {
                    if (i == j) continue;
                    if (!intersects(p[i], p[j])) {
                        inter += (float)(p[j].count - 1);
                    } else {
                        bool skip = r.raw() % 2;
                        if (!skip) {
                            double add = g_fuse_double ? std::fma(0.69, (double)p[j].count, (double)inter)
                                                       : (double)inter + 0.69 * (double)p[j].count;
                            inter = (float)add;
                        }
                    }
                }
                float score = g_fuse_float ? std::fmaf(scale, inter, (float)(p[i].count - 1))
                                           : (float)(p[i].count - 1) + scale * inter;
                if (score > maxScore) { maxScore = score; imax = i; }
            }
            return p[imax];
        }
        if (md == WEIGHTED_RANDOM) {  // pairs_counter.cuh:178-196
            float total = 0;
            for (int i = 0; i < size; i++) total += (float)p[i].count;
            float x = r.uniform() * total;
            float sum = 0;
            for (int i = 0; i < size; i++) {
                sum += (float)p[i].count;
                if (x <= sum) return p[i];
            }
            return p[size - 1];
        }
        return p[r.raw() % (uint32_t)size];
    }

    template <class R> void reduce(R &r) {  // additions_reducer.cuh:89-103
        if (scale < 0) scale = r.uniform() / 2;
        while (freshVariables < maxFresh) {
            update();
            if (!sub.any()) break;
            int md = mode == MIX ? (int)(r.raw() % MIX) : mode;
            Pair s = select(md, r);
            replace(s.i, s.j);
        }
    }

    void partialInitialize(const std::vector<std::pair<int, int>> &bestVars, int count) {
        for (int q = 0; q < count && q < (int)bestVars.size(); q++) replace(bestVars[q].first, bestVars[q].second);
    }
};

const int kModes[15] = {GREEDY_INTER, GREEDY_INTER, GREEDY_INTER, GREEDY_INTER, GREEDY_INTER, GREEDY_INTER,
                        GREEDY_INTER, GREEDY_INTER, GREEDY_ALT, GREEDY_ALT, GREEDY_ALT, GREEDY_ALT,
                        GREEDY_RANDOM, GREEDY_RANDOM, MIX};

}  // namespace

struct fgo_reducer_state {
    std::vector<std::pair<int, int>> vars[3];
};

// ------------------------------------------------------------ resizing
std::string sizeKey(const int n[3]) {  // getKey(scheme) with sorted sizes (utils.cu:3-25)
    int a[3] = {n[0], n[1], n[2]};
    std::sort(a, a + 3);
    return std::to_string(a[0]) + "x" + std::to_string(a[1]) + "x" + std::to_string(a[2]);
}

void loadBest(Z2 &s, const fgo_batch *b, int w, int cap) {
    for (int c = 0; c < 3; c++) s.n[c] = b->best_n ? b->best_n[w * 3 + c] : b->n[w * 3 + c];
    for (int c = 0; c < 3; c++) s.nn[c] = s.n[c] * s.n[(c + 1) % 3];
    s.m = b->best_m[w];
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < s.m; t++) s.x[c][t] = b->best_fac[facIndex(w, c, t, cap)];
}

void loadBest(ZT &s, const fgo_batch *b, int w, int cap) {
    for (int c = 0; c < 3; c++) s.n[c] = b->best_n ? b->best_n[w * 3 + c] : b->n[w * 3 + c];
    for (int c = 0; c < 3; c++) s.nn[c] = s.n[c] * s.n[(c + 1) % 3];
    s.m = b->best_m[w];
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < s.m; t++) {
            const size_t q = facIndex(w, c, t, cap);
            s.x[c][t].v = b->best_fac[q];
            s.x[c][t].s = b->best_sgn[q];
            s.x[c][t].ok = b->best_valid[q] != 0;
        }
}

// resizeKernel body (flip_graph.cu:575-613) for walk w; `best` holds every walk's best scheme.
template <class Scheme, class R>
void resizeStep(Scheme &s, R &r, const std::vector<Scheme> &best, int S, double p) {
    if ((double)r.uniform() > p) return;
    if ((double)r.uniform() < 0.5) s.swapSizeRandom(r);
    bool merged = false;
    for (int i = 0; i < 3 && !merged; i++) {
        const int index = (int)(r.raw() % (uint32_t)S);
        merged |= s.tryMerge(best[index], r);
    }
    if (merged) return;
    const double q = (double)r.uniform();
    if (q < 0.05) s.tryProject(r);
    else if (q < 0.55) s.tryProductWith(best[(int)(r.raw() % (uint32_t)S)]);
    else if (q < 0.85) s.tryProduct(r);
    else s.tryExtend(r);
}

// updateRanks (flip_graph.cu:249-266): the best rank per (sorted) size; a walk that
// improves it has its current scheme copied to its best slot; every walk's best rank
// becomes its size's.
template <class Scheme>
void updateRanks(std::map<std::string, int> &table, std::vector<Scheme> &cur, std::vector<Scheme> &best, fgo_batch *b,
                 int S, int cap) {
    std::vector<std::string> keys(S);
    for (int w = 0; w < S; w++) {
        keys[w] = sizeKey(cur[w].n);
        auto it = table.find(keys[w]);
        if (it == table.end() || cur[w].m < it->second) {
            table[keys[w]] = cur[w].m;
            best[w] = cur[w];
            storeBest(cur[w], b, w, cap);
        }
    }
    for (int w = 0; w < S; w++) b->best_rank[w] = table[keys[w]];
}

// FlipGraph::run with --resize-probability > 0 (flip_graph.cu:286-299): launches of every
// walk, then the resize step of every walk, then the best-rank table.  The table starts from
// the first walk's size at the naive rank, as the constructor sets it (flip_graph.cu:19), and
// an update over the starting schemes (FlipGraph::initialize, flip_graph.cu:190-198).
template <class Scheme, class R>
void runResize(const fgo_walk_cfg *cfg, int S, fgo_batch *b, std::vector<R> &rs) {
    const int cap = cfg->cap;
    std::vector<Scheme> cur(S), best(S);
    for (int w = 0; w < S; w++) {
        loadScheme(cur[w], b, w, cap);
        loadBest(best[w], b, w, cap);
        cur[w].status = best[w].status = &b->status[w];
        cur[w].retryCap = best[w].retryCap = retry_cap(cfg);
        cur[w].slotCap = best[w].slotCap = cap;
        setImplicit(cur[w], cfg->rng == FGO_RNG_FAST);  // the fast mode: implicit pairs, no lists
        setImplicit(best[w], cfg->rng == FGO_RNG_FAST);
        setMaxMatrix(cur[w], cfg->rng == FGO_RNG_FAST ? 56 : kMaxMatrix);
    }
    std::map<std::string, int> table;
    table[sizeKey(cur[0].n)] = cur[0].n[0] * cur[0].n[1] * cur[0].n[2];
    updateRanks(table, cur, best, b, S, cap);
    for (int L = 0; L < cfg->launches; L++) {
        for (int w = 0; w < S; w++) {
            if (b->status[w]) continue;
            walkLaunch(cur[w], rs[w], cfg, b, w);
            loadBest(best[w], b, w, cap);
        }
        for (int w = 0; w < S; w++) {
            if (b->status[w]) continue;
            // The fast mode's resize step keeps the reference's list order (each operator
            // rebuilds the lists, and its reductions follow them); its walk then drops them.
            const bool fast = cfg->rng == FGO_RNG_FAST;
            if (fast) setImplicit(cur[w], false);
            resizeStep(cur[w], rs[w], best, S, cfg->resize_p);
            if (fast) { setImplicit(cur[w], true); rebuildIfList(cur[w]); }
        }
        updateRanks(table, cur, best, b, S, cap);
    }
    for (int w = 0; w < S; w++) {
        storeScheme(cur[w], b, w, cap);
        b->rng_pos[w] = rs[w].pos;
    }
}

template <class Scheme>
void runWalksResize(const fgo_walk_cfg *cfg, int S, fgo_batch *b, const fgo_tape *tape) {
    if (cfg->rng == FGO_RNG_TAPE) {
        std::vector<RefDraws> rs(S);
        for (int w = 0; w < S; w++) {
            RefDraws &r = rs[w];
            r.d = tape->draws + tape->offsets[w];
            r.u = tape->uniforms + tape->offsets[w];
            r.n = tape->offsets[w + 1] - tape->offsets[w];
            r.pos = b->rng_pos[w];
            r.status = &b->status[w];
        }
        runResize<Scheme>(cfg, S, b, rs);
    } else {
        std::vector<FastDraws> rs(S);
        for (int w = 0; w < S; w++) {
            FastDraws &r = rs[w];
            r.key[0] = (uint32_t)cfg->seed;
            r.key[1] = (uint32_t)(cfg->seed >> 32);
            r.walk = (uint32_t)w;
            r.pos = b->rng_pos[w];
            r.status = &b->status[w];
        }
        runResize<Scheme>(cfg, S, b, rs);
    }
}

extern "C" {

void fgo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { philox(ctr, key, out); }

void fgo_set_fma(int fuse_float, int fuse_double) { g_fuse_float = fuse_float; g_fuse_double = fuse_double; }

int fgo_init_naive(const fgo_walk_cfg *cfg, int S, int n1, int n2, int n3, fgo_batch *b) {
    int bad = 0;
    if (cfg->ring == FGO_RING_ZB) {
        ZB *s = new ZB;
        for (int w = 0; w < S; w++) {
            s->status = &b->status[w];
            s->initNaive(n1, n2, n3);
            storeZB(*s, b, w, cfg->cap);
            storeBestZB(*s, b, w, cfg->cap);
            b->best_rank[w] = n1 * n2 * n3;
            b->flips[w] = 0;
            bad += b->status[w] != 0;
        }
        delete s;
        return bad;
    }
    if (cfg->ring == FGO_RING_Z2) {
        Z2 *s = new Z2;
        for (int w = 0; w < S; w++) {
            s->status = &b->status[w];
            s->initNaive(n1, n2, n3);
            storeZ2(*s, b, w, cfg->cap);
            storeBestZ2(*s, b, w, cfg->cap);
            b->best_rank[w] = n1 * n2 * n3;
            b->flips[w] = 0;
            bad += b->status[w] != 0;
        }
        delete s;
    } else {
        ZT *s = new ZT;
        for (int w = 0; w < S; w++) {
            s->status = &b->status[w];
            s->initNaive(n1, n2, n3);
            storeZT(*s, b, w, cfg->cap);
            storeBestZT(*s, b, w, cfg->cap);
            b->best_rank[w] = n1 * n2 * n3;
            b->flips[w] = 0;
            bad += b->status[w] != 0;
        }
        delete s;
    }
    return bad;
}

int fgo_walk(const fgo_walk_cfg *cfg, int S, fgo_batch *b, const fgo_tape *tape) {
    struct Flag {
        explicit Flag(int on) { g_ternarySandwich = on; }
        ~Flag() { g_ternarySandwich = 0; }
    } flag(cfg->zt_sandwich);
    if (cfg->ring == FGO_RING_ZB) {
        if (cfg->rng != FGO_RNG_FAST || cfg->resize_p > 0 || cfg->sandwich_p > 0 || cfg->basis_p > 0 || cfg->gauss_p > 0)
            return -1;
        runWalksZB(cfg, S, b);
        int bad = 0;
        for (int w = 0; w < S; w++) bad += b->status[w] != 0;
        return bad;
    }
    if (cfg->resize_p > 0) {
        if (cfg->rng == FGO_RNG_FAST && cfg->ring != FGO_RING_Z2) return -1;
        if (cfg->ring == FGO_RING_Z2) runWalksResize<Z2>(cfg, S, b, tape);
        else runWalksResize<ZT>(cfg, S, b, tape);
        int bad = 0;
        for (int w = 0; w < S; w++) bad += b->status[w] != 0;
        return bad;
    }
    if (cfg->ring == FGO_RING_Z2) runWalks<Z2>(cfg, S, b, tape);
    else runWalks<ZT>(cfg, S, b, tape);
    int bad = 0;
    for (int w = 0; w < S; w++) bad += b->status[w] != 0;
    return bad;
}

// ============================================================ proposal bound
// How many steps a better flip proposal can save the fast-mode walk (no reference
// counterpart; bounds what a learned proposal can gain).  greedy = 0: the uniform
// proposal (tryFlipImplicit).  greedy = 1: an exact one-step lookahead: every ordered
// equal pair and orientation is applied to a copy of the scheme (with the reduction
// test), and when some of them lower the rank one of those is taken uniformly, else
// the uniform proposal runs.  The rest of a step is the fast walk's (flip_graph.cu:
// 533-569): expansion when no pair exists or by its gate while m <= best + 2, plus
// after plus_iterations flips without a drop.  steps[w] = the steps walk w (Philox
// stream w of seed) took from the naive scheme until its rank first reached target,
// or -1 when it did not within max_steps.
namespace {
bool greedyFlip(Z2 &s, Z2 &tmp, std::vector<uint32_t> &cand, FastDraws &r) {
    cand.clear();
    for (int c = 0; c < 3; c++)
        for (int a = 0; a < s.m; a++)
            for (int b = 0; b < s.m; b++) {
                if (a == b || s.x[c][a] != s.x[c][b]) continue;
                for (int o = 0; o < 2; o++) {
                    tmp.m = s.m;
                    for (int q = 0; q < 3; q++) std::memcpy(tmp.x[q], s.x[q], sizeof(uint64_t) * s.m);
                    int i = c, j = c == 0 ? 1 : 0, k = c == 2 ? 1 : 2;
                    if (o) std::swap(j, k);
                    tmp.flip(i, j, k, a, b, true);
                    if (tmp.m < s.m) cand.push_back((uint32_t)(c << 24 | a << 14 | b << 4 | o));
                }
            }
    if (cand.empty()) return false;
    const uint32_t p = cand[r.below((uint32_t)cand.size())];
    const int c = (int)(p >> 24), a = (int)((p >> 14) & 1023), b = (int)((p >> 4) & 1023);
    int i = c, j = c == 0 ? 1 : 0, k = c == 2 ? 1 : 2;
    if (p & 1) std::swap(j, k);
    s.flip(i, j, k, a, b, true);
    return true;
}
}  // namespace

int fgo_lookahead_ttr(int n1, int n2, int n3, int walks, int target, int64_t max_steps, int plus_iterations,
                      double expand_p, int iterations, uint64_t seed, int greedy, int64_t *steps) {
    if (n1 < 1 || n2 < 1 || n3 < 1 || n1 * n2 * n3 > kMaxRank - 2 || n1 * n2 > 64 || n2 * n3 > 64 || n3 * n1 > 64)
        return -1;
    Z2 *s = new Z2, *tmp = new Z2;
    std::vector<uint32_t> cand;
    int32_t st = 0, tst = 0;
    int failed = 0;
    for (int w = 0; w < walks; w++) {
        st = 0;
        s->implicit = true;
        s->status = &st;
        s->initNaive(n1, n2, n3);
        *tmp = *s;
        tmp->status = &tst;
        FastDraws r;
        r.key[0] = (uint32_t)seed;
        r.key[1] = (uint32_t)(seed >> 32);
        r.walk = (uint32_t)w;
        r.pos = 0;
        r.status = &st;
        steps[w] = -1;
        int flipsCount = 0, best = s->m;
        for (int64_t it = 0; it < max_steps; it++) {
            const int rank = s->m;
            const bool flipped = (greedy && greedyFlip(*s, *tmp, cand, r)) || s->tryFlip(r, true);
            if (!flipped) {
                s->tryExpand(randint(1, 2, r), r);
                if (st) break;
                continue;
            }
            if (s->m < rank) flipsCount = 0;
            flipsCount++;
            if (s->m <= target) { steps[w] = it + 1; break; }
            if (s->m < best) best = s->m;
            if (r.gate(expand_p, iterations) && s->m <= best + 2) {
                if (s->tryExpand(randint(1, 2, r), r)) flipsCount = 0;
            }
            if (flipsCount >= plus_iterations && s->tryPlus(r)) flipsCount = 0;
            if (st) break;
        }
        failed += steps[w] < 0;
    }
    delete s;
    delete tmp;
    return failed;
}

int fgo_reduce_gauss(const fgo_walk_cfg *cfg, int S, fgo_batch *b, const fgo_tape *tape, int32_t *found) {
    if (cfg->ring != FGO_RING_Z2) return -1;
    Z2 *s = new Z2;
    for (int w = 0; w < S; w++) {
        loadScheme(*s, b, w, cfg->cap);
        s->status = &b->status[w];
        bool hit;
        if (cfg->rng == FGO_RNG_TAPE) {
            RefDraws r;
            r.d = tape->draws + tape->offsets[w];
            r.u = tape->uniforms + tape->offsets[w];
            r.n = tape->offsets[w + 1] - tape->offsets[w];
            r.pos = b->rng_pos[w];
            r.status = &b->status[w];
            hit = s->tryReduceGauss(r, false);
            b->rng_pos[w] = r.pos;
        } else {
            FastDraws r;
            r.key[0] = (uint32_t)cfg->seed;
            r.key[1] = (uint32_t)(cfg->seed >> 32);
            r.walk = (uint32_t)w;
            r.pos = b->rng_pos[w];
            r.status = &b->status[w];
            hit = s->tryReduceGauss(r, false);
            b->rng_pos[w] = r.pos;
        }
        found[w] = hit ? 1 : 0;
        storeScheme(*s, b, w, cfg->cap);
    }
    delete s;
    return 0;
}

int fgo_minimize(const fgo_walk_cfg *cfg, int S, fgo_batch *b, const fgo_tape *tape, int32_t *best_complexity) {
    if (cfg->ring == FGO_RING_Z2) runMinimize<Z2>(cfg, S, b, tape, best_complexity);
    else runMinimize<ZT>(cfg, S, b, tape, best_complexity);
    int bad = 0;
    for (int w = 0; w < S; w++) bad += b->status[w] != 0;
    return bad;
}

int fgo_validate(int ring, int S, int cap, const int32_t *n, const int32_t *m, const uint64_t *fac,
                 const uint64_t *sgn, const uint8_t *valid, uint8_t *valid_out) {
    int good = 0;
    for (int w = 0; w < S; w++) {
        int n0 = n[w * 3], n1 = n[w * 3 + 1], n2 = n[w * 3 + 2];
        int nn0 = n0 * n1, nn1 = n1 * n2, nn2 = n2 * n0, mm = m[w];
        bool ok = true;
        const uint64_t *u = fac + facIndex(w, 0, 0, cap), *v = fac + facIndex(w, 1, 0, cap), *x = fac + facIndex(w, 2, 0, cap);
        if (ring == FGO_RING_Z2) {
            // Bit-sliced over k: the reference's per-(i,j,k) XOR (scheme_z2.cu:3-29).
            for (int i = 0; i < nn0 && ok; i++)
                for (int j = 0; j < nn1 && ok; j++) {
                    uint64_t acc = 0;
                    for (int t = 0; t < mm; t++)
                        if (((u[t] >> i) & 1) && ((v[t] >> j) & 1)) acc ^= x[t];
                    for (int k = 0; k < nn2 && ok; k++) {
                        int target = (i % n1 == j / n2) && (i / n1 == k % n0) && (j % n2 == k / n0);
                        if ((int)((acc >> k) & 1) != target) ok = false;
                    }
                }
        } else {
            const uint64_t *us = sgn + facIndex(w, 0, 0, cap), *vs = sgn + facIndex(w, 1, 0, cap), *xs = sgn + facIndex(w, 2, 0, cap);
            auto coef = [](uint64_t vv, uint64_t ss, int idx) { int r = (int)((vv >> idx) & 1); return ((ss >> idx) & 1) ? -r : r; };
            for (int i = 0; i < nn0 && ok; i++)
                for (int j = 0; j < nn1 && ok; j++)
                    for (int k = 0; k < nn2 && ok; k++) {
                        int target = (i % n1 == j / n2) && (i / n1 == k % n0) && (j % n2 == k / n0);
                        int e = 0;
                        for (int t = 0; t < mm; t++) e += coef(u[t], us[t], i) * coef(v[t], vs[t], j) * coef(x[t], xs[t], k);
                        if (e != target) ok = false;
                    }
            for (int c = 0; c < 3 && ok; c++)
                for (int t = 0; t < mm; t++)
                    if (!valid[facIndex(w, c, t, cap)]) { ok = false; break; }
        }
        valid_out[w] = ok;
        good += ok;
    }
    return good;
}

int fgo_validate_zb(int S, int cap, const int32_t *n, const int32_t *m, const uint64_t *fac, const uint64_t *sgn,
                    const uint64_t *fac2, uint8_t *valid_out) {
    int good = 0;
    for (int w = 0; w < S; w++) {
        const int n0 = n[w * 3], n1 = n[w * 3 + 1], n2 = n[w * 3 + 2];
        const int nn0 = n0 * n1, nn1 = n1 * n2, nn2 = n2 * n0, mm = m[w];
        auto coef = [&](int c, int t, int e) {
            const size_t q = facIndex(w, c, t, cap);
            const int a = (fac[q] >> e) & 1 ? (((fac2[q] >> e) & 1) ? 2 : 1) : 0;
            return ((sgn[q] >> e) & 1) ? -a : a;
        };
        bool ok = true;
        for (int i = 0; i < nn0 && ok; i++)
            for (int j = 0; j < nn1 && ok; j++)
                for (int k = 0; k < nn2 && ok; k++) {
                    const int target = (i % n1 == j / n2) && (i / n1 == k % n0) && (j % n2 == k / n0);
                    int e = 0;
                    for (int t = 0; t < mm; t++) e += coef(0, t, i) * coef(1, t, j) * coef(2, t, k);
                    if (e != target) ok = false;
                }
        valid_out[w] = ok;
        good += ok;
    }
    return good;
}

int fgo_complexity(int ring, int S, int cap, const int32_t *n, const int32_t *m, const uint64_t *fac, int32_t *out) {
    (void)ring;
    for (int w = 0; w < S; w++) {
        int count = 0;
        for (int c = 0; c < 3; c++)
            for (int t = 0; t < m[w]; t++) count += popc64(fac[facIndex(w, c, t, cap)]);
        out[w] = count - 2 * m[w] - n[w * 3 + 2] * n[w * 3];
    }
    return 0;
}

// Reducer sizes per config.cuh:16-32 with AdditionsReducer's template order
// <maxExpressions, maxFresh, maxExpressionLength, maxSubexpressions>.
}  // extern "C"

// runReducersKernel (scheme_additions_reducer.cu:494-540) for reducers 0..count-1;
// reducer idx reduces scheme idx % schemes (coef [schemes][3][m][64], rank ranks[s]
// or m).  vars_out (may be NULL): [count][3][500][2] fresh variables.
static int reduce_impl(int n1, int n2, int n3, int m, const int8_t *coef, const int32_t *ranks, int schemes,
                       int count, int independent, const fgo_tape *tape, int rng, uint64_t seed, int32_t *out,
                       int32_t *modes, int64_t *consumed, const fgo_reducer_state *best,
                       fgo_reducer_state **best_out, int32_t *vars_out) {
    const int nn[3] = {n1 * n2, n2 * n3, n3 * n1};
    const int maxFresh[3] = {250, 250, 500};
    const int maxLen[3] = {32, 32, 175};
    const int maxSub[3] = {2016, 2016, 61075};
    int bad = 0;
    std::vector<Reducer> all((size_t)count * 3);
    for (int idx = 0; idx < count; idx++) {
        int32_t status = 0;
        RefDraws rt;
        FastDraws rf;
        if (rng == FGO_RNG_TAPE) {
            rt.d = tape->draws + tape->offsets[idx];
            rt.u = tape->uniforms + tape->offsets[idx];
            rt.n = tape->offsets[idx + 1] - tape->offsets[idx];
            rt.status = &status;
        } else {
            rf.key[0] = (uint32_t)seed;
            rf.key[1] = (uint32_t)(seed >> 32);
            rf.walk = (uint32_t)idx;
            rf.status = &status;
        }
        Reducer *R = &all[(size_t)idx * 3];
        for (int p = 0; p < 3; p++) {
            R[p].maxFresh = maxFresh[p];
            R[p].maxLen = maxLen[p];
            R[p].sub.maxPairs = maxSub[p];
        }
        // copySchemeToReducers (scheme_additions_reducer.cu:463-492) of schemes[idx % schemesCount]
        const int8_t *cf = coef + (size_t)(idx % schemes) * 3 * m * 64;
        const int ms = ranks ? ranks[idx % schemes] : m;
        std::vector<int> row(std::max(m, 64));
        for (int t = 0; t < ms; t++) {
            for (int i = 0; i < nn[0]; i++) row[i] = cf[((size_t)0 * m + t) * 64 + i];
            R[0].addExpression(row.data(), nn[0]);
        }
        for (int t = 0; t < ms; t++) {
            for (int i = 0; i < nn[1]; i++) row[i] = cf[((size_t)1 * m + t) * 64 + i];
            R[1].addExpression(row.data(), nn[1]);
        }
        for (int i = 0; i < nn[2]; i++) {
            for (int t = 0; t < ms; t++) row[t] = cf[((size_t)2 * m + t) * 64 + i];
            R[2].addExpression(row.data(), ms);
        }
        auto body = [&](auto &r) {
            for (int p = 0; p < 3; p++) R[p].setMode(idx == 0 ? GREEDY : kModes[r.raw() % 15]);
            static const std::vector<std::pair<int, int>> empty;
            const std::vector<std::pair<int, int>> *bv[3] = {&empty, &empty, &empty};
            if (best) for (int p = 0; p < 3; p++) bv[p] = &best->vars[p];
            if (independent) {
                for (int p = 0; p < 3; p++)
                    if ((double)r.uniform() < 0.3 && !bv[p]->empty())
                        R[p].partialInitialize(*bv[p], 1 + (int)(r.raw() % (uint32_t)bv[p]->size()));
            } else if ((double)r.uniform() < 0.3) {
                for (int p = 0; p < 3; p++)
                    if (!bv[p]->empty()) R[p].partialInitialize(*bv[p], 1 + (int)(r.raw() % (uint32_t)bv[p]->size()));
            }
            for (int p = 0; p < 3; p++) R[p].reduce(r);
        };
        if (rng == FGO_RNG_TAPE) { body(rt); if (consumed) consumed[idx] = rt.pos; }
        else { body(rf); if (consumed) consumed[idx] = rf.pos; }
        for (int p = 0; p < 3; p++) {
            out[idx * 9 + p * 3 + 0] = R[p].additions();
            out[idx * 9 + p * 3 + 1] = R[p].freshVariables;
            out[idx * 9 + p * 3 + 2] = R[p].naiveAdditions;
            if (modes) modes[idx * 3 + p] = R[p].mode;
            if (vars_out)
                for (size_t q = 0; q < R[p].vars.size() && q < 500; q++) {
                    vars_out[(((size_t)idx * 3 + p) * 500 + q) * 2] = R[p].vars[q].first;
                    vars_out[(((size_t)idx * 3 + p) * 500 + q) * 2 + 1] = R[p].vars[q].second;
                }
        }
        bad += status != 0;
    }
    if (best_out) {
        fgo_reducer_state *st = new fgo_reducer_state;
        // Per-component incumbents: lowest (additions, fresh) over reducers, first index on ties.
        for (int p = 0; p < 3; p++) {
            int bi = 0;
            for (int idx = 1; idx < count; idx++) {
                const Reducer &a = all[(size_t)idx * 3 + p], &c = all[(size_t)bi * 3 + p];
                if (a.additions() < c.additions() || (a.additions() == c.additions() && a.freshVariables < c.freshVariables)) bi = idx;
            }
            st->vars[p] = all[(size_t)bi * 3 + p].vars;
        }
        *best_out = st;
    }
    return bad;
}

extern "C" {

int fgo_reduce(int n1, int n2, int n3, int m, const int8_t *coef, int count, int independent,
               const fgo_tape *tape, int rng, uint64_t seed, int32_t *out, int32_t *modes,
               int64_t *consumed, const fgo_reducer_state *best, fgo_reducer_state **best_out) {
    return reduce_impl(n1, n2, n3, m, coef, nullptr, 1, count, independent, tape, rng, seed, out, modes, consumed,
                       best, best_out, nullptr);
}

int fgo_reduce_schemes(int n1, int n2, int n3, int m, const int8_t *coef, const int32_t *ranks, int schemes,
                       int count, int independent, const fgo_tape *tape, int32_t *out, int32_t *modes,
                       int64_t *consumed, const fgo_reducer_state *best, int32_t *vars_out) {
    return reduce_impl(n1, n2, n3, m, coef, ranks, schemes, count, independent, tape, FGO_RNG_TAPE, 0, out, modes,
                       consumed, best, nullptr, vars_out);
}

// flipSchemesKernel (scheme_additions_reducer.cu:448-460).
int fgo_flip_schemes(int n1, int n2, int n3, int m, const int8_t *coef0, int schemes, int max_flips,
                     const fgo_tape *tape, int8_t *coef_out, int32_t *ranks_out, int64_t *consumed) {
    const int nn[3] = {n1 * n2, n2 * n3, n3 * n1};
    std::memcpy(coef_out, coef0, (size_t)3 * m * 64);
    ranks_out[0] = m;
    if (consumed) consumed[0] = 0;
    int bad = 0;
    std::vector<ZT> scratch(1);
    ZT &z = scratch[0];
    for (int idx = 1; idx < schemes; idx++) {
        int32_t status = 0;
        RefDraws rt;
        rt.d = tape->draws + tape->offsets[idx];
        rt.u = tape->uniforms + tape->offsets[idx];
        rt.n = tape->offsets[idx + 1] - tape->offsets[idx];
        rt.status = &status;
        // schemes[0].copyTo(schemes[idx]) (scheme_integer.cu:66-79): terms, then initFlips
        z.status = &status;
        z.n[0] = n1; z.n[1] = n2; z.n[2] = n3;
        for (int c = 0; c < 3; c++) z.nn[c] = nn[c];
        z.m = m;
        for (int c = 0; c < 3; c++)
            for (int t = 0; t < m; t++) {
                Tern a;
                for (int e = 0; e < nn[c]; e++) {
                    const int8_t x = coef0[((size_t)c * m + t) * 64 + e];
                    if (x) a.v |= (uint64_t)1 << e;
                    if (x < 0) a.s |= (uint64_t)1 << e;
                }
                z.x[c][t] = a;
            }
        z.rebuildLists();
        const uint32_t flips = rt.raw() % (uint32_t)(max_flips + 1);
        for (uint32_t i = 0; i < flips; i++)
            if (!z.tryFlip(rt, true) || status) break;
        int8_t *out = coef_out + (size_t)idx * 3 * m * 64;
        for (int c = 0; c < 3; c++)
            for (int t = 0; t < m; t++)
                for (int e = 0; e < 64; e++)
                    out[((size_t)c * m + t) * 64 + e] = (int8_t)(t < z.m && e < nn[c] ? z.x[c][t].at(e) : 0);
        ranks_out[idx] = z.m;
        if (consumed) consumed[idx] = rt.pos;
        bad += status != 0;
    }
    return bad;
}

void fgo_reducer_state_free(fgo_reducer_state *s) { delete s; }

fgo_reducer_state *fgo_reducer_state_make(const int32_t *fresh, const int32_t *vars) {
    fgo_reducer_state *st = new fgo_reducer_state;
    for (int p = 0; p < 3; p++)
        for (int q = 0; q < fresh[p]; q++)
            st->vars[p].push_back({vars[(p * 500 + q) * 2], vars[(p * 500 + q) * 2 + 1]});
    return st;
}

}  // extern "C"
