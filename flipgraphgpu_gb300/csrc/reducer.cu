// Additions reducer: greedy / randomised common-subexpression elimination
// over the U rows, V rows and W columns of a scheme, one thread block per
// reducer.  Restates runReducersKernel (scheme_additions_reducer.cu:494-540),
// AdditionsReducer (additions_reducer.cuh) and PairsCounter (pairs_counter.cuh).
//
// The hot part, the pair-frequency count, is block parallel: every signed pair
// occurrence (expression e, positions i < j) gets its sequence number in the
// reference's insertion order; occurrences are counted in a shared-memory hash
// (atomicCAS / atomicAdd / atomicMin of the first occurrence), and the distinct
// pairs are then laid out by first occurrence, which is exactly the order the
// reference's PairsCounter stores them in.  The reference's partial sort
// (pairs_counter.cuh:73-101), the selection modes and every draw run on one
// thread, so the XORWOW stream is consumed exactly as the reference does.
#include <algorithm>
#include <cstdint>
#include <mutex>
#include <vector>

#include <string>

#include "../../include/flipgraph.h"
#include "fg_device.cuh"
#include "launch.h"

namespace fg {

namespace {

enum { GREEDY = 0, GREEDY_ALT = 1, GREEDY_RANDOM = 2, GREEDY_INTER = 3, WEIGHTED_RANDOM = 4, MIX = 5, RANDOM = 6 };

// Threads per reducer block (fg_reducer_config::threads, 0 = 128).  Many reducers over many
// schemes run best at 128 (post-search workload, 4,096 schemes x 32 reducers: 13.6 K runs/s,
// 10.6 K at 512); many reducers over one 4x4x4 rank-47 scheme at 512 (4,071 runs/s at 128,
// 5,557 at 256, 5,854 at 512).  The count never changes a result.
int reduce_threads(int requested) {
    if (requested <= 0) return 128;
    if (requested > 1024) return 1024;
    return (requested + 31) / 32 * 32;
}

__constant__ int c_modes[15] = {GREEDY_INTER, GREEDY_INTER, GREEDY_INTER, GREEDY_INTER, GREEDY_INTER,
                                GREEDY_INTER, GREEDY_INTER, GREEDY_INTER, GREEDY_ALT,   GREEDY_ALT,
                                GREEDY_ALT,   GREEDY_ALT,   GREEDY_RANDOM, GREEDY_RANDOM, MIX};

// Fresh-variable caps (config.cuh:29-31) and PairsCounter capacities (config.cuh:25-27).
__device__ __forceinline__ int max_fresh(int c) { return c == 2 ? 500 : 250; }
__device__ __forceinline__ int max_pairs(int c) { return c == 2 ? 61075 : 2016; }

struct ReduceDims {
    int E[3];      // expressions per component: m, m, nn2
    int L[3];      // initial max length (real variables): nn0, nn1, m
    int nocc;      // max pair occurrences over components (initial)
    int tbits;     // hash table size = 1 << tbits
};

// Shared-memory carve-up for one block.
struct RedSmem {
    int16_t *ex;      // [E][L] expression entries (signed variable ids)
    int16_t *es;      // [E] sizes
    int *off;         // [E+1] occurrence offsets
    uint32_t *hkey;   // [T]
    int *hcnt;        // [T]
    int *hfirst;      // [T]
    int *byfirst;     // [nocc] slot of the pair first seen at occurrence q, or -1
    int *pi, *pj, *pc;// [nocc] distinct pairs (insertion order, then sorted)
    int16_t *vars;    // [500][2] fresh variables of the component being reduced
};

__device__ __forceinline__ uint32_t pair_key(int i, int j) {  // canonizePair (pairs_counter.cuh:214-225)
    if (abs(i) > abs(j)) { int t = i; i = j; j = t; }
    if (i < 0) { i = -i; j = -j; }
    return ((uint32_t)i << 16) | ((uint32_t)j & 0xFFFFu);
}

__device__ __forceinline__ int key_i(uint32_t k) { return (int)(k >> 16); }
__device__ __forceinline__ int key_j(uint32_t k) { return (int)(int16_t)(k & 0xFFFFu); }

__device__ __forceinline__ uint32_t hash_slot(uint32_t key, int tbits) { return (key * 2654435761u) >> (32 - tbits); }

__device__ int block_sum(int v, int *scratch) {
    for (int d = 16; d; d >>= 1) v += __shfl_xor_sync(kFull, v, d);
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane_id() == 0) scratch[warp] = v;
    __syncthreads();
    int t = 0;
    for (int q = 0; q < nw; q++) t += scratch[q];
    __syncthreads();
    return t;
}

// Serial-thread state of one component's AdditionsReducer.
struct RedState {
    int E, real, fresh, naive, mode, maxFresh, maxPairs;
    float scale;
};

// binarySearch (additions_reducer.cuh:247-269) by absolute value.
__device__ __forceinline__ int bsearch_abs(const int16_t *e, int size, int value, int start) {
    int lo = start, hi = size - 1, va = abs(value);
    while (lo <= hi) {
        int mid = lo + (hi - lo) / 2;
        int ma = abs((int)e[mid]);
        if (ma < va) lo = mid + 1;
        else if (ma > va) hi = mid - 1;
        else return mid;
    }
    return -1;
}

// replaceSubexpression (additions_reducer.cuh:218-245), expressions in parallel.
__device__ void replace_pair(RedSmem &sm, RedState &st, int L, int pi, int pj) {
    const int var = st.real + st.fresh + 1;
    for (int e = threadIdx.x; e < st.E; e += blockDim.x) {
        int16_t *x = sm.ex + (size_t)e * L;
        int size = sm.es[e];
        if (size < 2) continue;
        int i = bsearch_abs(x, size, pi, 0);
        if (i == -1) continue;
        int j = bsearch_abs(x, size, pj, i + 1);
        if (j == -1) continue;
        int v;
        if (x[i] == pi && x[j] == pj) v = var;
        else if (x[i] == -pi && x[j] == -pj) v = -var;
        else continue;
        int w = i;
        for (int q = i + 1; q < size; q++)
            if (q != j) x[w++] = x[q];
        x[w] = (int16_t)v;
        sm.es[e] = (int16_t)(size - 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        sm.vars[2 * st.fresh] = (int16_t)pi;
        sm.vars[2 * st.fresh + 1] = (int16_t)pj;
    }
    st.fresh++;
    __syncthreads();
}

__device__ __forceinline__ bool intersects(int ai, int aj, int bi, int bj) {
    return ai == bi || ai == abs(bj) || abs(aj) == bi || abs(aj) == abs(bj);
}

// updateSubexpressions + sort (additions_reducer.cuh:207-216, pairs_counter.cuh:61-101).
// Leaves the sorted pairs in sm.pi/pj/pc [0, *size), returns maxCount; *top = topSize.
__device__ int count_pairs(RedSmem &sm, RedState &st, const ReduceDims &D, int L, int *size_out, int *top_out,
                           int *scratch) {
    const int T = 1 << D.tbits;
    // occurrence offsets (sequential prefix over expressions by thread 0)
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int e = 0; e < st.E; e++) {
            sm.off[e] = acc;
            int s = sm.es[e];
            acc += s * (s - 1) / 2;
        }
        sm.off[st.E] = acc;
    }
    for (int q = threadIdx.x; q < T; q += blockDim.x) { sm.hkey[q] = 0xFFFFFFFFu; sm.hcnt[q] = 0; sm.hfirst[q] = 0x7FFFFFFF; }
    __syncthreads();
    const int N = sm.off[st.E];
    for (int q = threadIdx.x; q < N; q += blockDim.x) sm.byfirst[q] = -1;
    for (int q = threadIdx.x; q < N; q += blockDim.x) {
        int lo = 0, hi = st.E - 1;  // last e with off[e] <= q
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (sm.off[mid] <= q) lo = mid; else hi = mid - 1;
        }
        const int e = lo, s = sm.es[e];
        int r = q - sm.off[e], i = 0;
        while (r >= s - 1 - i) { r -= s - 1 - i; i++; }
        const int j = i + 1 + r;
        const int16_t *x = sm.ex + (size_t)e * L;
        const uint32_t key = pair_key(x[i], x[j]);
        uint32_t h = hash_slot(key, D.tbits);
        for (;;) {
            uint32_t prev = atomicCAS(&sm.hkey[h], 0xFFFFFFFFu, key);
            if (prev == 0xFFFFFFFFu || prev == key) break;
            h = (h + 1) & (T - 1);
        }
        atomicAdd(&sm.hcnt[h], 1);
        atomicMin(&sm.hfirst[h], q);
    }
    __syncthreads();
    for (int q = threadIdx.x; q < T; q += blockDim.x)
        if (sm.hkey[q] != 0xFFFFFFFFu) sm.byfirst[sm.hfirst[q]] = q;
    __syncthreads();
    // Distinct pairs in first-occurrence order (= PairsCounter insertion order), capped:
    // a block-wide stream compaction of the occurrences that first saw a pair.
    int d0 = 0, localMax = 0;
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int base = 0; base < N; base += blockDim.x) {
        const int q = base + threadIdx.x;
        const int slot = q < N ? sm.byfirst[q] : -1;
        const unsigned bal = __ballot_sync(kFull, slot >= 0);
        __syncthreads();
        if (lane_id() == 0) scratch[warp] = __popc(bal);
        __syncthreads();
        int before = d0;
        for (int w = 0; w < warp; w++) before += scratch[w];
        int total = 0;
        for (int w = 0; w < nw; w++) total += scratch[w];
        if (slot >= 0) {
            const int d = before + __popc(bal & lanemask_lt());
            if (d < st.maxPairs) {
                const uint32_t k = sm.hkey[slot];
                sm.pi[d] = key_i(k);
                sm.pj[d] = key_j(k);
                sm.pc[d] = sm.hcnt[slot];
                if (sm.pc[d] > localMax) localMax = sm.pc[d];
            }
        }
        d0 += total;
    }
    for (int dd = 16; dd; dd >>= 1) localMax = max(localMax, __shfl_xor_sync(kFull, localMax, dd));
    __syncthreads();
    if (lane_id() == 0) scratch[warp] = localMax;
    __syncthreads();
    if (threadIdx.x == 0) {
        int d = d0 < st.maxPairs ? d0 : st.maxPairs, maxCount = 0;
        for (int w = 0; w < nw; w++) maxCount = max(maxCount, scratch[w]);
        // sort(): move max-count pairs to the front by swapping, then drop count-1 pairs.
        int top = 0, size = d;
        if (maxCount >= 2) {
            for (int i = 0; i < size; i++) {
                if (sm.pc[i] != maxCount) continue;
                if (i != top) {
                    int a = sm.pi[i], b = sm.pj[i], c = sm.pc[i];
                    sm.pi[i] = sm.pi[top]; sm.pj[i] = sm.pj[top]; sm.pc[i] = sm.pc[top];
                    sm.pi[top] = a; sm.pj[top] = b; sm.pc[top] = c;
                }
                top++;
            }
            int j = top;
            for (int i = top; i < size; i++)
                if (sm.pc[i] > 1) { sm.pi[j] = sm.pi[i]; sm.pj[j] = sm.pj[i]; sm.pc[j] = sm.pc[i]; j++; }
            size = j;
        } else {
            top = size;
        }
        scratch[32] = size;
        scratch[33] = top;
        scratch[34] = maxCount;
    }
    __syncthreads();
    *size_out = scratch[32];
    *top_out = scratch[33];
    int mc = scratch[34];
    __syncthreads();
    return mc;
}

// Greedy-intersections choice (pairs_counter.cuh:148-176) by the whole block.  The
// serial loop visits (i, j) in order and draws once per intersecting pair; here
// every thread scores a contiguous range of rows i in that same inner order,
// starting its copy of the reducer's XORWOW stream at the draw the serial loop
// would be at (prefix over the rows' intersecting-pair counts, then cuRAND's
// skipahead), and the first row with the largest score wins, as in the serial
// strict-greater scan.  The reducer's own stream then advances by all the draws.
__device__ int select_gi(const RedSmem &sm, float scale, int size, XorwowDraws &r, int *rowCnt, int *scratch) {
    __shared__ curandStateXORWOW_t base;
    __shared__ float wbest[32];
    __shared__ int widx[32], wtot[32];
    const int tid = threadIdx.x, nt = blockDim.x, warp = tid >> 5, nw = nt >> 5;
    for (int i = tid; i < size; i += nt) {
        const int ai = sm.pi[i], aj = sm.pj[i];
        int cnt = 0;
        for (int j = 0; j < size; j++) cnt += (j != i) & intersects(ai, aj, sm.pi[j], sm.pj[j]);
        rowCnt[i] = cnt;
    }
    __syncthreads();
    const int per = (size + nt - 1) / nt;
    const int lo = min(size, tid * per), hi = min(size, lo + per);
    int local = 0;
    for (int i = lo; i < hi; i++) local += rowCnt[i];
    int incl = local;  // inclusive scan over threads (ranges are in thread order)
    for (int d = 1; d < 32; d <<= 1) {
        const int o = __shfl_up_sync(kFull, incl, d);
        if (lane_id() >= d) incl += o;
    }
    if (lane_id() == 31) wtot[warp] = incl;
    if (tid == 0) base = r.st;
    __syncthreads();
    int start = incl - local, total = 0;
    for (int w = 0; w < nw; w++) {
        if (w < warp) start += wtot[w];
        total += wtot[w];
    }
    curandStateXORWOW_t s = base;
    if (start > 0) skipahead((unsigned long long)start, &s);
    float myBest = 0.0f;
    int myIdx = -1;
    for (int i = lo; i < hi; i++) {
        const int ai = sm.pi[i], aj = sm.pj[i];
        float inter = 0;
        for (int j = 0; j < size; j++) {
            if (i == j) continue;
            if (!intersects(ai, aj, sm.pi[j], sm.pj[j])) {
                inter += (float)(sm.pc[j] - 1);
            } else if (!(curand(&s) % 2)) {
                inter = (float)__fma_rn(0.69, (double)sm.pc[j], (double)inter);
            }
        }
        const float score = __fmaf_rn(scale, inter, (float)(sm.pc[i] - 1));
        if (score > myBest) { myBest = score; myIdx = i; }
    }
    // block arg-max: larger score first, then the smaller row
    for (int d = 16; d; d >>= 1) {
        const float os = __shfl_xor_sync(kFull, myBest, d);
        const int oi = __shfl_xor_sync(kFull, myIdx, d);
        if (oi >= 0 && (myIdx < 0 || os > myBest || (os == myBest && oi < myIdx))) { myBest = os; myIdx = oi; }
    }
    if (lane_id() == 0) { wbest[warp] = myBest; widx[warp] = myIdx; }
    __syncthreads();
    int imax = 0;
    if (tid == 0) {
        float b = 0.0f;
        int bi = -1;
        for (int w = 0; w < nw; w++)
            if (widx[w] >= 0 && (bi < 0 || wbest[w] > b || (wbest[w] == b && widx[w] < bi))) { b = wbest[w]; bi = widx[w]; }
        imax = bi < 0 ? 0 : bi;
        if (total > 0) skipahead((unsigned long long)total, &r.st);
        r.count += (uint64_t)total;
        scratch[38] = imax;
    }
    __syncthreads();
    imax = scratch[38];
    __syncthreads();
    return imax;
}

// selectSubexpression (additions_reducer.cuh:272-289) on thread 0; returns the pair index.
__device__ int select_pair(const RedSmem &sm, const RedState &st, int md, int size, int top, XorwowDraws &r) {
    if (md == GREEDY) return 0;
    if (md == GREEDY_ALT) return (int)(r.raw() % (uint32_t)top);
    if (md == GREEDY_RANDOM) {
        if (r.uniform() < st.scale) return (int)(r.raw() % (uint32_t)size);
        return (int)(r.raw() % (uint32_t)top);
    }
    if (md == GREEDY_INTER) {  // pairs_counter.cuh:148-176
        int imax = 0;
        float maxScore = 0;
        for (int i = 0; i < size; i++) {
            float inter = 0;
            for (int j = 0; j < size; j++) {
                if (i == j) continue;
                if (!intersects(sm.pi[i], sm.pj[i], sm.pi[j], sm.pj[j])) {
                    inter += (float)(sm.pc[j] - 1);
                } else if (!(r.raw() % 2)) {
                    inter = (float)__fma_rn(0.69, (double)sm.pc[j], (double)inter);
                }
            }
            float score = __fmaf_rn(st.scale, inter, (float)(sm.pc[i] - 1));
            if (score > maxScore) { maxScore = score; imax = i; }
        }
        return imax;
    }
    if (md == WEIGHTED_RANDOM) {  // pairs_counter.cuh:178-196
        float total = 0;
        for (int i = 0; i < size; i++) total += (float)sm.pc[i];
        float x = r.uniform() * total;
        float sum = 0;
        for (int i = 0; i < size; i++) {
            sum += (float)sm.pc[i];
            if (x <= sum) return i;
        }
        return size - 1;
    }
    return (int)(r.raw() % (uint32_t)size);
}

struct ReduceArgs {
    int count, schemes, n1, n2, n3, m;
    const int8_t *coef;              // [schemes][3][m][64]
    curandStateXORWOW_t *states;     // [count]
    int independent;
    int best_fresh[3];
    const int16_t *best_vars;        // [3][500][2]
    int32_t *out;                    // [count][13]: per component additions, fresh, naive, mode; draws
    float *out_scale;                // [count][3]
    int16_t *out_vars;               // [count][3][500][2] or null
    ReduceDims D;
    unsigned char *gscratch;         // non-null: per-block tables in global memory (slotBytes each)
    size_t slotBytes;
    const int32_t *ranks = nullptr;  // [schemes] rank of each scheme (null: all m); rows past it are zero
};

// One reducer (runReducersKernel body for reducer idx); its pair tables start at `base`.
__device__ void reduce_one(const ReduceArgs &A, int idx, unsigned char *base, int *scratch) {
    const ReduceDims &D = A.D;
    const int Lmax = max(D.L[0], max(D.L[1], D.L[2]));
    const int Emax = max(D.E[0], max(D.E[1], D.E[2]));
    const int T = 1 << D.tbits;
    RedSmem sm;
    unsigned char *p = base;
    sm.hkey = reinterpret_cast<uint32_t *>(p); p += 4 * (size_t)T;
    sm.hcnt = reinterpret_cast<int *>(p); p += 4 * (size_t)T;
    sm.hfirst = reinterpret_cast<int *>(p); p += 4 * (size_t)T;
    sm.byfirst = reinterpret_cast<int *>(p); p += 4 * (size_t)D.nocc;
    sm.pi = reinterpret_cast<int *>(p); p += 4 * (size_t)D.nocc;
    sm.pj = reinterpret_cast<int *>(p); p += 4 * (size_t)D.nocc;
    sm.pc = reinterpret_cast<int *>(p); p += 4 * (size_t)D.nocc;
    sm.off = reinterpret_cast<int *>(p); p += 4 * (size_t)(Emax + 1);
    sm.vars = reinterpret_cast<int16_t *>(p); p += 2 * 2 * 500;
    sm.es = reinterpret_cast<int16_t *>(p); p += 2 * (size_t)((Emax + 1) & ~1);
    sm.ex = reinterpret_cast<int16_t *>(p);

    XorwowDraws r;
    r.st = A.states[idx];
    r.count = 0;
    r.P = nullptr;
    const int8_t *coef = A.coef + (size_t)(idx % A.schemes) * 3 * A.m * 64;
    const int nn[3] = {A.n1 * A.n2, A.n2 * A.n3, A.n3 * A.n1};
    // A flipped scheme may have dropped rank (tryFlip reduces): it has fewer U and V
    // expressions and W has fewer real variables (addExpression(w, scheme.m)).
    const int ms = A.ranks ? A.ranks[idx % A.schemes] : A.m;

    // Modes (scheme_additions_reducer.cu:600-602): reducer 0 is plain greedy, no draws.
    int modes[3];
    for (int c = 0; c < 3; c++) modes[c] = idx == 0 ? GREEDY : c_modes[r.raw() % 15];
    // Partial initialisation draws (scheme_additions_reducer.cu:604-623).
    int partial[3] = {0, 0, 0};
    if (A.independent) {
        for (int c = 0; c < 3; c++)
            if ((double)r.uniform() < 0.3 && A.best_fresh[c] > 0) partial[c] = 1 + (int)(r.raw() % (uint32_t)A.best_fresh[c]);
    } else if ((double)r.uniform() < 0.3) {
        for (int c = 0; c < 3; c++)
            if (A.best_fresh[c] > 0) partial[c] = 1 + (int)(r.raw() % (uint32_t)A.best_fresh[c]);
    }
    for (int c = 0; c < 3; c++) {
        // copySchemeToReducers (scheme_additions_reducer.cu:463-492): naive expressions.
        RedState st;
        st.E = c < 2 ? ms : D.E[c];
        st.real = c < 2 ? nn[c] : ms;
        st.fresh = 0;
        st.mode = modes[c];
        st.maxFresh = max_fresh(c);
        st.maxPairs = max_pairs(c);
        const int L = Lmax;
        for (int e = threadIdx.x; e < st.E; e += blockDim.x) {
            int16_t *x = sm.ex + (size_t)e * L;
            int size = 0;
            if (c < 2) {
                for (int q = 0; q < nn[c]; q++) {
                    int v = coef[((size_t)c * A.m + e) * 64 + q];
                    if (v) x[size++] = (int16_t)(v > 0 ? q + 1 : -(q + 1));
                }
            } else {
                for (int t = 0; t < A.m; t++) {
                    int v = coef[((size_t)2 * A.m + t) * 64 + e];
                    if (v) x[size++] = (int16_t)(v > 0 ? t + 1 : -(t + 1));
                }
            }
            sm.es[e] = (int16_t)size;
        }
        __syncthreads();
        int naiveLocal = 0;
        for (int e = threadIdx.x; e < st.E; e += blockDim.x) naiveLocal += sm.es[e] - 1;
        st.naive = block_sum(naiveLocal, scratch);
        // partialInitialize (additions_reducer.cuh:129-136) from the incumbent's variables.
        for (int q = 0; q < partial[c] && q < A.best_fresh[c]; q++) {
            const int16_t *bv = A.best_vars + ((size_t)c * 500 + q) * 2;
            replace_pair(sm, st, L, bv[0], bv[1]);
        }
        // reduce (additions_reducer.cuh:89-103).
        st.scale = -1;
        if (threadIdx.x == 0) st.scale = r.uniform() / 2;
        while (st.fresh < st.maxFresh) {
            int size, top;
            int maxCount = count_pairs(sm, st, D, L, &size, &top, scratch);
            if (!(size > 0 && maxCount > 1)) break;
            if (threadIdx.x == 0) {
                scratch[37] = st.mode == MIX ? (int)(r.raw() % MIX) : st.mode;
                scratch[39] = __float_as_int(st.scale);
            }
            __syncthreads();
            const int md = scratch[37];
            if (md == GREEDY_INTER) {
                const int k = select_gi(sm, __int_as_float(scratch[39]), size, r, sm.byfirst, scratch);
                if (threadIdx.x == 0) {
                    scratch[35] = sm.pi[k];
                    scratch[36] = sm.pj[k];
                }
            } else if (threadIdx.x == 0) {
                const int k = select_pair(sm, st, md, size, top, r);
                scratch[35] = sm.pi[k];
                scratch[36] = sm.pj[k];
            }
            __syncthreads();
            int pi = scratch[35], pj = scratch[36];
            __syncthreads();
            replace_pair(sm, st, L, pi, pj);
        }
        int addLocal = 0;
        for (int e = threadIdx.x; e < st.E; e += blockDim.x) addLocal += sm.es[e] - 1;
        int adds = block_sum(addLocal, scratch) + st.fresh;
        if (threadIdx.x == 0) {
            A.out[idx * 13 + c * 4 + 0] = adds;
            A.out[idx * 13 + c * 4 + 1] = st.fresh;
            A.out[idx * 13 + c * 4 + 2] = st.naive;
            A.out[idx * 13 + c * 4 + 3] = st.mode;
            A.out_scale[idx * 3 + c] = st.scale;
        }
        if (A.out_vars)
            for (int q = threadIdx.x; q < 2 * st.fresh; q += blockDim.x)
                A.out_vars[((size_t)idx * 3 + c) * 1000 + q] = sm.vars[q];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        A.states[idx] = r.st;
        A.out[idx * 13 + 12] = (int32_t)r.count;
    }
}

// Reducers blockIdx.x, blockIdx.x + gridDim.x, ...; tables in dynamic shared memory, or in
// this block's global scratch slot when they do not fit on chip.
__global__ void k_reduce(ReduceArgs A) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int scratch[40];
    unsigned char *base = A.gscratch ? A.gscratch + (size_t)blockIdx.x * A.slotBytes : smem;
    for (int idx = blockIdx.x; idx < A.count; idx += gridDim.x) {
        reduce_one(A, idx, base, scratch);
        __syncthreads();
    }
}

__global__ void k_seed_reducers(curandStateXORWOW_t *st, int count, unsigned long long seed) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) curand_init(seed, (unsigned long long)i, 0ull, &st[i]);  // scheme_additions_reducer.cu:445
}

}  // namespace
}  // namespace fg

using namespace fg;

struct fg_reducer {
    fg_reducer_config cfg;
    int n1, n2, n3, m;
    ReduceDims D;
    int8_t *d_coef = nullptr;
    curandStateXORWOW_t *d_states = nullptr;
    int16_t *d_best = nullptr;
    int32_t *d_out = nullptr;
    float *d_scale = nullptr;
    int16_t *d_vars = nullptr;
    size_t smem = 0;
    unsigned char *d_scratch = nullptr;  // global-memory tables when they exceed shared memory
    size_t slotBytes = 0;
    int slots = 0;
    // --max-flips: the schemes 1.. are flipped copies of scheme 0 (fg_reducer_flip)
    bool ternary0 = false;      // scheme 0's coefficients are all in {-1, 0, 1}
    int32_t *d_ranks = nullptr; // [schemes] rank of each scheme after the last flip pass
    int32_t *d_pairs = nullptr; // [schemes] largest pair-occurrence count of a component
    int32_t *d_fstatus = nullptr;  // [schemes] walk status bits of the flip pass
    bool flipped = false;       // d_ranks holds the ranks fg_reducer_run must use
};

namespace {
fg_status rfail(fg_status s, const char *msg) {
    fg::last_error() = msg;
    return s;
}
#define RCUDA(call)                                                             \
    do {                                                                        \
        cudaError_t e_ = (call);                                                \
        if (e_ != cudaSuccess) return rfail(FG_ERR_CUDA, cudaGetErrorString(e_)); \
    } while (0)

// k_reduce's dynamic shared-memory limit is one setting per process and device.
// Every launcher only raises it, under one lock, to at least its launch's size:
// a launch on another thread can then never find it lowered below its own size.
std::mutex g_smem_limit_mu;

cudaError_t raise_reduce_smem_limit(size_t bytes) {
    std::lock_guard<std::mutex> lock(g_smem_limit_mu);
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, k_reduce);
    if (e != cudaSuccess) return e;
    if ((size_t)fa.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
    return cudaFuncSetAttribute(k_reduce, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

// Pair tables for expressions holding at most `nocc` pair occurrences: in shared
// memory when they fit, else one slot per resident block in global memory.
fg_status plan_tables(fg_reducer *h, long nocc) {
    ReduceDims &D = h->D;
    const int m = h->m, nn[3] = {h->n1 * h->n2, h->n2 * h->n3, h->n3 * h->n1};
    D.nocc = (int)nocc;
    D.tbits = 4;
    while ((1L << D.tbits) < 2 * nocc) D.tbits++;
    const int T = 1 << D.tbits;
    const int Lmax = nn[0] > nn[1] ? (nn[0] > m ? nn[0] : m) : (nn[1] > m ? nn[1] : m);
    const int Emax = m > nn[2] ? m : nn[2];
    const size_t bytes = (size_t)12 * T + (size_t)16 * D.nocc + 4 * (size_t)(Emax + 1) + 2000 +
                         2 * (size_t)((Emax + 1 + 1) & ~1) + 2 * (size_t)Emax * Lmax + 64;
    int optin = 0, sms = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->cfg.device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->cfg.device);
    if (h->d_scratch) cudaFree(h->d_scratch);
    h->d_scratch = nullptr;
    h->slotBytes = 0;
    h->slots = 0;
    h->smem = bytes;
    if (bytes > (size_t)optin) {
        // Tables in global memory (L2-resident per block), blocks loop over the reducers.
        h->slotBytes = (bytes + 255) / 256 * 256;
        h->slots = std::min(h->cfg.count, 4 * (sms > 0 ? sms : 1));
        h->smem = 0;
        if (cudaMalloc(&h->d_scratch, h->slotBytes * h->slots) != cudaSuccess) {
            h->d_scratch = nullptr;
            return rfail(FG_ERR_CAPACITY, "scheme too large for the reducer's global tables");
        }
    }
    return FG_OK;
}
}  // namespace

extern "C" {

fg_status fg_reducer_create(const fg_reducer_config *cfg, int n1, int n2, int n3, int m, const int8_t *coef,
                            fg_reducer **out) {
    if (!cfg || !coef || !out) return rfail(FG_ERR_ARG, "null argument");
    *out = nullptr;
    if (cfg->count <= 0 || cfg->schemes <= 0) return rfail(FG_ERR_ARG, "count and schemes must be positive");
    if (n1 <= 0 || n2 <= 0 || n3 <= 0 || n1 * n2 > 64 || n2 * n3 > 64 || n3 * n1 > 64 || m <= 0 || m > FG_MAX_RANK)
        return rfail(FG_ERR_ARG, "scheme sizes out of range");
    // Capacities of the reference's compiled configuration (config.cuh:16-27).
    if (n3 * n1 > 64) return rfail(FG_ERR_CAPACITY, "too many W expressions");
    fg_reducer *h = new fg_reducer;
    h->cfg = *cfg;
    h->n1 = n1; h->n2 = n2; h->n3 = n3; h->m = m;
    const int nn[3] = {n1 * n2, n2 * n3, n3 * n1};
    ReduceDims &D = h->D;
    D.E[0] = m; D.E[1] = m; D.E[2] = nn[2];
    D.L[0] = nn[0]; D.L[1] = nn[1]; D.L[2] = m;
    // Largest initial pair-occurrence count over schemes and components.
    long nocc = 1;
    for (int s = 0; s < cfg->schemes; s++) {
        const int8_t *cf = coef + (size_t)s * 3 * m * 64;
        for (int c = 0; c < 3; c++) {
            long tot = 0;
            for (int e = 0; e < D.E[c]; e++) {
                int size = 0;
                if (c < 2) { for (int q = 0; q < nn[c]; q++) size += cf[((size_t)c * m + e) * 64 + q] != 0; }
                else { for (int t = 0; t < m; t++) size += cf[((size_t)2 * m + t) * 64 + e] != 0; }
                tot += (long)size * (size - 1) / 2;
            }
            if (tot > nocc) nocc = tot;
        }
    }
    h->ternary0 = true;
    for (size_t q = 0; q < (size_t)3 * m * 64; q++) h->ternary0 &= coef[q] >= -1 && coef[q] <= 1;
    if (cudaSetDevice(cfg->device) != cudaSuccess) { delete h; return rfail(FG_ERR_CUDA, "cudaSetDevice failed"); }
    fg_status ps = plan_tables(h, nocc);
    if (ps != FG_OK) { delete h; return ps; }
    size_t ncoef = (size_t)cfg->schemes * 3 * m * 64;
    cudaError_t e = cudaMalloc(&h->d_coef, ncoef);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_coef, coef, ncoef, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_states, sizeof(curandStateXORWOW_t) * cfg->count);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_best, 2 * 3 * 500 * 2);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_out, 4 * 13 * (size_t)cfg->count);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_scale, 4 * 3 * (size_t)cfg->count);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_vars, 2 * (size_t)cfg->count * 3 * 1000);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_ranks, 4 * (size_t)cfg->schemes);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_pairs, 4 * (size_t)cfg->schemes);
    if (e == cudaSuccess) e = cudaMalloc(&h->d_fstatus, 4 * (size_t)cfg->schemes);
    if (e == cudaSuccess) {
        k_seed_reducers<<<(cfg->count + 127) / 128, 128>>>(h->d_states, cfg->count, (unsigned long long)cfg->seed);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        fg_reducer_destroy(h);
        return rfail(FG_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = h;
    return FG_OK;
}

fg_status fg_reducer_run(fg_reducer *h, int independent, const int32_t *best_fresh, const int32_t *best_vars,
                         int32_t *out_counts, float *out_scale, int32_t *out_vars) {
    if (!h || !out_counts) return rfail(FG_ERR_ARG, "null argument");
    RCUDA(cudaSetDevice(h->cfg.device));
    ReduceArgs A;
    A.count = h->cfg.count;
    A.schemes = h->cfg.schemes;
    A.n1 = h->n1; A.n2 = h->n2; A.n3 = h->n3; A.m = h->m;
    A.coef = h->d_coef;
    A.states = h->d_states;
    A.independent = independent;
    std::vector<int16_t> bv(3 * 500 * 2, 0);
    for (int c = 0; c < 3; c++) {
        A.best_fresh[c] = best_fresh ? best_fresh[c] : 0;
        if (A.best_fresh[c] < 0 || A.best_fresh[c] > 500) return rfail(FG_ERR_ARG, "best fresh count out of range");
        if (A.best_fresh[c] > 0 && !best_vars) return rfail(FG_ERR_ARG, "best_vars is null");
        for (int q = 0; q < 2 * A.best_fresh[c]; q++) bv[c * 1000 + q] = (int16_t)best_vars[c * 1000 + q];
    }
    RCUDA(cudaMemcpy(h->d_best, bv.data(), bv.size() * 2, cudaMemcpyHostToDevice));
    A.best_vars = h->d_best;
    A.out = h->d_out;
    A.out_scale = h->d_scale;
    A.out_vars = h->d_vars;
    A.D = h->D;
    A.gscratch = h->d_scratch;
    A.slotBytes = h->slotBytes;
    A.ranks = h->flipped ? h->d_ranks : nullptr;
    if (h->smem) RCUDA(raise_reduce_smem_limit(h->smem));
    k_reduce<<<h->d_scratch ? h->slots : A.count, reduce_threads(h->cfg.threads), h->smem>>>(A);
    RCUDA(cudaGetLastError());
    RCUDA(cudaMemcpy(out_counts, h->d_out, 4 * 13 * (size_t)A.count, cudaMemcpyDeviceToHost));
    if (out_scale) RCUDA(cudaMemcpy(out_scale, h->d_scale, 4 * 3 * (size_t)A.count, cudaMemcpyDeviceToHost));
    if (out_vars) {
        // The kernel writes each component's first 2 * fresh entries; the rest of the
        // row is returned as zero (the device buffer keeps earlier runs' pairs there).
        std::vector<int16_t> v((size_t)A.count * 3 * 1000);
        RCUDA(cudaMemcpy(v.data(), h->d_vars, v.size() * 2, cudaMemcpyDeviceToHost));
        for (int r = 0; r < A.count; r++)
            for (int c = 0; c < 3; c++) {
                const int used = 2 * out_counts[(size_t)r * 13 + c * 4 + 1];
                const size_t row = ((size_t)r * 3 + c) * 1000;
                for (int q = 0; q < 1000; q++) out_vars[row + q] = q < used ? v[row + q] : 0;
            }
    }
    return FG_OK;
}

fg_status fg_reducer_flip(fg_reducer *h, int max_flips, int32_t *ranks_out, int8_t *coef_out) {
    if (!h) return rfail(FG_ERR_ARG, "null handle");
    if (max_flips < 0) return rfail(FG_ERR_ARG, "max_flips must be >= 0");
    if (h->cfg.schemes > h->cfg.count)
        return rfail(FG_ERR_ARG, "the flip pass draws from the reducers' streams: schemes must not exceed count");
    if (!h->ternary0) return rfail(FG_ERR_ARG, "the flip pass needs scheme 0's coefficients in {-1, 0, 1}");
    RCUDA(cudaSetDevice(h->cfg.device));
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->cfg.device);
    const int S = h->cfg.schemes;
    std::vector<int32_t> ranks(S, h->m), pairs(S, h->D.nocc), status(S, 0);
    RCUDA(launch_flip_schemes(S, h->n1, h->n2, h->n3, h->m, max_flips, h->d_coef, h->d_states, h->d_ranks, h->d_pairs,
                              h->d_fstatus, sms, 0));
    RCUDA(cudaDeviceSynchronize());
    if (S > 1) {
        RCUDA(cudaMemcpy(ranks.data() + 1, h->d_ranks + 1, 4 * (size_t)(S - 1), cudaMemcpyDeviceToHost));
        RCUDA(cudaMemcpy(pairs.data() + 1, h->d_pairs + 1, 4 * (size_t)(S - 1), cudaMemcpyDeviceToHost));
        RCUDA(cudaMemcpy(status.data() + 1, h->d_fstatus + 1, 4 * (size_t)(S - 1), cudaMemcpyDeviceToHost));
    }
    RCUDA(cudaMemcpy(h->d_ranks, ranks.data(), 4, cudaMemcpyHostToDevice));  // scheme 0 is not flipped
    h->flipped = true;
    // Flips make expressions denser: grow the pair tables when a scheme needs more room.
    const long need = *std::max_element(pairs.begin(), pairs.end());
    if (need > h->D.nocc) {
        fg_status ps = plan_tables(h, need);
        if (ps != FG_OK) return ps;
    }
    if (ranks_out) std::copy(ranks.begin(), ranks.end(), ranks_out);
    if (coef_out) RCUDA(cudaMemcpy(coef_out, h->d_coef, (size_t)S * 3 * h->m * 64, cudaMemcpyDeviceToHost));
    for (int s = 1; s < S; s++)
        if (status[s]) return rfail(FG_ERR_WALK, "a scheme's flips stopped at a retry bound");
    return FG_OK;
}

fg_status fg_reducer_destroy(fg_reducer *h) {
    if (!h) return FG_OK;
    void *ptrs[] = {h->d_coef, h->d_states, h->d_best,  h->d_out,   h->d_scale,
                    h->d_vars, h->d_scratch, h->d_ranks, h->d_pairs, h->d_fstatus};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete h;
    return FG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- no-allocation variant
// fg_reducer_run_noalloc keeps every device buffer of one reducer pass in a
// single file-scope scratch array, so a call makes no device allocation.  All
// calls in the process share that array: calls that overlap in time (from two
// host threads, or two devices' calls interleaved) race on it and must be
// serialised by the caller.  Its pair tables live in shared memory only (the
// allocating path moves oversized tables to global memory; this one cannot).
namespace {

constexpr size_t kNoallocScratchBytes = (size_t)4 << 20;
constexpr int kNoallocMaxCount = 1024;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Device address of the scratch array on the current device.  Resolved on every
// call (a cheap runtime lookup), so a call after cudaDeviceReset, which ends the
// context and with it the old address, gets the new context's address.
cudaError_t noalloc_base(unsigned char **base) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    if (!p) return cudaErrorInvalidSymbol;
    *base = static_cast<unsigned char *>(p);
    return cudaSuccess;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

extern "C" {

fg_status fg_reducer_run_noalloc(const fg_reducer_config *cfg, int n1, int n2, int n3, int m, const int8_t *coef,
                                 int independent, const int32_t *best_fresh, const int32_t *best_vars,
                                 int32_t *out_counts, float *out_scale) {
    if (!cfg || !coef || !out_counts) return rfail(FG_ERR_ARG, "null argument");
    if (cfg->count <= 0 || cfg->schemes <= 0) return rfail(FG_ERR_ARG, "count and schemes must be positive");
    if (n1 <= 0 || n2 <= 0 || n3 <= 0 || n1 * n2 > 64 || n2 * n3 > 64 || n3 * n1 > 64 || m <= 0 || m > FG_MAX_RANK)
        return rfail(FG_ERR_ARG, "scheme sizes out of range");
    if (cfg->device < 0) return rfail(FG_ERR_ARG, "device out of range");
    if (cfg->count > kNoallocMaxCount) return rfail(FG_ERR_CAPACITY, "count above the no-allocation limit (1024)");
    int bf[3] = {0, 0, 0};
    for (int c = 0; c < 3; c++) {
        bf[c] = best_fresh ? best_fresh[c] : 0;
        if (bf[c] < 0 || bf[c] > 500) return rfail(FG_ERR_ARG, "best fresh count out of range");
        if (bf[c] > 0 && !best_vars) return rfail(FG_ERR_ARG, "best_vars is null");
    }
    // Scratch layout, each region on a 256-byte boundary.
    const size_t nCoef = (size_t)cfg->schemes * 3 * m * 64;
    const size_t oCoef = 0;
    const size_t oStates = align256(oCoef + nCoef);
    const size_t oBest = align256(oStates + sizeof(curandStateXORWOW_t) * (size_t)cfg->count);
    const size_t oOut = align256(oBest + (size_t)2 * 3 * 500 * 2);
    const size_t oScale = align256(oOut + (size_t)4 * 13 * cfg->count);
    const size_t total = oScale + (size_t)4 * 3 * cfg->count;
    if (total > kNoallocScratchBytes) return rfail(FG_ERR_CAPACITY, "schemes too large for the no-allocation scratch (4 MiB)");

    // Problem dimensions, as fg_reducer_create derives them.
    const int nn[3] = {n1 * n2, n2 * n3, n3 * n1};
    ReduceDims D;
    D.E[0] = m; D.E[1] = m; D.E[2] = nn[2];
    D.L[0] = nn[0]; D.L[1] = nn[1]; D.L[2] = m;
    long nocc = 1;
    for (int sc = 0; sc < cfg->schemes; sc++) {
        const int8_t *cf = coef + (size_t)sc * 3 * m * 64;
        for (int c = 0; c < 3; c++) {
            long tot = 0;
            for (int e = 0; e < D.E[c]; e++) {
                int size = 0;
                if (c < 2) { for (int q = 0; q < nn[c]; q++) size += cf[((size_t)c * m + e) * 64 + q] != 0; }
                else { for (int t = 0; t < m; t++) size += cf[((size_t)2 * m + t) * 64 + e] != 0; }
                tot += (long)size * (size - 1) / 2;
            }
            if (tot > nocc) nocc = tot;
        }
    }
    D.nocc = (int)nocc;
    D.tbits = 4;
    while ((1L << D.tbits) < 2 * nocc) D.tbits++;
    const int T = 1 << D.tbits;
    const int Lmax = nn[0] > nn[1] ? (nn[0] > m ? nn[0] : m) : (nn[1] > m ? nn[1] : m);
    const int Emax = m > nn[2] ? m : nn[2];
    const size_t smem = (size_t)12 * T + (size_t)16 * D.nocc + 4 * (size_t)(Emax + 1) + 2000 +
                        2 * (size_t)((Emax + 1 + 1) & ~1) + 2 * (size_t)Emax * Lmax + 64;

    RCUDA(cudaSetDevice(cfg->device));
    int optin = 0;
    RCUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, cfg->device));
    if (smem > (size_t)optin) return rfail(FG_ERR_CAPACITY, "scheme too large for the shared-memory reducer");
    unsigned char *base = nullptr;
    RCUDA(noalloc_base(&base));

    std::vector<int16_t> bv(3 * 500 * 2, 0);
    for (int c = 0; c < 3; c++)
        for (int q = 0; q < 2 * bf[c]; q++) bv[c * 1000 + q] = (int16_t)best_vars[c * 1000 + q];
    // Everything on the legacy default stream, in order.
    RCUDA(cudaMemcpy(base + oCoef, coef, nCoef, cudaMemcpyHostToDevice));
    RCUDA(cudaMemcpy(base + oBest, bv.data(), bv.size() * 2, cudaMemcpyHostToDevice));
    RCUDA(cudaMemset(base + oOut, 0, (size_t)4 * 13 * cfg->count));
    RCUDA(cudaMemset(base + oScale, 0, (size_t)4 * 3 * cfg->count));
    auto *states = reinterpret_cast<curandStateXORWOW_t *>(base + oStates);
    k_seed_reducers<<<(cfg->count + 127) / 128, 128>>>(states, cfg->count, (unsigned long long)cfg->seed);
    RCUDA(cudaGetLastError());
    RCUDA(raise_reduce_smem_limit(smem));

    ReduceArgs A;
    A.count = cfg->count;
    A.schemes = cfg->schemes;
    A.n1 = n1; A.n2 = n2; A.n3 = n3; A.m = m;
    A.coef = reinterpret_cast<const int8_t *>(base + oCoef);
    A.states = states;
    A.independent = independent;
    for (int c = 0; c < 3; c++) A.best_fresh[c] = bf[c];
    A.best_vars = reinterpret_cast<const int16_t *>(base + oBest);
    A.out = reinterpret_cast<int32_t *>(base + oOut);
    A.out_scale = reinterpret_cast<float *>(base + oScale);
    A.out_vars = nullptr;
    A.D = D;
    A.gscratch = nullptr;
    A.slotBytes = 0;
    k_reduce<<<A.count, reduce_threads(cfg->threads), smem>>>(A);
    RCUDA(cudaGetLastError());
    RCUDA(cudaMemcpy(out_counts, base + oOut, (size_t)4 * 13 * A.count, cudaMemcpyDeviceToHost));
    if (out_scale) RCUDA(cudaMemcpy(out_scale, base + oScale, (size_t)4 * 3 * A.count, cudaMemcpyDeviceToHost));
    return FG_OK;
}

}  // extern "C"
