// Fast-mode Z2 walk, one WARP per walk: the same semantics as the
// thread-per-walk kernel (SimtZ2: implicit pair enumeration in canonical
// order, Philox stream), for schemes large enough that one thread per walk
// is latency bound.
//
// The walk is stored compactly in shared memory, word (c, t) = factor | partner
// count << HS, and lane l owns terms t = S*l + q (q < S), so ascending term
// order is lane-major and every canonical-order search is one warp prefix sum
// plus a ballot.  A flip's count update touches each lane's S terms; the rare
// structural edits (reductions, zero terms, plus, split, expand, tryReduce)
// run on lane 0 through SimtZ2<W, 0> on the same words, with the stream
// handed over and back so both consume the same word sequence.
#pragma once
#include "fg_device.cuh"
#include "walk_simt.cuh"

namespace fg {

// Walk state handed to and back from the serial edits.
struct SerialCtx {
    int n0, n1, n2, cap, m, P0, P1, P2, status, result;
    uint32_t k0, k1, walk;
    unsigned long long count;
    const WalkParams *P;
};

// One structural edit of a compact walk, by SimtZ2<W, 0> on the calling
// thread with the walk's stream at x.count; op codes as WarpFast::OP_*.
template <class W>
__device__ __noinline__ void serial_op(W *s, SerialCtx &x, int op, int a0, int a1, int a2, int a3) {
    ThreadPhilox tp;
    tp.k0 = x.k0; tp.k1 = x.k1; tp.walk = x.walk; tp.count = x.count; tp.blk = -1; tp.P = x.P;
    SimtZ2<W, 0> z(tp);
    z.s = s; z.cap = x.cap;
    z.n0 = x.n0; z.n1 = x.n1; z.n2 = x.n2;
    z.nn0 = x.n0 * x.n1; z.nn1 = x.n1 * x.n2; z.nn2 = x.n2 * x.n0; z.full = x.n0 * x.n1 * x.n2;
    z.m = x.m; z.P0 = x.P0; z.P1 = x.P1; z.P2 = x.P2; z.status = x.status;
    int res = 0;
    switch (op) {
        case 0: {  // a flip (j = a0, a = a1, k = a2, b = a3) that zeroes a word
            const W newA = z.F(a0, a1) ^ z.F(a0, a3), newB = z.F(a2, a3) ^ z.F(a2, a1);
            z.setWord(a0, a1, newA);
            z.setWord(a2, a3, newB);
            z.removeZeroes();
            break;
        }
        case 1: z.reduce(a0, a1, a2); break;
        case 2: res = z.tryExpand(a0); break;
        case 3: res = z.tryPlus(); break;
        default: res = z.tryReduce(); break;
    }
    x.m = z.m; x.P0 = z.P0; x.P1 = z.P1; x.P2 = z.P2; x.status = z.status;
    x.count = tp.count; x.result = res;
}

template <class W, int S>
struct WarpFast {
    using Serial = SimtZ2<W, 0>;
    static_assert(S >= 1 && S <= 32, "terms per lane");
    static constexpr int HS = Serial::HS;
    static constexpr W FM = Serial::FM;
    static constexpr W ONE = Serial::ONE;
    enum { OP_ZEROFLIP, OP_REDUCE, OP_EXPAND, OP_PLUS, OP_TRYREDUCE };

    W *s;  // [3][cap] compact, this warp's walk
    int cap;
    int n0, n1, n2;
    int m;
    int P0, P1, P2;
    int status;
    PhiloxDraws &r;

    __device__ WarpFast(PhiloxDraws &rr) : r(rr) {}

    __device__ __forceinline__ W &A(int c, int t) const { return s[c * cap + t]; }
    __device__ __forceinline__ W F(int c, int t) const { return A(c, t) & FM; }
    __device__ __forceinline__ void addP(int c, int d) { if (c == 0) P0 += d; else if (c == 1) P1 += d; else P2 += d; }

    // Runs one structural edit on lane 0 (serial_op, not inlined: it keeps the
    // flip loop's register budget small), then publishes rank, pair totals,
    // status and stream position to the warp; returns the edit's result.
    __device__ int serial(int op, int a0 = 0, int a1 = 0, int a2 = 0, int a3 = 0) {
        __syncwarp();
        SerialCtx x;
        x.n0 = n0; x.n1 = n1; x.n2 = n2; x.cap = cap;
        x.m = m; x.P0 = P0; x.P1 = P1; x.P2 = P2; x.status = status; x.result = 0;
        x.k0 = r.k0; x.k1 = r.k1; x.walk = r.walk; x.count = r.count; x.P = r.P;
        if (lane_id() == 0) serial_op<W>(s, x, op, a0, a1, a2, a3);
        const int res = x.result;
        __syncwarp();
        m = __shfl_sync(kFull, x.m, 0);
        P0 = __shfl_sync(kFull, x.P0, 0);
        P1 = __shfl_sync(kFull, x.P1, 0);
        P2 = __shfl_sync(kFull, x.P2, 0);
        status = __shfl_sync(kFull, x.status, 0);
        r.count = __shfl_sync(kFull, x.count, 0);
        return __shfl_sync(kFull, res, 0);
    }

    // Partner counts from scratch, warp-parallel (lane l recounts its own terms).
    __device__ void rebuild() {
        __syncwarp();
        int tot[3] = {0, 0, 0};
#pragma unroll
        for (int c = 0; c < 3; c++) {
            W v[S];
            int h[S];
#pragma unroll
            for (int q = 0; q < S; q++) {
                const int t = S * lane_id() + q;
                v[q] = t < m ? F(c, t) : (W)0;
                h[q] = 0;
            }
            for (int u = 0; u < m; u++) {
                const W x = F(c, u);
#pragma unroll
                for (int q = 0; q < S; q++) h[q] += (x == v[q]) & (u != S * lane_id() + q);
            }
            __syncwarp();
            int loc = 0;
#pragma unroll
            for (int q = 0; q < S; q++) {
                const int t = S * lane_id() + q;
                if (t < m) { A(c, t) = v[q] | ((W)h[q] << HS); loc += h[q]; }
            }
#pragma unroll
            for (int d = 16; d; d >>= 1) loc += __shfl_xor_sync(kFull, loc, d);
            tot[c] = loc;
        }
        P0 = tot[0]; P1 = tot[1]; P2 = tot[2];
        __syncwarp();
    }

    // Uniform ordered equal pair in canonical order, then the flip (SimtZ2::tryFlip).
    __device__ bool tryFlip(bool checkReduce) {
        const int Ptot = P0 + P1 + P2;
        if (Ptot <= 0) return false;
        int q = (int)r.below((uint32_t)Ptot);
        int c;
        if (q < P0) c = 0;
        else if (q < P0 + P1) { c = 1; q -= P0; }
        else { c = 2; q -= P0 + P1; }
        // term a: prefix over the partner counts of component c
        W fv[S];
        int hc[S], loc = 0;
#pragma unroll
        for (int x = 0; x < S; x++) {
            const int t = S * lane_id() + x;
            const W w = t < m ? A(c, t) : (W)0;
            fv[x] = w & FM;
            hc[x] = (int)(w >> HS);
            loc += hc[x];
        }
        int incl = warp_inclusive_sum(loc);
        int owner = __ffs(__ballot_sync(kFull, incl > q)) - 1;
        if (owner < 0) { status |= ST_INTERNAL; return false; }
        int res = q - __shfl_sync(kFull, incl - loc, owner);
        int slot = 0;
#pragma unroll
        for (int x = 0; x < S; x++) {
            const bool here = res >= 0 && res < hc[x];
            if (here) slot = x;
            res = here ? -1 - res : (res >= 0 ? res - hc[x] : res);
        }
        const int a = S * owner + __shfl_sync(kFull, slot, owner);
        int k = __shfl_sync(kFull, -1 - res, owner);  // residual: rank of the partner
        const W va = F(c, a);
        // partner b: the k-th other term (ascending) carrying va
        unsigned mm = 0;
#pragma unroll
        for (int x = 0; x < S; x++) {
            const int t = S * lane_id() + x;
            if (t < m && t != a && fv[x] == va) mm |= 1u << x;
        }
        const int cnt = __popc(mm);
        incl = warp_inclusive_sum(cnt);
        owner = __ffs(__ballot_sync(kFull, incl > k)) - 1;
        if (owner < 0 || a >= m) { status |= ST_INTERNAL; return false; }
        k -= __shfl_sync(kFull, incl - cnt, owner);
        unsigned bits = __shfl_sync(kFull, mm, owner);
        for (int z = 0; z < k; z++) bits &= bits - 1;
        const int b = S * owner + __ffs(bits) - 1;
        int i = c, j = c == 0 ? 1 : 0, kk = c == 2 ? 1 : 2;
        if (r.coin()) { int tmp = j; j = kk; kk = tmp; }
        flip(i, j, kk, a, b, checkReduce);
        return true;
    }

    __device__ void flip(int i, int j, int k, int a, int b, bool checkReduce) {
        const W wja = A(j, a), wjb = A(j, b), wka = A(k, a), wkb = A(k, b);
        const W oldA = wja & FM, newA = oldA ^ (wjb & FM);
        const W oldB = wkb & FM, newB = oldB ^ (wka & FM);
        const int oldHa = (int)(wja >> HS), oldHb = (int)(wkb >> HS);
        const W xia = F(i, a), xka = wka & FM, xib = F(i, b), xjb = wjb & FM;
        if (!newA || !newB) {
            serial(OP_ZEROFLIP, j, a, k, b);
            return;
        }
        __syncwarp();
        if (lane_id() == 0) { A(j, a) = newA; A(k, b) = newB; }
        __syncwarp();
        int cA = 0, cB = 0;
        unsigned candJ = 0, candK = 0;
#pragma unroll
        for (int x = 0; x < S; x++) {
            const int t = S * lane_id() + x;
            if (t < m) {
                const W wj = A(j, t), wk = A(k, t);
                const W vj = wj & FM, vk = wk & FM;
                const bool oj = (vj == oldA) & (t != a), nj = (vj == newA) & (t != a);
                const bool ok = (vk == oldB) & (t != b), nk = (vk == newB) & (t != b);
                cA += nj;
                cB += nk;
                if (oj | nj) A(j, t) = wj + (nj ? ONE : (W)0) - (oj ? ONE : (W)0);
                if (ok | nk) A(k, t) = wk + (nk ? ONE : (W)0) - (ok ? ONE : (W)0);
                if (checkReduce && (nj | nk)) {
                    const W vi = F(i, t);
                    if (nj && (vi == xia || vk == xka)) candJ |= 1u << x;
                    if (nk && (vi == xib || vj == xjb)) candK |= 1u << x;
                }
            }
        }
        cA = (int)__reduce_add_sync(kFull, (unsigned)cA);
        cB = (int)__reduce_add_sync(kFull, (unsigned)cB);
        __syncwarp();
        if (lane_id() == 0) {
            A(j, a) = newA | ((W)cA << HS);
            A(k, b) = newB | ((W)cB << HS);
        }
        addP(j, 2 * (cA - oldHa));
        addP(k, 2 * (cB - oldHb));
        const unsigned any = __ballot_sync(kFull, (candJ | candK) != 0);
        if (any) {
            // First term (ascending) that triggers a reduction; j-part first at a term.
            const int owner = __ffs(any) - 1;
            const unsigned cj = __shfl_sync(kFull, candJ, owner), ck = __shfl_sync(kFull, candK, owner);
            const int x = __ffs(cj | ck) - 1;
            const int t = S * owner + x;
            const bool partJ = (cj >> x) & 1;
            // The reference tests, at the first such term, the j-part before the k-part.
            const W vi = F(i, t);
            if (partJ) serial(OP_REDUCE, vi == xia ? k : i, t, a);
            else serial(OP_REDUCE, vi == xib ? j : i, t, b);
        }
        __syncwarp();
    }

    __device__ bool tryExpand(int count) { return serial(OP_EXPAND, count) != 0; }
    __device__ bool tryPlus() { return serial(OP_PLUS) != 0; }
    __device__ bool tryReduce() { return serial(OP_TRYREDUCE) != 0; }
};

}  // namespace fg
