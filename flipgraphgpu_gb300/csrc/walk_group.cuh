// Fast-mode Z2 walk, one GROUP of G lanes per walk (32/G walks per warp; G =
// 32 is the one-warp-per-walk kernel): the same semantics as the thread-per-
// walk kernel (implicit pair enumeration in canonical order, Philox stream),
// a flip's O(m) work split over G lanes.  With G = 32 this slot-major layout
// measured 7-11 % faster than a lane-major warp kernel whose strided term
// accesses conflicted in shared memory.
//
// Layout: each walk is stored compactly in shared memory, word (c, t) =
// factor | partner count << HS at s[c * cap + t]; lane g of the group owns the
// terms t = x * G + g (x < S), so a group-wide access to slot x touches G
// consecutive words and, with the walks of a warp placed a multiple of 32
// words plus G apart, the warp's 32 lanes hit 32 different banks.  Ascending
// term order is slot-major: the canonical-order searches take one
// redux.sync (or ballot) per slot, a scan over the slot totals in registers,
// and one group scan inside the chosen slot.  Control flow may differ between
// the groups of a warp, so every warp-level primitive names the group's mask.
// Rare structural edits run on the group's lane 0 through SimtZ2<W, 0> on the
// same words (serial_op), with the stream position handed over and back.
#pragma once
#include "fg_device.cuh"
#include "walk_simt.cuh"
#include "walk_serial.cuh"

namespace fg {

// The walk's Philox stream (word q = Philox(ctr = (q/4 lo, q/4 hi, walk, 0), key)[q % 4]),
// refilled G blocks at a time (lane g computes block G*c + g) and served by a
// group shuffle per draw.
template <int G>
struct GroupDraws {
    uint32_t k0, k1, walk;
    uint64_t count;
    int64_t chunk;
    uint4 buf;
    const WalkParams *P;
    unsigned mask;
    int g;
    __device__ __forceinline__ uint32_t raw() {
        const int64_t c = (int64_t)(count / (uint64_t)(4 * G));
        if (c != chunk) {
            const uint64_t blk = (uint64_t)c * G + (uint64_t)g;
            buf = philox4x32_10(make_uint4((uint32_t)blk, (uint32_t)(blk >> 32), walk, 0u), k0, k1);
            chunk = c;
        }
        const uint32_t wq = (uint32_t)(count % (uint64_t)(4 * G));
        const uint32_t e = wq & 3u;
        const uint32_t v = e == 0 ? buf.x : e == 1 ? buf.y : e == 2 ? buf.z : buf.w;
        count++;
        return __shfl_sync(mask, v, (int)(wq >> 2), G);
    }
    __device__ __forceinline__ uint32_t below(uint32_t k) { return __umulhi(raw(), k); }
    __device__ __forceinline__ bool coin() { return raw() >> 31; }
    __device__ __forceinline__ bool gate_reduce() { return P->reduce_T != kGateOff && (uint64_t)raw() < P->reduce_T; }
    __device__ __forceinline__ bool gate_expand() { return P->expand_T != kGateOff && (uint64_t)raw() < P->expand_T; }
    __device__ __forceinline__ bool gate_sandwich() { return P->sandwich_T != kGateOff && (uint64_t)raw() < P->sandwich_T; }
    __device__ __forceinline__ bool gate_basis() { return P->basis_T != kGateOff && (uint64_t)raw() < P->basis_T; }
    __device__ __forceinline__ bool gate_gauss() { return P->gauss_T != kGateOff && (uint64_t)raw() < P->gauss_T; }
    __device__ __forceinline__ bool tie() { return raw() < 42949672u; }
};

// The G low bits set (G = 32: all).
template <int G> __host__ __device__ constexpr unsigned group_bits() { return G >= 32 ? 0xFFFFFFFFu : ((1u << G) - 1u); }

template <class W, int G, int S>
struct GroupFast {
    using Serial = SimtZ2<W, 0>;
    static_assert(G == 4 || G == 8 || G == 16 || G == 32, "lanes per walk");
    static_assert(S >= 1 && S <= 32, "terms per lane");
    static constexpr int HS = Serial::HS;
    static constexpr W FM = Serial::FM;
    static constexpr W ONE = Serial::ONE;
    enum { OP_ZEROFLIP, OP_REDUCE, OP_EXPAND, OP_PLUS, OP_TRYREDUCE, OP_SANDWICH, OP_BASIS, OP_GAUSS };

    W *s;  // [3][cap] compact, this group's walk
    int cap;
    int n0, n1, n2;
    int m;
    int P0, P1, P2;
    int status;
    GroupDraws<G> &r;
    unsigned mask;  // the group's lanes
    int g, gbase;   // lane in the group, first lane of the group in the warp

    __device__ GroupFast(GroupDraws<G> &rr) : r(rr) {}

    __device__ __forceinline__ W &A(int c, int t) const { return s[c * cap + t]; }
    __device__ __forceinline__ W F(int c, int t) const { return A(c, t) & FM; }
    __device__ __forceinline__ void addP(int c, int d) { if (c == 0) P0 += d; else if (c == 1) P1 += d; else P2 += d; }
    __device__ __forceinline__ unsigned gballot(bool p) const {
        return (__ballot_sync(mask, p) >> gbase) & group_bits<G>();
    }
    __device__ __forceinline__ int gsum(int v) const { return (int)__reduce_add_sync(mask, (unsigned)v); }
    __device__ __forceinline__ int gscan(int v) const {  // inclusive
#pragma unroll
        for (int d = 1; d < G; d <<= 1) {
            const int o = __shfl_up_sync(mask, v, d, G);
            if (g >= d) v += o;
        }
        return v;
    }

    __device__ int serial(int op, int a0 = 0, int a1 = 0, int a2 = 0, int a3 = 0) {
        __syncwarp(mask);
        SerialCtx x;
        x.n0 = n0; x.n1 = n1; x.n2 = n2; x.cap = cap;
        x.m = m; x.P0 = P0; x.P1 = P1; x.P2 = P2; x.status = status; x.result = 0;
        x.k0 = r.k0; x.k1 = r.k1; x.walk = r.walk; x.count = r.count; x.P = r.P;
        if (g == 0) {
            if (op >= OP_SANDWICH) serial_move<W>(s, x, op - OP_SANDWICH);
            else serial_op<W>(s, x, op, a0, a1, a2, a3);
        }
        __syncwarp(mask);
        m = __shfl_sync(mask, x.m, 0, G);
        P0 = __shfl_sync(mask, x.P0, 0, G);
        P1 = __shfl_sync(mask, x.P1, 0, G);
        P2 = __shfl_sync(mask, x.P2, 0, G);
        status = __shfl_sync(mask, x.status, 0, G);
        r.count = __shfl_sync(mask, x.count, 0, G);
        return __shfl_sync(mask, x.result, 0, G);
    }

    // Partner counts from scratch (lane g recounts its own terms).
    __device__ void rebuild() {
        __syncwarp(mask);
        // Counts go to the top byte of each word; the factor bits (compared below) stay
        // untouched, so the group's lanes may update their own words as they go.
        int tot[3] = {0, 0, 0};
        for (int c = 0; c < 3; c++) {
            int loc = 0;
#pragma unroll 1
            for (int x = 0; x < S; x++) {
                const int t = x * G + g;
                if (t >= m) break;
                const W v = F(c, t);
                int h = 0;
                for (int u = 0; u < m; u++) h += (F(c, u) == v) & (u != t);
                A(c, t) = v | ((W)h << HS);
                loc += h;
            }
            tot[c] = gsum(loc);
        }
        P0 = tot[0]; P1 = tot[1]; P2 = tot[2];
        __syncwarp(mask);
    }

    // Uniform ordered equal pair in canonical order (component, term, partner), orientation, flip.
    __device__ bool tryFlip(bool checkReduce) {
        const int Ptot = P0 + P1 + P2;
        if (Ptot <= 0) return false;
        int q = (int)r.below((uint32_t)Ptot);
        int c;
        if (q < P0) c = 0;
        else if (q < P0 + P1) { c = 1; q -= P0; }
        else { c = 2; q -= P0 + P1; }
        // slot of term a (slot totals by redux.sync), then the lane inside the slot
        int xs = -1, hv = 0;
#pragma unroll
        for (int x = 0; x < S; x++) {
            const int t = x * G + g;
            const int hx = t < m ? (int)(A(c, t) >> HS) : 0;
            const int tx = gsum(hx);
            if (xs < 0) {
                if (q < tx) { xs = x; hv = hx; }
                else q -= tx;
            }
        }
        if (xs < 0) { status |= ST_INTERNAL; return false; }
        const int incl = gscan(hv);
        const unsigned over = gballot(incl > q);
        if (!over) { status |= ST_INTERNAL; return false; }
        const int owner = __ffs(over) - 1;
        int k = q - __shfl_sync(mask, incl - hv, owner, G);  // rank of the partner among the other carriers
        const int a = xs * G + owner;
        const W va = F(c, a);
        // partner b: the k-th other term (ascending) carrying va
        int xb = -1;
        unsigned bits = 0;
#pragma unroll
        for (int x = 0; x < S; x++) {
            const int t = x * G + g;
            const unsigned bx = gballot(t < m && t != a && F(c, t) == va);
            const int cnt = __popc(bx);
            if (xb < 0) {
                if (k < cnt) { xb = x; bits = bx; }
                else k -= cnt;
            }
        }
        if (xb < 0) { status |= ST_INTERNAL; return false; }
        for (int z = 0; z < k; z++) bits &= bits - 1;
        const int b = xb * G + __ffs(bits) - 1;
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
        __syncwarp(mask);
        if (g == 0) { A(j, a) = newA; A(k, b) = newB; }
        __syncwarp(mask);
        int cA = 0, cB = 0;
        unsigned candJ = 0, candK = 0;
#pragma unroll
        for (int x = 0; x < S; x++) {
            const int t = x * G + g;
            if (t < m) {
                const W wj = A(j, t), wk = A(k, t);
                const W vj = wj & FM, vk = wk & FM;
                const bool oj = (vj == oldA) & (t != a), nj = (vj == newA) & (t != a);
                const bool ok = (vk == oldB) & (t != b), nk = (vk == newB) & (t != b);
                cA += nj;
                cB += nk;
                // unconditional write-back (no divergence; 0-3 % faster)
                A(j, t) = wj + (nj ? ONE : (W)0) - (oj ? ONE : (W)0);
                A(k, t) = wk + (nk ? ONE : (W)0) - (ok ? ONE : (W)0);
                if (checkReduce && (nj | nk)) {
                    const W vi = F(i, t);
                    if (nj && (vi == xia || vk == xka)) candJ |= 1u << x;
                    if (nk && (vi == xib || vj == xjb)) candK |= 1u << x;
                }
            }
        }
        cA = gsum(cA);
        cB = gsum(cB);
        __syncwarp(mask);
        if (g == 0) {
            A(j, a) = newA | ((W)cA << HS);
            A(k, b) = newB | ((W)cB << HS);
        }
        addP(j, 2 * (cA - oldHa));
        addP(k, 2 * (cB - oldHb));
        // First term (ascending) that triggers a reduction; its j-part is tested before its k-part.
        const unsigned cj = candJ | candK;
        const unsigned key = cj ? (unsigned)((__ffs(cj) - 1) * G + g) : 0xFFFFFFFFu;
        const unsigned tmin = __reduce_min_sync(mask, key);
        if (tmin != 0xFFFFFFFFu) {
            const int t = (int)tmin, owner = t % G, x = t / G;
            const bool partJ = (__shfl_sync(mask, candJ, owner, G) >> x) & 1u;
            const W vi = F(i, t);
            if (partJ) serial(OP_REDUCE, vi == xia ? k : i, t, a);
            else serial(OP_REDUCE, vi == xib ? j : i, t, b);
        }
        __syncwarp(mask);
    }

    __device__ bool tryExpand(int count) { return serial(OP_EXPAND, count) != 0; }
    __device__ bool tryPlus() { return serial(OP_PLUS) != 0; }
    __device__ bool tryReduce() { return serial(OP_TRYREDUCE) != 0; }
    __device__ void sandwich() { serial(OP_SANDWICH); }
    __device__ void swapBasis() { serial(OP_BASIS); }
    __device__ bool tryReduceGauss() { return serial(OP_GAUSS) != 0; }
};

}  // namespace fg
