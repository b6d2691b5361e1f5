// Kernel templates over both rings: walk / minimize / list rebuild, one warp per walk.
#pragma once
#include "fg_device.cuh"
#include "walk_z2.cuh"
#include "walk_zt.cuh"
#include "walk_moves.cuh"

namespace fg {

// Per-warp shared-memory footprint of a Z2 walk: factors [3][cap] + lists [3][500].
__host__ __device__ inline size_t walk_smem_bytes(int cap) {
    return (size_t)3 * cap * sizeof(uint64_t) + (size_t)3 * kListCap * sizeof(uint32_t);
}

template <class R> struct DrawsIO;

template <> struct DrawsIO<XorwowDraws> {
    static __device__ XorwowDraws load(const DevBatch &B, const WalkParams &P, int w, const WalkHeader &h) {
        XorwowDraws r;
        r.st = B.xorwow[w];
        r.count = h.draws;
        r.P = &P;
        return r;
    }
    static __device__ void store(const DevBatch &B, int w, const XorwowDraws &r) {
        if (lane_id() == 0) B.xorwow[w] = r.st;
    }
};

template <> struct DrawsIO<PhiloxDraws> {
    static __device__ PhiloxDraws load(const DevBatch &B, const WalkParams &P, int w, const WalkHeader &h) {
        PhiloxDraws r;
        r.k0 = P.key0;
        r.k1 = P.key1;
        r.walk = (uint32_t)w;
        r.count = h.draws;
        r.chunk = -1;
        r.P = &P;
        return r;
    }
    static __device__ void store(const DevBatch &, int, const PhiloxDraws &) {}
};

// ---------------------------------------------------------------- per-ring I/O
template <class Wk> struct RingIO;

template <class R, int S> struct RingIO<Z2Walk<R, S>> {
    using Walker = Z2Walk<R, S>;
    static __host__ __device__ size_t smem(int cap) { return walk_smem_bytes(cap); }
    static __device__ void bind(Walker &z, unsigned char *base, int cap) {
        z.x = reinterpret_cast<uint64_t *>(base);
        z.L = reinterpret_cast<uint32_t *>(z.x + 3 * cap);
    }
    static __device__ void load(Walker &z, const DevBatch &B, int w) {
        const uint64_t *src = B.fac + (size_t)w * 3 * B.cap;
        for (int q = lane_id(); q < 3 * B.cap; q += 32) z.x[q] = src[q];
    }
    static __device__ void store(Walker &z, const DevBatch &B, int w, bool best) {
        uint64_t *dst = (best ? B.best_fac : B.fac) + (size_t)w * 3 * B.cap;
        for (int q = lane_id(); q < 3 * B.cap; q += 32) dst[q] = (q % B.cap) < z.m ? z.x[q] : 0;
    }
    static __device__ int complexity(const Walker &z) {
        int c = 0;
        for (int t = lane_id(); t < z.m; t += 32) c += __popcll(z.X(0, t)) + __popcll(z.X(1, t)) + __popcll(z.X(2, t));
#pragma unroll
        for (int d = 16; d; d >>= 1) c += __shfl_xor_sync(kFull, c, d);
        return c - 2 * z.m - z.nn2;
    }
};

template <class R, int S> struct RingIO<ZTWalk<R, S>> {
    using Walker = ZTWalk<R, S>;
    static __host__ __device__ size_t smem(int cap) { return zt_smem_bytes(cap); }
    static __device__ void bind(Walker &z, unsigned char *base, int cap) {
        z.xv = reinterpret_cast<uint64_t *>(base);
        z.xs = z.xv + 3 * cap;
        z.xo = reinterpret_cast<uint8_t *>(z.xs + 3 * cap);
        z.L = reinterpret_cast<uint32_t *>(z.xo + ((size_t)3 * cap + 7) / 8 * 8);
        z.J = reinterpret_cast<uint16_t *>(z.L + 3 * kListCap);
    }
    static __device__ void load(Walker &z, const DevBatch &B, int w) {
        const size_t o = (size_t)w * 3 * B.cap;
        for (int q = lane_id(); q < 3 * B.cap; q += 32) {
            z.xv[q] = B.fac[o + q];
            z.xs[q] = B.sgn[o + q];
            z.xo[q] = B.valid[o + q];
        }
    }
    static __device__ void store(Walker &z, const DevBatch &B, int w, bool best) {
        const size_t o = (size_t)w * 3 * B.cap;
        uint64_t *dv = best ? B.best_fac : B.fac;
        uint64_t *ds = best ? B.best_sgn : B.sgn;
        uint8_t *dk = best ? B.best_valid : B.valid;
        for (int q = lane_id(); q < 3 * B.cap; q += 32) {
            bool in = (q % B.cap) < z.m;
            dv[o + q] = in ? z.xv[q] : 0;
            ds[o + q] = in ? z.xs[q] : 0;
            dk[o + q] = in ? z.xo[q] : 0;
        }
    }
    static __device__ int complexity(const Walker &z) {  // scheme_integer.cu:139-147
        int c = 0;
        for (int t = lane_id(); t < z.m; t += 32)
            c += __popcll(z.xv[t]) + __popcll(z.xv[z.cap + t]) + __popcll(z.xv[2 * z.cap + t]);
#pragma unroll
        for (int d = 16; d; d >>= 1) c += __shfl_xor_sync(kFull, c, d);
        return c - 2 * z.m - z.nn2;
    }
};

template <class Walker>
__device__ __forceinline__ void walk_bind(Walker &z, const DevBatch &B, const WalkHeader &h, int w,
                                          unsigned char *base) {
    RingIO<Walker>::bind(z, base, B.cap);
    RingIO<Walker>::load(z, B, w);
    for (int c = 0; c < 3; c++) {
        const uint32_t *ls = B.lists + ((size_t)w * 3 + c) * kListCap;
        for (int q = lane_id(); q < h.list_size[c]; q += 32) z.L[c * kListCap + q] = ls[q];
    }
    z.cap = B.cap;
    z.n0 = h.n[0]; z.n1 = h.n[1]; z.n2 = h.n[2];
    z.nn0 = z.n0 * z.n1; z.nn1 = z.n1 * z.n2; z.nn2 = z.n2 * z.n0;
    z.full = z.n0 * z.n1 * z.n2;
    z.m = h.m;
    z.sz0 = h.list_size[0]; z.sz1 = h.list_size[1]; z.sz2 = h.list_size[2];
    z.status = h.status;
    __syncwarp();
}

template <class Walker>
__device__ __forceinline__ void walk_store(Walker &z, const DevBatch &B, int w) {
    __syncwarp();
    RingIO<Walker>::store(z, B, w, false);
    for (int c = 0; c < 3; c++) {
        uint32_t *ls = B.lists + ((size_t)w * 3 + c) * kListCap;
        int s = z.sz(c);
        for (int q = lane_id(); q < kListCap; q += 32) ls[q] = q < s ? z.L[c * kListCap + q] : 0u;
    }
}

// randomWalkKernel (flip_graph.cu:520-573) for one walk, `iterations` steps.
template <class Walker, class R>
__device__ void walk_one(const DevBatch &B, const WalkParams &P, int w, unsigned char *base) {
    const WalkHeader h = B.hdr[w];
    R r = DrawsIO<R>::load(B, P, w, h);
    Walker z(r);
    walk_bind(z, B, h, w, base);
    int flipsCount = h.flips, bestRank = h.best_rank, bestM = h.best_m;
    uint64_t accepted = 0;
    const int iterations = P.random_iterations ? randint(1, P.iterations, r) : P.iterations;
    for (int it = 0; it < iterations; it++) {
        const int rank = z.m;
        if (!z.tryFlip(true)) {
            z.tryExpand(randint(1, 2, r));
            if (z.status) break;
            continue;
        }
        accepted++;
        if (z.m < rank) flipsCount = 0;
        flipsCount++;
        if (z.m < bestRank || (z.m == bestRank && r.tie())) {
            bestRank = z.m;
            bestM = z.m;
            RingIO<Walker>::store(z, B, w, true);
            if (B.best_n && lane_id() == 0) {
                B.best_n[w * 3 + 0] = z.n0;
                B.best_n[w * 3 + 1] = z.n1;
                B.best_n[w * 3 + 2] = z.n2;
            }
        }
        if (r.gate_reduce()) z.tryReduce();
        if (r.gate_gauss()) z.tryReduceGauss();  // not in the reference's walk
        if (r.gate_expand() && z.m <= bestM + 2) {
            if (z.tryExpand(randint(1, 2, r))) flipsCount = 0;
        }
        if (r.gate_sandwich()) sandwich_move(z);  // flip_graph.cu:560-561
        if (r.gate_basis()) basis_move(z);        // flip_graph.cu:563-564
        if (flipsCount >= P.plus_iterations && z.tryPlus()) flipsCount = 0;
        if (z.status) break;
    }
    walk_store(z, B, w);
    DrawsIO<R>::store(B, w, r);
    if (lane_id() == 0) {
        WalkHeader o = h;
        o.m = z.m;
        o.flips = flipsCount;
        o.best_rank = bestRank;
        o.best_m = bestM;
        o.status = z.status;
        o.list_size[0] = z.sz0; o.list_size[1] = z.sz1; o.list_size[2] = z.sz2;
        o.draws = r.count;
        o.flips_done = accepted;
        B.hdr[w] = o;
    }
}

// minimizeKernel (complexity_minimizer.cu:245-263) for one walk.
template <class Walker, class R>
__device__ void minimize_one(const DevBatch &B, const WalkParams &P, int w, unsigned char *base, int32_t *bestC) {
    const WalkHeader h = B.hdr[w];
    R r = DrawsIO<R>::load(B, P, w, h);
    Walker z(r);
    walk_bind(z, B, h, w, base);
    int best = bestC[w];
    int bestM = h.best_m;
    uint64_t accepted = 0;
    for (int it = 0; it < P.iterations; it++) {
        if (!z.tryFlip(false)) break;
        accepted++;
        int c = RingIO<Walker>::complexity(z);
        if (c < best) {
            best = c;
            bestM = z.m;
            RingIO<Walker>::store(z, B, w, true);
        }
        if (z.status) break;
    }
    walk_store(z, B, w);
    DrawsIO<R>::store(B, w, r);
    if (lane_id() == 0) {
        WalkHeader o = h;
        o.m = z.m;
        o.best_m = bestM;
        o.status = z.status;
        o.list_size[0] = z.sz0; o.list_size[1] = z.sz1; o.list_size[2] = z.sz2;
        o.draws = r.count;
        o.flips_done = accepted;
        B.hdr[w] = o;
        bestC[w] = best;
    }
}

template <class Walker, class R>
__global__ void k_walk(DevBatch B, WalkParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5;
    unsigned char *base = smem + RingIO<Walker>::smem(B.cap) * warp;
    for (int w = blockIdx.x * wpb + warp; w < B.S; w += gridDim.x * wpb) walk_one<Walker, R>(B, P, w, base);
}

template <class Walker, class R>
__global__ void k_minimize(DevBatch B, WalkParams P, int32_t *bestC) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5;
    unsigned char *base = smem + RingIO<Walker>::smem(B.cap) * warp;
    for (int w = blockIdx.x * wpb + warp; w < B.S; w += gridDim.x * wpb) minimize_one<Walker, R>(B, P, w, base, bestC);
}

// Rebuilds every walk's lists from its factors (initFlips).
template <class Walker>
__global__ void k_rebuild(DevBatch B) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5;
    unsigned char *base = smem + RingIO<Walker>::smem(B.cap) * warp;
    for (int w = blockIdx.x * wpb + warp; w < B.S; w += gridDim.x * wpb) {
        WalkHeader h = B.hdr[w];
        h.list_size[0] = h.list_size[1] = h.list_size[2] = 0;
        PhiloxDraws unused;
        Walker z(unused);
        walk_bind(z, B, h, w, base);
        z.rebuild();
        walk_store(z, B, w);
        if (lane_id() == 0) {
            B.hdr[w].list_size[0] = z.sz0;
            B.hdr[w].list_size[1] = z.sz1;
            B.hdr[w].list_size[2] = z.sz2;
        }
    }
}

}  // namespace fg
