// Kernel templates: walk / minimize / init / verify, one warp per walk.
#pragma once
#include "fg_device.cuh"
#include "walk_z2.cuh"

namespace fg {

// Per-warp shared-memory footprint of a walk: factors [3][cap] + lists [3][500].
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

template <class R, int S>
__device__ __forceinline__ void z2_load(Z2Walk<R, S> &z, const DevBatch &B, const WalkHeader &h, int w) {
    const int cap = B.cap;
    const uint64_t *src = B.fac + (size_t)w * 3 * cap;
    for (int q = lane_id(); q < 3 * cap; q += 32) z.x[q] = src[q];
    for (int c = 0; c < 3; c++) {
        const uint32_t *ls = B.lists + ((size_t)w * 3 + c) * kListCap;
        for (int q = lane_id(); q < h.list_size[c]; q += 32) z.L[c * kListCap + q] = ls[q];
    }
    z.cap = cap;
    z.n0 = h.n[0]; z.n1 = h.n[1]; z.n2 = h.n[2];
    z.nn0 = z.n0 * z.n1; z.nn1 = z.n1 * z.n2; z.nn2 = z.n2 * z.n0;
    z.full = z.n0 * z.n1 * z.n2;
    z.m = h.m;
    z.sz0 = h.list_size[0]; z.sz1 = h.list_size[1]; z.sz2 = h.list_size[2];
    z.status = h.status;
    __syncwarp();
}

// Writes factors (zero beyond m) and lists (zero beyond size) back to HBM.
template <class R, int S>
__device__ __forceinline__ void z2_store(Z2Walk<R, S> &z, const DevBatch &B, int w) {
    const int cap = B.cap;
    __syncwarp();
    uint64_t *dst = B.fac + (size_t)w * 3 * cap;
    for (int q = lane_id(); q < 3 * cap; q += 32) dst[q] = (q % cap) < z.m ? z.x[q] : 0;
    for (int c = 0; c < 3; c++) {
        uint32_t *ls = B.lists + ((size_t)w * 3 + c) * kListCap;
        int s = z.sz(c);
        for (int q = lane_id(); q < kListCap; q += 32) ls[q] = q < s ? z.L[c * kListCap + q] : 0u;
    }
}

template <class R, int S>
__device__ __forceinline__ void z2_copy_best(Z2Walk<R, S> &z, const DevBatch &B, int w) {
    const int cap = B.cap;
    uint64_t *dst = B.best_fac + (size_t)w * 3 * cap;
    for (int q = lane_id(); q < 3 * cap; q += 32) dst[q] = (q % cap) < z.m ? z.x[q] : 0;
}

// randomWalkKernel (flip_graph.cu:520-573) for one walk, `iterations` steps.
template <class R, int S>
__device__ void z2_walk_one(const DevBatch &B, const WalkParams &P, int w, uint64_t *xs, uint32_t *Ls) {
    const WalkHeader h = B.hdr[w];
    R r = DrawsIO<R>::load(B, P, w, h);
    Z2Walk<R, S> z(r);
    z.x = xs;
    z.L = Ls;
    z2_load(z, B, h, w);
    int flipsCount = h.flips, bestRank = h.best_rank, bestM = h.best_m;
    uint64_t accepted = 0;
    for (int it = 0; it < P.iterations; it++) {
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
            z2_copy_best(z, B, w);
        }
        if (r.gate_reduce()) z.tryReduce();
        if (r.gate_expand() && z.m <= bestM + 2) {
            if (z.tryExpand(randint(1, 2, r))) flipsCount = 0;
        }
        r.gate_zero();  // sandwiching (probability 0)
        r.gate_zero();  // basis change (probability 0)
        if (flipsCount >= P.plus_iterations && z.tryPlus()) flipsCount = 0;
        if (z.status) break;
    }
    z2_store(z, B, w);
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

// Warp sum of popcounts over the current scheme: complexity (scheme_z2.cu:127-139).
template <class R, int S>
__device__ __forceinline__ int z2_complexity(const Z2Walk<R, S> &z) {
    int c = 0;
#pragma unroll
    for (int s = 0; s < S; s++) {
        int t = 32 * s + lane_id();
        if (t < z.m) c += __popcll(z.X(0, t)) + __popcll(z.X(1, t)) + __popcll(z.X(2, t));
    }
#pragma unroll
    for (int d = 16; d; d >>= 1) c += __shfl_xor_sync(kFull, c, d);
    return c - 2 * z.m - z.nn2;
}

// minimizeKernel (complexity_minimizer.cu:245-263) for one walk.
template <class R, int S>
__device__ void z2_minimize_one(const DevBatch &B, const WalkParams &P, int w, uint64_t *xs, uint32_t *Ls,
                                int32_t *bestC) {
    const WalkHeader h = B.hdr[w];
    R r = DrawsIO<R>::load(B, P, w, h);
    Z2Walk<R, S> z(r);
    z.x = xs;
    z.L = Ls;
    z2_load(z, B, h, w);
    int best = bestC[w];
    int bestM = h.best_m;
    uint64_t accepted = 0;
    for (int it = 0; it < P.iterations; it++) {
        if (!z.tryFlip(false)) break;
        accepted++;
        int c = z2_complexity(z);
        if (c < best) {
            best = c;
            bestM = z.m;
            z2_copy_best(z, B, w);
        }
        if (z.status) break;
    }
    z2_store(z, B, w);
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

template <class R, int S>
__global__ void k_walk_z2(DevBatch B, WalkParams P) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5;
    const size_t per = walk_smem_bytes(B.cap);
    uint64_t *xs = reinterpret_cast<uint64_t *>(smem + per * warp);
    uint32_t *Ls = reinterpret_cast<uint32_t *>(xs + 3 * B.cap);
    for (int w = blockIdx.x * wpb + warp; w < B.S; w += gridDim.x * wpb) z2_walk_one<R, S>(B, P, w, xs, Ls);
}

template <class R, int S>
__global__ void k_minimize_z2(DevBatch B, WalkParams P, int32_t *bestC) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5;
    const size_t per = walk_smem_bytes(B.cap);
    uint64_t *xs = reinterpret_cast<uint64_t *>(smem + per * warp);
    uint32_t *Ls = reinterpret_cast<uint32_t *>(xs + 3 * B.cap);
    for (int w = blockIdx.x * wpb + warp; w < B.S; w += gridDim.x * wpb) z2_minimize_one<R, S>(B, P, w, xs, Ls, bestC);
}

// Rebuilds the lists of every walk from its factors (initFlips); used after
// naive initialisation and after host-provided records without lists.
template <int S>
__global__ void k_rebuild_lists_z2(DevBatch B) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5;
    const size_t per = walk_smem_bytes(B.cap);
    uint64_t *xs = reinterpret_cast<uint64_t *>(smem + per * warp);
    uint32_t *Ls = reinterpret_cast<uint32_t *>(xs + 3 * B.cap);
    for (int w = blockIdx.x * wpb + warp; w < B.S; w += gridDim.x * wpb) {
        WalkHeader h = B.hdr[w];
        h.list_size[0] = h.list_size[1] = h.list_size[2] = 0;
        PhiloxDraws unused;
        Z2Walk<PhiloxDraws, S> z(unused);
        z.x = xs;
        z.L = Ls;
        z2_load(z, B, h, w);
        z.rebuild();
        z2_store(z, B, w);
        if (lane_id() == 0) {
            B.hdr[w].list_size[0] = z.sz0;
            B.hdr[w].list_size[1] = z.sz1;
            B.hdr[w].list_size[2] = z.sz2;
        }
    }
}

}  // namespace fg
