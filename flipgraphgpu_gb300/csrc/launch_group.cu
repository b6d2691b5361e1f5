// Fast-mode group-per-walk Z2 kernel (GroupFast: G lanes per walk) and its launcher.
#include "kernels.cuh"
#include "launch.h"
#include "walk_group.cuh"

namespace fg {

namespace {

// Global [3][cap] record slots [0, hi) from the compact [3][scap] words (factors
// only, zero from m on); the group's lanes stride by G.
template <class W, int G, int S>
__device__ __forceinline__ void group_store(uint64_t *dst, const W *base, int cap, int scap, int m, int hi, int g) {
    for (int c = 0; c < 3; c++)
        for (int t = g; t < hi; t += G)
            dst[c * cap + t] = t < m ? (uint64_t)(base[c * scap + t] & GroupFast<W, G, S>::FM) : 0ull;
}

template <class W, int G, int S>
__device__ void group_walk_one(const DevBatch &B, const WalkParams &P, int w, W *base, int scap, unsigned mask, int g,
                               int gbase) {
    WalkHeader &hw = B.hdr[w];
    GroupDraws<G> r;
    r.k0 = P.key0; r.k1 = P.key1; r.walk = (uint32_t)w; r.count = hw.draws; r.chunk = -1; r.P = &P;
    r.mask = mask; r.g = g;
    GroupFast<W, G, S> z(r);
    z.s = base;
    z.cap = scap;
    z.n0 = hw.n[0]; z.n1 = hw.n[1]; z.n2 = hw.n[2];
    z.m = hw.m;
    z.status = hw.status;
    z.mask = mask; z.g = g; z.gbase = gbase;
    const uint64_t *src = B.fac + (size_t)w * 3 * B.cap;
    for (int q = g; q < 3 * scap; q += G) {
        const int c = q / scap, t = q - c * scap;
        base[q] = t < z.m ? (W)src[c * B.cap + t] : (W)0;
    }
    z.rebuild();
    int flipsCount = hw.flips, bestRank = hw.best_rank, bestM = hw.best_m;
    uint64_t accepted = 0;
    bool copied = false;
    uint64_t *bdst = B.best_fac + (size_t)w * 3 * B.cap;
    // with resizing on, each launch runs randint(1, iterations) steps (flip_graph.cu:531)
    const int iterations = P.random_iterations ? randint(1, P.iterations, r) : P.iterations;
    for (int it = 0; it < iterations; it++) {
        const int rank = z.m;
        if (!z.tryFlip(true)) {
            if (z.status) break;
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
            __syncwarp(mask);
            group_store<W, G, S>(bdst, base, B.cap, scap, z.m, z.m, g);
            copied = true;
        }
        if (r.gate_reduce()) z.tryReduce();
        if (r.gate_gauss()) z.tryReduceGauss();  // not in the reference's walk
        if (r.gate_expand() && z.m <= bestM + 2) {
            if (z.tryExpand(randint(1, 2, r))) flipsCount = 0;
        }
        if (r.gate_sandwich()) z.sandwich();  // flip_graph.cu:560-561
        if (r.gate_basis()) z.swapBasis();    // flip_graph.cu:563-564
        if (flipsCount >= P.plus_iterations && z.tryPlus()) flipsCount = 0;
        if (z.status) break;
    }
    __syncwarp(mask);
    group_store<W, G, S>(B.fac + (size_t)w * 3 * B.cap, base, B.cap, scap, z.m, B.cap, g);
    if (copied)
        for (int c = 0; c < 3; c++)
            for (int t = (bestM < 0 ? 0 : bestM) + g; t < B.cap; t += G) bdst[c * B.cap + t] = 0ull;
    __syncwarp(mask);
    if (g == 0) {
        if (copied && B.best_n)  // resizing: the best scheme's sizes
            for (int c = 0; c < 3; c++) B.best_n[w * 3 + c] = hw.n[c];
        hw.m = z.m;
        hw.flips = flipsCount;
        hw.best_rank = bestRank;
        hw.best_m = bestM;
        hw.status = z.status;
        hw.list_size[0] = hw.list_size[1] = hw.list_size[2] = 0;
        hw.draws = r.count;
        hw.flips_done = accepted;
    }
}

// minimizeKernel (complexity_minimizer.cu:190-214) for one walk, G lanes: flips without
// reduction tests, the complexity after every flip (a group sum of popcounts), the lowest
// one's scheme kept as the best; the same results as the thread-per-walk minimizer.
template <class W, int G, int S>
__device__ void group_minimize_one(const DevBatch &B, const WalkParams &P, int w, W *base, int scap, unsigned mask,
                                   int g, int gbase, int32_t *bestC) {
    WalkHeader &hw = B.hdr[w];
    GroupDraws<G> r;
    r.k0 = P.key0; r.k1 = P.key1; r.walk = (uint32_t)w; r.count = hw.draws; r.chunk = -1; r.P = &P;
    r.mask = mask; r.g = g;
    GroupFast<W, G, S> z(r);
    z.s = base;
    z.cap = scap;
    z.n0 = hw.n[0]; z.n1 = hw.n[1]; z.n2 = hw.n[2];
    z.m = hw.m;
    z.status = hw.status;
    z.mask = mask; z.g = g; z.gbase = gbase;
    const uint64_t *src = B.fac + (size_t)w * 3 * B.cap;
    for (int q = g; q < 3 * scap; q += G) {
        const int c = q / scap, t = q - c * scap;
        base[q] = t < z.m ? (W)src[c * B.cap + t] : (W)0;
    }
    z.rebuild();
    const int nn2 = z.n2 * z.n0;
    int best = bestC[w], bestM = hw.best_m;
    bool copied = false;
    uint64_t accepted = 0;
    uint64_t *bdst = B.best_fac + (size_t)w * 3 * B.cap;
    for (int it = 0; it < P.iterations; it++) {
        if (!z.tryFlip(false)) break;
        accepted++;
        int pop = 0;
        for (int x = 0; x < S; x++) {
            const int t = x * G + g;
            if (t < z.m)
                pop += __popcll((unsigned long long)z.F(0, t)) + __popcll((unsigned long long)z.F(1, t)) +
                       __popcll((unsigned long long)z.F(2, t));
        }
        const int cplx = z.gsum(pop) - 2 * z.m - nn2;
        if (cplx < best) {
            best = cplx;
            bestM = z.m;
            __syncwarp(mask);
            group_store<W, G, S>(bdst, base, B.cap, scap, z.m, z.m, g);
            copied = true;
        }
        if (z.status) break;
    }
    __syncwarp(mask);
    group_store<W, G, S>(B.fac + (size_t)w * 3 * B.cap, base, B.cap, scap, z.m, B.cap, g);
    if (copied)
        for (int c = 0; c < 3; c++)
            for (int t = (bestM < 0 ? 0 : bestM) + g; t < B.cap; t += G) bdst[c * B.cap + t] = 0ull;
    __syncwarp(mask);
    if (g == 0) {
        hw.m = z.m;
        hw.best_m = bestM;
        hw.status = z.status;
        hw.list_size[0] = hw.list_size[1] = hw.list_size[2] = 0;
        hw.draws = r.count;
        hw.flips_done = accepted;
        bestC[w] = best;
    }
}

template <class W, int G, int S>
__global__ void k_minimize_group(DevBatch B, WalkParams P, int first, int count, int scap, int ws, int32_t *bestC) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int GPW = 32 / G;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    const int gi = lane / G, g = lane % G, gbase = gi * G;
    const unsigned mask = group_bits<G>() << gbase;
    W *base = reinterpret_cast<W *>(smem) + (size_t)(warp * GPW + gi) * ws;
    for (int q0 = (blockIdx.x * wpb + warp) * GPW; q0 < count; q0 += gridDim.x * wpb * GPW) {
        const int q = q0 + gi;
        if (q < count) group_minimize_one<W, G, S>(B, P, first + q, base, scap, mask, g, gbase, bestC);
    }
}

// Walks [first, first + count), 32/G per warp; `ws` = words between walks in shared memory.
template <class W, int G, int S>
__global__ void k_walk_group(DevBatch B, WalkParams P, int first, int count, int scap, int ws) {
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int GPW = 32 / G;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    const int gi = lane / G, g = lane % G, gbase = gi * G;
    const unsigned mask = group_bits<G>() << gbase;
    W *base = reinterpret_cast<W *>(smem) + (size_t)(warp * GPW + gi) * ws;
    for (int q0 = (blockIdx.x * wpb + warp) * GPW; q0 < count; q0 += gridDim.x * wpb * GPW) {
        const int q = q0 + gi;
        if (q < count) group_walk_one<W, G, S>(B, P, first + q, base, scap, mask, g, gbase);
    }
}

// bestC == nullptr: the walk; else the minimizer with bestC as the running best complexities.
template <class W, int G, int S>
cudaError_t group_t(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int sms, cudaStream_t s,
                    int32_t *bestC = nullptr) {
    if (scap > G * S) return cudaErrorInvalidValue;
    const int wpb = 4;
    // Walks of a warp start (32k + G) words apart: slot x of the 32/G groups hits 32 distinct banks.
    const int ws = (3 * scap + 31) / 32 * 32 + G;
    const size_t smem = (size_t)wpb * (32 / G) * ws * sizeof(W);
    const void *fn = bestC ? (const void *)k_minimize_group<W, G, S> : (const void *)k_walk_group<W, G, S>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int blocks = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, 32 * wpb, smem);
    if (e != cudaSuccess) return e;
    if (blocks < 1) return cudaErrorInvalidConfiguration;
    const int perBlock = wpb * (32 / G);
    const int need = (count + perBlock - 1) / perBlock;
    const int grid = need < blocks * sms ? need : blocks * sms;
    if (bestC) k_minimize_group<W, G, S><<<grid, 32 * wpb, smem, s>>>(B, P, first, count, scap, ws, bestC);
    else k_walk_group<W, G, S><<<grid, 32 * wpb, smem, s>>>(B, P, first, count, scap, ws);
    return cudaGetLastError();
}

template <class W>
cudaError_t group_w(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int lanes, int sms,
                    cudaStream_t s) {
    const int minLanes = scap <= 64 ? 4 : (scap <= 128 ? 8 : 16);
    if (lanes < minLanes) lanes = minLanes;  // 0 = automatic; too few lanes for the slots: widen
    if (lanes == 4) {
        if (scap <= 16) return group_t<W, 4, 4>(B, P, first, count, scap, sms, s);
        if (scap <= 32) return group_t<W, 4, 8>(B, P, first, count, scap, sms, s);
        if (scap <= 64) return group_t<W, 4, 16>(B, P, first, count, scap, sms, s);
        return cudaErrorInvalidValue;
    }
    if (lanes == 8) {
        if (scap <= 64) return group_t<W, 8, 8>(B, P, first, count, scap, sms, s);
        if (scap <= 128) return group_t<W, 8, 16>(B, P, first, count, scap, sms, s);
        return cudaErrorInvalidValue;
    }
    if (lanes == 16) {
        if (scap <= 256) return group_t<W, 16, 16>(B, P, first, count, scap, sms, s);
        if (scap <= 352) return group_t<W, 16, 22>(B, P, first, count, scap, sms, s);
        return cudaErrorInvalidValue;
    }
    if (lanes == 32) {  // one walk per warp, terms slot-major (conflict-free)
        if (scap <= 32) return group_t<W, 32, 1>(B, P, first, count, scap, sms, s);
        if (scap <= 64) return group_t<W, 32, 2>(B, P, first, count, scap, sms, s);
        if (scap <= 128) return group_t<W, 32, 4>(B, P, first, count, scap, sms, s);
        if (scap <= 352) return group_t<W, 32, 11>(B, P, first, count, scap, sms, s);
        return cudaErrorInvalidValue;
    }
    return cudaErrorInvalidValue;
}

// The minimizer, one warp per walk (slot-major, 32 lanes).
template <class W>
cudaError_t minimize_w(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int sms,
                       int32_t *bestC, cudaStream_t s) {
    if (scap <= 32) return group_t<W, 32, 1>(B, P, first, count, scap, sms, s, bestC);
    if (scap <= 64) return group_t<W, 32, 2>(B, P, first, count, scap, sms, s, bestC);
    if (scap <= 128) return group_t<W, 32, 4>(B, P, first, count, scap, sms, s, bestC);
    if (scap <= 352) return group_t<W, 32, 11>(B, P, first, count, scap, sms, s, bestC);
    return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t launch_minimize_group(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int wide,
                                  int sms, int32_t *bestC, cudaStream_t s) {
    if (scap < 1 || scap > B.cap) return cudaErrorInvalidValue;
    return wide ? minimize_w<unsigned long long>(B, P, first, count, scap, sms, bestC, s)
                : minimize_w<uint32_t>(B, P, first, count, scap, sms, bestC, s);
}

cudaError_t launch_walk_group(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int wide,
                              int lanes, int sms, cudaStream_t s) {
    if (scap < 1 || scap > B.cap) return cudaErrorInvalidValue;
    return wide ? group_w<unsigned long long>(B, P, first, count, scap, lanes, sms, s)
                : group_w<uint32_t>(B, P, first, count, scap, lanes, sms, s);
}

}  // namespace fg
