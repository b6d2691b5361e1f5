// Fast-mode warp-per-walk Z2 kernel (WarpFast) and its launcher.
#include "kernels.cuh"
#include "launch.h"
#include "walk_warpfast.cuh"

namespace fg {

namespace {

// Global [3][cap] record from the compact [3][scap] words (factors only):
// slots [0, m) and, when `tail`, zeros in [m, cap).
template <class W, int S>
__device__ __forceinline__ void store_compact(uint64_t *dst, const W *base, int cap, int scap, int m, bool tail) {
    const int hi = tail ? cap : m;
    for (int c = 0; c < 3; c++)
        for (int t = lane_id(); t < hi; t += 32)
            dst[c * cap + t] = t < m ? (uint64_t)(base[c * scap + t] & WarpFast<W, S>::FM) : 0ull;
}

__device__ __forceinline__ void clear_tail(uint64_t *dst, int cap, int from) {
    for (int c = 0; c < 3; c++)
        for (int t = (from < 0 ? 0 : from) + lane_id(); t < cap; t += 32) dst[c * cap + t] = 0ull;
}

template <class W, int S>
__device__ void warpfast_walk_one(const DevBatch &B, const WalkParams &P, int w, W *base, int scap) {
    WalkHeader &hw = B.hdr[w];
    PhiloxDraws r;
    r.k0 = P.key0; r.k1 = P.key1; r.walk = (uint32_t)w; r.count = hw.draws; r.chunk = -1; r.P = &P;
    WarpFast<W, S> z(r);
    z.s = base;
    z.cap = scap;
    z.n0 = hw.n[0]; z.n1 = hw.n[1]; z.n2 = hw.n[2];
    z.m = hw.m;
    z.status = hw.status;
    const uint64_t *src = B.fac + (size_t)w * 3 * B.cap;
    for (int q = lane_id(); q < 3 * scap; q += 32) {
        const int c = q / scap, t = q - c * scap;
        base[q] = t < z.m ? (W)src[c * B.cap + t] : (W)0;
    }
    z.rebuild();
    int flipsCount = hw.flips, bestRank = hw.best_rank, bestM = hw.best_m;
    bool copied = false;
    uint64_t accepted = 0;
    uint64_t *bdst = B.best_fac + (size_t)w * 3 * B.cap;
    for (int it = 0; it < P.iterations; it++) {
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
            __syncwarp();
            store_compact<W, S>(bdst, base, B.cap, scap, z.m, false);
            copied = true;
        }
        if (r.gate_reduce()) z.tryReduce();
        if (r.gate_expand() && z.m <= bestM + 2) {
            if (z.tryExpand(randint(1, 2, r))) flipsCount = 0;
        }
        if (flipsCount >= P.plus_iterations && z.tryPlus()) flipsCount = 0;
        if (z.status) break;
    }
    __syncwarp();
    uint64_t *dst = B.fac + (size_t)w * 3 * B.cap;
    store_compact<W, S>(dst, base, B.cap, scap, z.m, true);
    if (copied) clear_tail(bdst, B.cap, bestM);
    if (lane_id() == 0) {
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

// Walks [first, first + count), one warp each (grid-stride over walks).
template <class W, int S>
__global__ void k_walk_warpfast(DevBatch B, WalkParams P, int first, int count, int scap) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5;
    W *base = reinterpret_cast<W *>(smem) + (size_t)warp * 3 * scap;
    for (int q = blockIdx.x * wpb + warp; q < count; q += gridDim.x * wpb)
        warpfast_walk_one<W, S>(B, P, first + q, base, scap);
}

template <class W, int S>
cudaError_t warpfast_t(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int sms,
                       cudaStream_t s) {
    const int wpb = 4;
    const size_t smem = (size_t)wpb * 3 * scap * sizeof(W);
    cudaError_t e = cudaFuncSetAttribute(k_walk_warpfast<W, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int blocks = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_walk_warpfast<W, S>, 32 * wpb, smem);
    if (e != cudaSuccess) return e;
    if (blocks < 1) return cudaErrorInvalidConfiguration;
    const int need = (count + wpb - 1) / wpb;
    const int grid = need < blocks * sms ? need : blocks * sms;
    k_walk_warpfast<W, S><<<grid, 32 * wpb, smem, s>>>(B, P, first, count, scap);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_walk_warpfast(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int wide,
                                 int sms, cudaStream_t s) {
    if (scap < 1 || scap > B.cap) return cudaErrorInvalidValue;
    switch (slots_for_cap(scap) | (wide << 8)) {
        case 1: return warpfast_t<uint32_t, 1>(B, P, first, count, scap, sms, s);
        case 2: return warpfast_t<uint32_t, 2>(B, P, first, count, scap, sms, s);
        case 4: return warpfast_t<uint32_t, 4>(B, P, first, count, scap, sms, s);
        case 11: return warpfast_t<uint32_t, 11>(B, P, first, count, scap, sms, s);
        case 256 + 1: return warpfast_t<unsigned long long, 1>(B, P, first, count, scap, sms, s);
        case 256 + 2: return warpfast_t<unsigned long long, 2>(B, P, first, count, scap, sms, s);
        case 256 + 4: return warpfast_t<unsigned long long, 4>(B, P, first, count, scap, sms, s);
        case 256 + 11: return warpfast_t<unsigned long long, 11>(B, P, first, count, scap, sms, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace fg
