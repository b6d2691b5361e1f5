// Per-(ring, slot count) launchers of the warp-per-walk kernels; each
// launch_<ring>_s<S>.cu instantiates one pair so variants compile in parallel.
#pragma once
#include "kernels.cuh"
#include "launch.h"

namespace fg {

template <int RING, class R, int S> struct WalkerOf;
template <class R, int S> struct WalkerOf<0, R, S> { using type = Z2Walk<R, S>; };
template <class R, int S> struct WalkerOf<1, R, S> { using type = ZTWalk<R, S>; };

template <class K> inline cudaError_t set_smem(K kernel, size_t smem) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <int RING, class R, int S>
cudaError_t walk_rs(const DevBatch &B, const WalkParams &P, int wpb, int grid, cudaStream_t s) {
    using Wk = typename WalkerOf<RING, R, S>::type;
    size_t smem = RingIO<Wk>::smem(B.cap) * wpb;
    cudaError_t e = set_smem(k_walk<Wk, R>, smem);
    if (e != cudaSuccess) return e;
    k_walk<Wk, R><<<grid, 32 * wpb, smem, s>>>(B, P);
    return cudaGetLastError();
}

template <int RING, class R, int S>
cudaError_t minimize_rs(const DevBatch &B, const WalkParams &P, int wpb, int grid, int32_t *bestC, cudaStream_t s) {
    using Wk = typename WalkerOf<RING, R, S>::type;
    size_t smem = RingIO<Wk>::smem(B.cap) * wpb;
    cudaError_t e = set_smem(k_minimize<Wk, R>, smem);
    if (e != cudaSuccess) return e;
    k_minimize<Wk, R><<<grid, 32 * wpb, smem, s>>>(B, P, bestC);
    return cudaGetLastError();
}

template <int RING, class R, int S> int occupancy_rs(int cap, int wpb) {
    using Wk = typename WalkerOf<RING, R, S>::type;
    int blocks = 0;
    size_t smem = RingIO<Wk>::smem(cap) * wpb;
    if (set_smem(k_walk<Wk, R>, smem) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_walk<Wk, R>, 32 * wpb, smem) != cudaSuccess) return 0;
    return blocks;
}

template <int RING, int S>
cudaError_t walk_s(const DevBatch &B, const WalkParams &P, int rng, int wpb, int grid, cudaStream_t s) {
    return rng == RNG_XORWOW ? walk_rs<RING, XorwowDraws, S>(B, P, wpb, grid, s)
                             : walk_rs<RING, PhiloxDraws, S>(B, P, wpb, grid, s);
}

template <int RING, int S>
cudaError_t minimize_s(const DevBatch &B, const WalkParams &P, int rng, int wpb, int grid, int32_t *bestC,
                       cudaStream_t s) {
    return rng == RNG_XORWOW ? minimize_rs<RING, XorwowDraws, S>(B, P, wpb, grid, bestC, s)
                             : minimize_rs<RING, PhiloxDraws, S>(B, P, wpb, grid, bestC, s);
}

template <int RING, int S> cudaError_t rebuild_s(const DevBatch &B, int wpb, int grid, cudaStream_t s) {
    using Wk = typename WalkerOf<RING, PhiloxDraws, S>::type;
    size_t smem = RingIO<Wk>::smem(B.cap) * wpb;
    cudaError_t e = set_smem(k_rebuild<Wk>, smem);
    if (e != cudaSuccess) return e;
    k_rebuild<Wk><<<grid, 32 * wpb, smem, s>>>(B);
    return cudaGetLastError();
}

template <int RING, int S> int occupancy_s(int cap, int rng, int wpb) {
    return rng == RNG_XORWOW ? occupancy_rs<RING, XorwowDraws, S>(cap, wpb) : occupancy_rs<RING, PhiloxDraws, S>(cap, wpb);
}

#define FG_INSTANTIATE(RING, S)                                                                                \
    template cudaError_t walk_s<RING, S>(const DevBatch &, const WalkParams &, int, int, int, cudaStream_t);   \
    template cudaError_t minimize_s<RING, S>(const DevBatch &, const WalkParams &, int, int, int, int32_t *,   \
                                             cudaStream_t);                                                    \
    template cudaError_t rebuild_s<RING, S>(const DevBatch &, int, int, cudaStream_t);                         \
    template int occupancy_s<RING, S>(int, int, int);

}  // namespace fg
