// Per-slot-count Z2 launchers; each launch_z2_sN.cu instantiates one S so the
// kernel variants compile in parallel translation units.
#pragma once
#include "kernels.cuh"
#include "launch.h"

namespace fg {

template <class K> inline cudaError_t set_smem(K kernel, size_t smem) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <int S>
cudaError_t walk_z2_s(const DevBatch &B, const WalkParams &P, int rng, int wpb, int grid, cudaStream_t s) {
    size_t smem = walk_smem_bytes(B.cap) * wpb;
    if (rng == RNG_XORWOW) {
        cudaError_t e = set_smem(k_walk_z2<XorwowDraws, S>, smem);
        if (e != cudaSuccess) return e;
        k_walk_z2<XorwowDraws, S><<<grid, 32 * wpb, smem, s>>>(B, P);
    } else {
        cudaError_t e = set_smem(k_walk_z2<PhiloxDraws, S>, smem);
        if (e != cudaSuccess) return e;
        k_walk_z2<PhiloxDraws, S><<<grid, 32 * wpb, smem, s>>>(B, P);
    }
    return cudaGetLastError();
}

template <int S>
cudaError_t minimize_z2_s(const DevBatch &B, const WalkParams &P, int rng, int wpb, int grid, int32_t *bestC,
                          cudaStream_t s) {
    size_t smem = walk_smem_bytes(B.cap) * wpb;
    if (rng == RNG_XORWOW) {
        cudaError_t e = set_smem(k_minimize_z2<XorwowDraws, S>, smem);
        if (e != cudaSuccess) return e;
        k_minimize_z2<XorwowDraws, S><<<grid, 32 * wpb, smem, s>>>(B, P, bestC);
    } else {
        cudaError_t e = set_smem(k_minimize_z2<PhiloxDraws, S>, smem);
        if (e != cudaSuccess) return e;
        k_minimize_z2<PhiloxDraws, S><<<grid, 32 * wpb, smem, s>>>(B, P, bestC);
    }
    return cudaGetLastError();
}

template <int S> cudaError_t rebuild_z2_s(const DevBatch &B, int wpb, int grid, cudaStream_t s) {
    size_t smem = walk_smem_bytes(B.cap) * wpb;
    cudaError_t e = set_smem(k_rebuild_lists_z2<S>, smem);
    if (e != cudaSuccess) return e;
    k_rebuild_lists_z2<S><<<grid, 32 * wpb, smem, s>>>(B);
    return cudaGetLastError();
}

template <int S> int occupancy_z2_s(int cap, int rng, int wpb) {
    int blocks = 0;
    size_t smem = walk_smem_bytes(cap) * wpb;
    cudaError_t e;
    if (rng == RNG_XORWOW) {
        if (set_smem(k_walk_z2<XorwowDraws, S>, smem) != cudaSuccess) return 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_walk_z2<XorwowDraws, S>, 32 * wpb, smem);
    } else {
        if (set_smem(k_walk_z2<PhiloxDraws, S>, smem) != cudaSuccess) return 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_walk_z2<PhiloxDraws, S>, 32 * wpb, smem);
    }
    return e == cudaSuccess ? blocks : 0;
}

#define FG_INSTANTIATE_Z2(S)                                                                                   \
    template cudaError_t walk_z2_s<S>(const DevBatch &, const WalkParams &, int, int, int, cudaStream_t);      \
    template cudaError_t minimize_z2_s<S>(const DevBatch &, const WalkParams &, int, int, int, int32_t *,      \
                                          cudaStream_t);                                                       \
    template cudaError_t rebuild_z2_s<S>(const DevBatch &, int, int, cudaStream_t);                            \
    template int occupancy_z2_s<S>(int, int, int);

}  // namespace fg
