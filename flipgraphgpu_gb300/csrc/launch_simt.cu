// Fast-mode (SIMT, one thread per walk) Z2 walk kernel and launcher.
#include "launch.h"
#include "walk_simt.cuh"

namespace fg {

namespace {

// Words between components of a walk in shared memory: the slot count rounded up
// to a multiple of 4, so the pair search reads whole groups of 4 without bounds tests.
__host__ __device__ __forceinline__ int simt_ld(int scap) { return (scap + 3) / 4 * 4; }

// Snapshot of the live terms; the slots past the final best rank are cleared
// once at the end of the launch (simt_clear_best_tail).
template <class W>
__device__ __forceinline__ void simt_copy_best(const SimtZ2<W> &z, const DevBatch &B, int w) {
    uint64_t *dst = B.best_fac + (size_t)w * 3 * B.cap;
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < z.m; t++) dst[c * B.cap + t] = (uint64_t)z.F(c, t);
}

__device__ __forceinline__ void simt_clear_best_tail(const DevBatch &B, int w, int bestM) {
    uint64_t *dst = B.best_fac + (size_t)w * 3 * B.cap;
    for (int c = 0; c < 3; c++)
        for (int t = bestM < 0 ? 0 : bestM; t < B.cap; t++) dst[c * B.cap + t] = 0ull;
}

// randomWalkKernel (flip_graph.cu:520-573) for one walk, one thread.  MV: the gates of the
// rare moves (Gauss reduction, sandwiching, basis changes) are compiled in (a run with their
// probabilities 0 takes the kernel without them: their calls alone cost the walk loop a
// quarter of its speed).
template <class W, bool MV>
__device__ void simt_walk_one(const DevBatch &B, const WalkParams &P, int w, W *s, int scap) {
    const WalkHeader h = B.hdr[w];
    ThreadPhilox r;
    r.k0 = P.key0; r.k1 = P.key1; r.walk = (uint32_t)w; r.count = h.draws; r.blk = -1; r.P = &P;
    SimtZ2<W> z(r);
    z.s = s;
    z.cap = scap;
    z.ld = simt_ld(scap);
    z.n0 = h.n[0]; z.n1 = h.n[1]; z.n2 = h.n[2];
    z.nn0 = z.n0 * z.n1; z.nn1 = z.n1 * z.n2; z.nn2 = z.n2 * z.n0;
    z.full = z.n0 * z.n1 * z.n2;
    z.m = h.m;
    z.status = h.status;
    const uint64_t *src = B.fac + (size_t)w * 3 * B.cap;
    for (int c = 0; c < 3; c++)  // slots past the rank stay zero (SimtZ2::pickPair relies on it)
        for (int t = 0; t < z.ld; t++) z.A(c, t) = t < z.m ? (W)src[c * B.cap + t] : (W)0;
    z.rebuild();
    int flipsCount = h.flips, bestRank = h.best_rank, bestM = h.best_m;
    uint64_t accepted = 0;
    bool copied = false;
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
            simt_copy_best(z, B, w);
            copied = true;
        }
        if (r.gate_reduce()) z.tryReduce();
        if constexpr (MV) {
            if (r.gate_gauss()) z.tryReduceGauss();  // not in the reference's walk
        }
        if (r.gate_expand() && z.m <= bestM + 2) {
            if (z.tryExpand(randint(1, 2, r))) flipsCount = 0;
        }
        if constexpr (MV) {
            if (r.gate_sandwich()) z.sandwich();  // flip_graph.cu:560-561
            if (r.gate_basis()) z.swapBasis();    // flip_graph.cu:563-564
        }
        if (flipsCount >= P.plus_iterations && z.tryPlus()) flipsCount = 0;
        if (z.status) break;
    }
    uint64_t *dst = B.fac + (size_t)w * 3 * B.cap;
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < B.cap; t++) dst[c * B.cap + t] = t < z.m ? (uint64_t)z.F(c, t) : 0ull;
    if (copied) simt_clear_best_tail(B, w, bestM);
    if (copied && B.best_n)  // resizing: the best scheme's sizes
        for (int c = 0; c < 3; c++) B.best_n[w * 3 + c] = h.n[c];
    WalkHeader o = h;
    o.m = z.m;
    o.flips = flipsCount;
    o.best_rank = bestRank;
    o.best_m = bestM;
    o.status = z.status;
    o.list_size[0] = o.list_size[1] = o.list_size[2] = 0;
    o.draws = r.count;
    o.flips_done = accepted;
    B.hdr[w] = o;
}

// minimizeKernel (complexity_minimizer.cu:190-214) for one walk in the fast mode: flips
// without reduction tests (a zero factor still removes its term), the complexity
// (sum of factor popcounts - 2m - n3*n1, scheme_z2.cu:127-139) after every flip, the
// lowest one's scheme kept as the best.  Same stream and pair order as the walk.
template <class W>
__device__ void simt_minimize_one(const DevBatch &B, const WalkParams &P, int w, W *s, int scap, int32_t *bestC) {
    const WalkHeader h = B.hdr[w];
    ThreadPhilox r;
    r.k0 = P.key0; r.k1 = P.key1; r.walk = (uint32_t)w; r.count = h.draws; r.blk = -1; r.P = &P;
    SimtZ2<W> z(r);
    z.s = s;
    z.cap = scap;
    z.ld = simt_ld(scap);
    z.n0 = h.n[0]; z.n1 = h.n[1]; z.n2 = h.n[2];
    z.nn0 = z.n0 * z.n1; z.nn1 = z.n1 * z.n2; z.nn2 = z.n2 * z.n0;
    z.full = z.n0 * z.n1 * z.n2;
    z.m = h.m;
    z.status = h.status;
    const uint64_t *src = B.fac + (size_t)w * 3 * B.cap;
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < z.ld; t++) z.A(c, t) = t < z.m ? (W)src[c * B.cap + t] : (W)0;
    z.rebuild();
    int best = bestC[w], bestM = h.best_m;
    bool copied = false;
    uint64_t accepted = 0;
    for (int it = 0; it < P.iterations; it++) {
        if (!z.tryFlip(false)) break;
        accepted++;
        int pop = 0;
        for (int t = 0; t < z.m; t++)
            pop += __popcll((unsigned long long)z.F(0, t)) + __popcll((unsigned long long)z.F(1, t)) +
                   __popcll((unsigned long long)z.F(2, t));
        const int cplx = pop - 2 * z.m - z.nn2;
        if (cplx < best) {
            best = cplx;
            bestM = z.m;
            simt_copy_best(z, B, w);
            copied = true;
        }
        if (z.status) break;
    }
    uint64_t *dst = B.fac + (size_t)w * 3 * B.cap;
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < B.cap; t++) dst[c * B.cap + t] = t < z.m ? (uint64_t)z.F(c, t) : 0ull;
    if (copied) simt_clear_best_tail(B, w, bestM);
    WalkHeader o = h;
    o.m = z.m;
    o.best_m = bestM;
    o.status = z.status;
    o.list_size[0] = o.list_size[1] = o.list_size[2] = 0;
    o.draws = r.count;
    o.flips_done = accepted;
    B.hdr[w] = o;
    bestC[w] = best;
}

template <class W>
__global__ void k_minimize_simt(DevBatch B, WalkParams P, int first, int count, int scap, int32_t *bestC) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    W *s = reinterpret_cast<W *>(smem) + (size_t)warp * 3 * simt_ld(scap) * 32 + lane;
    for (int base = (blockIdx.x * wpb + warp) * 32; base < count; base += gridDim.x * wpb * 32) {
        const int q = base + lane;
        if (q < count) simt_minimize_one<W>(B, P, first + q, s, scap, bestC);
    }
}

// Walks [first, first + count) of the batch; scap = slots per walk in shared memory.
template <class W, bool MV>
__global__ void k_walk_simt(DevBatch B, WalkParams P, int first, int count, int scap) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    W *s = reinterpret_cast<W *>(smem) + (size_t)warp * 3 * simt_ld(scap) * 32 + lane;
    for (int base = (blockIdx.x * wpb + warp) * 32; base < count; base += gridDim.x * wpb * 32) {
        const int q = base + lane;
        if (q < count) simt_walk_one<W, MV>(B, P, first + q, s, scap);
    }
}

template <class W> size_t simt_smem(int scap, int wpb) { return (size_t)wpb * 3 * simt_ld(scap) * 32 * sizeof(W); }

template <class W>
cudaError_t minimize_simt_t(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int wpb, int sms,
                            int32_t *bestC, cudaStream_t s) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (simt_smem<W>(scap, 1) > (size_t)optin) return cudaErrorInvalidConfiguration;
    while (wpb > 1 && simt_smem<W>(scap, wpb) > (size_t)optin) wpb--;
    const size_t smem = simt_smem<W>(scap, wpb);
    cudaError_t e = cudaFuncSetAttribute(k_minimize_simt<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int blocks = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_minimize_simt<W>, 32 * wpb, smem);
    if (e != cudaSuccess) return e;
    if (blocks < 1) return cudaErrorInvalidConfiguration;
    const int need = (count + 32 * wpb - 1) / (32 * wpb);
    const int grid = need < blocks * sms ? need : blocks * sms;
    k_minimize_simt<W><<<grid, 32 * wpb, smem, s>>>(B, P, first, count, scap, bestC);
    return cudaGetLastError();
}

template <class W, bool MV>
cudaError_t walk_simt_t(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int wpb, int sms,
                        cudaStream_t s) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const size_t perWarp = simt_smem<W>(scap, 1);
    if (perWarp > (size_t)optin) return cudaErrorInvalidConfiguration;  // rank too large for this mode
    while (wpb > 1 && simt_smem<W>(scap, wpb) > (size_t)optin) wpb--;
    size_t smem = simt_smem<W>(scap, wpb);
    cudaError_t e = cudaFuncSetAttribute(k_walk_simt<W, MV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int blocks = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_walk_simt<W, MV>, 32 * wpb, smem);
    if (e != cudaSuccess) return e;
    if (blocks < 1) return cudaErrorInvalidConfiguration;
    int need = (count + 32 * wpb - 1) / (32 * wpb);
    int grid = need < blocks * sms ? need : blocks * sms;
    k_walk_simt<W, MV><<<grid, 32 * wpb, smem, s>>>(B, P, first, count, scap);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_walk_simt(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int wide,
                             int wpb, int sms, cudaStream_t s) {
    const bool moves = P.sandwich_T != kGateOff || P.basis_T != kGateOff || P.gauss_T != kGateOff;
    if (wide) return moves ? walk_simt_t<unsigned long long, true>(B, P, first, count, scap, wpb, sms, s)
                           : walk_simt_t<unsigned long long, false>(B, P, first, count, scap, wpb, sms, s);
    return moves ? walk_simt_t<uint32_t, true>(B, P, first, count, scap, wpb, sms, s)
                 : walk_simt_t<uint32_t, false>(B, P, first, count, scap, wpb, sms, s);
}

cudaError_t launch_minimize_simt(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int wide,
                                 int wpb, int sms, int32_t *bestC, cudaStream_t s) {
    if (wide) return minimize_simt_t<unsigned long long>(B, P, first, count, scap, wpb, sms, bestC, s);
    return minimize_simt_t<uint32_t>(B, P, first, count, scap, wpb, sms, bestC, s);
}

}  // namespace fg
