// List-mode Z2 walk kernel, one thread per walk (walk_simt_list.cuh), and its launcher.
#include "launch.h"
#include "walk_simt_list.cuh"

namespace fg {

namespace {

template <class R> struct ThreadDrawsIO;

template <> struct ThreadDrawsIO<ThreadXorwow> {
    static __device__ ThreadXorwow load(const DevBatch &B, const WalkParams &P, int w, const WalkHeader &h) {
        ThreadXorwow r;
        r.st = B.xorwow[w];
        r.count = h.draws;
        r.P = &P;
        return r;
    }
    static __device__ void store(const DevBatch &B, int w, const ThreadXorwow &r) { B.xorwow[w] = r.st; }
};

template <> struct ThreadDrawsIO<ThreadPhilox> {
    static __device__ ThreadPhilox load(const DevBatch &, const WalkParams &P, int w, const WalkHeader &h) {
        ThreadPhilox r;
        r.k0 = P.key0; r.k1 = P.key1; r.walk = (uint32_t)w; r.count = h.draws; r.blk = -1; r.P = &P;
        return r;
    }
    static __device__ void store(const DevBatch &, int, const ThreadPhilox &) {}
};

// The walk's current scheme (or best scheme) back to its records: every slot up to the
// records' cap, zero past the rank.
template <class W, class R>
__device__ void store_factors(const SimtListZ2<W, R> &z, uint64_t *dst, int cap) {
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < cap; t++) dst[c * cap + t] = t < z.m ? (uint64_t)z.X(c, t) : 0ull;
}

// randomWalkKernel (flip_graph.cu:520-573) for one walk, one thread: the loop of the
// warp-per-walk walk_one with the same draw sites (sandwiching, basis and Gauss moves
// are off for this kernel; their gates still take the reference's draws).
template <class W, class R>
__device__ void simt_list_walk_one(const DevBatch &B, const WalkParams &P, int w, W *s, int ld, uint32_t *Lw) {
    const WalkHeader h = B.hdr[w];
    R r = ThreadDrawsIO<R>::load(B, P, w, h);
    SimtListZ2<W, R> z(r);
    z.x = s;
    z.L = Lw;
    z.ld = ld;
    z.cap = ld < B.cap ? ld : B.cap;
    z.n0 = h.n[0]; z.n1 = h.n[1]; z.n2 = h.n[2];
    z.nn0 = z.n0 * z.n1; z.nn1 = z.n1 * z.n2; z.nn2 = z.n2 * z.n0;
    z.full = z.n0 * z.n1 * z.n2;
    z.m = h.m;
    z.sz0 = h.list_size[0]; z.sz1 = h.list_size[1]; z.sz2 = h.list_size[2];
    z.status = h.status;
    const uint64_t *src = B.fac + (size_t)w * 3 * B.cap;
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < ld; t++) z.setX(c, t, t < h.m ? (W)src[c * B.cap + t] : (W)0);
    for (int c = 0; c < 3; c++) {
        const uint32_t *ls = B.lists + ((size_t)w * 3 + c) * kListCap;
        for (int q = 0; q < h.list_size[c]; q++) z.setLq(c, q, ls[q]);
    }
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
            store_factors(z, B.best_fac + (size_t)w * 3 * B.cap, B.cap);
            if (B.best_n) {
                B.best_n[w * 3 + 0] = z.n0;
                B.best_n[w * 3 + 1] = z.n1;
                B.best_n[w * 3 + 2] = z.n2;
            }
        }
        if (r.gate_reduce()) z.tryReduce();
        r.gate_gauss();  // off for this kernel: takes the draw the warp kernel's gate takes
        if (r.gate_expand() && z.m <= bestM + 2) {
            if (z.tryExpand(randint(1, 2, r))) flipsCount = 0;
        }
        r.gate_sandwich();  // probability 0 for this kernel; the gates' draws are kept
        r.gate_basis();
        if (flipsCount >= P.plus_iterations && z.tryPlus()) flipsCount = 0;
        if (z.status) break;
    }
    store_factors(z, B.fac + (size_t)w * 3 * B.cap, B.cap);
    for (int c = 0; c < 3; c++) {
        uint32_t *ls = B.lists + ((size_t)w * 3 + c) * kListCap;
        const int sc = z.sz(c);
        for (int q = 0; q < kListCap; q++) ls[q] = q < sc ? z.Lq(c, q) : 0u;
    }
    ThreadDrawsIO<R>::store(B, w, r);
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

// Walks [first, first + count); ld factor slots per walk in shared memory; lists in the
// scratch, walk w's column at lists + ((w / 32) * 3 * kListCap * 32) + w % 32.
template <class W, class R>
__global__ void k_walk_simt_list(DevBatch B, WalkParams P, int first, int count, int ld, uint32_t *lists) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    W *s = reinterpret_cast<W *>(smem) + (size_t)warp * 3 * ld * 32 + lane;
    for (int base = (blockIdx.x * wpb + warp) * 32; base < count; base += gridDim.x * wpb * 32) {
        const int q = base + lane;
        if (q < count) {
            const int w = first + q;
            uint32_t *Lw = lists + (size_t)(w >> 5) * 3 * kListCap * 32 + (w & 31);
            simt_list_walk_one<W, R>(B, P, w, s, ld, Lw);
        }
    }
}

template <class W> size_t list_smem(int ld, int wpb) { return (size_t)wpb * 3 * ld * 32 * sizeof(W); }

template <class W, class R>
cudaError_t walk_simt_list_t(const DevBatch &B, const WalkParams &P, int first, int count, int ld, int wpb, int sms,
                             uint32_t *lists, cudaStream_t s) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (list_smem<W>(ld, 1) > (size_t)optin) return cudaErrorInvalidConfiguration;
    while (wpb > 1 && list_smem<W>(ld, wpb) > (size_t)optin) wpb--;
    const size_t smem = list_smem<W>(ld, wpb);
    cudaError_t e = cudaFuncSetAttribute(k_walk_simt_list<W, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int blocks = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_walk_simt_list<W, R>, 32 * wpb, smem);
    if (e != cudaSuccess) return e;
    if (blocks < 1) return cudaErrorInvalidConfiguration;
    const int need = (count + 32 * wpb - 1) / (32 * wpb);
    const int grid = need < blocks * sms ? need : blocks * sms;
    k_walk_simt_list<W, R><<<grid, 32 * wpb, smem, s>>>(B, P, first, count, ld, lists);
    return cudaGetLastError();
}

}  // namespace

size_t simt_list_smem_per_warp(int scap, int wide) { return (size_t)3 * scap * 32 * (wide ? 8 : 4); }

size_t simt_list_scratch_words(int walks) { return (size_t)((walks + 31) / 32) * 32 * 3 * kListCap; }

cudaError_t launch_walk_simt_list(const DevBatch &B, const WalkParams &P, int rng, int first, int count, int scap,
                                  int wide, int wpb, int sms, uint32_t *lists, cudaStream_t s) {
    if (rng == RNG_XORWOW) {
        if (wide) return walk_simt_list_t<unsigned long long, ThreadXorwow>(B, P, first, count, scap, wpb, sms, lists, s);
        return walk_simt_list_t<uint32_t, ThreadXorwow>(B, P, first, count, scap, wpb, sms, lists, s);
    }
    if (wide) return walk_simt_list_t<unsigned long long, ThreadPhilox>(B, P, first, count, scap, wpb, sms, lists, s);
    return walk_simt_list_t<uint32_t, ThreadPhilox>(B, P, first, count, scap, wpb, sms, lists, s);
}

}  // namespace fg
