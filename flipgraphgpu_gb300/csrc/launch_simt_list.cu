// List-mode walk kernels, one thread per walk (Z2: walk_simt_list.cuh, ZT:
// walk_simt_list_zt.cuh), and their launcher.
#include <vector>

#include "launch.h"
#include "walk_simt_list.cuh"
#include "walk_simt_list_zt.cuh"

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

// Per-ring binding of a thread's walk to its shared-memory column (32 walks interleaved by
// lane) and its scratch column, and the record I/O.  Slots past the rank are written as zero.
template <class Z> struct ListRing;

template <class W, class R> struct ListRing<SimtListZ2<W, R>> {
    static constexpr int kWords = 1;  // factor words per (component, slot)
    static constexpr int kScratchVecs = 3 * kListVecs;
    static __device__ void bind(SimtListZ2<W, R> &z, unsigned char *col, uint4 *scr, const uint2 *) {
        z.x = reinterpret_cast<W *>(col);
        z.V = scr;
    }
    static __device__ void load(SimtListZ2<W, R> &z, const DevBatch &B, int w, int m) {
        const uint64_t *src = B.fac + (size_t)w * 3 * B.cap;
        for (int c = 0; c < 3; c++)
            for (int t = 0; t < z.ld; t++) z.setX(c, t, t < m ? (W)src[c * B.cap + t] : (W)0);
    }
    static __device__ void store(const SimtListZ2<W, R> &z, const DevBatch &B, int w, bool best) {
        uint64_t *dst = (best ? B.best_fac : B.fac) + (size_t)w * 3 * B.cap;
        for (int c = 0; c < 3; c++)
            for (int t = 0; t < B.cap; t++) dst[c * B.cap + t] = t < z.m ? (uint64_t)z.X(c, t) : 0ull;
    }
};

template <class R> struct ListRing<SimtListZT<R>> {
    static constexpr int kWords = 2;  // values and signs
    static constexpr int kScratchVecs = 3 * kListVecs + kPermVecs;
    static __device__ void bind(SimtListZT<R> &z, unsigned char *col, uint4 *scr, const uint2 *mg) {
        z.xv = reinterpret_cast<uint32_t *>(col);
        z.xs = z.xv + (size_t)3 * z.ld * 32;
        z.V = scr;
        z.J = scr + ((size_t)3 * kListVecs << 5);
        z.mg = mg;
    }
    // 64-bit record words in, 32-bit words out: every factor's bits 32-63 must copy bit 31
    // and, above 16 entries, every factor must be valid (the host routes other batches to
    // the warp kernel; a word that breaks this stops the walk with ST_INTERNAL, its record
    // untouched, rather than being cut).
    static __device__ void load(SimtListZT<R> &z, const DevBatch &B, int w, int m) {
        const size_t o = (size_t)w * 3 * B.cap;
        const int nnmax = max(z.nn0, max(z.nn1, z.nn2));
        z.mk = nnmax > 16 ? 0u : kInvalidMark;
        for (int c = 0; c < 3; c++)
            for (int t = 0; t < z.ld; t++) {
                const bool in = t < m;
                const size_t q = o + c * B.cap + t;
                const uint64_t v = in ? B.fac[q] : 0ull, sg = in ? B.sgn[q] : 0ull;
                const bool ok = !in || B.valid[q];
                if ((uint64_t)(int64_t)(int32_t)v != v || (uint64_t)(int64_t)(int32_t)sg != sg || (!ok && !z.mk))
                    z.status |= ST_INTERNAL;
                z.xv[z.at(c, t)] = (uint32_t)v;
                z.xs[z.at(c, t)] = (uint32_t)sg | (ok ? 0u : z.mk);
            }
    }
    static __device__ void store(const SimtListZT<R> &z, const DevBatch &B, int w, bool best) {
        const size_t o = (size_t)w * 3 * B.cap;
        uint64_t *dv = best ? B.best_fac : B.fac;
        uint64_t *ds = best ? B.best_sgn : B.sgn;
        uint8_t *dk = best ? B.best_valid : B.valid;
        for (int c = 0; c < 3; c++)
            for (int t = 0; t < B.cap; t++) {
                const bool in = t < z.m;
                const uint32_t sg = in ? z.xs[z.at(c, t)] : 0u, v = in ? z.xv[z.at(c, t)] : 0u;
                dv[o + c * B.cap + t] = (uint64_t)(int64_t)(int32_t)v;
                ds[o + c * B.cap + t] = (uint64_t)(int64_t)(int32_t)(sg & ~z.mk);
                dk[o + c * B.cap + t] = in && !(sg & z.mk) ? 1 : 0;
            }
    }
};

// randomWalkKernel (flip_graph.cu:520-573) for one walk, one thread: the loop of the
// warp-per-walk walk_one with the same draw sites (sandwiching, basis and Gauss moves
// are off for this kernel; their gates still take the reference's draws).
template <class Z, class R>
__device__ void simt_list_walk_one(const DevBatch &B, const WalkParams &P, int w, unsigned char *col, int ld,
                                   uint4 *scr, const uint2 *mg) {
    const WalkHeader h = B.hdr[w];
    R r = ThreadDrawsIO<R>::load(B, P, w, h);
    Z z(r);
    z.ld = ld;
    ListRing<Z>::bind(z, col, scr, mg);
    z.cap = ld < B.cap ? ld : B.cap;
    z.n0 = h.n[0]; z.n1 = h.n[1]; z.n2 = h.n[2];
    z.nn0 = z.n0 * z.n1; z.nn1 = z.n1 * z.n2; z.nn2 = z.n2 * z.n0;
    z.full = z.n0 * z.n1 * z.n2;
    z.m = h.m;
    z.sz0 = h.list_size[0]; z.sz1 = h.list_size[1]; z.sz2 = h.list_size[2];
    z.status = h.status;
    ListRing<Z>::load(z, B, w, h.m);
    if (z.status & ~h.status) {  // a record the ring's words cannot hold: the walk stops, its record untouched
        B.hdr[w].status = z.status;
        return;
    }
    for (int c = 0; c < 3; c++) {
        const uint32_t *ls = B.lists + ((size_t)w * 3 + c) * kListCap;
        for (int q = 0; q < h.list_size[c]; q++) z.setLq(c, q, pack16((int)(ls[q] >> 16), (int)(ls[q] & 0xFFFFu)));
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
            ListRing<Z>::store(z, B, w, true);
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
    ListRing<Z>::store(z, B, w, false);
    for (int c = 0; c < 3; c++) {
        uint32_t *ls = B.lists + ((size_t)w * 3 + c) * kListCap;
        const int sc = z.sz(c);
        for (int q = 0; q < kListCap; q++) {
            const uint32_t e = q < sc ? z.Lq(c, q) : 0u;
            ls[q] = q < sc ? ((e >> 8) << 16) | (e & 0xFFu) : 0u;
        }
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

// Walks [first, first + count); ld (<= 256) slots per walk in shared memory (kWords words
// of wb bytes per slot and component); walk w's scratch column of 16-byte vectors at
// scratch + (w / 32) * kScratchVecs * 32 + w % 32.
template <class Z, class R, int WB>
__global__ void k_walk_simt_list(DevBatch B, WalkParams P, int first, int count, int ld, uint4 *scratch,
                                 const uint2 *mg) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    unsigned char *col = smem + ((size_t)warp * ListRing<Z>::kWords * 3 * ld * 32 + lane) * WB;
    for (int base = (blockIdx.x * wpb + warp) * 32; base < count; base += gridDim.x * wpb * 32) {
        const int q = base + lane;
        if (q < count) {
            const int w = first + q;
            uint4 *scr = scratch + (size_t)(w >> 5) * ListRing<Z>::kScratchVecs * 32 + (w & 31);
            simt_list_walk_one<Z, R>(B, P, w, col, ld, scr, mg);
        }
    }
}

template <class Z, class R, int WB>
cudaError_t walk_simt_list_t(const DevBatch &B, const WalkParams &P, int first, int count, int ld, int wpb, int sms,
                             uint4 *scratch, const uint2 *mg, cudaStream_t s) {
    if (ld > 256) return cudaErrorInvalidValue;  // list entries hold slot indices in 8 bits
    auto smemFor = [&](int k) { return (size_t)k * ListRing<Z>::kWords * 3 * ld * 32 * WB; };
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (smemFor(1) > (size_t)optin) return cudaErrorInvalidConfiguration;
    while (wpb > 1 && smemFor(wpb) > (size_t)optin) wpb--;
    const size_t smem = smemFor(wpb);
    cudaError_t e = cudaFuncSetAttribute(k_walk_simt_list<Z, R, WB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    int blocks = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_walk_simt_list<Z, R, WB>, 32 * wpb, smem);
    if (e != cudaSuccess) return e;
    if (blocks < 1) return cudaErrorInvalidConfiguration;
    const int need = (count + 32 * wpb - 1) / (32 * wpb);
    const int grid = need < blocks * sms ? need : blocks * sms;
    k_walk_simt_list<Z, R, WB><<<grid, 32 * wpb, smem, s>>>(B, P, first, count, ld, scratch, mg);
    return cudaGetLastError();
}

}  // namespace

// Factor word bytes of the Z2 list kernel: 4 for factors of at most 32 entries, else 8.  (16-bit
// words for factors of at most 16 entries measured slower on GB300: 2.62 against 3.21 G flips/s on
// the six-shape batch; the extra resident warps crowd the L1 that serves the list scans.)
int simt_list_word_bytes(int nnmax) { return nnmax <= 32 ? 4 : 8; }

size_t simt_list_smem_per_warp(int ring, int scap, int nnmax) {
    return ring == 1 ? (size_t)2 * 3 * scap * 32 * 4 : (size_t)3 * scap * 32 * simt_list_word_bytes(nnmax);
}

// The lists (and for ZT the permutation draws) of every walk, then the remainder table.
size_t simt_list_walk_bytes(int ring, int walks) {
    const int vecs = ring == 1 ? 3 * kListVecs + kPermVecs : 3 * kListVecs;
    return (size_t)((walks + 31) / 32) * 32 * vecs * sizeof(uint4);
}

size_t simt_list_scratch_bytes(int ring, int walks) {
    return simt_list_walk_bytes(ring, walks) + (size_t)kRemTableSize * sizeof(uint2);
}

cudaError_t simt_list_init_scratch(int ring, int walks, void *scratch, cudaStream_t s) {
    std::vector<uint2> t(kRemTableSize, make_uint2(0u, 1u));
    for (uint32_t d = 2; d < (uint32_t)kRemTableSize; d++) {
        uint32_t l = 0;
        while ((1u << l) < d) l++;
        t[d] = make_uint2((uint32_t)((((uint64_t)((1u << l) - d)) << 32) / d + 1), l);
    }
    unsigned char *dst = static_cast<unsigned char *>(scratch) + simt_list_walk_bytes(ring, walks);
    cudaError_t e = cudaMemcpyAsync(dst, t.data(), t.size() * sizeof(uint2), cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s);  // the host table goes out of scope
}

cudaError_t launch_walk_simt_list(int ring, const DevBatch &B, const WalkParams &P, int rng, int first, int count,
                                  int scap, int nnmax, int wpb, int sms, void *scratch, cudaStream_t s) {
    const int wb = simt_list_word_bytes(nnmax);
    uint4 *v = static_cast<uint4 *>(scratch);
    const uint2 *mg = reinterpret_cast<const uint2 *>(static_cast<unsigned char *>(scratch) +
                                                      simt_list_walk_bytes(ring, B.S));
    using U64 = unsigned long long;
    if (ring == 1) {
        if (rng == RNG_XORWOW) return walk_simt_list_t<SimtListZT<ThreadXorwow>, ThreadXorwow, 4>(B, P, first, count, scap, wpb, sms, v, mg, s);
        return walk_simt_list_t<SimtListZT<ThreadPhilox>, ThreadPhilox, 4>(B, P, first, count, scap, wpb, sms, v, mg, s);
    }
    if (rng == RNG_XORWOW) {
        if (wb == 8) return walk_simt_list_t<SimtListZ2<U64, ThreadXorwow>, ThreadXorwow, 8>(B, P, first, count, scap, wpb, sms, v, mg, s);
        return walk_simt_list_t<SimtListZ2<uint32_t, ThreadXorwow>, ThreadXorwow, 4>(B, P, first, count, scap, wpb, sms, v, mg, s);
    }
    if (wb == 8) return walk_simt_list_t<SimtListZ2<U64, ThreadPhilox>, ThreadPhilox, 8>(B, P, first, count, scap, wpb, sms, v, mg, s);
    return walk_simt_list_t<SimtListZ2<uint32_t, ThreadPhilox>, ThreadPhilox, 4>(B, P, first, count, scap, wpb, sms, v, mg, s);
}

}  // namespace fg
