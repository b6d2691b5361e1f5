// Bounded-integer (ZB) walk kernel (ZBWalk, one warp per walk) and its exact
// integer verification.
#include "launch.h"
#include "walk_zb.cuh"

namespace fg {

namespace {

// Records of walk w, components [3][cap] as sign-magnitude masks.
struct ZBRecord {
    uint64_t *fac, *sgn, *fac2;
};

__device__ __forceinline__ ZBRecord zb_record(const DevBatch &B, int w, bool best) {
    const size_t o = (size_t)w * 3 * B.cap;
    return best ? ZBRecord{B.best_fac + o, B.best_sgn + o, B.best_fac2 + o} : ZBRecord{B.fac + o, B.sgn + o, B.fac2 + o};
}

// Slots [0, hi) of a record from the walk's planes (zero from m on).
__device__ void zb_store(const ZBWalk &z, const ZBRecord &d, int cap, int hi) {
    for (int c = 0; c < 3; c++)
        for (int t = lane_id(); t < hi; t += 32) {
            uint64_t nz = 0, neg = 0, two = 0;
            if (t < z.m) v3toMasks(z.get(c, t), nz, neg, two);
            d.fac[c * cap + t] = nz;
            d.sgn[c * cap + t] = neg;
            d.fac2[c * cap + t] = two;
        }
}

__device__ void zb_walk_one(const DevBatch &B, const WalkParams &P, int w, uint64_t *base, int scap) {
    WalkHeader &hw = B.hdr[w];
    PhiloxDraws r;
    r.k0 = P.key0; r.k1 = P.key1; r.walk = (uint32_t)w; r.count = hw.draws; r.chunk = -1; r.P = &P;
    ZBWalk z(r);
    z.X = base;
    z.H = reinterpret_cast<uint16_t *>(base + 9 * scap);
    z.cap = scap;
    z.nslot = (scap + 31) / 32;
    z.n0 = hw.n[0]; z.n1 = hw.n[1]; z.n2 = hw.n[2];
    z.full = z.n0 * z.n1 * z.n2;
    z.nnc[0] = z.n0 * z.n1; z.nnc[1] = z.n1 * z.n2; z.nnc[2] = z.n2 * z.n0;
    for (int c = 0; c < 3; c++) z.Lc[c] = z.nnc[c] >= 64 ? ~0ull : ((1ull << z.nnc[c]) - 1);
    z.m = hw.m;
    z.status = hw.status;
    const ZBRecord src = zb_record(B, w, false);
    for (int q = lane_id(); q < 3 * scap; q += 32) {
        const int c = q / scap, t = q - c * scap;
        const Vec3 v = t < z.m ? v3fromMasks(src.fac[c * B.cap + t], src.sgn[c * B.cap + t], src.fac2[c * B.cap + t])
                               : Vec3{0, 0, 0};
        uint64_t *p = base + (size_t)c * 3 * scap + t;
        p[0] = v.b0; p[scap] = v.b1; p[2 * scap] = v.b2;
    }
    z.rebuildCounts();
    int flipsCount = hw.flips, bestRank = hw.best_rank, bestM = hw.best_m;
    bool copied = false;
    uint64_t accepted = 0;
    const ZBRecord best = zb_record(B, w, true);
    for (int it = 0; it < P.iterations; it++) {
        const int rank = z.m;
        const int f = z.tryFlip();
        if (f == 0) {
            if (z.status) break;
            z.tryExpand(randint(1, 2, r));
            if (z.status) break;
            continue;
        }
        if (f < 0) continue;  // the proposal left the bound
        accepted++;
        if (z.m < rank) flipsCount = 0;
        flipsCount++;
        if (z.m < bestRank || (z.m == bestRank && r.tie())) {
            bestRank = z.m;
            bestM = z.m;
            __syncwarp();
            zb_store(z, best, B.cap, z.m);
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
    zb_store(z, src, B.cap, B.cap);
    if (copied)
        for (int c = 0; c < 3; c++)
            for (int t = (bestM < 0 ? 0 : bestM) + lane_id(); t < B.cap; t += 32) {
                best.fac[c * B.cap + t] = 0;
                best.sgn[c * B.cap + t] = 0;
                best.fac2[c * B.cap + t] = 0;
            }
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

// Walks [first, first + count), one warp each (grid-stride over walks).  Six
// 4-warp blocks per SM (80 registers) measured 7-11 % faster than the
// unbounded build's four (118 registers), its few spills notwithstanding.
__global__ void __launch_bounds__(128, 6) k_walk_zb(DevBatch B, WalkParams P, int first, int count, int scap) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5;
    uint64_t *base = reinterpret_cast<uint64_t *>(smem) + (size_t)warp * zb_words(scap);
    for (int q = blockIdx.x * wpb + warp; q < count; q += gridDim.x * wpb) zb_walk_one(B, P, first + q, base, scap);
}

__device__ __forceinline__ int zb_coef(uint64_t nz, uint64_t neg, uint64_t two, int e) {
    const int a = (int)((nz >> e) & 1) << (int)((two >> e) & 1);
    return ((neg >> e) & 1) ? -a : a;
}

// Exact integer Brent check, one warp per walk: every (i, j, k) equation
// sum_t u_t[i] v_t[j] w_t[k] equals its 0/1 target.
__global__ void k_verify_zb(DevBatch B, int best, uint8_t *out) {
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cap = B.cap;
    for (int w = blockIdx.x * wpb + warp; w < B.S; w += gridDim.x * wpb) {
        const WalkHeader h = B.hdr[w];
        const ZBRecord s = zb_record(B, w, best);
        const int n0 = h.n[0], n1 = h.n[1], n2 = h.n[2];
        const int nn0 = n0 * n1, nn1 = n1 * n2, nn2 = n2 * n0;
        const int m = best ? h.best_m : h.m;
        bool ok = m >= 0 && m <= cap;
        const int eqs = nn0 * nn1 * nn2;
        for (int q = lane; ok && q < eqs; q += 32) {
            const int i = q / (nn1 * nn2), j = (q / nn2) % nn1, k = q % nn2;
            const int target = (i % n1 == j / n2) && (i / n1 == k % n0) && (j % n2 == k / n0);
            int e = 0;
            for (int t = 0; t < m; t++) {
                const int a = zb_coef(s.fac[t], s.sgn[t], s.fac2[t], i);
                if (!a) continue;
                const int b = zb_coef(s.fac[cap + t], s.sgn[cap + t], s.fac2[cap + t], j);
                if (!b) continue;
                e += a * b * zb_coef(s.fac[2 * cap + t], s.sgn[2 * cap + t], s.fac2[2 * cap + t], k);
            }
            ok = e == target;
        }
        ok = __all_sync(kFull, ok);
        if (lane == 0) {
            out[w] = ok;
            if (!best) B.hdr[w].valid = ok;
        }
        __syncwarp();
    }
}

}  // namespace

cudaError_t launch_walk_zb(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int sms,
                           cudaStream_t s) {
    if (scap < 1 || scap > B.cap || scap > kMaxRank + 2) return cudaErrorInvalidValue;
    const int wpb = 4;
    const size_t smem = (size_t)wpb * zb_words(scap) * sizeof(uint64_t);
    cudaError_t e = cudaFuncSetAttribute(k_walk_zb, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int blocks = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_walk_zb, 32 * wpb, smem);
    if (e != cudaSuccess) return e;
    if (blocks < 1) return cudaErrorInvalidConfiguration;
    const int need = (count + wpb - 1) / wpb;
    const int grid = need < blocks * sms ? need : blocks * sms;
    k_walk_zb<<<grid, 32 * wpb, smem, s>>>(B, P, first, count, scap);
    return cudaGetLastError();
}

cudaError_t launch_verify_zb(const DevBatch &B, int best, uint8_t *out, cudaStream_t s) {
    const int wpb = 4;
    k_verify_zb<<<(B.S + wpb - 1) / wpb, 32 * wpb, 0, s>>>(B, best, out);
    return cudaGetLastError();
}

}  // namespace fg
