// The additions reducer's flip pass for --max-flips > 0 (flipSchemesKernel,
// scheme_additions_reducer.cu:448-460): before each reduction after the first,
// scheme s (1 <= s < schemes) becomes scheme 0 after curand() % (maxFlips + 1)
// ternary flips (SchemeInteger::tryFlip with its reductions, scheme_integer.cu:
// 907-975), drawn from reducer s's own XORWOW stream, which the reducer then
// continues.  One warp per scheme, the ZT walk's shared-memory layout.
#include "launch.h"
#include "walk_zt.cuh"

namespace fg {

namespace {

struct FlipArgs {
    int schemes, n1, n2, n3, m, maxFlips;
    int8_t *coef;                     // [schemes][3][m][64]: scheme 0 read, 1.. written
    curandStateXORWOW_t *states;      // reducer streams [>= schemes]
    int32_t *ranks, *pairs, *status;  // [schemes]
};

// One warp's shared memory: a ZT walk of m slots, rounded to 16 bytes.
__host__ __device__ inline size_t flip_warp_bytes(int m) { return (zt_smem_bytes(m) + 15) / 16 * 16; }

__device__ __forceinline__ int warp_sum(int v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

template <int S>
__global__ void k_flip_schemes(FlipArgs A) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = lane_id();
    unsigned char *base = smem + flip_warp_bytes(A.m) * warp;
    const int m = A.m, cap = A.m;
    const int nn[3] = {A.n1 * A.n2, A.n2 * A.n3, A.n3 * A.n1};
    for (int s = 1 + blockIdx.x * wpb + warp; s < A.schemes; s += gridDim.x * wpb) {
        XorwowDraws r;
        r.st = A.states[s];
        r.count = 0;
        r.P = nullptr;  // tryFlip takes no gate draws
        ZTWalk<XorwowDraws, S> z(r);
        z.xv = reinterpret_cast<uint64_t *>(base);
        z.xs = z.xv + 3 * cap;
        z.xo = reinterpret_cast<uint8_t *>(z.xs + 3 * cap);
        z.L = reinterpret_cast<uint32_t *>(z.xo + ((size_t)3 * cap + 7) / 8 * 8);
        z.J = reinterpret_cast<uint16_t *>(z.L + 3 * kListCap);
        z.cap = cap;
        z.n0 = A.n1; z.n1 = A.n2; z.n2 = A.n3;
        z.nn0 = nn[0]; z.nn1 = nn[1]; z.nn2 = nn[2];
        z.full = A.n1 * A.n2 * A.n3;
        z.m = m;
        z.sz0 = z.sz1 = z.sz2 = 0;
        z.status = 0;
        // schemes[0].copyTo(schemes[s]) (scheme_integer.cu:66-79): the terms, then initFlips.
        for (int q = lane; q < 3 * m; q += 32) {
            const int c = q / m, t = q - c * m;
            const int8_t *row = A.coef + ((size_t)c * m + t) * 64;
            uint64_t v = 0, g = 0;
            for (int e = 0; e < nn[c]; e++) {
                if (row[e]) v |= 1ull << e;
                if (row[e] < 0) g |= 1ull << e;
            }
            z.xv[q] = v;
            z.xs[q] = g;
            z.xo[q] = 1;
        }
        __syncwarp();
        z.rebuild();
        const uint32_t flips = r.raw() % (uint32_t)(A.maxFlips + 1);
        for (uint32_t i = 0; i < flips; i++)
            if (!z.tryFlip(true) || z.status) break;
        __syncwarp();
        // The flipped scheme as the reducer's coefficient rows (rows past its rank zero).
        int8_t *out = A.coef + (size_t)s * 3 * m * 64;
        for (int q = lane; q < 3 * m * 64; q += 32) {
            const int c = q / (m * 64), t = (q / 64) % m, e = q % 64;
            int8_t val = 0;
            if (t < z.m && e < nn[c]) {
                const uint64_t v = z.xv[c * cap + t], g = z.xs[c * cap + t];
                val = (int8_t)(((v >> e) & 1) ? (((g >> e) & 1) ? -1 : 1) : 0);
            }
            out[q] = val;
        }
        // Largest pair-occurrence count of its three components (sizes the pair tables).
        int pu = 0, pv = 0, pw = 0;
        for (int t = lane; t < z.m; t += 32) {
            const int a = __popcll(z.xv[t]), b = __popcll(z.xv[cap + t]);
            pu += a * (a - 1) / 2;
            pv += b * (b - 1) / 2;
        }
        for (int e = lane; e < nn[2]; e += 32) {
            int k = 0;
            for (int t = 0; t < z.m; t++) k += (int)((z.xv[2 * cap + t] >> e) & 1);
            pw += k * (k - 1) / 2;
        }
        pu = warp_sum(pu);
        pv = warp_sum(pv);
        pw = warp_sum(pw);
        if (lane == 0) {
            A.states[s] = r.st;
            A.ranks[s] = z.m;
            A.pairs[s] = max(pu, max(pv, pw));
            A.status[s] = z.status;
        }
        __syncwarp();
    }
}

template <int S>
cudaError_t launch_flip(const FlipArgs &A, int sms, cudaStream_t st) {
    const int wpb = 4;
    const size_t smem = flip_warp_bytes(A.m) * wpb;
    cudaError_t e = cudaFuncSetAttribute(k_flip_schemes<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int need = (A.schemes - 1 + wpb - 1) / wpb;
    const int cap = 4 * (sms > 0 ? sms : 1);
    const int grid = need < 1 ? 1 : (need < cap ? need : cap);
    k_flip_schemes<S><<<grid, 32 * wpb, smem, st>>>(A);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_flip_schemes(int schemes, int n1, int n2, int n3, int m, int maxFlips, int8_t *coef,
                                curandStateXORWOW_t *states, int32_t *ranks, int32_t *pairs, int32_t *status, int sms,
                                cudaStream_t st) {
    if (schemes < 2) return cudaSuccess;
    if (m < 1 || m > kMaxRank + 2 || maxFlips < 0) return cudaErrorInvalidValue;
    const FlipArgs A{schemes, n1, n2, n3, m, maxFlips, coef, states, ranks, pairs, status};
    const int groups = (m + 31) / 32;
    if (groups <= 1) return launch_flip<1>(A, sms, st);
    if (groups <= 2) return launch_flip<2>(A, sms, st);
    if (groups <= 4) return launch_flip<4>(A, sms, st);
    return launch_flip<11>(A, sms, st);
}

}  // namespace fg
