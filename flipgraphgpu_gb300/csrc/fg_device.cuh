// Device-side building blocks shared by the walk, minimizer and verification
// kernels: batch layout, draw policies and warp-cooperative FlipSet lists.
//
// Execution model: one warp owns one walk.  Every lane runs the same
// (warp-uniform) control flow; lanes own terms t = lane + 32*s of the scheme
// for the parallel scans, and lane 0 performs the rare serial edits
// (term compaction, plus/split) on the warp's shared-memory copy.
#pragma once
#include <cstdint>
#include <curand_kernel.h>

namespace fg {

constexpr int kMaxRank = 350;   // reference config.cuh:10
constexpr int kListCap = 500;   // reference config.cuh:14 (FlipSet capacity)
constexpr unsigned kFull = 0xffffffffu;
constexpr int kRetryCap = 1 << 20;  // bound on the reference's unbounded retry loops
enum : int { ST_RETRY = 2, ST_OVERFLOW = 4, ST_INTERNAL = 8 };  // ST_INTERNAL: pair counts inconsistent

// Per-walk header in HBM (64 bytes).
struct WalkHeader {
    int32_t n[3];
    int32_t m;
    int32_t flips;       // flips since the last rank drop
    int32_t best_rank;
    int32_t best_m;
    int32_t status;
    int32_t list_size[3];
    int32_t valid;       // last verification result
    uint64_t draws;      // draws consumed since seeding
    uint64_t flips_done; // accepted flips in the last launch
};
static_assert(sizeof(WalkHeader) == 64, "header layout");

// Device records: walk w owns fac[w*3*cap ...], lists[w*3*500 ...] etc., so a
// warp reads and writes its own walk with contiguous, coalesced accesses.
struct DevBatch {
    int S, cap;
    WalkHeader *hdr;
    uint64_t *fac, *sgn;
    uint8_t *valid;
    uint32_t *lists;
    uint64_t *best_fac, *best_sgn;
    uint8_t *best_valid;
    curandStateXORWOW_t *xorwow;  // reference stream states (FG_RNG_XORWOW)
    int32_t *best_n;              // [S][3] sizes of the best scheme (resizing), or null
    uint64_t *fac2, *best_fac2;   // ZB: |c| = 2 masks (fac = nonzero, sgn = negative)
};

constexpr uint64_t kGateOff = ~0ull;

struct WalkParams {
    int iterations;
    int plus_iterations;
    // Reference gates: curand_uniform() * iterations < p  <=>  product < gate_f (the
    // least float >= p), so the comparison stays in single precision.
    float reduce_gate_f, expand_gate_f, sandwich_gate_f, basis_gate_f, tie_gate_f;
    // Philox gates: draw < threshold, threshold = floor(p / iterations * 2^32);
    // kGateOff (p <= 0) = never fires and takes no draw.
    uint64_t reduce_T, expand_T, sandwich_T, basis_T;
    // Gauss (XOR) reduction gate (no reference counterpart in the walk): off takes no draw.
    int gauss_on;
    float gauss_gate_f;
    uint64_t gauss_T;
    int zt_sandwich;  // ZT: sandwiching by signed permutations (the reference's move is empty)
    uint32_t key0, key1;  // Philox key (seed)
    int random_iterations;  // resizing on: each launch runs randint(1, iterations) steps (flip_graph.cu:531)
    int retry_cap;          // bound on the reference's unbounded retry loops (> 0)
    int max_matrix;         // resizing: most entries a grown factor may hold (64; 56 in the fast mode)
};

// The retry bound of a walk's parameters; kRetryCap where a caller runs without them
// (the additions reducer's flip pass).
__device__ __forceinline__ int retry_cap_of(const WalkParams *P) {
    return P && P->retry_cap > 0 ? P->retry_cap : kRetryCap;
}

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ unsigned lanemask_lt() { return (1u << lane_id()) - 1u; }

// ---------------------------------------------------------------- draws
// Reference stream: cuRAND XORWOW, replicated in every lane (all lanes advance
// identical copies, so no broadcast is needed).  Draw sites follow the
// reference exactly: curand() % k, curand() % 2, float gates.
struct XorwowDraws {
    curandStateXORWOW_t st;
    uint64_t count;
    const WalkParams *P;
    __device__ __forceinline__ uint32_t raw() { count++; return curand(&st); }
    __device__ __forceinline__ float uniform() { count++; return curand_uniform(&st); }
    __device__ __forceinline__ uint32_t below(uint32_t k) { return raw() % k; }
    __device__ __forceinline__ bool coin() { return raw() & 1u; }
    __device__ __forceinline__ bool gate_reduce() { return uniform() * (float)P->iterations < P->reduce_gate_f; }
    __device__ __forceinline__ bool gate_expand() { return uniform() * (float)P->iterations < P->expand_gate_f; }
    __device__ __forceinline__ bool gate_sandwich() { return uniform() * (float)P->iterations < P->sandwich_gate_f; }
    __device__ __forceinline__ bool gate_basis() { return uniform() * (float)P->iterations < P->basis_gate_f; }
    __device__ __forceinline__ bool gate_gauss() { return P->gauss_on && uniform() * (float)P->iterations < P->gauss_gate_f; }
    __device__ __forceinline__ bool tie() { return uniform() < P->tie_gate_f; }
    __device__ __forceinline__ uint64_t mask(int nn) { return (uint64_t)raw() % ((uint64_t)1 << nn); }
};

// Philox4x32-10 block function (Salmon, Moraes, Dror, Shaw, SC'11).
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    }
    return c;
}

// Fast stream: word q of walk w is Philox(ctr = (q/4 lo, q/4 hi, w, 0), key)[q % 4].
// A warp computes 32 consecutive blocks at once (lane l -> block 32*c + l), i.e.
// 128 words per refill, and serves them in order with one shuffle per draw.
struct PhiloxDraws {
    uint32_t k0, k1, walk;
    uint64_t count;   // next word index
    int64_t chunk;    // 128-word chunk held in buf
    uint4 buf;
    const WalkParams *P;
    __device__ __forceinline__ uint32_t raw() {
        int64_t c = (int64_t)(count >> 7);
        if (c != chunk) {
            uint64_t blk = ((uint64_t)c << 5) + (uint64_t)lane_id();
            buf = philox4x32_10(make_uint4((uint32_t)blk, (uint32_t)(blk >> 32), walk, 0u), k0, k1);
            chunk = c;
        }
        uint32_t wq = (uint32_t)count & 127u;
        uint32_t e = wq & 3u;
        uint32_t v = e == 0 ? buf.x : e == 1 ? buf.y : e == 2 ? buf.z : buf.w;
        count++;
        return __shfl_sync(kFull, v, (int)(wq >> 2));
    }
    __device__ __forceinline__ float uniform() { return (float)(raw() >> 8) * (1.0f / 16777216.0f); }
    __device__ __forceinline__ uint32_t below(uint32_t k) { return __umulhi(raw(), k); }
    __device__ __forceinline__ bool coin() { return raw() >> 31; }
    __device__ __forceinline__ bool gate(uint64_t T) { return T != kGateOff && (uint64_t)raw() < T; }
    __device__ __forceinline__ bool gate_reduce() { return gate(P->reduce_T); }
    __device__ __forceinline__ bool gate_expand() { return gate(P->expand_T); }
    __device__ __forceinline__ bool gate_sandwich() { return gate(P->sandwich_T); }
    __device__ __forceinline__ bool gate_basis() { return gate(P->basis_T); }
    __device__ __forceinline__ bool gate_gauss() { return gate(P->gauss_T); }
    __device__ __forceinline__ bool tie() { return raw() < 42949672u; }
    __device__ __forceinline__ uint64_t mask(int nn) { return nn >= 32 ? (uint64_t)raw() : (uint64_t)(raw() & ((1u << nn) - 1u)); }
};

template <class R> __device__ __forceinline__ int randint(int a, int b, R &r) { return a + (int)r.below((uint32_t)(b - a + 1)); }

// ---------------------------------------------------------------- FlipSet lists
__device__ __forceinline__ bool touches(uint32_t v, uint32_t idx) { return (v >> 16) == idx || (v & 0xFFFFu) == idx; }

// First position >= from holding a pair that touches idx (sz when none).
__device__ __forceinline__ int list_next_match(const uint32_t *L, int sz, uint32_t idx, int from) {
    for (int base = from; base < sz; base += 32) {
        int q = base + lane_id();
        bool hit = q < sz && touches(L[q], idx);
        unsigned b = __ballot_sync(kFull, hit);
        if (b) return base + __ffs(b) - 1;
    }
    return sz;
}

// FlipSet::remove(index) (flip_set.cu:27-31): removes every pair touching idx by
// swapping in the last element and re-checking it.  The matches are located with
// ballots; only those positions are visited, giving the reference's exact order.
__device__ __forceinline__ int list_remove_index(uint32_t *L, int sz, uint32_t idx) {
    int p = list_next_match(L, sz, idx, 0);
    while (p < sz) {
        sz--;
        if (p == sz) break;
        uint32_t v = L[sz];
        __syncwarp();
        if (lane_id() == 0) L[p] = v;
        __syncwarp();
        if (touches(v, idx)) continue;
        p = list_next_match(L, sz, idx, p + 1);
    }
    return sz;
}

// Appends (hi, t) for every t whose bit is set in masks[s] (t = 32*s + lane), in
// ascending t, dropping pairs past the capacity as FlipSet::add does (flip_set.cu:7-13).
template <int S>
__device__ __forceinline__ int list_append(uint32_t *L, int sz, uint32_t hi, const unsigned (&masks)[S]) {
    int base = sz;
#pragma unroll
    for (int s = 0; s < S; s++) {
        unsigned msk = masks[s];
        if ((msk >> lane_id()) & 1u) {
            int pos = base + __popc(msk & lanemask_lt());
            if (pos < kListCap) L[pos] = (hi << 16) | (uint32_t)(32 * s + lane_id());
        }
        base += __popc(msk);
    }
    __syncwarp();
    return base < kListCap ? base : kListCap;
}

// Inclusive warp prefix sum.
__device__ __forceinline__ int warp_inclusive_sum(int v) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        int o = __shfl_up_sync(kFull, v, d);
        if (lane_id() >= d) v += o;
    }
    return v;
}

// Least float f with (double)f >= p: float products compared against it give the
// same answer as the reference's float-to-double comparison with p.
inline float ceil_to_float(double p) {
    float f = (float)p;
    if ((double)f < p) f = nextafterf(f, __builtin_huge_valf());
    return f;
}

}  // namespace fg
