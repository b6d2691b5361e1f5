// C-ABI of libflipgraph (include/flipgraph.h): handle lifetime, record
// transfer, launches, exact verification and test-support streams.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/flipgraph.h"
#include "launch.h"
#include "learned.h"

using namespace fg;

namespace fg {
std::string &last_error() {
    thread_local std::string err;
    return err;
}
}  // namespace fg

namespace {

fg_status fail(fg_status st, const std::string &msg) {
    fg::last_error() = msg;
    return st;
}

#define FG_CUDA(call)                                                                              \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail(FG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));          \
    } while (0)

// ---------------------------------------------------------------- small kernels
__global__ void k_init_xorwow(curandStateXORWOW_t *st, int S, unsigned long long seed) {
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w < S) curand_init(seed, (unsigned long long)w, 0ull, &st[w]);  // flip_graph.cu:450
}

// initializeNaive (scheme_z2.cu:32-55 / scheme_integer.cu:41-64) + initializeSchemesKernel
// (flip_graph.cu:510-518); lists are built afterwards by the rebuild kernel.
__global__ void k_init_naive(DevBatch B, int n1_, int n2_, int n3_, const int32_t *shapes, int zt) {
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= B.S) return;
    const int n1 = shapes ? shapes[w * 3] : n1_, n2 = shapes ? shapes[w * 3 + 1] : n2_, n3 = shapes ? shapes[w * 3 + 2] : n3_;
    const int cap = B.cap;
    uint64_t *f = B.fac + (size_t)w * 3 * cap, *bf = B.best_fac + (size_t)w * 3 * cap;
    for (int q = 0; q < 3 * cap; q++) { f[q] = 0; bf[q] = 0; }
    if (zt) {
        uint64_t *g = B.sgn + (size_t)w * 3 * cap, *bg = B.best_sgn + (size_t)w * 3 * cap;
        uint8_t *v = B.valid + (size_t)w * 3 * cap, *bv = B.best_valid + (size_t)w * 3 * cap;
        for (int q = 0; q < 3 * cap; q++) { g[q] = 0; bg[q] = 0; v[q] = 0; bv[q] = 0; }
    }
    if (B.fac2) {  // ZB: signs and |c| = 2 masks start at zero
        uint64_t *g = B.sgn + (size_t)w * 3 * cap, *bg = B.best_sgn + (size_t)w * 3 * cap;
        uint64_t *t2 = B.fac2 + (size_t)w * 3 * cap, *bt2 = B.best_fac2 + (size_t)w * 3 * cap;
        for (int q = 0; q < 3 * cap; q++) { g[q] = 0; bg[q] = 0; t2[q] = 0; bt2[q] = 0; }
    }
    for (int i = 0; i < n1; i++)
        for (int j = 0; j < n3; j++)
            for (int k = 0; k < n2; k++) {
                int t = (i * n3 + j) * n2 + k;
                uint64_t a = 1ull << (i * n2 + k), b = 1ull << (k * n3 + j), c = 1ull << (j * n1 + i);
                f[t] = bf[t] = a;
                f[cap + t] = bf[cap + t] = b;
                f[2 * cap + t] = bf[2 * cap + t] = c;
                if (zt)
                    for (int q = 0; q < 3; q++) {
                        B.valid[(size_t)w * 3 * cap + q * cap + t] = 1;
                        B.best_valid[(size_t)w * 3 * cap + q * cap + t] = 1;
                    }
            }
    if (B.best_n) { B.best_n[w * 3] = n1; B.best_n[w * 3 + 1] = n2; B.best_n[w * 3 + 2] = n3; }
    WalkHeader h = B.hdr[w];
    h.n[0] = n1; h.n[1] = n2; h.n[2] = n3;
    h.m = n1 * n2 * n3;
    h.flips = 0;
    h.best_rank = n1 * n2 * n3;
    h.best_m = n1 * n2 * n3;
    h.status = 0;
    h.list_size[0] = h.list_size[1] = h.list_size[2] = 0;
    h.valid = 0;
    h.flips_done = 0;
    B.hdr[w] = h;
}

// Exact Brent check (scheme_z2.cu:3-29), one warp per walk, bit-sliced over k:
// for every (i, j), XOR over terms of [u_t(i) & v_t(j)] * w_t must equal the
// single target bit k = (j % n2) * n0 + i / n1 when i % n1 == j / n2, else 0.
__global__ void k_verify_z2(DevBatch B, int best, uint8_t *out) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cap = B.cap;
    uint64_t *x = reinterpret_cast<uint64_t *>(smem) + (size_t)warp * 3 * cap;
    for (int w = blockIdx.x * wpb + warp; w < B.S; w += gridDim.x * wpb) {
        const WalkHeader h = B.hdr[w];
        const uint64_t *src = (best ? B.best_fac : B.fac) + (size_t)w * 3 * cap;
        for (int q = lane; q < 3 * cap; q += 32) x[q] = src[q];
        __syncwarp();
        const int32_t *dims = best && B.best_n ? B.best_n + w * 3 : h.n;
        const int n0 = dims[0], n1 = dims[1], n2 = dims[2];
        const int nn0 = n0 * n1, nn1 = n1 * n2, nn2 = n2 * n0;
        const int m = best ? h.best_m : h.m;
        const uint64_t kmask = nn2 >= 64 ? ~0ull : ((1ull << nn2) - 1);
        bool ok = m >= 0 && m <= cap;
        for (int q = lane; ok && q < nn0 * nn1; q += 32) {
            const int i = q / nn1, j = q % nn1;
            uint64_t acc = 0;
            for (int t = 0; t < m; t++)
                if (((x[t] >> i) & (x[cap + t] >> j)) & 1ull) acc ^= x[2 * cap + t];
            uint64_t target = (i % n1 == j / n2) ? (1ull << ((j % n2) * n0 + i / n1)) : 0ull;
            ok = (acc & kmask) == target;
        }
        ok = __all_sync(kFull, ok);
        if (lane == 0) {
            out[w] = ok;
            if (!best) B.hdr[w].valid = ok;
        }
        __syncwarp();
    }
}

// Exact integer Brent check (scheme_integer.cu:3-38), one warp per walk: every
// (i, j, k) equation sum_t u_t[i] v_t[j] w_t[k] equals its 0/1 target, and no
// coefficient carries the overflow flag.
__global__ void k_verify_zt(DevBatch B, int best, uint8_t *out) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cap = B.cap;
    uint64_t *xv = reinterpret_cast<uint64_t *>(smem) + (size_t)warp * 6 * cap;
    uint64_t *xs = xv + 3 * cap;
    for (int w = blockIdx.x * wpb + warp; w < B.S; w += gridDim.x * wpb) {
        const WalkHeader h = B.hdr[w];
        const int32_t *dims = best && B.best_n ? B.best_n + w * 3 : h.n;
        const size_t o = (size_t)w * 3 * cap;
        const uint64_t *sv = best ? B.best_fac : B.fac, *ss = best ? B.best_sgn : B.sgn;
        const uint8_t *sk = best ? B.best_valid : B.valid;
        const int m = best ? h.best_m : h.m;
        bool ok = m >= 0 && m <= cap;
        for (int q = lane; q < 3 * cap; q += 32) {
            xv[q] = sv[o + q];
            xs[q] = ss[o + q];
            if ((q % cap) < m && !sk[o + q]) ok = false;
        }
        __syncwarp();
        const int n0 = dims[0], n1 = dims[1], n2 = dims[2];
        const int nn0 = n0 * n1, nn1 = n1 * n2, nn2 = n2 * n0;
        for (int q = lane; ok && q < nn0 * nn1 * nn2; q += 32) {
            const int i = q / (nn1 * nn2), j = (q / nn2) % nn1, k = q % nn2;
            int e = 0;
            for (int t = 0; t < m; t++) {
                int cu = (int)((xv[t] >> i) & 1), cv = (int)((xv[cap + t] >> j) & 1), cw = (int)((xv[2 * cap + t] >> k) & 1);
                if (cu & cv & cw) {
                    int sg = (int)(((xs[t] >> i) ^ (xs[cap + t] >> j) ^ (xs[2 * cap + t] >> k)) & 1);
                    e += sg ? -1 : 1;
                }
            }
            const int target = (i % n1 == j / n2) && (i / n1 == k % n0) && (j % n2 == k / n0);
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

__global__ void k_tape(unsigned long long seed, int first, int count, int draws, uint32_t *d, float *u) {
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= count) return;
    curandStateXORWOW_t a, b;
    curand_init(seed, (unsigned long long)(first + w), 0ull, &a);
    b = a;
    for (int q = 0; q < draws; q++) {
        d[(size_t)w * draws + q] = curand(&a);
        u[(size_t)w * draws + q] = curand_uniform(&b);
    }
}

__global__ void k_philox(const uint4 *ctr, int count, uint32_t k0, uint32_t k1, uint4 *out) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < count) out[q] = philox4x32_10(ctr[q], k0, k1);
}

}  // namespace

// ---------------------------------------------------------------- handle
// A run of consecutive walks sharing one shared-memory layout in fast mode.
struct Segment {
    int first, count, scap, wide, nnmax;
    int kind = -1, lanes = 0, wpb = 0;  // fg_autotune's choice (kind -1: none; wpb: warps per block, thread kernel)
};

constexpr int kSideStreams = 8;

struct fg_handle {
    fg_config cfg;
    int dev = 0, sms = 0, wpb = 4, grid = 1;
    cudaStream_t stream = nullptr;
    cudaStream_t side[kSideStreams] = {};
    cudaEvent_t fork = nullptr, join[kSideStreams] = {};
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    std::vector<Segment> segs;
    std::vector<int> launchOrder;  // segments by ascending work (slots x walks), launched in this order
    LearnedBuffers learned;
    LearnedGraph learnedGraph;  // the learned step loop, captured once per set of arguments
    LearnedConfig lcfg;
    fg_mlp *mlp = nullptr;
    int simtMaxCap = -1;                  // fg_set_fast_split: thread per walk up to this slot count (-1: off)
    int fastKernel = -1, groupLanes = 0;  // fg_set_fast_kernel override (-1: per-segment choice)
    int listKernel = -1;                  // fg_set_list_kernel override (-1: automatic)
    void *d_listScratch = nullptr;        // thread-per-walk list kernel: lists interleaved by walk
    // Fast mode: the walk launches of one step (all segments, forked and joined) as a CUDA
    // graph, captured on first use and dropped whenever the launch plan changes.
    cudaGraphExec_t walkGraph = nullptr;
    bool graphPrimed = false;  // the plan's kernels ran once directly (attributes set) before capture
    DevBatch B{};
    WalkParams P{};
    int32_t *d_bestC = nullptr;
    // resizing: best rank per size key (FlipGraph::n2bestRank) and its device-side helpers
    std::map<std::string, int> table;
    bool tableReady = false;
    int32_t *d_copyList = nullptr, *d_bestRanks = nullptr;
    uint8_t *d_valid = nullptr;
    bool ready = false;
    // ZT: every live factor of the records valid, with bits 32-63 copying bit 31 (what the
    // thread-per-walk list kernel's 32-bit words hold for factors of 17-31 entries)
    bool ternaryWordsOk = true;
};

namespace {

template <class T> fg_status dalloc(T **p, size_t count) {
    *p = nullptr;
    if (!count) return FG_OK;
    FG_CUDA(cudaMalloc((void **)p, count * sizeof(T)));
    FG_CUDA(cudaMemset(*p, 0, count * sizeof(T)));
    return FG_OK;
}

void compute_params(fg_handle *h) {
    const fg_config &c = h->cfg;
    WalkParams &P = h->P;
    P.iterations = c.iterations;
    P.plus_iterations = c.plus_iterations;
    P.reduce_gate_f = ceil_to_float(c.reduce_p);
    P.expand_gate_f = ceil_to_float(c.expand_p);
    P.sandwich_gate_f = ceil_to_float(c.sandwich_p);
    P.basis_gate_f = ceil_to_float(c.basis_p);
    P.tie_gate_f = ceil_to_float(0.01);
    auto thr = [&](double p) -> uint64_t {
        if (!(p > 0)) return kGateOff;
        double q = p / (double)c.iterations;
        return q >= 1.0 ? (1ull << 32) : (uint64_t)(q * 4294967296.0);
    };
    P.reduce_T = thr(c.reduce_p);
    P.expand_T = thr(c.expand_p);
    P.sandwich_T = thr(c.sandwich_p);
    P.basis_T = thr(c.basis_p);
    P.gauss_on = c.gauss_p > 0 ? 1 : 0;
    P.gauss_gate_f = ceil_to_float(c.gauss_p);
    P.gauss_T = thr(c.gauss_p);
    P.zt_sandwich = c.zt_sandwich;
    P.key0 = (uint32_t)c.seed;
    P.key1 = (uint32_t)(c.seed >> 32);
    P.random_iterations = c.resize_p > 0 ? 1 : 0;
    P.retry_cap = c.retry_cap > 0 ? c.retry_cap : kRetryCap;
    // the fast mode's words keep the partner count in their top byte: factors of at most 56 entries
    P.max_matrix = c.mode == FG_MODE_FAST ? 56 : 64;
}

int verify_grid(fg_handle *h) { return (h->B.S + 3) / 4; }
size_t verify_smem(fg_handle *h) { return (size_t)4 * 3 * h->B.cap * sizeof(uint64_t); }

fg_status launch_verify(fg_handle *h, int best) {
    if (h->cfg.ring == FG_RING_ZB) {
        FG_CUDA(launch_verify_zb(h->B, best, h->d_valid, h->stream));
        return FG_OK;
    }
    if (h->cfg.ring == FG_RING_ZT) {
        size_t smem = 2 * verify_smem(h);
        FG_CUDA(cudaFuncSetAttribute(k_verify_zt, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_verify_zt<<<verify_grid(h), 128, smem, h->stream>>>(h->B, best, h->d_valid);
    } else {
        size_t smem = verify_smem(h);
        FG_CUDA(cudaFuncSetAttribute(k_verify_z2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_verify_z2<<<verify_grid(h), 128, smem, h->stream>>>(h->B, best, h->d_valid);
    }
    FG_CUDA(cudaGetLastError());
    return FG_OK;
}

// Fast-mode segments: maximal runs of walks with the same slot count and word
// width.  Slots = max(rank, n1*n2*n3) rounded up to 4 (ranks never exceed it:
// plus and split stop at n1*n2*n3, scheme_z2.cu:1030,1053,1081).  Too many
// segments (shapes interleaved walk by walk) collapse into one segment sized
// for the largest walk.
void drop_graph(fg_handle *h) {
    if (h->walkGraph) cudaGraphExecDestroy(h->walkGraph);
    h->walkGraph = nullptr;
    h->graphPrimed = false;
}

void plan_segments(fg_handle *h, const std::vector<WalkHeader> &hdr) {
    const int S = h->B.S, cap = h->B.cap;
    std::vector<Segment> segs;
    int maxScap = 4, anyWide = 0, maxNN = 0;
    for (int w = 0; w < S; w++) {
        const WalkHeader &o = hdr[w];
        int full = o.n[0] * o.n[1] * o.n[2];
        int need = o.m > full ? o.m : full;
        int scap = (need + 3) / 4 * 4;
        if (scap > cap) scap = cap;
        int nnmax = o.n[0] * o.n[1];
        if (o.n[1] * o.n[2] > nnmax) nnmax = o.n[1] * o.n[2];
        if (o.n[2] * o.n[0] > nnmax) nnmax = o.n[2] * o.n[0];
        int wide = nnmax > 24;
        if (scap > maxScap) maxScap = scap;
        anyWide |= wide;
        if (!segs.empty() && segs.back().scap == scap && segs.back().wide == wide && segs.back().first + segs.back().count == w) {
            segs.back().count++;
            if (nnmax > segs.back().nnmax) segs.back().nnmax = nnmax;
        } else {
            segs.push_back({w, 1, scap, wide, nnmax});
        }
        if (nnmax > maxNN) maxNN = nnmax;
    }
    if ((int)segs.size() > kSideStreams) segs.assign(1, Segment{0, S, maxScap, anyWide, maxNN});
    h->segs = segs;
    // Segments launch in ascending order of work, whatever the order of the shapes in the
    // batch.  Measured on GB300 with the six-shape batch (65,536 walks, 2x2x2 .. 4x4x4):
    // smallest first 3.35 G (bit-exact lists) and 5.3 G (fast) verified flips/s, largest
    // first 2.76 G and 4.25 G.
    h->launchOrder.resize(segs.size());
    for (size_t i = 0; i < segs.size(); i++) h->launchOrder[i] = (int)i;
    std::stable_sort(h->launchOrder.begin(), h->launchOrder.end(), [&](int a, int b) {
        return (long long)segs[a].scap * segs[a].count < (long long)segs[b].scap * segs[b].count;
    });
    drop_graph(h);
}

// Fast mode kernel choice for a segment.  One thread per walk does O(m) work
// per flip for 32 walks at once but needs many walks to hide its latency and
// 3 * slots * 32 words of shared memory per warp; one warp per walk does a
// fixed ~300 warp instructions per flip and fills the GPU with few walks.
// Measured crossovers on GB300 (fast mode, 1000 iterations): thread per walk
// wins up to 32 slots from 2 walk-warps per SM, up to 64 slots from 8, up to
// 80 slots from 16; warp per walk wins everywhere else.  `count` is the whole
// batch: the segments run concurrently and share the SMs.
bool thread_per_walk(int scap, int count, int sms) {
    const double warpsPerSM = (double)count / 32.0 / (sms > 0 ? sms : 1);
    if (scap <= 32) return warpsPerSM >= 2.0;
    if (scap <= 64) return warpsPerSM >= 8.0;
    if (scap <= 80) return warpsPerSM >= 16.0;
    return false;
}

bool uses_lists(const fg_handle *h) {
    return h->cfg.mode == FG_MODE_REFERENCE || h->cfg.mode == FG_MODE_PHILOX_LISTS;
}

fg_status refresh_plan(fg_handle *h) {
    std::vector<WalkHeader> hdr(h->B.S);
    FG_CUDA(cudaMemcpy(hdr.data(), h->B.hdr, sizeof(WalkHeader) * h->B.S, cudaMemcpyDeviceToHost));
    plan_segments(h, hdr);
    return FG_OK;
}

// FlipGraph::updateRanks (flip_graph.cu:249-266) with resizing on: per size key
// (sizes sorted, utils.cu:3-25) the best rank; a walk that improves it has its
// current scheme copied to its best slot, and every walk's best rank becomes its
// key's.  The table starts, as FlipGraph's constructor and initialize() set it
// (flip_graph.cu:19,190-198), from the first walk's size at the naive rank.
fg_status update_ranks(fg_handle *h) {
    const int S = h->B.S;
    std::vector<WalkHeader> hdr(S);
    FG_CUDA(cudaMemcpyAsync(hdr.data(), h->B.hdr, sizeof(WalkHeader) * S, cudaMemcpyDeviceToHost, h->stream));
    FG_CUDA(cudaStreamSynchronize(h->stream));
    auto key = [](const int32_t *n) {
        int a[3] = {n[0], n[1], n[2]};
        std::sort(a, a + 3);
        return std::to_string(a[0]) + "x" + std::to_string(a[1]) + "x" + std::to_string(a[2]);
    };
    if (!h->tableReady) {
        h->table.clear();
        h->table[key(hdr[0].n)] = hdr[0].n[0] * hdr[0].n[1] * hdr[0].n[2];
        h->tableReady = true;
    }
    std::vector<std::string> keys(S);
    std::vector<int32_t> copies, ranks(S);
    for (int w = 0; w < S; w++) {
        keys[w] = key(hdr[w].n);
        auto it = h->table.find(keys[w]);
        if (it == h->table.end() || hdr[w].m < it->second) {
            h->table[keys[w]] = hdr[w].m;
            copies.push_back(w);
        }
    }
    for (int w = 0; w < S; w++) ranks[w] = h->table[keys[w]];
    if (!copies.empty())
        FG_CUDA(cudaMemcpyAsync(h->d_copyList, copies.data(), 4 * copies.size(), cudaMemcpyHostToDevice, h->stream));
    FG_CUDA(cudaMemcpyAsync(h->d_bestRanks, ranks.data(), 4 * (size_t)S, cudaMemcpyHostToDevice, h->stream));
    FG_CUDA(launch_copy_best(h->B, h->d_copyList, (int)copies.size(), h->d_bestRanks, h->stream));
    FG_CUDA(cudaStreamSynchronize(h->stream));
    return FG_OK;
}

// Fast-mode kernel of segment g: fg_set_fast_kernel's override, else fg_autotune's
// choice, else fg_set_fast_split's split, else the measured crossover.
void segment_kernel(const fg_handle *h, const Segment &g, int &kind, int &lanes, int &wpb) {
    lanes = 32;
    // static warps per block of the thread kernel: 4 (six-shape batch on GB300: 5.42 G flips/s
    // against 5.28 G with 2 and 5.30 G with 8)
    wpb = h->cfg.walks_per_block > 0 ? h->cfg.walks_per_block : 4;
    if (h->fastKernel >= 0) { kind = h->fastKernel; lanes = kind == FG_FAST_GROUP ? h->groupLanes : 32; return; }
    if (g.kind >= 0) {
        kind = g.kind;
        lanes = g.lanes;
        if (g.wpb > 0) wpb = g.wpb;
        return;
    }
    if (h->simtMaxCap >= 0) kind = g.scap <= h->simtMaxCap ? FG_FAST_THREAD : FG_FAST_WARP;
    else kind = thread_per_walk(g.scap, h->B.S, h->sms) ? FG_FAST_THREAD : FG_FAST_WARP;
}

cudaError_t launch_segment(const fg_handle *h, const Segment &g, int kind, int lanes, int wpb, cudaStream_t st) {
    if (h->cfg.ring == FG_RING_ZB) return launch_walk_zb(h->B, h->P, g.first, g.count, g.scap, h->sms, st);
    if (kind == FG_FAST_THREAD) return launch_walk_simt(h->B, h->P, g.first, g.count, g.scap, g.wide, wpb, h->sms, st);
    if (kind == FG_FAST_GROUP) return launch_walk_group(h->B, h->P, g.first, g.count, g.scap, g.wide, lanes, h->sms, st);
    return launch_walk_group(h->B, h->P, g.first, g.count, g.scap, g.wide, 32, h->sms, st);  // one warp per walk
}

// Every segment's kernel, one side stream each, forked from and joined into h->stream.
cudaError_t launch_segments(fg_handle *h) {
    cudaError_t e;
    if (h->segs.size() == 1) {
        int kind, lanes, wpb;
        segment_kernel(h, h->segs[0], kind, lanes, wpb);
        return launch_segment(h, h->segs[0], kind, lanes, wpb, h->stream);
    }
    if ((e = cudaEventRecord(h->fork, h->stream)) != cudaSuccess) return e;
    for (const int i : h->launchOrder) {
        const Segment &g = h->segs[i];
        int kind, lanes, wpb;
        segment_kernel(h, g, kind, lanes, wpb);
        if ((e = cudaStreamWaitEvent(h->side[i], h->fork, 0)) != cudaSuccess) return e;
        if ((e = launch_segment(h, g, kind, lanes, wpb, h->side[i])) != cudaSuccess) return e;
        if ((e = cudaEventRecord(h->join[i], h->side[i])) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(h->stream, h->join[i], 0)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// List modes: the thread-per-walk list kernel covers both rings, with resizing (between
// launches; the segments are re-planned after each resize step), without sandwiching, basis
// changes or the Gauss reduction (their moves run in the warp kernel).
bool list_thread_possible(const fg_config &c) {
    return (c.ring == FG_RING_Z2 || c.ring == FG_RING_ZT) &&
           (c.mode == FG_MODE_REFERENCE || c.mode == FG_MODE_PHILOX_LISTS) &&
           !(c.sandwich_p > 0) && !(c.basis_p > 0) && !(c.gauss_p > 0);
}

// Automatic choice: thread per walk when every segment's factors fit a block's shared
// memory and the batch gives at least kListThreadWarpsPerSM warps of walks per SM (with
// fewer walks one warp per walk fills the GPU better).  Measured on GB300, reference
// stream, 3x3x3: Z2 with 8,192 walks (1.7 warps per SM) 1.14 G flips/s with a thread per
// walk against 0.78 G with a warp, 4,096 walks 0.57 G against 0.70 G; ZT with 16,384 walks
// (3.4 warps per SM) 285 M against 205 M, 8,192 walks 150 M against 198 M.
constexpr double kListThreadWarpsPerSM[2] = {1.5, 3.0};  // Z2, ZT

bool list_thread_chosen(const fg_handle *h) {
    if (h->listKernel == FG_LIST_WARP || !list_thread_possible(h->cfg)) return false;
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->dev);
    for (const Segment &g : h->segs) {
        if (g.scap > 256 || simt_list_smem_per_warp(h->cfg.ring, g.scap, g.nnmax) > (size_t)optin) return false;
        // ternary words: 31 entries (a naive factor of 32 entries sets bit 31 without copying it
        // upwards); above 16 the records must suit them (no overflow mark)
        if (h->cfg.ring == FG_RING_ZT && (g.nnmax > 31 || (g.nnmax > 16 && !h->ternaryWordsOk))) return false;
    }
    if (h->listKernel == FG_LIST_THREAD) return true;
    // With resizing the automatic choice keeps one warp per walk: the walks' sizes spread out,
    // the segments collapse into one sized for the largest scheme, and on GB300 (16,384 walks
    // from 3x3x3, resize 0.2, six launches of up to 1,000 steps) one thread per walk measured
    // 335 M verified flips/s against 361 M for Z2 (49 M against 42 M for ZT).
    if (h->cfg.resize_p > 0) return false;
    return (double)h->B.S / 32.0 / (h->sms > 0 ? h->sms : 1) >= kListThreadWarpsPerSM[h->cfg.ring == FG_RING_ZT];
}

// Static warps per block of the thread-per-walk list kernel: walks_per_block when given
// (at most 16), else 6 for Z2 batches of several shape segments and 4 otherwise.  Measured on
// GB300 (reference stream, verified flips/s, 4 against 6): Z2 six shapes 2x2x2..4x4x4,
// 65,536 walks 3.35 G against 3.65 G, 16,384 walks 1.09 G against 1.35 G; Z2 3x3x3, 3x3x4,
// 4x4x4, 65,536 walks 2.53 G against 2.84 G; ZT six shapes of at most 16 entries, 65,536
// walks 2.04 G against 1.92 G; ZT 3x3x3 + 2x4x4 1.62 G against 0.95 G; one shape (16,384
// walks of 3x3x3 or 4x4x4, both rings) 4 best by 1-8 %.
int list_wpb(const fg_handle *h) {
    if (h->cfg.walks_per_block > 0) return std::min(h->cfg.walks_per_block, 16);
    return h->cfg.ring == FG_RING_Z2 && h->segs.size() > 1 ? 6 : 4;
}

// With resizing, the kernels that run per shape segment (the fast mode's, and the
// thread-per-walk list kernel when requested) need the segments re-planned after each resize.
bool segments_follow_sizes(const fg_handle *h) {
    return h->cfg.mode == FG_MODE_FAST || (list_thread_possible(h->cfg) && h->listKernel == FG_LIST_THREAD);
}

// One thread-per-walk list launch per segment, forked from and joined into h->stream.
cudaError_t launch_list_segments(fg_handle *h) {
    cudaError_t e;
    if (!h->d_listScratch) {
        e = cudaMalloc(&h->d_listScratch, simt_list_scratch_bytes(h->cfg.ring, h->B.S));
        if (e != cudaSuccess) { h->d_listScratch = nullptr; return e; }
        e = simt_list_init_scratch(h->cfg.ring, h->B.S, h->d_listScratch, h->stream);
        if (e != cudaSuccess) return e;
    }
    const int rng = h->cfg.mode == FG_MODE_REFERENCE ? RNG_XORWOW : RNG_PHILOX;
    // warps per block: the autotuner's choice for the segment, else the static one
    auto wpbOf = [&](const Segment &g) { return g.wpb > 0 ? g.wpb : list_wpb(h); };
    if (h->segs.size() == 1) {
        const Segment &g = h->segs[0];
        return launch_walk_simt_list(h->cfg.ring, h->B, h->P, rng, g.first, g.count, g.scap, g.nnmax, wpbOf(g),
                                     h->sms, h->d_listScratch, h->stream);
    }
    if ((e = cudaEventRecord(h->fork, h->stream)) != cudaSuccess) return e;
    for (const int i : h->launchOrder) {
        const Segment &g = h->segs[i];
        if ((e = cudaStreamWaitEvent(h->side[i], h->fork, 0)) != cudaSuccess) return e;
        if ((e = launch_walk_simt_list(h->cfg.ring, h->B, h->P, rng, g.first, g.count, g.scap, g.nnmax, wpbOf(g),
                                       h->sms, h->d_listScratch, h->side[i])) != cudaSuccess)
            return e;
        if ((e = cudaEventRecord(h->join[i], h->side[i])) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(h->stream, h->join[i], 0)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// Launches one walk pass over every walk on h->stream (fast mode: one kernel
// per segment on side streams, forked from and joined back into h->stream).
fg_status launch_walks(fg_handle *h) {
    if (h->cfg.mode == FG_MODE_LEARNED) {
        for (const Segment &g : h->segs)
            if (g.nnmax > 21) return fail(FG_ERR_CAPACITY, "the learned mode takes factors of at most 21 entries");
        FG_CUDA(learned_launch(h->learned, h->B, h->P, h->lcfg, h->mlp, h->stream, &h->learnedGraph));
        return FG_OK;
    }
    if (h->cfg.mode != FG_MODE_FAST) {
        if (list_thread_chosen(h)) {
            FG_CUDA(launch_list_segments(h));
            return FG_OK;
        }
        // a forced thread kernel that does not fit: an error for fixed sizes; with resizing the
        // sizes change from launch to launch, and such a launch takes the warp kernel
        if (h->listKernel == FG_LIST_THREAD && !(h->cfg.resize_p > 0))
            return fail(FG_ERR_CAPACITY, "the thread-per-walk list kernel does not fit these schemes' slots");
        FG_CUDA(launch_walk(h->cfg.ring, h->B, h->P, h->cfg.mode == FG_MODE_REFERENCE ? RNG_XORWOW : RNG_PHILOX,
                            h->wpb, h->grid, h->stream));
        return FG_OK;
    }
    if (h->cfg.ring != FG_RING_ZB)
        for (const Segment &g : h->segs)
            if (g.nnmax > 56) return fail(FG_ERR_CAPACITY, "fast mode holds factors of at most 56 entries");
    if (h->walkGraph) {
        FG_CUDA(cudaGraphLaunch(h->walkGraph, h->stream));
        return FG_OK;
    }
    if (!h->graphPrimed) {  // first step of a plan: direct launches (they set the kernels' attributes)
        FG_CUDA(launch_segments(h));
        h->graphPrimed = true;
        return FG_OK;
    }
    // Capture this step's launches once; later steps replay the graph.
    cudaGraph_t g = nullptr;
    FG_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeRelaxed));
    cudaError_t le = launch_segments(h);
    cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
    if (le != cudaSuccess || ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return fail(FG_ERR_CUDA, cudaGetErrorString(le != cudaSuccess ? le : ce));
    }
    cudaError_t ie = cudaGraphInstantiate(&h->walkGraph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
        h->walkGraph = nullptr;
        return fail(FG_ERR_CUDA, cudaGetErrorString(ie));
    }
    FG_CUDA(cudaGraphLaunch(h->walkGraph, h->stream));
    return FG_OK;
}

}  // namespace

extern "C" {

const char *fg_last_error(void) { return fg::last_error().c_str(); }
const char *fg_version(void) { return "flipgraph-gb300 0.1 (sm_103a)"; }

fg_status fg_create(const fg_config *cfg, fg_handle **out) {
    if (!cfg || !out) return fail(FG_ERR_ARG, "null argument");
    *out = nullptr;
    if (cfg->walks <= 0) return fail(FG_ERR_ARG, "walks must be positive");
    if (cfg->ring != FG_RING_Z2 && cfg->ring != FG_RING_ZT && cfg->ring != FG_RING_ZB) return fail(FG_ERR_ARG, "unknown ring");
    if (cfg->ring == FG_RING_ZB && cfg->mode != FG_MODE_FAST)
        return fail(FG_ERR_ARG, "the bounded-integer ring (ZB) runs in the fast mode");
    if (cfg->ring == FG_RING_ZB && (cfg->resize_p > 0 || cfg->sandwich_p > 0 || cfg->basis_p > 0 || cfg->gauss_p > 0))
        return fail(FG_ERR_ARG, "resizing, sandwiching, basis changes and the Gauss reduction are not defined for ZB");
    if (cfg->ring == FG_RING_ZT && (cfg->mode == FG_MODE_FAST || cfg->mode == FG_MODE_LEARNED))
        return fail(FG_ERR_ARG, "the fast and learned modes are available for the Z2 ring; use a list mode for ZT");
    if (cfg->mode != FG_MODE_REFERENCE && cfg->mode != FG_MODE_PHILOX_LISTS && cfg->mode != FG_MODE_FAST &&
        cfg->mode != FG_MODE_LEARNED)
        return fail(FG_ERR_ARG, "unknown mode");
    if (cfg->cap <= 0 || slots_for_cap(cfg->cap) == 0 || cfg->cap > FG_MAX_RANK + 2)
        return fail(FG_ERR_CAPACITY, "cap must be in [1, 352]");
    if (cfg->resize_p > 0 && cfg->mode != FG_MODE_REFERENCE && cfg->mode != FG_MODE_PHILOX_LISTS &&
        !(cfg->mode == FG_MODE_FAST && cfg->ring == FG_RING_Z2))
        return fail(FG_ERR_ARG, "resizing runs in a list mode (reference or philox) or the Z2 fast mode");
    if ((cfg->sandwich_p > 0 || cfg->basis_p > 0) && cfg->mode != FG_MODE_REFERENCE && cfg->mode != FG_MODE_PHILOX_LISTS &&
        !(cfg->mode == FG_MODE_FAST && cfg->ring == FG_RING_Z2))
        return fail(FG_ERR_ARG, "sandwiching and basis-change moves run in a list mode (reference or philox) or the Z2 fast mode");
    if (cfg->gauss_p > 0 && (cfg->ring != FG_RING_Z2 || cfg->mode == FG_MODE_LEARNED))
        return fail(FG_ERR_ARG, "the Gauss reduction runs on the Z2 ring in a list mode (reference or philox) or the fast mode");
    if (cfg->resize_p > 0 && cfg->cap < FG_MAX_RANK)
        return fail(FG_ERR_CAPACITY, "resizing needs cap >= 350 (products reach the maximal rank)");
    if (cfg->iterations <= 0) return fail(FG_ERR_ARG, "iterations must be positive");
    if (cfg->retry_cap < 0) return fail(FG_ERR_ARG, "retry_cap must be >= 0 (0 = the default bound)");
    fg_handle *h = new fg_handle;
    h->cfg = *cfg;
    h->dev = cfg->device;
    if (cudaSetDevice(h->dev) != cudaSuccess) { delete h; return fail(FG_ERR_CUDA, "cudaSetDevice failed"); }
    cudaDeviceGetAttribute(&h->sms, cudaDevAttrMultiProcessorCount, h->dev);
    h->wpb = cfg->walks_per_block > 0 ? cfg->walks_per_block : 4;
    const int S = cfg->walks, cap = cfg->cap;
    h->B.S = S;
    h->B.cap = cap;
    fg_status st = FG_OK;
    size_t nf = (size_t)S * 3 * cap;
    if ((st = dalloc(&h->B.hdr, (size_t)S)) || (st = dalloc(&h->B.fac, nf)) || (st = dalloc(&h->B.best_fac, nf)) ||
        (st = dalloc(&h->B.lists, (size_t)S * 3 * kListCap)) || (st = dalloc(&h->d_bestC, (size_t)S)) ||
        (st = dalloc(&h->d_valid, (size_t)S))) {
        fg_destroy(h);
        return st;
    }
    if (cfg->ring == FG_RING_ZT) {
        if ((st = dalloc(&h->B.sgn, nf)) || (st = dalloc(&h->B.best_sgn, nf)) || (st = dalloc(&h->B.valid, nf)) ||
            (st = dalloc(&h->B.best_valid, nf))) {
            fg_destroy(h);
            return st;
        }
    }
    if (cfg->ring == FG_RING_ZB) {
        if ((st = dalloc(&h->B.sgn, nf)) || (st = dalloc(&h->B.best_sgn, nf)) || (st = dalloc(&h->B.fac2, nf)) ||
            (st = dalloc(&h->B.best_fac2, nf))) {
            fg_destroy(h);
            return st;
        }
    }
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        fg_destroy(h);
        return fail(FG_ERR_CUDA, "stream creation failed");
    }
    for (auto &e : h->ev) cudaEventCreate(&e);
    cudaEventCreateWithFlags(&h->fork, cudaEventDisableTiming);
    for (int i = 0; i < kSideStreams; i++) {
        cudaStreamCreateWithFlags(&h->side[i], cudaStreamNonBlocking);
        cudaEventCreateWithFlags(&h->join[i], cudaEventDisableTiming);
    }
    compute_params(h);
    if (cfg->mode == FG_MODE_REFERENCE) {
        if ((st = dalloc(&h->B.xorwow, (size_t)S))) { fg_destroy(h); return st; }
        k_init_xorwow<<<(S + 127) / 128, 128, 0, h->stream>>>(h->B.xorwow, S, (unsigned long long)cfg->seed);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(h->stream) != cudaSuccess) {
            fg_destroy(h);
            return fail(FG_ERR_CUDA, "seeding failed");
        }
    }
    if (cfg->resize_p > 0 && ((st = dalloc(&h->B.best_n, (size_t)S * 3)) || (st = dalloc(&h->d_copyList, (size_t)S)) ||
                              (st = dalloc(&h->d_bestRanks, (size_t)S)))) {
        fg_destroy(h);
        return st;
    }
    if (cfg->mode == FG_MODE_LEARNED) {
        cudaError_t le = learned_alloc(h->learned, S, cap, 1);
        if (le != cudaSuccess) {
            fg_destroy(h);
            return fail(FG_ERR_CUDA, cudaGetErrorString(le));
        }
    }
    int occ = occupancy_walk(cfg->ring, cap, cfg->mode == FG_MODE_REFERENCE ? RNG_XORWOW : RNG_PHILOX, h->wpb);
    if (occ <= 0) occ = 1;
    int need = (S + h->wpb - 1) / h->wpb;
    h->grid = need < occ * h->sms ? need : occ * h->sms;
    *out = h;
    return FG_OK;
}

fg_status fg_destroy(fg_handle *h) {
    if (!h) return FG_OK;
    cudaSetDevice(h->dev);
    if (h->stream) cudaStreamSynchronize(h->stream);
    h->learnedGraph.reset();
    learned_free(h->learned);
    drop_graph(h);
    void *ptrs[] = {h->B.hdr, h->B.fac, h->B.sgn, h->B.valid, h->B.lists, h->B.best_fac, h->B.best_sgn,
                    h->B.best_valid, h->B.xorwow, h->d_bestC, h->d_valid, h->B.best_n, h->d_copyList,
                    h->d_bestRanks, h->B.fac2, h->B.best_fac2, h->d_listScratch};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (auto &e : h->ev)
        if (e) cudaEventDestroy(e);
    for (int i = 0; i < kSideStreams; i++) {
        if (h->side[i]) cudaStreamDestroy(h->side[i]);
        if (h->join[i]) cudaEventDestroy(h->join[i]);
    }
    if (h->fork) cudaEventDestroy(h->fork);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return FG_OK;
}

fg_status fg_init_naive(fg_handle *h, int n1, int n2, int n3) {
    if (!h) return fail(FG_ERR_ARG, "null handle");
    if (n1 <= 0 || n2 <= 0 || n3 <= 0 || n1 * n2 > 64 || n2 * n3 > 64 || n3 * n1 > 64)
        return fail(FG_ERR_ARG, "matrix sizes exceed 64 elements");
    if (n1 * n2 * n3 > h->B.cap) return fail(FG_ERR_CAPACITY, "naive rank exceeds cap");
    FG_CUDA(cudaSetDevice(h->dev));
    k_init_naive<<<(h->B.S + 127) / 128, 128, 0, h->stream>>>(h->B, n1, n2, n3, nullptr, h->cfg.ring == FG_RING_ZT);
    FG_CUDA(cudaGetLastError());
    if (uses_lists(h)) FG_CUDA(launch_rebuild(h->cfg.ring, h->B, h->wpb, h->grid, h->stream));
    FG_CUDA(cudaStreamSynchronize(h->stream));
    fg_status st = refresh_plan(h);
    if (st) return st;
    h->ready = true;
    h->ternaryWordsOk = true;
    h->tableReady = false;
    return FG_OK;
}

fg_status fg_init_naive_shapes(fg_handle *h, const int32_t *shapes) {
    if (!h || !shapes) return fail(FG_ERR_ARG, "null argument");
    const int S = h->B.S;
    for (int w = 0; w < S; w++) {
        int n1 = shapes[w * 3], n2 = shapes[w * 3 + 1], n3 = shapes[w * 3 + 2];
        if (n1 <= 0 || n2 <= 0 || n3 <= 0 || n1 * n2 > 64 || n2 * n3 > 64 || n3 * n1 > 64)
            return fail(FG_ERR_ARG, "matrix sizes exceed 64 elements");
        if (n1 * n2 * n3 > h->B.cap) return fail(FG_ERR_CAPACITY, "naive rank exceeds cap");
    }
    FG_CUDA(cudaSetDevice(h->dev));
    int32_t *d = nullptr;
    FG_CUDA(cudaMalloc(&d, (size_t)S * 12));
    cudaError_t e = cudaMemcpy(d, shapes, (size_t)S * 12, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_init_naive<<<(S + 127) / 128, 128, 0, h->stream>>>(h->B, 0, 0, 0, d, h->cfg.ring == FG_RING_ZT);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && uses_lists(h)) e = launch_rebuild(h->cfg.ring, h->B, h->wpb, h->grid, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(d);
    if (e != cudaSuccess) return fail(FG_ERR_CUDA, cudaGetErrorString(e));
    fg_status st = refresh_plan(h);
    if (st) return st;
    h->ready = true;
    h->ternaryWordsOk = true;
    h->tableReady = false;
    return FG_OK;
}

fg_status fg_set_proposal(fg_handle *h, fg_mlp *mlp, int candidates, float temperature, float min_entropy) {
    if (!h) return fail(FG_ERR_ARG, "null handle");
    if (h->cfg.mode != FG_MODE_LEARNED) return fail(FG_ERR_STATE, "the proposal is set in the learned mode");
    if (candidates < 1 || candidates > 16 || !(temperature > 0.0f) || !(min_entropy >= 0.0f))
        return fail(FG_ERR_ARG, "candidates in [1, 16], temperature > 0, min_entropy >= 0");
    FG_CUDA(cudaSetDevice(h->dev));
    FG_CUDA(cudaStreamSynchronize(h->stream));
    h->learnedGraph.reset();  // the captured step loop names the old network's and buffers' addresses
    if (candidates != h->learned.K) FG_CUDA(learned_alloc(h->learned, h->B.S, h->B.cap, candidates));
    h->mlp = mlp;
    h->lcfg.K = candidates;
    h->lcfg.invTemp = 1.0f / temperature;
    h->lcfg.minEntropy = min_entropy;
    return FG_OK;
}

fg_status fg_collect_records(fg_handle *h, int every, int horizon, int launches, int64_t capacity, uint64_t *features,
                             float *labels, int64_t *count) {
    if (!h || !features || !labels || !count) return fail(FG_ERR_ARG, "null argument");
    if (h->cfg.mode != FG_MODE_LEARNED || h->learned.K != 1)
        return fail(FG_ERR_STATE, "records are collected in the learned mode with one candidate");
    if (!h->ready) return fail(FG_ERR_STATE, "records not initialised");
    if (every <= 0 || horizon <= 0 || launches < 0 || capacity <= 0) return fail(FG_ERR_ARG, "bad argument");
    FG_CUDA(cudaSetDevice(h->dev));
    FG_CUDA(cudaStreamSynchronize(h->stream));
    FG_CUDA(learned_alloc_records(h->learned, capacity, 1024));
    h->lcfg.recordEvery = every;
    fg_status st = FG_OK;
    for (int L = 0; L < launches && st == FG_OK; L++) st = launch_walks(h);
    h->lcfg.recordEvery = 0;
    std::vector<uint64_t> f;
    std::vector<float> y;
    cudaError_t e = st == FG_OK ? learned_take_records(h->learned, horizon, f, y, h->stream) : cudaSuccess;
    cudaError_t e2 = learned_alloc_records(h->learned, 0, 0);
    if (st) return st;
    if (e != cudaSuccess || e2 != cudaSuccess) return fail(FG_ERR_CUDA, cudaGetErrorString(e != cudaSuccess ? e : e2));
    const size_t n = std::min(y.size(), (size_t)capacity);
    std::copy(f.begin(), f.begin() + n * 3, features);
    std::copy(y.begin(), y.begin() + n, labels);
    *count = (int64_t)n;
    return FG_OK;
}

fg_status fg_rebuild_lists(fg_handle *h) {
    if (!h) return fail(FG_ERR_ARG, "null handle");
    if (!h->ready) return fail(FG_ERR_STATE, "records not initialised");
    FG_CUDA(cudaSetDevice(h->dev));
    if (uses_lists(h)) FG_CUDA(launch_rebuild(h->cfg.ring, h->B, h->wpb, h->grid, h->stream));
    FG_CUDA(cudaStreamSynchronize(h->stream));
    return FG_OK;
}

fg_status fg_set_list_kernel(fg_handle *h, int kernel) {
    if (!h) return fail(FG_ERR_ARG, "null handle");
    if (kernel < -1 || kernel > FG_LIST_THREAD) return fail(FG_ERR_ARG, "kernel in -1..1");
    if (kernel == FG_LIST_THREAD && !list_thread_possible(h->cfg))
        return fail(FG_ERR_ARG, "the thread-per-walk list kernel runs in a list mode without resizing, "
                                "sandwiching, basis changes or the Gauss reduction");
    h->listKernel = kernel;
    if (h->ready && h->cfg.resize_p > 0 && kernel == FG_LIST_THREAD) return refresh_plan(h);  // sizes may have moved
    return FG_OK;
}

fg_status fg_set_fast_kernel(fg_handle *h, int kernel, int lanes) {
    if (!h) return fail(FG_ERR_ARG, "null handle");
    if (kernel < -1 || kernel > FG_FAST_WARP || !(lanes == 0 || lanes == 4 || lanes == 8 || lanes == 16 || lanes == 32))
        return fail(FG_ERR_ARG, "kernel in -1..2, lanes 0, 4, 8, 16 or 32");
    h->fastKernel = kernel;
    h->groupLanes = lanes;
    drop_graph(h);
    return FG_OK;
}

fg_status fg_autotune(fg_handle *h, int iterations, int32_t *kinds, int32_t *lanes, int32_t *warps) {
    if (!h || iterations <= 0) return fail(FG_ERR_ARG, "bad argument");
    if (!h->ready) return fail(FG_ERR_STATE, "records not initialised");
    const bool fast = h->cfg.mode == FG_MODE_FAST && h->cfg.ring == FG_RING_Z2;
    const bool lists = !fast && uses_lists(h) && list_thread_chosen(h);
    if (!fast && !lists)
        return fail(FG_ERR_ARG, "the autotuner chooses among the Z2 fast-mode kernels and the warps per block "
                                "of the thread-per-walk list kernel");
    FG_CUDA(cudaSetDevice(h->dev));
    FG_CUDA(cudaStreamSynchronize(h->stream));
    const size_t S = (size_t)h->B.S, nf = S * 3 * h->B.cap;
    // Snapshot of everything a launch changes (records, best schemes, lists, cuRAND states);
    // every trial starts from it and it is put back at the end, so tuning leaves
    // trajectories and stream positions untouched.
    struct Region {
        void *p;
        size_t bytes;
    };
    std::vector<Region> regs = {{h->B.hdr, S * sizeof(WalkHeader)}, {h->B.fac, nf * 8}, {h->B.best_fac, nf * 8}};
    if (h->B.best_n) regs.push_back({h->B.best_n, S * 3 * sizeof(int32_t)});  // resizing: best sizes
    if (lists) {
        regs.push_back({h->B.lists, S * 3 * kListCap * sizeof(uint32_t)});
        if (h->B.xorwow) regs.push_back({h->B.xorwow, S * sizeof(curandStateXORWOW_t)});
        if (h->cfg.ring == FG_RING_ZT)
            for (Region r : {Region{h->B.sgn, nf * 8}, Region{h->B.best_sgn, nf * 8}, Region{h->B.valid, nf},
                             Region{h->B.best_valid, nf}})
                regs.push_back(r);
    }
    size_t total = 0;
    for (const Region &r : regs) total += (r.bytes + 255) / 256 * 256;
    unsigned char *snap = nullptr;
    if (cudaMalloc(&snap, total) != cudaSuccess) return fail(FG_ERR_CUDA, "autotune snapshot allocation failed");
    auto restore = [&](bool save) -> cudaError_t {
        size_t off = 0;
        for (const Region &r : regs) {
            void *dst = save ? (void *)(snap + off) : r.p;
            const void *src = save ? r.p : (const void *)(snap + off);
            cudaError_t e = cudaMemcpyAsync(dst, src, r.bytes, cudaMemcpyDeviceToDevice, h->stream);
            if (e != cudaSuccess) return e;
            off += (r.bytes + 255) / 256 * 256;
        }
        return cudaSuccess;
    };
    cudaError_t e = restore(true);
    const int savedIterations = h->P.iterations;
    h->P.iterations = iterations;
    drop_graph(h);
    // Fast mode (kind, lanes, warps per block): thread per walk with 2, 4, 8 warps per block;
    // 8, 16, 32 lanes per walk.  List modes: the thread-per-walk list kernel with 2, 4, 6, 8
    // warps per block.  Warps per block change how the concurrently launched segments share
    // the SMs.  Measured on GB300, six-shape batch, every segment alike: the bit-exact list
    // kernel 3.35 G flips/s with 4, 3.65 G with 6; the fast kernel 5.42 G with 4, 4.36 G with 6.
    const int fastCand[6][3] = {{FG_FAST_THREAD, 0, 2}, {FG_FAST_THREAD, 0, 4}, {FG_FAST_THREAD, 0, 8},
                                {FG_FAST_GROUP, 8, 0},  {FG_FAST_GROUP, 16, 0}, {FG_FAST_WARP, 32, 0}};
    const int listCand[4][3] = {{FG_FAST_THREAD, 0, 2}, {FG_FAST_THREAD, 0, 4}, {FG_FAST_THREAD, 0, 6},
                                {FG_FAST_THREAD, 0, 8}};
    const int (*cand)[3] = fast ? fastCand : listCand;
    const int nCand = fast ? 6 : 4;
    auto launchAll = [&]() { return fast ? launch_segments(h) : launch_list_segments(h); };
    // The segments run concurrently, so a choice is judged by the whole step.  One timing: from
    // the snapshot an untimed launch (kernel attributes), then from the snapshot a timed one.
    auto timeOnce = [&](float &ms) -> cudaError_t {
        cudaError_t te;
        if ((te = restore(false)) != cudaSuccess) return te;
        launchAll();
        if ((te = restore(false)) != cudaSuccess) return te;
        cudaEventRecord(h->ev[0], h->stream);
        cudaError_t le = launchAll();
        cudaEventRecord(h->ev[1], h->stream);
        if ((te = cudaStreamSynchronize(h->stream)) != cudaSuccess) return te;
        ms = 1e30f;
        if (le != cudaSuccess) {  // a candidate a segment cannot run (e.g. shared memory)
            cudaGetLastError();
            return cudaSuccess;
        }
        cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]);
        return cudaSuccess;
    };
    // A candidate replaces the configuration in place only when, timed in the order in place,
    // candidate, candidate, in place (so that a drift of the clocks over the tuning cancels),
    // its two steps take less than kMargin of the other two: launches of segments on side
    // streams share the SMs in an order that varies from run to run, and the clocks fall as
    // the tuning heats the GPU, so small differences do not carry over.
    constexpr float kMargin = 0.97f;
    auto better = [&](const std::vector<Segment> &inPlace, const std::vector<Segment> &candidate,
                      bool &yes) -> cudaError_t {
        float t[4];
        const std::vector<Segment> *order[4] = {&inPlace, &candidate, &candidate, &inPlace};
        for (int q = 0; q < 4; q++) {
            h->segs = *order[q];
            cudaError_t te = timeOnce(t[q]);
            if (te != cudaSuccess) return te;
        }
        h->segs = inPlace;
        yes = t[1] + t[2] < kMargin * (t[0] + t[3]);
        return cudaSuccess;
    };
    for (Segment &g : h->segs) {  // explicit static choice as the starting point
        if (fast) {
            int k, l, w;
            g.kind = -1;
            segment_kernel(h, g, k, l, w);
            g.kind = k; g.lanes = l; g.wpb = k == FG_FAST_THREAD ? w : 0;
        } else {
            g.kind = FG_FAST_THREAD; g.lanes = 0; g.wpb = list_wpb(h);
        }
    }
    // First one warps-per-block value for every thread-per-walk segment at once (the segments
    // share the SMs, so a common value can beat every single-segment change).
    for (int w : {2, 4, 6, 8}) {
        if (e != cudaSuccess) break;
        if (fast && w == 6) continue;
        std::vector<Segment> cand = h->segs;
        bool differs = false;
        for (Segment &g : cand)
            if (g.kind == FG_FAST_THREAD && g.wpb != w) { g.wpb = w; differs = true; }
        if (!differs) continue;
        const std::vector<Segment> inPlace = h->segs;
        bool yes = false;
        if ((e = better(inPlace, cand, yes)) != cudaSuccess) break;
        h->segs = yes ? cand : inPlace;
    }
    // Then each segment in turn, the others fixed (one sweep of coordinate descent).
    for (size_t i = 0; e == cudaSuccess && i < h->segs.size(); i++) {
        for (int c = 0; c < nCand && e == cudaSuccess; c++) {
            const Segment &g = h->segs[i];
            if (cand[c][0] == g.kind && cand[c][2] == g.wpb && (g.kind == FG_FAST_THREAD || cand[c][1] == g.lanes))
                continue;  // the configuration in place
            const std::vector<Segment> inPlace = h->segs;
            std::vector<Segment> next = inPlace;
            next[i].kind = cand[c][0]; next[i].lanes = cand[c][1]; next[i].wpb = cand[c][2];
            bool yes = false;
            if ((e = better(inPlace, next, yes)) != cudaSuccess) break;
            h->segs = yes ? next : inPlace;
        }
    }
    h->P.iterations = savedIterations;
    cudaError_t re = restore(false);
    if (e == cudaSuccess) e = re;
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(snap);
    drop_graph(h);
    if (e != cudaSuccess) return fail(FG_ERR_CUDA, cudaGetErrorString(e));
    for (size_t i = 0; i < h->segs.size(); i++) {
        if (kinds) kinds[i] = h->segs[i].kind;
        if (lanes) lanes[i] = h->segs[i].lanes;
        if (warps) warps[i] = h->segs[i].wpb;
    }
    return FG_OK;
}

int fg_segment_count(fg_handle *h) { return h ? (int)h->segs.size() : 0; }

fg_status fg_set_fast_split(fg_handle *h, int simt_max_cap) {
    if (!h || simt_max_cap < -1) return fail(FG_ERR_ARG, "bad argument");
    h->simtMaxCap = simt_max_cap;
    drop_graph(h);
    return FG_OK;
}

fg_status fg_get_counters(fg_handle *h, int32_t *m, int32_t *best_rank, int32_t *best_m, int32_t *flips_since_drop,
                          uint64_t *flips_last_launch, uint8_t *valid) {
    if (!h) return fail(FG_ERR_ARG, "null handle");
    FG_CUDA(cudaSetDevice(h->dev));
    FG_CUDA(cudaStreamSynchronize(h->stream));
    const int S = h->B.S;
    std::vector<WalkHeader> hdr(S);
    FG_CUDA(cudaMemcpy(hdr.data(), h->B.hdr, sizeof(WalkHeader) * S, cudaMemcpyDeviceToHost));
    for (int w = 0; w < S; w++) {
        if (m) m[w] = hdr[w].m;
        if (best_rank) best_rank[w] = hdr[w].best_rank;
        if (best_m) best_m[w] = hdr[w].best_m;
        if (flips_since_drop) flips_since_drop[w] = hdr[w].flips;
        if (flips_last_launch) flips_last_launch[w] = hdr[w].flips_done;
        if (valid) valid[w] = (uint8_t)hdr[w].valid;
    }
    return FG_OK;
}

fg_status fg_get_scheme(fg_handle *h, int walk, int best, int32_t *n, int32_t *m, uint64_t *fac, uint64_t *sgn,
                        uint8_t *valid) {
    if (!h || walk < 0 || walk >= h->B.S) return fail(FG_ERR_ARG, "bad walk index");
    FG_CUDA(cudaSetDevice(h->dev));
    FG_CUDA(cudaStreamSynchronize(h->stream));
    WalkHeader hd;
    FG_CUDA(cudaMemcpy(&hd, h->B.hdr + walk, sizeof(WalkHeader), cudaMemcpyDeviceToHost));
    if (n) for (int c = 0; c < 3; c++) n[c] = hd.n[c];
    if (n && best && h->B.best_n) FG_CUDA(cudaMemcpy(n, h->B.best_n + walk * 3, 12, cudaMemcpyDeviceToHost));
    if (m) *m = best ? hd.best_m : hd.m;
    const size_t o = (size_t)walk * 3 * h->B.cap, nf = (size_t)3 * h->B.cap;
    if (fac) FG_CUDA(cudaMemcpy(fac, (best ? h->B.best_fac : h->B.fac) + o, nf * 8, cudaMemcpyDeviceToHost));
    if (h->cfg.ring == FG_RING_ZT) {
        if (sgn) FG_CUDA(cudaMemcpy(sgn, (best ? h->B.best_sgn : h->B.sgn) + o, nf * 8, cudaMemcpyDeviceToHost));
        if (valid) FG_CUDA(cudaMemcpy(valid, (best ? h->B.best_valid : h->B.valid) + o, nf, cudaMemcpyDeviceToHost));
    }
    return FG_OK;
}

fg_status fg_get_scheme_zb(fg_handle *h, int walk, int best, int32_t *n, int32_t *m, uint64_t *fac, uint64_t *sgn,
                           uint64_t *fac2) {
    if (!h || h->cfg.ring != FG_RING_ZB) return fail(FG_ERR_ARG, "not a ZB handle");
    fg_status st = fg_get_scheme(h, walk, best, n, m, fac, nullptr, nullptr);
    if (st) return st;
    const size_t o = (size_t)walk * 3 * h->B.cap, nf = (size_t)3 * h->B.cap;
    if (sgn) FG_CUDA(cudaMemcpy(sgn, (best ? h->B.best_sgn : h->B.sgn) + o, nf * 8, cudaMemcpyDeviceToHost));
    if (fac2) FG_CUDA(cudaMemcpy(fac2, (best ? h->B.best_fac2 : h->B.fac2) + o, nf * 8, cudaMemcpyDeviceToHost));
    return FG_OK;
}

fg_status fg_host_alloc(uint64_t bytes, void **out) {
    if (!out) return fail(FG_ERR_ARG, "null argument");
    FG_CUDA(cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault));
    return FG_OK;
}

fg_status fg_host_free(void *p) {
    if (p) FG_CUDA(cudaFreeHost(p));
    return FG_OK;
}

fg_status fg_set_records(fg_handle *h, const fg_records *rec) {
    if (!h || !rec || !rec->n || !rec->m || !rec->fac) return fail(FG_ERR_ARG, "null argument");
    // The list modes take the FlipSets from the records; the fast modes keep no lists.
    if (uses_lists(h) && (!rec->list_size || !rec->list_pairs)) return fail(FG_ERR_ARG, "list modes need the lists");
    if (h->cfg.ring == FG_RING_ZT && (!rec->sgn || !rec->valid)) return fail(FG_ERR_ARG, "ZT records need sgn and valid");
    if (h->cfg.ring == FG_RING_ZB && (!rec->sgn || !rec->fac2)) return fail(FG_ERR_ARG, "ZB records need sgn and fac2");
    FG_CUDA(cudaSetDevice(h->dev));
    const int S = h->B.S, cap = h->B.cap;
    size_t nf = (size_t)S * 3 * cap;
    // Everything the kernels index by is checked before anything is copied, so a
    // rejected record leaves the handle as it was: sizes (the matrix entries index
    // factor bits; best sizes only where resizing reads them), ranks (slots) and, in
    // the list modes, every pair (two distinct slots below the rank).
    auto shape_ok = [](const int32_t *n) {
        for (int c = 0; c < 3; c++)
            if (n[c] <= 0 || n[c] > 64) return false;
        return n[0] * n[1] <= 64 && n[1] * n[2] <= 64 && n[2] * n[0] <= 64;
    };
    for (int w = 0; w < S; w++) {
        if (!shape_ok(rec->n + w * 3) || (h->B.best_n && rec->best_n && !shape_ok(rec->best_n + w * 3)))
            return fail(FG_ERR_ARG, "record " + std::to_string(w) + ": matrix sizes out of range");
        const int m = rec->m[w], bm = rec->best_m ? rec->best_m[w] : m;
        if (m < 0 || m > cap || bm < 0 || bm > cap)
            return fail(FG_ERR_CAPACITY, "record " + std::to_string(w) + ": rank exceeds cap");
        if (!uses_lists(h)) continue;
        for (int c = 0; c < 3; c++) {
            const int size = rec->list_size[w * 3 + c];
            if (size < 0 || size > kListCap) return fail(FG_ERR_CAPACITY, "record " + std::to_string(w) + ": list size");
            const uint32_t *pairs = rec->list_pairs + ((size_t)w * 3 + c) * kListCap;
            for (int q = 0; q < size; q++) {
                const int a = (int)(pairs[q] >> 16), b = (int)(pairs[q] & 0xFFFFu);
                if (a >= m || b >= m || a == b)
                    return fail(FG_ERR_ARG, "record " + std::to_string(w) + ": list pair outside the scheme");
            }
        }
    }
    std::vector<WalkHeader> hdr(S);
    FG_CUDA(cudaMemcpy(hdr.data(), h->B.hdr, sizeof(WalkHeader) * S, cudaMemcpyDeviceToHost));
    for (int w = 0; w < S; w++) {
        WalkHeader &o = hdr[w];
        for (int c = 0; c < 3; c++) o.n[c] = rec->n[w * 3 + c];
        o.m = rec->m[w];
        for (int c = 0; c < 3; c++) o.list_size[c] = uses_lists(h) ? rec->list_size[w * 3 + c] : 0;
        o.flips = rec->flips ? rec->flips[w] : 0;
        o.best_rank = rec->best_rank ? rec->best_rank[w] : o.m;
        o.best_m = rec->best_m ? rec->best_m[w] : o.m;
        o.status = rec->status ? rec->status[w] : 0;
        o.valid = 0;
    }
    FG_CUDA(cudaMemcpy(h->B.hdr, hdr.data(), sizeof(WalkHeader) * S, cudaMemcpyHostToDevice));
    FG_CUDA(cudaMemcpy(h->B.fac, rec->fac, nf * sizeof(uint64_t), cudaMemcpyHostToDevice));
    if (uses_lists(h))
        FG_CUDA(cudaMemcpy(h->B.lists, rec->list_pairs, (size_t)S * 3 * kListCap * 4, cudaMemcpyHostToDevice));
    if (h->B.best_n) {
        std::vector<int32_t> bn((size_t)S * 3);
        for (int w = 0; w < S; w++)
            for (int c = 0; c < 3; c++) bn[w * 3 + c] = rec->best_n ? rec->best_n[w * 3 + c] : rec->n[w * 3 + c];
        FG_CUDA(cudaMemcpy(h->B.best_n, bn.data(), bn.size() * 4, cudaMemcpyHostToDevice));
    }
    FG_CUDA(cudaMemcpy(h->B.best_fac, rec->best_fac ? rec->best_fac : rec->fac, nf * sizeof(uint64_t),
                       cudaMemcpyHostToDevice));
    if (h->cfg.ring == FG_RING_ZT) {
        h->ternaryWordsOk = true;
        auto sext32 = [](uint64_t x) { return (uint64_t)(int64_t)(int32_t)(uint32_t)x; };
        for (int w = 0; w < S && h->ternaryWordsOk; w++)
            for (int c = 0; c < 3; c++)
                for (int t = 0; t < rec->m[w]; t++) {
                    const size_t q = ((size_t)w * 3 + c) * cap + t;
                    if (!rec->valid[q] || sext32(rec->fac[q]) != rec->fac[q] || sext32(rec->sgn[q]) != rec->sgn[q])
                        h->ternaryWordsOk = false;
                }
        FG_CUDA(cudaMemcpy(h->B.sgn, rec->sgn, nf * 8, cudaMemcpyHostToDevice));
        FG_CUDA(cudaMemcpy(h->B.valid, rec->valid, nf, cudaMemcpyHostToDevice));
        FG_CUDA(cudaMemcpy(h->B.best_sgn, rec->best_sgn ? rec->best_sgn : rec->sgn, nf * 8, cudaMemcpyHostToDevice));
        FG_CUDA(cudaMemcpy(h->B.best_valid, rec->best_valid ? rec->best_valid : rec->valid, nf, cudaMemcpyHostToDevice));
    }
    if (h->cfg.ring == FG_RING_ZB) {
        FG_CUDA(cudaMemcpy(h->B.sgn, rec->sgn, nf * 8, cudaMemcpyHostToDevice));
        FG_CUDA(cudaMemcpy(h->B.fac2, rec->fac2, nf * 8, cudaMemcpyHostToDevice));
        FG_CUDA(cudaMemcpy(h->B.best_sgn, rec->best_sgn ? rec->best_sgn : rec->sgn, nf * 8, cudaMemcpyHostToDevice));
        FG_CUDA(cudaMemcpy(h->B.best_fac2, rec->best_fac2 ? rec->best_fac2 : rec->fac2, nf * 8, cudaMemcpyHostToDevice));
    }
    plan_segments(h, hdr);
    h->ready = true;
    h->tableReady = false;
    return FG_OK;
}

fg_status fg_get_records(fg_handle *h, fg_records *rec) {
    if (!h || !rec) return fail(FG_ERR_ARG, "null argument");
    FG_CUDA(cudaSetDevice(h->dev));
    FG_CUDA(cudaStreamSynchronize(h->stream));
    const int S = h->B.S, cap = h->B.cap;
    size_t nf = (size_t)S * 3 * cap;
    std::vector<WalkHeader> hdr(S);
    FG_CUDA(cudaMemcpy(hdr.data(), h->B.hdr, sizeof(WalkHeader) * S, cudaMemcpyDeviceToHost));
    for (int w = 0; w < S; w++) {
        const WalkHeader &o = hdr[w];
        if (rec->n) for (int c = 0; c < 3; c++) rec->n[w * 3 + c] = o.n[c];
        if (rec->m) rec->m[w] = o.m;
        if (rec->list_size) for (int c = 0; c < 3; c++) rec->list_size[w * 3 + c] = o.list_size[c];
        if (rec->flips) rec->flips[w] = o.flips;
        if (rec->best_rank) rec->best_rank[w] = o.best_rank;
        if (rec->best_m) rec->best_m[w] = o.best_m;
        if (rec->rng_pos) rec->rng_pos[w] = (int64_t)o.draws;
        if (rec->status) rec->status[w] = o.status;
    }
    if (rec->best_n) {
        if (h->B.best_n) FG_CUDA(cudaMemcpy(rec->best_n, h->B.best_n, (size_t)S * 12, cudaMemcpyDeviceToHost));
        else for (int w = 0; w < S; w++) for (int c = 0; c < 3; c++) rec->best_n[w * 3 + c] = hdr[w].n[c];
    }
    if (rec->fac) FG_CUDA(cudaMemcpy(rec->fac, h->B.fac, nf * 8, cudaMemcpyDeviceToHost));
    if (rec->best_fac) FG_CUDA(cudaMemcpy(rec->best_fac, h->B.best_fac, nf * 8, cudaMemcpyDeviceToHost));
    if (rec->list_pairs) {
        if (uses_lists(h))
            FG_CUDA(cudaMemcpy(rec->list_pairs, h->B.lists, (size_t)S * 3 * kListCap * 4, cudaMemcpyDeviceToHost));
        else
            std::memset(rec->list_pairs, 0, (size_t)S * 3 * kListCap * 4);  // the fast modes keep no lists
    }
    if (h->cfg.ring == FG_RING_ZT) {
        if (rec->sgn) FG_CUDA(cudaMemcpy(rec->sgn, h->B.sgn, nf * 8, cudaMemcpyDeviceToHost));
        if (rec->valid) FG_CUDA(cudaMemcpy(rec->valid, h->B.valid, nf, cudaMemcpyDeviceToHost));
        if (rec->best_sgn) FG_CUDA(cudaMemcpy(rec->best_sgn, h->B.best_sgn, nf * 8, cudaMemcpyDeviceToHost));
        if (rec->best_valid) FG_CUDA(cudaMemcpy(rec->best_valid, h->B.best_valid, nf, cudaMemcpyDeviceToHost));
    }
    if (h->cfg.ring == FG_RING_ZB) {
        if (rec->sgn) FG_CUDA(cudaMemcpy(rec->sgn, h->B.sgn, nf * 8, cudaMemcpyDeviceToHost));
        if (rec->fac2) FG_CUDA(cudaMemcpy(rec->fac2, h->B.fac2, nf * 8, cudaMemcpyDeviceToHost));
        if (rec->best_sgn) FG_CUDA(cudaMemcpy(rec->best_sgn, h->B.best_sgn, nf * 8, cudaMemcpyDeviceToHost));
        if (rec->best_fac2) FG_CUDA(cudaMemcpy(rec->best_fac2, h->B.best_fac2, nf * 8, cudaMemcpyDeviceToHost));
    }
    return FG_OK;
}

fg_status run_launches(fg_handle *h, int launches, fg_stats *stats, bool resizing);

fg_status fg_run(fg_handle *h, int launches, fg_stats *stats) {
    if (!h) return fail(FG_ERR_ARG, "null handle");
    return run_launches(h, launches, stats, h->cfg.resize_p > 0);
}

fg_status fg_run_walks(fg_handle *h, int launches, fg_stats *stats) {
    if (!h) return fail(FG_ERR_ARG, "null handle");
    return run_launches(h, launches, stats, false);
}

fg_status fg_resize(fg_handle *h) {
    if (!h) return fail(FG_ERR_ARG, "null handle");
    if (!(h->cfg.resize_p > 0)) return fail(FG_ERR_STATE, "the handle was created without resizing");
    if (!h->ready) return fail(FG_ERR_STATE, "records not initialised");
    FG_CUDA(cudaSetDevice(h->dev));
    FG_CUDA(launch_resize(h->cfg.ring, h->B, h->P, h->cfg.mode == FG_MODE_REFERENCE ? RNG_XORWOW : RNG_PHILOX, h->cfg.resize_p,
                          h->wpb, h->grid, uses_lists(h), h->stream));
    FG_CUDA(cudaStreamSynchronize(h->stream));
    if (segments_follow_sizes(h)) return refresh_plan(h);  // shape segments follow the new sizes
    return FG_OK;
}

fg_status fg_get_sizes(fg_handle *h, int32_t *n, int32_t *best_n) {
    if (!h) return fail(FG_ERR_ARG, "null handle");
    FG_CUDA(cudaSetDevice(h->dev));
    FG_CUDA(cudaStreamSynchronize(h->stream));
    const int S = h->B.S;
    std::vector<WalkHeader> hdr(S);
    FG_CUDA(cudaMemcpy(hdr.data(), h->B.hdr, sizeof(WalkHeader) * S, cudaMemcpyDeviceToHost));
    for (int w = 0; w < S; w++)
        for (int c = 0; c < 3; c++) {
            if (n) n[w * 3 + c] = hdr[w].n[c];
            if (best_n && !h->B.best_n) best_n[w * 3 + c] = hdr[w].n[c];
        }
    if (best_n && h->B.best_n) FG_CUDA(cudaMemcpy(best_n, h->B.best_n, (size_t)S * 12, cudaMemcpyDeviceToHost));
    return FG_OK;
}

fg_status fg_copy_to_best(fg_handle *h, const int32_t *walks, int count) {
    if (!h || (count > 0 && !walks) || count < 0 || count > h->B.S) return fail(FG_ERR_ARG, "bad argument");
    if (!h->B.best_n) return fail(FG_ERR_STATE, "the handle was created without resizing");
    for (int i = 0; i < count; i++)
        if (walks[i] < 0 || walks[i] >= h->B.S) return fail(FG_ERR_ARG, "walk index out of range");
    FG_CUDA(cudaSetDevice(h->dev));
    if (count) FG_CUDA(cudaMemcpyAsync(h->d_copyList, walks, 4 * (size_t)count, cudaMemcpyHostToDevice, h->stream));
    FG_CUDA(launch_copy_best(h->B, h->d_copyList, count, nullptr, h->stream));
    FG_CUDA(cudaStreamSynchronize(h->stream));
    return FG_OK;
}

fg_status fg_set_best_ranks(fg_handle *h, const int32_t *ranks) {
    if (!h || !ranks) return fail(FG_ERR_ARG, "null argument");
    if (!h->B.best_n) return fail(FG_ERR_STATE, "the handle was created without resizing");
    FG_CUDA(cudaSetDevice(h->dev));
    FG_CUDA(cudaMemcpyAsync(h->d_bestRanks, ranks, 4 * (size_t)h->B.S, cudaMemcpyHostToDevice, h->stream));
    FG_CUDA(launch_copy_best(h->B, h->d_copyList, 0, h->d_bestRanks, h->stream));
    FG_CUDA(cudaStreamSynchronize(h->stream));
    return FG_OK;
}

fg_status run_launches(fg_handle *h, int launches, fg_stats *stats, bool resizing) {
    if (!h) return fail(FG_ERR_ARG, "null handle");
    if (!h->ready) return fail(FG_ERR_STATE, "records not initialised");
    if (launches < 0) return fail(FG_ERR_ARG, "launches must be >= 0");
    FG_CUDA(cudaSetDevice(h->dev));
    const int S = h->B.S;
    fg_stats acc{};
    acc.min_rank = acc.min_best_rank = 1 << 30;
    std::vector<WalkHeader> hdr(S);
    if (resizing && !h->tableReady) {
        fg_status us = update_ranks(h);
        if (us) return us;
    }
    for (int L = 0; L < launches; L++) {
        FG_CUDA(cudaEventRecord(h->ev[0], h->stream));
        fg_status ls = launch_walks(h);
        if (ls) return ls;
        if (resizing) {
            FG_CUDA(launch_resize(h->cfg.ring, h->B, h->P, h->cfg.mode == FG_MODE_REFERENCE ? RNG_XORWOW : RNG_PHILOX,
                                  h->cfg.resize_p, h->wpb, h->grid, uses_lists(h), h->stream));
            fg_status us = update_ranks(h);
            if (us) return us;
            if (segments_follow_sizes(h) && (us = refresh_plan(h))) return us;  // segments follow the sizes
        }
        FG_CUDA(cudaEventRecord(h->ev[1], h->stream));
        fg_status st = launch_verify(h, 0);
        if (st) return st;
        FG_CUDA(cudaEventRecord(h->ev[2], h->stream));
        FG_CUDA(cudaMemcpyAsync(hdr.data(), h->B.hdr, sizeof(WalkHeader) * S, cudaMemcpyDeviceToHost, h->stream));
        FG_CUDA(cudaStreamSynchronize(h->stream));
        float a = 0, b = 0;
        cudaEventElapsedTime(&a, h->ev[0], h->ev[1]);
        cudaEventElapsedTime(&b, h->ev[1], h->ev[2]);
        acc.kernel_ms += a;
        acc.verify_ms += b;
        for (int w = 0; w < S; w++) {
            acc.flips += hdr[w].flips_done;
            if (hdr[w].valid) acc.verified_flips += hdr[w].flips_done;
        }
    }
    for (int w = 0; w < S && launches > 0; w++) {
        acc.walks_valid += hdr[w].valid != 0;
        acc.walks_failed += hdr[w].status != 0;
        if (hdr[w].m < acc.min_rank) acc.min_rank = hdr[w].m;
        if (hdr[w].best_rank < acc.min_best_rank) acc.min_best_rank = hdr[w].best_rank;
    }
    if (stats) *stats = acc;
    if (acc.walks_failed) return fail(FG_ERR_WALK, "some walks reported a nonzero status");
    return FG_OK;
}

fg_status fg_minimize(fg_handle *h, int32_t *best_complexity) {
    if (!h || !best_complexity) return fail(FG_ERR_ARG, "null argument");
    if (!h->ready) return fail(FG_ERR_STATE, "records not initialised");
    FG_CUDA(cudaSetDevice(h->dev));
    const int S = h->B.S;
    FG_CUDA(cudaMemcpyAsync(h->d_bestC, best_complexity, (size_t)S * 4, cudaMemcpyHostToDevice, h->stream));
    if (h->cfg.mode == FG_MODE_FAST && h->cfg.ring == FG_RING_Z2) {  // per shape segment, the walk's kernel choice
        for (const Segment &g : h->segs) {
            if (g.nnmax > 56) return fail(FG_ERR_CAPACITY, "fast mode holds factors of at most 56 entries");
            int kind, lanes, wpb;
            segment_kernel(h, g, kind, lanes, wpb);
            if (kind == FG_FAST_THREAD)
                FG_CUDA(launch_minimize_simt(h->B, h->P, g.first, g.count, g.scap, g.wide, wpb, h->sms, h->d_bestC,
                                             h->stream));
            else
                FG_CUDA(launch_minimize_group(h->B, h->P, g.first, g.count, g.scap, g.wide, h->sms, h->d_bestC,
                                              h->stream));
        }
    } else {
        if (!uses_lists(h)) return fail(FG_ERR_ARG, "the minimizer runs in a list mode or the Z2 fast mode");
        FG_CUDA(launch_minimize(h->cfg.ring, h->B, h->P, h->cfg.mode == FG_MODE_REFERENCE ? RNG_XORWOW : RNG_PHILOX,
                                h->wpb, h->grid, h->d_bestC, h->stream));
    }
    FG_CUDA(cudaMemcpyAsync(best_complexity, h->d_bestC, (size_t)S * 4, cudaMemcpyDeviceToHost, h->stream));
    FG_CUDA(cudaStreamSynchronize(h->stream));
    return FG_OK;
}

fg_status fg_validate(fg_handle *h, int best, uint8_t *out) {
    if (!h || !out) return fail(FG_ERR_ARG, "null argument");
    FG_CUDA(cudaSetDevice(h->dev));
    fg_status st = launch_verify(h, best);
    if (st) return st;
    FG_CUDA(cudaMemcpyAsync(out, h->d_valid, h->B.S, cudaMemcpyDeviceToHost, h->stream));
    FG_CUDA(cudaStreamSynchronize(h->stream));
    return FG_OK;
}

fg_status fg_xorwow_tape(uint64_t seed, int first_walk, int count, int draws, int device, uint32_t *out_draws,
                         float *out_uniforms) {
    if (count <= 0 || draws < 0 || !out_draws || !out_uniforms) return fail(FG_ERR_ARG, "bad tape arguments");
    FG_CUDA(cudaSetDevice(device));
    size_t n = (size_t)count * draws;
    uint32_t *d = nullptr;
    float *u = nullptr;
    FG_CUDA(cudaMalloc(&d, n * 4 + 4));
    if (cudaMalloc(&u, n * 4 + 4) != cudaSuccess) { cudaFree(d); return fail(FG_ERR_CUDA, "tape allocation"); }
    k_tape<<<(count + 63) / 64, 64>>>((unsigned long long)seed, first_walk, count, draws, d, u);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out_draws, d, n * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(out_uniforms, u, n * 4, cudaMemcpyDeviceToHost);
    cudaFree(d);
    cudaFree(u);
    if (e != cudaSuccess) return fail(FG_ERR_CUDA, cudaGetErrorString(e));
    return FG_OK;
}

fg_status fg_philox_blocks(const uint32_t *ctr, int count, uint32_t key0, uint32_t key1, int device, uint32_t *out) {
    if (count <= 0 || !ctr || !out) return fail(FG_ERR_ARG, "bad philox arguments");
    FG_CUDA(cudaSetDevice(device));
    uint4 *dc = nullptr, *dout = nullptr;
    const size_t bytes = (size_t)count * 16;
    FG_CUDA(cudaMalloc(&dc, bytes));
    if (cudaMalloc(&dout, bytes) != cudaSuccess) { cudaFree(dc); return fail(FG_ERR_CUDA, "allocation"); }
    cudaError_t e = cudaMemcpy(dc, ctr, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_philox<<<(count + 127) / 128, 128>>>(dc, count, key0, key1, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, bytes, cudaMemcpyDeviceToHost);
    cudaFree(dc);
    cudaFree(dout);
    if (e != cudaSuccess) return fail(FG_ERR_CUDA, cudaGetErrorString(e));
    return FG_OK;
}

}  // extern "C"
