// Learned-proposal Z2 walk.
//
// The walks of a batch advance in lockstep, one flip proposal per step:
//   step kernel  - every walk finishes its pending iteration (picks one of its
//                  K candidates from the scores, applies the flip and the rest
//                  of the fast walk's iteration: best snapshot, reduce/expand
//                  gates, plus transition), then draws K candidate flips
//                  (uniform ordered equal pair + orientation, the fast walk's
//                  draws) and writes their 192 features;
//   MLP          - scores all S*K candidates on the tensor cores (mlp.cu).
// With K = 1 no score is read and no extra draw is made, so the walk consumes
// its Philox stream exactly like the fast kernels and reproduces them.  The
// walk state lives in global memory (one 32-bit word per factor, walks
// interleaved so that a warp's 32 walks touch consecutive words), which for
// 65,536 walks of rank <= 64 is 50 MB and stays in L2.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "learned.h"
#include "mlp.h"
#include "walk_simt.cuh"

namespace fg {

namespace {

using Z = SimtZ2<uint32_t, -1>;

__device__ __forceinline__ uint32_t therm8(int x) { return x <= 0 ? 0u : ((1u << (x < 8 ? x : 8)) - 1u); }

__device__ __forceinline__ void bind(Z &z, const LearnedBuffers &L, const WalkHeader &h, int w) {
    z.s = L.words + w;
    z.rsh = L.sh;
    z.cap = L.scap;
    z.ld = L.scap;
    z.n0 = h.n[0]; z.n1 = h.n[1]; z.n2 = h.n[2];
    z.nn0 = z.n0 * z.n1; z.nn1 = z.n1 * z.n2; z.nn2 = z.n2 * z.n0;
    z.full = z.n0 * z.n1 * z.n2;
}

__device__ __forceinline__ uint64_t term_code(const Z &z, int t) {
    return (uint64_t)z.F(0, t) | ((uint64_t)z.F(1, t) << 21) | ((uint64_t)z.F(2, t) << 42);
}

// Features of candidate flip (component c, orientation o, terms a, b).
__device__ void features(const Z &z, int c, int o, int a, int b, int gap, int plateau, uint64_t *f) {
    int j = c == 0 ? 1 : 0, k = c == 2 ? 1 : 2;
    if (o) { int tmp = j; j = k; k = tmp; }
    const uint32_t newA = z.F(j, a) ^ z.F(j, b), newB = z.F(k, b) ^ z.F(k, a);
    int pa = 0, pb = 0;
    for (int t = 0; t < z.m; t++) {
        pa += (t != a) & (z.F(j, t) == newA);
        pb += (t != b) & (z.F(k, t) == newB);
    }
    const int hca = (int)(z.A(c, a) >> Z::HS);
    f[0] = term_code(z, a);
    f[1] = term_code(z, b);
    f[2] = (1ull << c) | ((uint64_t)o << 3) | ((uint64_t)therm8(pa) << 8) | ((uint64_t)therm8(pb) << 16) |
           ((uint64_t)therm8(hca) << 24) | ((uint64_t)therm8(gap) << 32) | ((uint64_t)therm8(__popc(newA)) << 40) |
           ((uint64_t)therm8(__popc(newB)) << 48) | ((uint64_t)therm8(plateau) << 56);
}

__global__ void k_learned_load(DevBatch B, WalkParams P, LearnedBuffers L) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= L.S) return;
    const WalkHeader h = B.hdr[w];
    ThreadPhilox r;
    r.k0 = P.key0; r.k1 = P.key1; r.walk = (uint32_t)w; r.count = h.draws; r.blk = -1; r.P = &P;
    Z z(r);
    bind(z, L, h, w);
    z.m = h.m;
    z.status = h.status;
    const uint64_t *src = B.fac + (size_t)w * 3 * B.cap;
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < L.scap; t++) z.A(c, t) = t < h.m ? (uint32_t)src[c * B.cap + t] : 0u;
    z.rebuild();
    LWalk s = L.lw[w];
    s.m = z.m; s.P0 = z.P0; s.P1 = z.P1; s.P2 = z.P2; s.status = z.status;
    s.flips = h.flips; s.bestRank = h.best_rank; s.bestM = h.best_m;
    s.it = 0; s.pending = 0; s.copied = 0;
    s.draws = h.draws; s.accepted = 0;
    L.lw[w] = s;  // total and ndrops persist across launches
}

__global__ void k_learned_step(DevBatch B, WalkParams P, LearnedBuffers L, LearnedConfig C, int useScores) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= L.S) return;
    LWalk s = L.lw[w];
    if (!s.pending && (s.status || s.it >= P.iterations)) return;
    const WalkHeader h = B.hdr[w];
    ThreadPhilox r;
    r.k0 = P.key0; r.k1 = P.key1; r.walk = (uint32_t)w; r.count = s.draws; r.blk = -1; r.P = &P;
    Z z(r);
    bind(z, L, h, w);
    z.m = s.m; z.P0 = s.P0; z.P1 = s.P1; z.P2 = s.P2; z.status = s.status;
    const int K = L.K;
    if (s.pending) {
        int ci = 0;
        if (K > 1) {
            bool uniform = !useScores;
            float p[16];
            float Zs = 0.0f;
            if (!uniform) {
                float mx = -INFINITY;
                for (int q = 0; q < K; q++) mx = fmaxf(mx, L.scores[(size_t)w * K + q]);
                for (int q = 0; q < K; q++) {
                    p[q] = expf((L.scores[(size_t)w * K + q] - mx) * C.invTemp);
                    Zs += p[q];
                }
                float H = 0.0f;
                for (int q = 0; q < K; q++) {
                    const float pq = p[q] / Zs;
                    if (pq > 0.0f) H -= pq * logf(pq);
                }
                uniform = !(Zs > 0.0f) || !(H >= C.minEntropy);  // also catches NaN scores
            }
            if (uniform) {
                ci = (int)r.below((uint32_t)K);
            } else {
                const float u = (float)(r.raw() >> 8) * (1.0f / 16777216.0f) * Zs;
                float acc = 0.0f;
                ci = K - 1;
                for (int q = 0; q < K; q++) {
                    acc += p[q];
                    if (u < acc) { ci = q; break; }
                }
            }
        }
        const uint32_t cd = L.cand[(size_t)w * K + ci];
        const int c = (int)(cd & 3u), o = (int)((cd >> 2) & 1u), a = (int)((cd >> 3) & 511u), b = (int)((cd >> 12) & 511u);
        int j = c == 0 ? 1 : 0, k = c == 2 ? 1 : 2;
        if (o) { int tmp = j; j = k; k = tmp; }
        const int rank = z.m;
        z.flip(c, j, k, a, b, true);
        s.accepted++;
        s.total++;
        if (C.recordEvery > 0 && s.total % (unsigned long long)C.recordEvery == 0) {
            const unsigned long long slot = atomicAdd(L.recCount, 1ull);
            if ((long long)slot < L.recCap) {
                const uint64_t *f = L.feat + ((size_t)w * K + ci) * 3;
                L.recFeat[slot * 3 + 0] = f[0];
                L.recFeat[slot * 3 + 1] = f[1];
                L.recFeat[slot * 3 + 2] = f[2];
                L.recWalk[slot] = (uint32_t)w;
                L.recFlip[slot] = (uint32_t)s.total;
            }
        }
        bool dropped = z.m < rank;
        if (z.m < rank) s.flips = 0;
        s.flips++;
        if (z.m < s.bestRank || (z.m == s.bestRank && r.tie())) {
            s.bestRank = z.m;
            s.bestM = z.m;
            uint64_t *dst = B.best_fac + (size_t)w * 3 * B.cap;
            for (int cc = 0; cc < 3; cc++)
                for (int t = 0; t < z.m; t++) dst[cc * B.cap + t] = z.F(cc, t);
            s.copied = 1;
        }
        if (r.gate_reduce()) {
            const int before = z.m;
            z.tryReduce();
            dropped |= z.m < before;
        }
        if (r.gate_expand() && z.m <= s.bestM + 2) {
            if (z.tryExpand(randint(1, 2, r))) s.flips = 0;
        }
        if (s.flips >= P.plus_iterations && z.tryPlus()) s.flips = 0;
        if (dropped && L.drops) {
            if (s.ndrops < L.dropCap) L.drops[(size_t)w * L.dropCap + s.ndrops] = (uint32_t)s.total;
            s.ndrops++;
        }
        s.it++;
        s.pending = 0;
    }
    // Next proposal (iterations without an equal pair expand and are consumed here).
    while (!z.status && s.it < P.iterations) {
        if (z.P0 + z.P1 + z.P2 <= 0) {
            z.tryExpand(randint(1, 2, r));
            s.it++;
            continue;
        }
        bool ok = true;
        for (int q = 0; q < K && ok; q++) {
            int c, a, b;
            ok = z.pickPair(c, a, b);
            if (!ok) break;
            const int o = r.coin() ? 1 : 0;
            L.cand[(size_t)w * K + q] = (uint32_t)c | ((uint32_t)o << 2) | ((uint32_t)a << 3) | ((uint32_t)b << 12);
            features(z, c, o, a, b, z.m - s.bestRank, s.flips / 6250, L.feat + ((size_t)w * K + q) * 3);
        }
        if (ok) s.pending = 1;
        break;
    }
    s.m = z.m; s.P0 = z.P0; s.P1 = z.P1; s.P2 = z.P2; s.status = z.status;
    s.draws = r.count;
    L.lw[w] = s;
}

__global__ void k_learned_store(DevBatch B, LearnedBuffers L) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= L.S) return;
    const LWalk s = L.lw[w];
    uint64_t *dst = B.fac + (size_t)w * 3 * B.cap;
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < B.cap; t++)
            dst[c * B.cap + t] = t < s.m ? (uint64_t)(L.words[((size_t)(c * L.scap + t) << L.sh) + w] & Z::FM) : 0ull;
    if (s.copied) {
        uint64_t *bd = B.best_fac + (size_t)w * 3 * B.cap;
        for (int c = 0; c < 3; c++)
            for (int t = s.bestM < 0 ? 0 : s.bestM; t < B.cap; t++) bd[c * B.cap + t] = 0ull;
    }
    WalkHeader &h = B.hdr[w];
    h.m = s.m;
    h.flips = s.flips;
    h.best_rank = s.bestRank;
    h.best_m = s.bestM;
    h.status = s.status;
    h.list_size[0] = h.list_size[1] = h.list_size[2] = 0;
    h.draws = s.draws;
    h.flips_done = s.accepted;
}

template <class T> cudaError_t dalloc(T **p, size_t n) { return cudaMalloc(reinterpret_cast<void **>(p), n * sizeof(T)); }

}  // namespace

cudaError_t learned_alloc(LearnedBuffers &L, int S, int scap, int K) {
    learned_free(L);
    int sh = 0;
    while ((1 << sh) < S) sh++;
    L.S = S;
    L.Spad = 1 << sh;
    L.sh = sh;
    L.scap = scap;
    L.K = K;
    cudaError_t e;
    if ((e = dalloc(&L.words, (size_t)3 * scap * L.Spad)) || (e = dalloc(&L.lw, (size_t)S)) ||
        (e = dalloc(&L.cand, (size_t)S * K)) || (e = dalloc(&L.feat, (size_t)S * K * 3)) ||
        (e = dalloc(&L.scores, (size_t)S * K))) {
        learned_free(L);
        return e;
    }
    if ((e = cudaMemset(L.lw, 0, sizeof(LWalk) * S)) || (e = cudaMemset(L.words, 0, sizeof(uint32_t) * 3 * scap * L.Spad)) ||
        (e = cudaMemset(L.feat, 0, sizeof(uint64_t) * 3 * S * K)))
        learned_free(L);
    return e;
}

cudaError_t learned_alloc_records(LearnedBuffers &L, long long recCap, int dropCap) {
    void *ps[] = {L.recFeat, L.recWalk, L.recFlip, L.recCount, L.drops};
    for (void *p : ps)
        if (p) cudaFree(p);
    L.recFeat = nullptr; L.recWalk = L.recFlip = nullptr; L.recCount = nullptr; L.drops = nullptr;
    L.recCap = 0; L.dropCap = 0;
    if (recCap <= 0) return cudaSuccess;
    cudaError_t e;
    if ((e = dalloc(&L.recFeat, (size_t)recCap * 3)) || (e = dalloc(&L.recWalk, (size_t)recCap)) ||
        (e = dalloc(&L.recFlip, (size_t)recCap)) || (e = dalloc(&L.recCount, 1)) ||
        (e = dalloc(&L.drops, (size_t)L.S * dropCap)))
        return e;
    L.recCap = recCap;
    L.dropCap = dropCap;
    if ((e = cudaMemset(L.recCount, 0, sizeof(unsigned long long)))) return e;
    // fresh drop logs and flip counters
    std::vector<LWalk> lw(L.S);
    if ((e = cudaMemcpy(lw.data(), L.lw, sizeof(LWalk) * L.S, cudaMemcpyDeviceToHost))) return e;
    for (auto &x : lw) { x.ndrops = 0; x.total = 0; }
    return cudaMemcpy(L.lw, lw.data(), sizeof(LWalk) * L.S, cudaMemcpyHostToDevice);
}

void learned_free(LearnedBuffers &L) {
    learned_alloc_records(L, 0, 0);
    void *ps[] = {L.words, L.lw, L.cand, L.feat, L.scores};
    for (void *p : ps)
        if (p) cudaFree(p);
    L = LearnedBuffers{};
}

namespace {

cudaError_t learned_steps(LearnedBuffers &L, const DevBatch &B, const WalkParams &P, const LearnedConfig &C,
                          fg_mlp *mlp, int useScores, cudaStream_t s) {
    const int threads = 128, blocks = (L.S + threads - 1) / threads;
    cudaError_t e = cudaSuccess;
    for (int step = 0; step <= P.iterations && !e; step++) {
        k_learned_step<<<blocks, threads, 0, s>>>(B, P, L, C, useScores);
        e = cudaGetLastError();
        if (!e && useScores && step < P.iterations) e = mlp_score_device(mlp, L.feat, L.S * L.K, L.scores, s);
    }
    return e;
}

template <class T> void append_bytes(std::vector<unsigned char> &k, const T &v) {
    const unsigned char *p = reinterpret_cast<const unsigned char *>(&v);
    k.insert(k.end(), p, p + sizeof(T));
}

// The step loop, through G's graph when G is given (see LearnedGraph).
cudaError_t learned_steps_graph(LearnedBuffers &L, const DevBatch &B, const WalkParams &P, const LearnedConfig &C,
                                fg_mlp *mlp, int useScores, cudaStream_t s, LearnedGraph *G) {
    if (!G) return learned_steps(L, B, P, C, mlp, useScores, s);
    std::vector<unsigned char> key;
    append_bytes(key, B);
    append_bytes(key, P);
    append_bytes(key, C);
    append_bytes(key, L);
    append_bytes(key, mlp);
    append_bytes(key, mlp_workspace_epoch(mlp));
    append_bytes(key, useScores);
    if (key != G->key) {  // new arguments: run directly once
        G->reset();
        G->key = key;
        G->primed = true;
        return learned_steps(L, B, P, C, mlp, useScores, s);
    }
    if (G->exec) return cudaGraphLaunch(G->exec, s);
    if (G->failed) return learned_steps(L, B, P, C, mlp, useScores, s);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed);
    if (e) return e;
    const cudaError_t le = learned_steps(L, B, P, C, mlp, useScores, s);
    const cudaError_t ce = cudaStreamEndCapture(s, &g);
    if (le == cudaSuccess && ce == cudaSuccess) e = cudaGraphInstantiate(&G->exec, g, 0);
    else e = le != cudaSuccess ? le : ce;
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {  // not capturable here: direct launches from now on
        cudaGetLastError();
        G->exec = nullptr;
        G->failed = true;
        return learned_steps(L, B, P, C, mlp, useScores, s);
    }
    return cudaGraphLaunch(G->exec, s);
}

}  // namespace

cudaError_t learned_launch(LearnedBuffers &L, const DevBatch &B, const WalkParams &P, const LearnedConfig &C,
                           fg_mlp *mlp, cudaStream_t s, LearnedGraph *G) {
    const int threads = 128, blocks = (L.S + threads - 1) / threads;
    k_learned_load<<<blocks, threads, 0, s>>>(B, P, L);
    cudaError_t e = cudaGetLastError();
    const int useScores = (L.K > 1 && mlp) ? 1 : 0;
    if (!e) e = learned_steps_graph(L, B, P, C, mlp, useScores, s, G);
    if (!e) {
        k_learned_store<<<blocks, threads, 0, s>>>(B, L);
        e = cudaGetLastError();
    }
    return e;
}

cudaError_t learned_take_records(LearnedBuffers &L, int horizon, std::vector<uint64_t> &feat, std::vector<float> &label,
                                 cudaStream_t s) {
    feat.clear();
    label.clear();
    if (!L.recCap) return cudaSuccess;
    unsigned long long cnt = 0;
    cudaError_t e = cudaMemcpyAsync(&cnt, L.recCount, sizeof(cnt), cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaStreamSynchronize(s);
    if (e) return e;
    const size_t n = (size_t)std::min<unsigned long long>(cnt, (unsigned long long)L.recCap);
    std::vector<uint64_t> rf(n * 3);
    std::vector<uint32_t> rw(n), rfl(n), drops((size_t)L.S * L.dropCap);
    std::vector<LWalk> lw(L.S);
    if (n) {
        if (!e) e = cudaMemcpyAsync(rf.data(), L.recFeat, sizeof(uint64_t) * 3 * n, cudaMemcpyDeviceToHost, s);
        if (!e) e = cudaMemcpyAsync(rw.data(), L.recWalk, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s);
        if (!e) e = cudaMemcpyAsync(rfl.data(), L.recFlip, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s);
    }
    if (!e) e = cudaMemcpyAsync(drops.data(), L.drops, sizeof(uint32_t) * drops.size(), cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaMemcpyAsync(lw.data(), L.lw, sizeof(LWalk) * L.S, cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaStreamSynchronize(s);
    if (e) return e;
    feat.reserve(n * 3);
    label.reserve(n);
    for (size_t i = 0; i < n; i++) {
        const int w = (int)rw[i];
        const uint32_t f = rfl[i];
        const int nd = lw[w].ndrops, logged = std::min(nd, L.dropCap);
        const uint32_t *d = drops.data() + (size_t)w * L.dropCap;
        const uint32_t *it = std::lower_bound(d, d + logged, f);
        float y;
        if (it != d + logged) {
            y = (*it < (uint64_t)f + (uint64_t)horizon) ? 1.0f : 0.0f;
        } else if (nd > L.dropCap) {
            continue;  // later drops were not logged
        } else if (lw[w].total + 1 >= (unsigned long long)f + (unsigned long long)horizon) {
            y = 0.0f;
        } else {
            continue;  // the walk has not yet run `horizon` flips past this record
        }
        feat.push_back(rf[i * 3]);
        feat.push_back(rf[i * 3 + 1]);
        feat.push_back(rf[i * 3 + 2]);
        label.push_back(y);
    }
    return cudaSuccess;
}

}  // namespace fg
