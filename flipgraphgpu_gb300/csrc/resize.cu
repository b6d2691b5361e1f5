// Resize meta-operators of the Z2 walk (resizeKernel, flip_graph.cu:575-613;
// scheme_z2.cu:184-310, 643-979, 1165-1275), one warp per walk.
//
// After each walk launch a walk, with probability p, may transpose its sizes
// (swapSize), merge another walk's best scheme along one size, or else project
// out a row/column, take the tensor product with another walk's best scheme,
// double one size (block product) or extend one size by one.  Every operator
// remaps each term's three bit matrices independently, so lanes take terms
// t = lane, lane + 32, ...; draws are replicated in every lane (the reference's
// stream and draw order), structural edits that need order (compaction,
// reductions, list rebuilds) reuse the walk's warp code.  Matrix c is
// n[c] x n[c+1] (W transposed), entry (i, j) at bit i * n[c+1] + j.
#include "kernels.cuh"
#include "launch.h"
#include "walk_moves.cuh"

namespace fg {

namespace {

constexpr int kMaxExtensionN = 16;  // config.cuh:37
constexpr int kMinProjectN = 2;     // config.cuh:34
constexpr int kMaxRankRef = 350;    // config.cuh:10

__device__ __forceinline__ uint64_t bit(uint64_t v, int k) { return (v >> k) & 1ull; }

// Entry (i, j) of a rows x cols matrix to (i + di, j + dj) of a matrix with newCols columns.
__device__ Vec place(Vec a, int rows, int cols, int newCols, int di, int dj) {
    Vec o{0, 0};
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++) {
            const int from = i * cols + j, to = (i + di) * newCols + j + dj;
            o.v |= bit(a.v, from) << to;
            o.s |= bit(a.s, from) << to;
        }
    return o;
}

template <class Z>
__device__ __forceinline__ void set_sizes(Z &z, int a, int b, int c) {
    z.n0 = a; z.n1 = b; z.n2 = c;
    z.nn0 = a * b; z.nn1 = b * c; z.nn2 = c * a;
    z.full = a * b * c;
}

template <class Z>
__device__ __forceinline__ int nsz(const Z &z, int i) { return i == 0 ? z.n0 : (i == 1 ? z.n1 : z.n2); }

// Another walk's best scheme, read in place from the records.
struct BestView {
    const uint64_t *fac, *sgn;  // [3][cap]; sgn null for Z2
    int cap, n[3], m;
    __device__ Vec X(int c, int t) const { return Vec{fac[c * cap + t], sgn ? sgn[c * cap + t] : 0}; }
};

__device__ BestView best_view(const DevBatch &B, int index) {
    BestView o;
    o.fac = B.best_fac + (size_t)index * 3 * B.cap;
    o.sgn = B.best_sgn ? B.best_sgn + (size_t)index * 3 * B.cap : nullptr;
    o.cap = B.cap;
    o.m = B.hdr[index].best_m;
    for (int c = 0; c < 3; c++) o.n[c] = B.best_n[index * 3 + c];
    return o;
}

template <class Z>
__device__ void swap_size(Z &z, int p1, int p2) {  // scheme_z2.cu:916-979, scheme_integer.cu:843-905
    using O = RingOps<Z>;
    if (p1 == p2) return;
    if (p1 > p2) { int t = p1; p1 = p2; p2 = t; }
    int idx[3];
    if (p1 == 0 && p2 == 1) { idx[0] = 0; idx[1] = 2; idx[2] = 1; }
    else if (p1 == 0 && p2 == 2) { idx[0] = 1; idx[1] = 0; idx[2] = 2; }
    else { idx[0] = 2; idx[1] = 1; idx[2] = 0; }
    int g[3];
    for (int q = 0; q < 3; q++) g[q] = nsz(z, (idx[q] + 1) % 3);
    __syncwarp();
    for (int t = lane_id(); t < z.m; t += 32) {
        Vec v[3];
        for (int c = 0; c < 3; c++) {  // new matrix c is the transpose of old matrix idx[c]
            const int rows = g[c], cols = g[(c + 1) % 3];
            const Vec a = O::get(z, idx[c], t);
            Vec o{0, 0};
            for (int i = 0; i < rows; i++)
                for (int j = 0; j < cols; j++) {
                    o.v |= bit(a.v, j * rows + i) << (i * cols + j);
                    o.s |= bit(a.s, j * rows + i) << (i * cols + j);
                }
            v[c] = o;
        }
        for (int c = 0; c < 3; c++) O::put(z, c, t, v[c]);
    }
    __syncwarp();
    set_sizes(z, g[0], g[1], g[2]);
    O::fixSigns(z);
    z.rebuild();
}

template <class Z>
__device__ void reduce_all(Z &z) {  // while (tryReduce()) ; bounded
    for (int guard = 0; z.tryReduce(); guard++)
        if (guard > retry_cap_of(z.r.P)) { z.status |= ST_RETRY; return; }
}

template <class Z>
__device__ void project(Z &z, int p, int q) {  // scheme_z2.cu:643-653, scheme_integer.cu:573-584
    using O = RingOps<Z>;
    const int rc = (p + 2) % 3;  // matrix losing column q
    const int n[3] = {z.n0, z.n1, z.n2};
    __syncwarp();
    for (int t = lane_id(); t < z.m; t += 32) {
        {  // matrix p: drop row q
            const int rows = n[p], cols = n[(p + 1) % 3];
            const Vec a = O::get(z, p, t);
            Vec o{0, 0};
            for (int i = 0, i2 = 0; i < rows; i++) {
                if (i == q) continue;
                for (int j = 0; j < cols; j++) {
                    o.v |= bit(a.v, i * cols + j) << (i2 * cols + j);
                    o.s |= bit(a.s, i * cols + j) << (i2 * cols + j);
                }
                i2++;
            }
            O::put(z, p, t, o);
        }
        {  // matrix rc: drop column q
            const int rows = n[rc], cols = n[(rc + 1) % 3];
            const Vec a = O::get(z, rc, t);
            Vec o{0, 0};
            for (int i = 0; i < rows; i++)
                for (int j = 0, j2 = 0; j < cols; j++) {
                    if (j == q) continue;
                    o.v |= bit(a.v, i * cols + j) << (i * (cols - 1) + j2);
                    o.s |= bit(a.s, i * cols + j) << (i * (cols - 1) + j2);
                    j2++;
                }
            O::put(z, rc, t, o);
        }
    }
    __syncwarp();
    int g[3] = {n[0], n[1], n[2]};
    g[p]--;
    set_sizes(z, g[0], g[1], g[2]);
    z.removeZeroes();
    O::fixSigns(z);
    z.rebuild();
}

template <class Z>
__device__ void extend(Z &z, int p) {  // scheme_z2.cu:655-687, scheme_integer.cu:586-618 (old sizes)
    using O = RingOps<Z>;
    const int a = z.n0, b = z.n1, c = z.n2;
    const int col = p == 0 ? 2 : (p == 1 ? 0 : 1);  // matrix gaining a column (addColumn)
    const int cr = col == 0 ? a : (col == 1 ? b : c), cc = col == 0 ? b : (col == 1 ? c : a);
    const int m0 = z.m;
    __syncwarp();
    for (int t = lane_id(); t < m0; t += 32) O::put(z, col, t, place(O::get(z, col, t), cr, cc, cc + 1, 0, 0));
    // new terms, in the reference's loop order, each a single +1 entry per matrix
    const int outer = p == 0 ? c : a, inner = p == 0 ? b : (p == 1 ? c : b);
    for (int q = lane_id(); q < outer * inner; q += 32) {
        const int i = q / inner, j = q % inner, t = m0 + q;
        uint64_t u, v, w;
        if (p == 0) { u = 1ull << (a * b + j); v = 1ull << (j * c + i); w = 1ull << (i * (a + 1) + a); }
        else if (p == 1) { u = 1ull << (i * (b + 1) + b); v = 1ull << (b * c + j); w = 1ull << (j * a + i); }
        else { u = 1ull << (i * b + j); v = 1ull << (j * (c + 1) + c); w = 1ull << (c * a + i); }
        O::put(z, 0, t, Vec{u, 0});
        O::put(z, 1, t, Vec{v, 0});
        O::put(z, 2, t, Vec{w, 0});
    }
    __syncwarp();
    z.m = m0 + outer * inner;
    int g[3] = {a, b, c};
    g[p]++;
    set_sizes(z, g[0], g[1], g[2]);
    z.rebuild();
}

template <class Z>
__device__ void product(Z &z, int p) {  // scheme_z2.cu:689-747, scheme_integer.cu:620-678
    using O = RingOps<Z>;
    const int n[3] = {z.n0, z.n1, z.n2};
    int g[3] = {n[0], n[1], n[2]}, d[3];
    g[p] *= 2;
    for (int q = 0; q < 3; q++) d[q] = q == p ? n[q] : 0;
    const int m0 = z.m;
    __syncwarp();
    for (int t = lane_id(); t < m0; t += 32)
        for (int c = 0; c < 3; c++) {
            const int c1 = (c + 1) % 3;
            const Vec v = O::get(z, c, t);
            O::put(z, c, t, place(v, n[c], n[c1], g[c1], 0, 0));
            O::put(z, c, t + m0, place(v, n[c], n[c1], g[c1], d[c], d[c1]));
        }
    __syncwarp();
    z.m = 2 * m0;
    set_sizes(z, g[0], g[1], g[2]);
    z.rebuild();
}

template <class Z>
__device__ void merge(Z &z, const BestView &o, int p) {  // scheme_z2.cu:749-817, scheme_integer.cu:680-745
    using O = RingOps<Z>;
    const int n[3] = {z.n0, z.n1, z.n2};
    int g[3], d[3];
    for (int q = 0; q < 3; q++) {
        g[q] = q == p ? n[q] + o.n[q] : n[q];
        d[q] = q == p ? n[q] : 0;
    }
    const int m0 = z.m;
    __syncwarp();
    for (int t = lane_id(); t < m0; t += 32)
        for (int c = 0; c < 3; c++) O::put(z, c, t, place(O::get(z, c, t), n[c], n[(c + 1) % 3], g[(c + 1) % 3], 0, 0));
    for (int t = lane_id(); t < o.m; t += 32)
        for (int c = 0; c < 3; c++) {
            const int c1 = (c + 1) % 3;
            O::put(z, c, m0 + t, place(o.X(c, t), o.n[c], o.n[c1], g[c1], d[c], d[c1]));
        }
    __syncwarp();
    z.m = m0 + o.m;
    set_sizes(z, g[0], g[1], g[2]);
    z.rebuild();
}

// Tensor product with another walk's best scheme (scheme_z2.cu:819-862,
// scheme_integer.cu:747-841): term (t1, t2) -> t1 * m2 + t2, coefficients
// multiplied.  The walk's own terms are read from a copy in its global record,
// since the new terms overwrite them.
template <class Z>
__device__ void product_with(Z &z, const BestView &o, uint64_t *ownV, uint64_t *ownS) {
    using O = RingOps<Z>;
    const int a0 = z.n0, a1 = z.n1, a2 = z.n2, m1 = z.m;
    __syncwarp();
    O::stash(z, ownV, ownS);
    __syncwarp();
    const int an[3] = {a0, a1, a2};
    int g[3];
    for (int c = 0; c < 3; c++) g[c] = an[c] * o.n[c];
    for (int t = lane_id(); t < m1 * o.m; t += 32) {
        const int t1 = t / o.m, t2 = t % o.m;
        for (int c = 0; c < 3; c++) {
            const int c1 = (c + 1) % 3;
            const Vec va{ownV[c * z.cap + t1], ownS ? ownS[c * z.cap + t1] : 0}, vb = o.X(c, t2);
            Vec v{0, 0};
            for (int e1 = 0; e1 < an[c] * an[c1]; e1++) {
                if (!bit(va.v, e1)) continue;
                const int r1 = e1 / an[c1], q1 = e1 % an[c1];
                for (int e2 = 0; e2 < o.n[c] * o.n[c1]; e2++) {
                    if (!bit(vb.v, e2)) continue;
                    const int r2 = e2 / o.n[c1], q2 = e2 % o.n[c1];
                    const int to = (r1 * o.n[c] + r2) * g[c1] + q1 * o.n[c1] + q2;
                    v.v |= 1ull << to;
                    v.s |= (bit(va.s, e1) ^ bit(vb.s, e2)) << to;
                }
            }
            O::put(z, c, t, v);
        }
    }
    __syncwarp();
    z.m = m1 * o.m;
    set_sizes(z, g[0], g[1], g[2]);
    z.rebuild();
}

// scheme_z2.cu:260-294; maxMatrix = the reference's 64 (config.cuh:11), 56 in the fast mode.
__device__ bool valid_grown(const int g[3], int rank, int maxN, int maxMatrix) {
    if (rank > kMaxRankRef) return false;
    for (int q = 0; q < 3; q++)
        if (g[q] * g[(q + 1) % 3] > maxMatrix || g[q] > maxN) return false;
    return true;
}

template <class Z, class R>
__device__ bool try_project(Z &z, R &r) {  // scheme_z2.cu:1165-1185, scheme_integer.cu:1103-1123
    const int n[3] = {z.n0, z.n1, z.n2};
    int idx[3], size = 0;
    for (int i = 0; i < 3; i++)
        if (n[i] - 1 >= kMinProjectN && n[(i + 1) % 3] >= kMinProjectN && n[(i + 2) % 3] >= kMinProjectN) idx[size++] = i;
    if (!size) return false;
    const int p = idx[r.raw() % (uint32_t)size];
    const int q = (int)(r.raw() % (uint32_t)n[p]);
    project(z, p, q);
    reduce_all(z);
    return true;
}

template <class Z, class R>
__device__ bool try_extend(Z &z, R &r) {  // scheme_z2.cu:1187-1206, scheme_integer.cu:1125-1144
    int idx[3], size = 0;
    for (int i = 0; i < 3; i++) {
        int g[3] = {z.n0, z.n1, z.n2};
        g[i] += 1;
        if (valid_grown(g, z.m + g[(i + 1) % 3] * g[(i + 2) % 3], kMaxExtensionN, r.P->max_matrix)) idx[size++] = i;
    }
    if (!size) return false;
    extend(z, idx[r.raw() % (uint32_t)size]);
    reduce_all(z);
    return true;
}

template <class Z, class R>
__device__ bool try_product(Z &z, R &r) {  // scheme_z2.cu:1208-1223, scheme_integer.cu:1146-1161
    int idx[3], size = 0;
    for (int i = 0; i < 3; i++) {
        int g[3] = {z.n0, z.n1, z.n2};
        g[i] *= 2;
        if (valid_grown(g, z.m * 2, kMaxExtensionN, r.P->max_matrix)) idx[size++] = i;
    }
    if (!size) return false;
    product(z, idx[r.raw() % (uint32_t)size]);
    return true;
}

template <class Z, class R>
__device__ bool try_merge(Z &z, const BestView &o, R &r) {  // scheme_z2.cu:1225-1254, scheme_integer.cu:1163-1192
    if (z.m + o.m > kMaxRankRef) return false;
    const int n[3] = {z.n0, z.n1, z.n2};
    const bool eq0 = n[0] == o.n[0], eq1 = n[1] == o.n[1], eq2 = n[2] == o.n[2];
    const int s0 = n[0] + o.n[0], s1 = n[1] + o.n[1], s2 = n[2] + o.n[2];
    const int mx = r.P->max_matrix;
    int p[3], size = 0;
    if (s0 <= kMaxExtensionN && s0 * n[1] <= mx && s0 * n[2] <= mx && eq1 && eq2) p[size++] = 0;
    if (eq0 && s1 <= kMaxExtensionN && n[0] * s1 <= mx && n[2] * s1 <= mx && eq2) p[size++] = 1;
    if (eq0 && eq1 && s2 <= kMaxExtensionN && n[0] * s2 <= mx && n[1] * s2 <= mx) p[size++] = 2;
    if (!size) return false;
    merge(z, o, p[r.raw() % (uint32_t)size]);
    return true;
}

template <class Z>
__device__ bool try_product_with(Z &z, const BestView &o, uint64_t *ownV, uint64_t *ownS, int maxMatrix) {  // scheme_z2.cu:1256-1275
    if (z.m * o.m > kMaxRankRef) return false;
    const int n[3] = {z.n0, z.n1, z.n2};
    int g[3];
    for (int q = 0; q < 3; q++) g[q] = n[q] * o.n[q];
    for (int q = 0; q < 3; q++)
        if (g[q] > kMaxExtensionN || g[q] * g[(q + 1) % 3] > maxMatrix) return false;
    product_with(z, o, ownV, ownS);
    return true;
}

// resizeKernel (flip_graph.cu:575-613) for walk w.
template <class Walker, class R>
__device__ void resize_one(const DevBatch &B, const WalkParams &P, int w, unsigned char *base, double p, int keepLists) {
    const WalkHeader h = B.hdr[w];
    if (h.status) return;
    R r = DrawsIO<R>::load(B, P, w, h);
    if ((double)r.uniform() > p) {
        DrawsIO<R>::store(B, w, r);
        if (lane_id() == 0) B.hdr[w].draws = r.count;
        return;
    }
    Walker z(r);
    walk_bind(z, B, h, w, base);
    if ((double)r.uniform() < 0.5) {  // swapSize(state), scheme_z2.cu:1315-1323
        int p1, p2;
        do {
            p1 = (int)(r.raw() % 3u);
            p2 = (int)(r.raw() % 3u);
        } while (p1 == p2);
        swap_size(z, p1, p2);
    }
    bool merged = false;
    for (int i = 0; i < 3 && !merged; i++) {
        const int index = (int)(r.raw() % (uint32_t)B.S);
        merged |= try_merge(z, best_view(B, index), r);
    }
    if (!merged) {
        const double q = (double)r.uniform();
        if (q < 0.05) try_project(z, r);
        else if (q < 0.55)
            try_product_with(z, best_view(B, (int)(r.raw() % (uint32_t)B.S)), B.fac + (size_t)w * 3 * B.cap,
                             B.sgn ? B.sgn + (size_t)w * 3 * B.cap : nullptr, P.max_matrix);
        else if (q < 0.85) try_product(z, r);
        else try_extend(z, r);
    }
    walk_store(z, B, w);
    DrawsIO<R>::store(B, w, r);
    if (lane_id() == 0) {
        WalkHeader o = B.hdr[w];
        o.n[0] = z.n0; o.n[1] = z.n1; o.n[2] = z.n2;
        o.m = z.m;
        o.status = z.status;
        // the fast mode keeps no lists: its walks count partners when they load
        o.list_size[0] = keepLists ? z.sz0 : 0;
        o.list_size[1] = keepLists ? z.sz1 : 0;
        o.list_size[2] = keepLists ? z.sz2 : 0;
        o.draws = r.count;
        B.hdr[w] = o;
    }
}

template <class Walker, class R>
__global__ void k_resize(DevBatch B, WalkParams P, double p, int keepLists) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int wpb = blockDim.x >> 5, warp = threadIdx.x >> 5;
    unsigned char *base = smem + RingIO<Walker>::smem(B.cap) * warp;
    for (int w = blockIdx.x * wpb + warp; w < B.S; w += gridDim.x * wpb) resize_one<Walker, R>(B, P, w, base, p, keepLists);
}

// The per-size best-rank table's copies (FlipGraph::updateRanks, flip_graph.cu:257-261):
// walk w's current scheme becomes its best.
__global__ void k_copy_best(DevBatch B, const int32_t *walks, int count, const int32_t *bestRank) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (warp < count) {
        const int w = walks[warp];
        const size_t o = (size_t)w * 3 * B.cap;
        const int m = B.hdr[w].m;
        for (int q = lane_id(); q < 3 * B.cap; q += 32) {
            const bool live = (q % B.cap) < m;
            B.best_fac[o + q] = live ? B.fac[o + q] : 0ull;
            if (B.sgn) {
                B.best_sgn[o + q] = live ? B.sgn[o + q] : 0ull;
                B.best_valid[o + q] = live ? B.valid[o + q] : 0;
            }
        }
        if (lane_id() == 0) {
            B.hdr[w].best_m = m;
            for (int c = 0; c < 3; c++) B.best_n[w * 3 + c] = B.hdr[w].n[c];
        }
    }
    // every walk's best rank becomes its size's (one thread per walk)
    if (bestRank)
        for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < B.S; w += gridDim.x * blockDim.x)
            B.hdr[w].best_rank = bestRank[w];
}

template <class Walker, class R>
cudaError_t resize_t(const DevBatch &B, const WalkParams &P, double p, int wpb, int grid, int keepLists, cudaStream_t s) {
    const size_t smem = RingIO<Walker>::smem(B.cap) * wpb;
    cudaError_t e = cudaFuncSetAttribute(k_resize<Walker, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e) return e;
    k_resize<Walker, R><<<grid, 32 * wpb, smem, s>>>(B, P, p, keepLists);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_resize(int ring, const DevBatch &B, const WalkParams &P, int rng, double p, int wpb, int grid,
                          int keepLists, cudaStream_t s) {
    if (slots_for_cap(B.cap) != 11 || !B.best_n) return cudaErrorInvalidValue;
    if (ring == 0)
        return rng == RNG_XORWOW ? resize_t<Z2Walk<XorwowDraws, 11>, XorwowDraws>(B, P, p, wpb, grid, keepLists, s)
                                 : resize_t<Z2Walk<PhiloxDraws, 11>, PhiloxDraws>(B, P, p, wpb, grid, keepLists, s);
    return rng == RNG_XORWOW ? resize_t<ZTWalk<XorwowDraws, 11>, XorwowDraws>(B, P, p, wpb, grid, keepLists, s)
                             : resize_t<ZTWalk<PhiloxDraws, 11>, PhiloxDraws>(B, P, p, wpb, grid, keepLists, s);
}

cudaError_t launch_copy_best(const DevBatch &B, const int32_t *walks, int count, const int32_t *bestRank, cudaStream_t s) {
    const int threads = 256;
    int blocks = (count * 32 + threads - 1) / threads;
    const int walkBlocks = (B.S + threads - 1) / threads;
    if (blocks < walkBlocks) blocks = walkBlocks;
    if (blocks < 1) blocks = 1;
    k_copy_best<<<blocks, threads, 0, s>>>(B, walks, count, bestRank);
    return cudaGetLastError();
}

}  // namespace fg
