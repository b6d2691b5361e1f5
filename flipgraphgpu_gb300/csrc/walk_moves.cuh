// Basis moves of the list-mode walkers (randomWalkKernel's sandwiching and
// basis gates, flip_graph.cu:560-564): sandwiching conjugates every term by
// random invertible GF(2) matrices (scheme_z2.cu:444-529,1277-1300; empty for
// the ternary ring, scheme_integer.cu:1215-1217), swapBasis trades two basis
// vectors (scheme_z2.cu:864-914,1302-1313; scheme_integer.cu:791-841,1219-1233).
// One warp per walk: lanes transform terms, draws are replicated in every lane.
// Also the ring access shared with the resize operators (resize.cu).
#pragma once
#include "gf2.cuh"
#include "walk_z2.cuh"
#include "walk_zt.cuh"

namespace fg {

// A coefficient vector: Z2 factor bits in v (s = 0); ZT values in v, signs in s
// (a negative entry's sign bit moves with its value bit).
struct Vec {
    uint64_t v, s;
};

// Ring access for the two walkers: word (c, t) of the walk in shared memory.
template <class Z> struct RingOps;
template <class R, int S> struct RingOps<Z2Walk<R, S>> {
    using Z = Z2Walk<R, S>;
    __device__ static Vec get(const Z &z, int c, int t) { return Vec{z.x[c * z.cap + t], 0}; }
    __device__ static void put(Z &z, int c, int t, Vec w) { z.x[c * z.cap + t] = w.v; }
    __device__ static bool fixSigns(Z &) { return false; }
    __device__ static void stash(const Z &z, uint64_t *ownV, uint64_t *) {
        for (int q = lane_id(); q < 3 * z.cap; q += 32) ownV[q] = z.x[q];
    }
};
template <class R, int S> struct RingOps<ZTWalk<R, S>> {
    using Z = ZTWalk<R, S>;
    __device__ static Vec get(const Z &z, int c, int t) { return Vec{z.xv[c * z.cap + t], z.xs[c * z.cap + t]}; }
    __device__ static void put(Z &z, int c, int t, Vec w) {
        const int q = c * z.cap + t;
        z.xv[q] = w.v;
        z.xs[q] = w.s & w.v;
        z.xo[q] = 1;
    }
    __device__ static bool fixSigns(Z &z) { return z.fixSigns(); }
    __device__ static void stash(const Z &z, uint64_t *ownV, uint64_t *ownS) {
        for (int q = lane_id(); q < 3 * z.cap; q += 32) { ownV[q] = z.xv[q]; ownS[q] = z.xs[q]; }
    }
};

// The reference's ternary sandwiching is empty (only its gate draw is taken).
// Opt-in (WalkParams::zt_sandwich, no reference counterpart): conjugation by
// random signed permutation matrices, which keeps every coefficient in
// {-1, 0, 1}; entry (i, j) of u X v^-1 is sign_u(i) sign_v(j) X(p_u(i), p_v(j)).
template <class R>
__device__ void signed_permutation(int n, int *p, uint32_t &signs, R &r) {
    for (int i = 0; i < n; i++) p[i] = i;
    for (int i = n - 1; i > 0; i--) {  // randomPermutation, random.cuh:9-22
        const int j = (int)r.below((uint32_t)(i + 1));
        const int t = p[i]; p[i] = p[j]; p[j] = t;
    }
    signs = r.raw() & (n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u));
}

__device__ __forceinline__ void conj_signed(uint64_t xv, uint64_t xs, const int *pl, uint32_t sl, const int *pr,
                                            uint32_t sr, int n1, int n2, uint64_t &v, uint64_t &sg) {
    v = 0;
    sg = 0;
    for (int i = 0; i < n1; i++)
        for (int j = 0; j < n2; j++) {
            const int src = pl[i] * n2 + pr[j], dst = i * n2 + j;
            if (!((xv >> src) & 1)) continue;
            v |= 1ull << dst;
            if ((((xs >> src) & 1) ^ ((sl >> i) & 1) ^ ((sr >> j) & 1)) != 0) sg |= 1ull << dst;
        }
}

template <class R, int S>
__device__ __noinline__ void sandwich_move(ZTWalk<R, S> &z) {
    if (!z.r.P->zt_sandwich || z.n0 > 16 || z.n1 > 16 || z.n2 > 16) return;
    int pu[16], pv[16], pw[16];
    uint32_t su, sv, sw;
    signed_permutation(z.n0, pu, su, z.r);
    signed_permutation(z.n1, pv, sv, z.r);
    signed_permutation(z.n2, pw, sw, z.r);
    __syncwarp();
    for (int t = lane_id(); t < z.m; t += 32) {
        uint64_t v, sg;
        conj_signed(z.xv[t], z.xs[t], pu, su, pv, sv, z.n0, z.n1, v, sg);
        z.xv[t] = v; z.xs[t] = sg; z.xo[t] = 1;
        conj_signed(z.xv[z.cap + t], z.xs[z.cap + t], pv, sv, pw, sw, z.n1, z.n2, v, sg);
        z.xv[z.cap + t] = v; z.xs[z.cap + t] = sg; z.xo[z.cap + t] = 1;
        conj_signed(z.xv[2 * z.cap + t], z.xs[2 * z.cap + t], pw, sw, pu, su, z.n2, z.n0, v, sg);
        z.xv[2 * z.cap + t] = v; z.xs[2 * z.cap + t] = sg; z.xo[2 * z.cap + t] = 1;
    }
    __syncwarp();
    z.fixSigns();
    z.rebuild();
}

template <class R, int S>
__device__ __noinline__ void sandwich_move(Z2Walk<R, S> &z) {
    // Matrices are sized for n <= 16 as in the reference (config.cuh:40, MAX_SANDWICHING_N).
    if (z.n0 > 16 || z.n1 > 16 || z.n2 > 16) return;
    uint32_t u[16], u1[16], v[16], v1[16], w[16], w1[16];
    if (!invertible_gf2(z.n0, u, u1, z.r, z.status) || !invertible_gf2(z.n1, v, v1, z.r, z.status) ||
        !invertible_gf2(z.n2, w, w1, z.r, z.status))
        return;
    __syncwarp();
    for (int t = lane_id(); t < z.m; t += 32) {
        uint64_t *x = z.x + t;
        x[0] = conj_gf2(x[0], u, v1, z.n0, z.n1);
        x[z.cap] = conj_gf2(x[z.cap], v, w1, z.n1, z.n2);
        x[2 * z.cap] = conj_gf2(x[2 * z.cap], w, u1, z.n2, z.n0);
    }
    __syncwarp();
    z.rebuild();
}

template <class Z>
__device__ __noinline__ void basis_move(Z &z) {
    using O = RingOps<Z>;
    const bool rowsMove = z.r.raw() % 2;
    int a, b;
    if (rowsMove) { a = (int)(z.r.raw() % (uint32_t)z.n0); b = (int)(z.r.raw() % (uint32_t)z.n0); }
    else { a = (int)(z.r.raw() % (uint32_t)z.n2); b = (int)(z.r.raw() % (uint32_t)z.n2); }
    auto perm = [&](int q) { return q == a ? b : (q == b ? a : q); };
    __syncwarp();
    for (int t = lane_id(); t < z.m; t += 32) {
        if (rowsMove) {  // rows of U and columns of W
            const Vec u0 = O::get(z, 0, t), w0 = O::get(z, 2, t);
            Vec u{0, 0}, w{0, 0};
            for (int i = 0; i < z.n0; i++)
                for (int j = 0; j < z.n1; j++) {
                    const int from = perm(i) * z.n1 + j, to = i * z.n1 + j;
                    u.v |= ((u0.v >> from) & 1ull) << to;
                    u.s |= ((u0.s >> from) & 1ull) << to;
                }
            for (int i = 0; i < z.n2; i++)
                for (int j = 0; j < z.n0; j++) {
                    const int from = i * z.n0 + perm(j), to = i * z.n0 + j;
                    w.v |= ((w0.v >> from) & 1ull) << to;
                    w.s |= ((w0.s >> from) & 1ull) << to;
                }
            O::put(z, 0, t, u);
            O::put(z, 2, t, w);
        } else {  // columns of V and rows of W
            const Vec v0 = O::get(z, 1, t), w0 = O::get(z, 2, t);
            Vec v{0, 0}, w{0, 0};
            for (int i = 0; i < z.n1; i++)
                for (int j = 0; j < z.n2; j++) {
                    const int from = i * z.n2 + perm(j), to = i * z.n2 + j;
                    v.v |= ((v0.v >> from) & 1ull) << to;
                    v.s |= ((v0.s >> from) & 1ull) << to;
                }
            for (int i = 0; i < z.n2; i++)
                for (int j = 0; j < z.n0; j++) {
                    const int from = perm(i) * z.n0 + j, to = i * z.n0 + j;
                    w.v |= ((w0.v >> from) & 1ull) << to;
                    w.s |= ((w0.s >> from) & 1ull) << to;
                }
            O::put(z, 1, t, v);
            O::put(z, 2, t, w);
        }
    }
    __syncwarp();
    if (O::fixSigns(z)) z.rebuild();  // ternary only; Z2 lists stay valid
}

}  // namespace fg
