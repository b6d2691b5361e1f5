// GF(2) matrices of the sandwiching move (scheme_z2.cu:444-529): a random
// invertible matrix with its inverse, and the conjugation of one factor.
// Shared by the warp-per-walk list kernels and the fast-mode walkers.
#pragma once
#include "fg_device.cuh"

namespace fg {

// Random invertible n x n GF(2) matrix (row i = low n bits of one draw, entry (i, j)
// = bit j) and its inverse by Gauss-Jordan on [M | I]; redrawn until invertible.
template <class R>
__device__ bool invertible_gf2(int n, uint32_t *m, uint32_t *inv, R &r, int &status) {
    const uint32_t low = n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u);
    for (int guard = 0, cap = retry_cap_of(r.P); guard <= cap; guard++) {
        uint64_t aug[16];
        for (int i = 0; i < n; i++) {
            m[i] = r.raw() & low;
            aug[i] = (uint64_t)m[i] | (1ull << (n + i));
        }
        bool ok = true;
        for (int col = 0; col < n && ok; col++) {
            int piv = -1;
            for (int row = col; row < n; row++)
                if ((aug[row] >> col) & 1) { piv = row; break; }
            if (piv < 0) { ok = false; break; }
            const uint64_t t = aug[col]; aug[col] = aug[piv]; aug[piv] = t;
            for (int row = 0; row < n; row++)
                if (row != col && ((aug[row] >> col) & 1)) aug[row] ^= aug[col];
        }
        if (!ok) continue;
        for (int i = 0; i < n; i++) inv[i] = (uint32_t)(aug[i] >> n) & low;
        return true;
    }
    status |= ST_RETRY;
    return false;
}

// left (n1 x n1) * X (n1 x n2, entry (i, j) at bit i*n2 + j) * right (n2 x n2) over GF(2).
__device__ __forceinline__ uint64_t conj_gf2(uint64_t x, const uint32_t *left, const uint32_t *right, int n1, int n2) {
    const uint64_t rowMask = n2 >= 64 ? ~0ull : ((1ull << n2) - 1);
    uint64_t out = 0;
    for (int i = 0; i < n1; i++) {
        uint64_t r1 = 0;
        for (int k = 0; k < n1; k++)
            if ((left[i] >> k) & 1) r1 ^= (x >> (k * n2)) & rowMask;
        uint64_t r2 = 0;
        for (int k = 0; k < n2; k++)
            if ((r1 >> k) & 1) r2 ^= right[k];
        out |= (r2 & rowMask) << (i * n2);
    }
    return out;
}

}  // namespace fg
