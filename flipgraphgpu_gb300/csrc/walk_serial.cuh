// Rare structural edits of a compactly stored fast-mode Z2 walk (word (c, t) =
// factor | partner count << HS at s[c * cap + t]), run on one thread through
// SimtZ2<W, 0> on the same words while the other lanes of the walk wait: the
// group kernel (walk_group.cuh) hands its walk state and stream position over
// and takes them back, so both consume the same Philox word sequence.
#pragma once
#include "fg_device.cuh"
#include "walk_simt.cuh"

namespace fg {

// Walk state handed to and back from the serial edits.
struct SerialCtx {
    int n0, n1, n2, cap, m, P0, P1, P2, status, result;
    uint32_t k0, k1, walk;
    unsigned long long count;
    const WalkParams *P;
};

// One structural edit of a compact walk, by SimtZ2<W, 0> on the calling
// thread with the walk's stream at x.count; op codes as GroupFast::OP_*.
template <class W>
__device__ __noinline__ void serial_op(W *s, SerialCtx &x, int op, int a0, int a1, int a2, int a3) {
    ThreadPhilox tp;
    tp.k0 = x.k0; tp.k1 = x.k1; tp.walk = x.walk; tp.count = x.count; tp.blk = -1; tp.P = x.P;
    SimtZ2<W, 0> z(tp);
    z.s = s; z.cap = x.cap; z.ld = x.cap;
    z.n0 = x.n0; z.n1 = x.n1; z.n2 = x.n2;
    z.nn0 = x.n0 * x.n1; z.nn1 = x.n1 * x.n2; z.nn2 = x.n2 * x.n0; z.full = x.n0 * x.n1 * x.n2;
    z.m = x.m; z.P0 = x.P0; z.P1 = x.P1; z.P2 = x.P2; z.status = x.status;
    int res = 0;
    switch (op) {
        case 0: {  // a flip (j = a0, a = a1, k = a2, b = a3) that zeroes a word
            const W newA = z.F(a0, a1) ^ z.F(a0, a3), newB = z.F(a2, a3) ^ z.F(a2, a1);
            z.setWord(a0, a1, newA);
            z.setWord(a2, a3, newB);
            z.removeZeroes();
            break;
        }
        case 1: z.reduce(a0, a1, a2); break;
        case 2: res = z.tryExpand(a0); break;
        case 3: res = z.tryPlus(); break;
        default: res = z.tryReduce(); break;
    }
    x.m = z.m; x.P0 = z.P0; x.P1 = z.P1; x.P2 = z.P2; x.status = z.status;
    x.count = tp.count; x.result = res;
}

// A rare move of a compact walk, as serial_op: move 0 sandwiching, 1 a basis change, 2 the
// Gauss reduction (x.result: it reduced); kept apart so that their matrices and index
// arrays do not enlarge serial_op's frame.
template <class W>
__device__ __noinline__ void serial_move(W *s, SerialCtx &x, int move) {
    ThreadPhilox tp;
    tp.k0 = x.k0; tp.k1 = x.k1; tp.walk = x.walk; tp.count = x.count; tp.blk = -1; tp.P = x.P;
    SimtZ2<W, 0> z(tp);
    z.s = s; z.cap = x.cap; z.ld = x.cap;
    z.n0 = x.n0; z.n1 = x.n1; z.n2 = x.n2;
    z.nn0 = x.n0 * x.n1; z.nn1 = x.n1 * x.n2; z.nn2 = x.n2 * x.n0; z.full = x.n0 * x.n1 * x.n2;
    z.m = x.m; z.P0 = x.P0; z.P1 = x.P1; z.P2 = x.P2; z.status = x.status;
    int res = 0;
    if (move == 0) z.sandwich();
    else if (move == 1) z.swapBasis();
    else res = z.tryReduceGauss();
    x.m = z.m; x.P0 = z.P0; x.P1 = z.P1; x.P2 = z.P2; x.status = z.status;
    x.count = tp.count; x.result = res;
}

}  // namespace fg
