// Internal launch interface between the C-ABI (capi.cu) and the kernel
// translation units.  Not part of the public ABI.
#pragma once
#include <string>
#include <cuda_runtime.h>
#include "fg_device.cuh"

namespace fg {

enum { RNG_XORWOW = 0, RNG_PHILOX = 1 };

// Message of the last failing C-ABI call on this thread (fg_last_error).
std::string &last_error();

// Smallest supported slots-per-lane S with 32*S >= cap (0 when cap is too large).
int slots_for_cap(int cap);

// Warp-per-walk kernels (list modes); ring 0 = Z2, 1 = ZT.
cudaError_t launch_walk(int ring, const DevBatch &B, const WalkParams &P, int rng, int wpb, int grid, cudaStream_t s);
cudaError_t launch_minimize(int ring, const DevBatch &B, const WalkParams &P, int rng, int wpb, int grid,
                            int32_t *bestC, cudaStream_t s);
cudaError_t launch_rebuild(int ring, const DevBatch &B, int wpb, int grid, cudaStream_t s);
// Max resident blocks per SM of the walk kernel for this configuration.
int occupancy_walk(int ring, int cap, int rng, int wpb);

// Fast mode: thread-per-walk kernel over walks [first, first + count), `scap`
// factor slots per walk in shared memory; wide = 64-bit words (nn > 24).
cudaError_t launch_walk_simt(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int wide,
                             int wpb, int sms, cudaStream_t s);
// List modes (resize, sandwiching, basis and Gauss moves off): thread-per-walk walk over
// walks [first, first + count) with the reference's FlipSet lists; ring 0 = Z2, 1 = ZT
// (factors of at most 16 entries); rng RNG_XORWOW (bit-exact) or RNG_PHILOX.  `scratch`
// holds simt_list_scratch_bytes(ring, S) bytes (16-byte aligned); scap <= 256; nnmax = the
// segment's largest factor size (Z2 factor words of 16, 32 or 64 bits follow from it).
cudaError_t launch_walk_simt_list(int ring, const DevBatch &B, const WalkParams &P, int rng, int first, int count,
                                  int scap, int nnmax, int wpb, int sms, void *scratch, cudaStream_t s);
size_t simt_list_smem_per_warp(int ring, int scap, int nnmax);
size_t simt_list_scratch_bytes(int ring, int walks);
// Fills the scratch's constant part (the remainder table the ZT draws use); once, after allocation.
cudaError_t simt_list_init_scratch(int ring, int walks, void *scratch, cudaStream_t s);
// Fast mode complexity minimizer (minimizeKernel), one thread per walk; bestC[w] is the
// walk's best complexity so far, lowered in place.
cudaError_t launch_minimize_simt(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int wide,
                                 int wpb, int sms, int32_t *bestC, cudaStream_t s);
// The same minimizer, one warp per walk (for few walks or large schemes).
cudaError_t launch_minimize_group(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int wide,
                                  int sms, int32_t *bestC, cudaStream_t s);
// Resize meta-operators (one warp per walk, Z2, cap 352) and the best-rank table's copies.
// keepLists = 0 (fast mode): the walks' list sizes are left at zero.
cudaError_t launch_resize(int ring, const DevBatch &B, const WalkParams &P, int rng, double p, int wpb, int grid,
                          int keepLists, cudaStream_t s);
cudaError_t launch_copy_best(const DevBatch &B, const int32_t *walks, int count, const int32_t *bestRank, cudaStream_t s);
// Fast mode, `lanes` (4, 8, 16 or 32; 0 = by slot count) lanes per walk (same semantics as
// launch_walk_simt); 32 lanes is the one-warp-per-walk kernel.
cudaError_t launch_walk_group(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int wide,
                              int lanes, int sms, cudaStream_t s);
// Bounded-integer (ZB, |c| <= 2) fast-mode walk, one warp per walk, and its exact integer check.
cudaError_t launch_walk_zb(const DevBatch &B, const WalkParams &P, int first, int count, int scap, int sms,
                           cudaStream_t s);
cudaError_t launch_verify_zb(const DevBatch &B, int best, uint8_t *out, cudaStream_t s);
// Additions reducer, --max-flips: schemes [1, schemes) of coef ([schemes][3][m][64], ternary)
// become scheme 0 after up to maxFlips ZT flips drawn from states[s]; ranks, pairs (largest
// pair-occurrence count of a component) and status are written for those schemes.
cudaError_t launch_flip_schemes(int schemes, int n1, int n2, int n3, int m, int maxFlips, int8_t *coef,
                                curandStateXORWOW_t *states, int32_t *ranks, int32_t *pairs, int32_t *status, int sms,
                                cudaStream_t st);

}  // namespace fg
