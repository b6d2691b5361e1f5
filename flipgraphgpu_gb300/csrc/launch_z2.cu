// Z2 launch dispatch over the slot count S (terms per lane), 32*S >= cap.
#include "launch.h"

namespace fg {

template <int S> cudaError_t walk_z2_s(const DevBatch &, const WalkParams &, int, int, int, cudaStream_t);
template <int S> cudaError_t minimize_z2_s(const DevBatch &, const WalkParams &, int, int, int, int32_t *, cudaStream_t);
template <int S> cudaError_t rebuild_z2_s(const DevBatch &, int, int, cudaStream_t);
template <int S> int occupancy_z2_s(int, int, int);

int slots_for_cap(int cap) {
    if (cap <= 32) return 1;
    if (cap <= 64) return 2;
    if (cap <= 128) return 4;
    if (cap <= 352) return 11;
    return 0;
}

#define FG_DISPATCH_S(CAP, EXPR, FAIL)                      \
    switch (slots_for_cap(CAP)) {                           \
        case 1: { constexpr int SS = 1; return EXPR; }      \
        case 2: { constexpr int SS = 2; return EXPR; }      \
        case 4: { constexpr int SS = 4; return EXPR; }      \
        case 11: { constexpr int SS = 11; return EXPR; }    \
        default: return FAIL;                               \
    }

cudaError_t launch_walk_z2(const DevBatch &B, const WalkParams &P, int rng, int wpb, int grid, cudaStream_t s) {
    FG_DISPATCH_S(B.cap, walk_z2_s<SS>(B, P, rng, wpb, grid, s), cudaErrorInvalidValue)
}

cudaError_t launch_minimize_z2(const DevBatch &B, const WalkParams &P, int rng, int wpb, int grid, int32_t *bestC,
                               cudaStream_t s) {
    FG_DISPATCH_S(B.cap, minimize_z2_s<SS>(B, P, rng, wpb, grid, bestC, s), cudaErrorInvalidValue)
}

cudaError_t launch_rebuild_z2(const DevBatch &B, int wpb, int grid, cudaStream_t s) {
    FG_DISPATCH_S(B.cap, rebuild_z2_s<SS>(B, wpb, grid, s), cudaErrorInvalidValue)
}

int occupancy_walk_z2(int cap, int rng, int wpb) { FG_DISPATCH_S(cap, occupancy_z2_s<SS>(cap, rng, wpb), 0) }

}  // namespace fg
