// Warp-per-walk launch dispatch over ring and slot count S (terms per lane, 32*S >= cap).
#include "launch.h"

namespace fg {

template <int RING, int S> cudaError_t walk_s(const DevBatch &, const WalkParams &, int, int, int, cudaStream_t);
template <int RING, int S>
cudaError_t minimize_s(const DevBatch &, const WalkParams &, int, int, int, int32_t *, cudaStream_t);
template <int RING, int S> cudaError_t rebuild_s(const DevBatch &, int, int, cudaStream_t);
template <int RING, int S> int occupancy_s(int, int, int);

int slots_for_cap(int cap) {
    if (cap <= 32) return 1;
    if (cap <= 64) return 2;
    if (cap <= 128) return 4;
    if (cap <= 352) return 11;
    return 0;
}

#define FG_DISPATCH(RING, CAP, EXPR, FAIL)                                        \
    switch (slots_for_cap(CAP) | ((RING) << 8)) {                                 \
        case 1: { constexpr int RR = 0, SS = 1; return EXPR; }                    \
        case 2: { constexpr int RR = 0, SS = 2; return EXPR; }                    \
        case 4: { constexpr int RR = 0, SS = 4; return EXPR; }                    \
        case 11: { constexpr int RR = 0, SS = 11; return EXPR; }                  \
        case 256 + 1: { constexpr int RR = 1, SS = 1; return EXPR; }              \
        case 256 + 2: { constexpr int RR = 1, SS = 2; return EXPR; }              \
        case 256 + 4: { constexpr int RR = 1, SS = 4; return EXPR; }              \
        case 256 + 11: { constexpr int RR = 1, SS = 11; return EXPR; }            \
        default: return FAIL;                                                     \
    }

cudaError_t launch_walk(int ring, const DevBatch &B, const WalkParams &P, int rng, int wpb, int grid, cudaStream_t s) {
    FG_DISPATCH(ring, B.cap, (walk_s<RR, SS>(B, P, rng, wpb, grid, s)), cudaErrorInvalidValue)
}

cudaError_t launch_minimize(int ring, const DevBatch &B, const WalkParams &P, int rng, int wpb, int grid,
                            int32_t *bestC, cudaStream_t s) {
    FG_DISPATCH(ring, B.cap, (minimize_s<RR, SS>(B, P, rng, wpb, grid, bestC, s)), cudaErrorInvalidValue)
}

cudaError_t launch_rebuild(int ring, const DevBatch &B, int wpb, int grid, cudaStream_t s) {
    FG_DISPATCH(ring, B.cap, (rebuild_s<RR, SS>(B, wpb, grid, s)), cudaErrorInvalidValue)
}

int occupancy_walk(int ring, int cap, int rng, int wpb) { FG_DISPATCH(ring, cap, (occupancy_s<RR, SS>(cap, rng, wpb)), 0) }

}  // namespace fg
