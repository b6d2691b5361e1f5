/* CPU oracle for the flip-graph hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain C++ restatement of the reference's (dronperminov/FlipGraphGPU)
 * algorithms on the search path, used by tests/ and bench.py's CPU baseline
 * as the checker of the CUDA library.  The product never links it.
 *
 * Parity is pinned against the reference's own CUDA build: the fixtures in
 * tests/golden/ were produced by the reference kernels on a GB300
 * (tests/golden/make_golden.py) and the oracle must reproduce them byte for
 * byte from the recorded XORWOW draw tapes.
 *
 * Data exchange uses the canonical walk-record layout below (shared with the
 * CUDA library's C-ABI, include/flipgraph.h) so tests compare raw arrays.
 */
#ifndef FG_ORACLE_H
#define FG_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Draw source and pair enumeration.  FGO_RNG_TAPE replays recorded cuRAND
 * XORWOW outputs (both the curand() word and the curand_uniform() float of
 * every draw), which is the reference's stream, over the reference's FlipSet
 * lists; FGO_RNG_PHILOX is the library's Philox4x32-10 stream (keyed by the
 * seed, one counter stream per walk) over the same lists; FGO_RNG_FAST is the
 * Philox stream with implicit pair enumeration (no lists: an ordered equal
 * pair is drawn uniformly in canonical order), the library's fast mode. */
enum { FGO_RNG_TAPE = 0, FGO_RNG_PHILOX = 1, FGO_RNG_FAST = 2 };
enum { FGO_RING_Z2 = 0, FGO_RING_ZT = 1, FGO_RING_ZB = 2 /* integers, |c| <= 2 (fast mode only) */ };

typedef struct {
    int32_t ring;             /* FGO_RING_* */
    int32_t rng;              /* FGO_RNG_* */
    int32_t cap;              /* factor slots per walk record (>= every rank reached) */
    int32_t iterations;       /* walk steps per launch (randomWalkKernel's maxIterations) */
    int32_t plus_iterations;  /* flips without a rank drop before a plus transition */
    int32_t launches;         /* consecutive launches to emulate */
    double expand_p;          /* --expand-probability (divided by iterations per step) */
    double reduce_p;          /* --reduce-probability (divided by iterations per step) */
    uint64_t seed;            /* Philox key (FGO_RNG_PHILOX) */
    double resize_p;          /* --resize-probability; > 0: random iterations per launch, a resize
                                 step after every launch and the per-shape best-rank table
                                 (flip_graph.cu:236,286-299,249-277,575-613) */
    double sandwich_p;        /* --sandwiching-probability (Z2; the ternary move is empty) */
    double basis_p;           /* --basis-probability */
    double gauss_p;           /* Gauss (XOR) reduction per step, gauss_p / iterations (Z2; not in the
                                 reference's walk, whose tryReduceGauss is never called) */
    int32_t zt_sandwich;      /* ZT: 1 = sandwiching by random signed permutations (the reference's
                                 ternary sandwiching is empty); 0 = as the reference */
    int32_t retry_cap;        /* bound on the reference's unbounded retry loops; 0 = 2^20 */
} fgo_walk_cfg;

/* Structure-of-arrays batch of S walk records.  Factor arrays are [S][3][cap];
 * for ZT the ternary factor of slot (w,c,t) is (fac, sgn, valid) exactly as
 * the reference's Addition (values, signs, valid); for Z2 sgn/valid are NULL.
 * Lists are the reference's three FlipSets: sizes [S][3], pairs [S][3][500]
 * packed (a << 16) | b. */
typedef struct {
    int32_t *n;          /* [S][3] */
    int32_t *m;          /* [S] */
    uint64_t *fac;       /* [S][3][cap] */
    uint64_t *sgn;       /* ZT only */
    uint8_t *valid;      /* ZT only */
    int32_t *list_size;  /* [S][3] */
    uint32_t *list_pairs;/* [S][3][500] */
    int32_t *flips;      /* [S] flips since the last rank drop (flip_graph.cu:540-543) */
    int32_t *best_rank;  /* [S] */
    int32_t *best_m;     /* [S] */
    uint64_t *best_fac;  /* [S][3][cap] */
    uint64_t *best_sgn;  /* ZT only */
    uint8_t *best_valid; /* ZT only */
    int64_t *rng_pos;    /* [S] draws consumed so far (tape position / Philox word index) */
    int32_t *status;     /* [S] 0 ok; bit 1 tape exhausted; bit 2 capped retry loop; bit 4 slot overflow */
    int64_t *accepted;   /* [S] accepted flips, accumulated (may be NULL) */
    int32_t *best_n;     /* [S][3] sizes of the best scheme (resize; may be NULL = n) */
    uint64_t *fac2;      /* ZB only: [S][3][cap] |c| = 2 mask (fac = nonzero, sgn = negative) */
    uint64_t *best_fac2; /* ZB only */
} fgo_batch;

/* Tape: draws for walk w are tape_draws[tape_off[w] .. tape_off[w+1]). */
typedef struct {
    const uint32_t *draws;
    const float *uniforms;
    const int64_t *offsets;  /* [S+1] */
} fgo_tape;

/* Sets every walk to the naive n1 x n2 x n3 scheme (scheme_z2.cu:32-55), builds
 * its lists, and initialises best := current, best_rank := n1*n2*n3, flips := 0
 * (flip_graph.cu:453-457,510-518). */
int fgo_init_naive(const fgo_walk_cfg *cfg, int S, int n1, int n2, int n3, fgo_batch *b);

/* Runs cfg->launches launches of randomWalkKernel (flip_graph.cu:520-573) on
 * every walk, in place.  Returns the number of walks with a nonzero status. */
int fgo_walk(const fgo_walk_cfg *cfg, int S, fgo_batch *b, const fgo_tape *tape);

/* One call of SchemeZ2::tryReduceGauss (scheme_z2.cu:1156-1163; never called by the
 * reference's walk) on every Z2 record, exactly as the reference does it: zero
 * factors stay and the lists are not rebuilt.  found[w] = 1 when a combination
 * was folded (rank one less).  Returns -1 for the ternary ring. */
int fgo_reduce_gauss(const fgo_walk_cfg *cfg, int S, fgo_batch *b, const fgo_tape *tape, int32_t *found);

/* One launch of minimizeKernel (complexity_minimizer.cu:190-214): flips with
 * checkReduce=false; best_* receives the lowest-complexity scheme seen and
 * best_complexity[w] its complexity.  Lists are rebuilt from the factors. */
int fgo_minimize(const fgo_walk_cfg *cfg, int S, fgo_batch *b, const fgo_tape *tape,
                 int32_t *best_complexity);

/* Exact integer Brent check of ZB records (coefficient = (fac ? (fac2 ? 2 : 1) : 0),
 * negative where sgn is set). */
int fgo_validate_zb(int S, int cap, const int32_t *n, const int32_t *m, const uint64_t *fac, const uint64_t *sgn,
                    const uint64_t *fac2, uint8_t *valid_out);

/* Exact Brent check (scheme_z2.cu:3-29 / scheme_integer.cu:3-38) of every
 * record; valid_out[w] = 1 when it reproduces the n1 x n2 x n3 tensor. */
int fgo_validate(int ring, int S, int cap, const int32_t *n, const int32_t *m, const uint64_t *fac,
                 const uint64_t *sgn, const uint8_t *valid, uint8_t *valid_out);

/* complexity = popcount(u,v,w) - 2m - nn2 (scheme_z2.cu:127-139). */
int fgo_complexity(int ring, int S, int cap, const int32_t *n, const int32_t *m, const uint64_t *fac,
                   int32_t *out);

/* Additions reducer, one runReducersKernel launch (scheme_additions_reducer.cu:494-540)
 * for reducers 0..count-1 over one scheme (coefficients in {-1,0,1}: coef[3][m][64]
 * as int8 rows u[t][0..nn0), v[t][0..nn1), w[t][0..nn2)).  Reducers start from the
 * naive expressions; `best` (may be NULL) is the incumbent used for partial
 * initialisation with `independent` semantics.  Outputs per reducer r:
 * out[r*9 + {0,1,2}] = U additions, U fresh vars, U naive additions; {3..5} V; {6..8} W.
 * modes[r*3 + {0,1,2}] = selection mode of U, V, W. */
typedef struct fgo_reducer_state fgo_reducer_state;
int fgo_reduce(int n1, int n2, int n3, int m, const int8_t *coef, int count, int independent,
               const fgo_tape *tape, int rng, uint64_t seed, int32_t *out, int32_t *modes,
               int64_t *consumed, const fgo_reducer_state *best, fgo_reducer_state **best_out);
void fgo_reducer_state_free(fgo_reducer_state *s);
/* runReducersKernel over several schemes (--max-flips): reducer r reduces scheme
 * r % schemes of coef [schemes][3][m][64] at rank ranks[s] (NULL: m), draws from
 * tape walk r.  vars_out (may be NULL): [count][3][500][2] fresh variables of
 * every reducer (the "together" incumbent is one reducer's three lists). */
int fgo_reduce_schemes(int n1, int n2, int n3, int m, const int8_t *coef, const int32_t *ranks, int schemes,
                       int count, int independent, const fgo_tape *tape, int32_t *out, int32_t *modes,
                       int64_t *consumed, const fgo_reducer_state *best, int32_t *vars_out);
/* flipSchemesKernel (scheme_additions_reducer.cu:448-460): scheme s in [1, schemes)
 * := scheme 0 (coef0 [3][m][64], lists by initFlips) after curand() % (max_flips + 1)
 * SchemeInteger::tryFlip calls with reductions, stopping at the first without a
 * flip; stream s is tape walk s.  coef_out [schemes][3][m][64] (scheme 0 copied,
 * rows past a rank zero), ranks_out [schemes], consumed [schemes] draws. */
int fgo_flip_schemes(int n1, int n2, int n3, int m, const int8_t *coef0, int schemes, int max_flips,
                     const fgo_tape *tape, int8_t *coef_out, int32_t *ranks_out, int64_t *consumed);
/* Incumbent from explicit fresh-variable lists: fresh [3], vars [3][500][2]. */
fgo_reducer_state *fgo_reducer_state_make(const int32_t *fresh, const int32_t *vars);

/* Selects whether the multiply-adds of the greedy-intersections score are
 * evaluated fused (as nvcc contracts them by default) or unfused. */
void fgo_set_fma(int fuse_float, int fuse_double);

/* Steps from the naive scheme to rank `target` of fast-mode Z2 walks under the uniform
 * proposal (greedy = 0) or an exact one-step lookahead that takes a rank-lowering flip
 * whenever one exists (greedy = 1); steps[w] = -1 when walk w did not get there within
 * max_steps.  Returns the number of such walks, -1 for an unsupported shape. */
int fgo_lookahead_ttr(int n1, int n2, int n3, int walks, int target, int64_t max_steps, int plus_iterations,
                      double expand_p, int iterations, uint64_t seed, int greedy, int64_t *steps);

/* Philox4x32-10 block function (Salmon et al., SC'11) for known-answer tests. */
void fgo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

#ifdef __cplusplus
}
#endif
#endif
