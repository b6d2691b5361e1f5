/* flipgraph.h -- C ABI of the GB300 flip-graph search library (libflipgraph.so).
 *
 * The reference (dronperminov/FlipGraphGPU) has no library API: its three
 * executables drive CUDA kernels directly from host classes.  This header is
 * the boundary those host classes cross in this project; each entry point
 * names the reference code it replaces.  Plain C types only: pointers and
 * sizes, no CUDA or C++ types.  Every call returns an fg_status; no call
 * exits the process (the reference's CUDA_CHECK does, utils.cuh:12-19).
 *
 * Ownership: the library owns all device memory of a handle; the caller
 * owns every host buffer passed in.  One handle must not be used from two
 * threads at once.
 */
#ifndef FLIPGRAPH_H
#define FLIPGRAPH_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    FG_OK = 0,
    FG_ERR_ARG = 1,       /* invalid argument (sizes, null pointers, unsupported combination) */
    FG_ERR_CUDA = 2,      /* a CUDA runtime call failed; fg_last_error() has the message */
    FG_ERR_CAPACITY = 3,  /* a scheme does not fit the handle's slot / list capacity */
    FG_ERR_STATE = 4,     /* call order violated (e.g. run before init) */
    FG_ERR_WALK = 5       /* a walk hit a retry bound or overflow; see the status array */
} fg_status;

/* FG_RING_ZB: integer coefficients bounded by |c| <= 2, FG_MODE_FAST only; no
 * reference counterpart (the reference's integer ring is ZT, {-1, 0, 1}). */
typedef enum { FG_RING_Z2 = 0, FG_RING_ZT = 1, FG_RING_ZB = 2 } fg_ring;

/* Walk mode.
 * FG_MODE_REFERENCE: the reference's stream -- cuRAND XORWOW with
 *   curand_init(seed, walk_index, 0) per walk (flip_graph.cu:445-451) -- drawn
 *   at exactly the reference's draw sites over the reference's FlipSet lists,
 *   so trajectories match the reference bit for bit.  One warp per walk.
 * FG_MODE_PHILOX_LISTS: the same list semantics with the Philox4x32-10 stream
 *   (multiply-high ranges, integer gate thresholds).  One warp per walk.
 * FG_MODE_FAST: Philox stream, implicit pair enumeration (no lists: an ordered
 *   equal-factor pair is drawn uniformly in canonical order -- the reference's
 *   proposal distribution), one thread or one warp per walk.  The throughput mode.
 * FG_MODE_LEARNED: the fast mode's walk stepped in lockstep over the batch so
 *   that each step draws K candidate flips per walk, scores them with the
 *   learned network (fg_set_proposal) and samples one.  Without a network, or
 *   with K = 1, the proposal is the uniform one (K = 1 reproduces FG_MODE_FAST
 *   exactly).  Z2 only, factors of at most 21 entries.  No reference
 *   counterpart. */
typedef enum { FG_MODE_REFERENCE = 0, FG_MODE_PHILOX_LISTS = 1, FG_MODE_FAST = 2, FG_MODE_LEARNED = 3 } fg_mode;

/* Walk status bits (per walk). */
enum { FG_WALK_RETRY = 2, FG_WALK_OVERFLOW = 4, FG_WALK_INTERNAL = 8 /* fast mode: pair counts inconsistent */ };

/* Mirrors the options of the reference's flip_graph executable
 * (main_flip_graph.cu:10-25) that reach the walk kernel
 * (randomWalkKernel, flip_graph.cu:520). */
typedef struct {
    int32_t ring;             /* fg_ring */
    int32_t mode;             /* fg_mode */
    int32_t walks;            /* --schemes */
    int32_t cap;              /* factor slots per walk: >= max(initial rank, n1*n2*n3) */
    uint64_t seed;            /* --seed (nonzero; the CLI maps 0 to time(0) as the reference does) */
    int32_t iterations;       /* --max-iterations: walk steps per launch */
    int32_t plus_iterations;  /* --plus-iterations */
    double expand_p;          /* --expand-probability (per step: expand_p / iterations) */
    double reduce_p;          /* --reduce-probability (per step: reduce_p / iterations) */
    int32_t device;           /* CUDA device ordinal */
    int32_t walks_per_block;  /* 0 = library default */
    double resize_p;          /* --resize-probability: > 0 turns on the resize meta-operators
                                 (list modes on both rings, the fast mode on Z2; cap >= 350): each
                                 launch runs a random number of steps, then resizes walks and
                                 updates the best rank per size (flip_graph.cu:286-299,575-613,
                                 249-266); in the fast mode grown factors hold at most 56 entries */
    double sandwich_p;        /* --sandwiching-probability (list modes, Z2 fast mode; per step:
                                 sandwich_p / iterations): conjugate every term by random invertible
                                 GF(2) matrices and rebuild the lists (scheme_z2.cu:1277-1300; a no-op
                                 that still takes its gate draw on ZT, scheme_integer.cu:1215-1217) */
    double basis_p;           /* --basis-probability (list modes, Z2 fast mode; per step: basis_p / iterations):
                                 swap two basis vectors (scheme_z2.cu:1302-1313,
                                 scheme_integer.cu:1219-1233) */
    double gauss_p;           /* Z2, list and fast modes: per step with probability gauss_p / iterations, the
                                 Gauss (XOR) reduction SchemeZ2::tryReduceGauss (scheme_z2.cu:312-442,
                                 1156-1163), which the reference defines but its walk never calls;
                                 0 (default) takes no draw, keeping the reference's trajectories */
    int32_t zt_sandwich;      /* ZT: 1 = the sandwiching move conjugates by random signed permutation
                                 matrices (coefficients stay in {-1, 0, 1}); 0 (default) = the
                                 reference's empty ternary move (scheme_integer.cu:1215-1217) */
    int32_t retry_cap;        /* bound on the loops the reference leaves unbounded (tryPlus's pair
                                 rejection, scheme_z2.cu:1036-1039, scheme_integer.cu:984-987;
                                 trySplitExisted, scheme_integer.cu:1029-1033; while (tryReduce()),
                                 the invertible-matrix redraw): a walk that exceeds it stops with
                                 FG_WALK_RETRY in its status and fg_run returns FG_ERR_WALK.
                                 0 = the library default, 2^20 */
} fg_config;

/* Host-side walk records, structure of arrays over `walks` records with
 * `cap` factor slots each.  Factor arrays are [walks][3][cap]: for Z2 a
 * factor is a bitmask over the n_i*n_{i+1} matrix entries (bit r = entry r,
 * W stored transposed as in scheme_z2.cu:47-49); for ZT it is the
 * reference's Addition (values, signs, valid) split over fac / sgn / valid.
 * Lists are the three FlipSets of equal-factor pairs (flip_set.cu), sizes
 * [walks][3] and pairs [walks][3][500] packed (a << 16) | b, in the
 * reference's order.  Unused slots and list entries read as zero. */
typedef struct {
    int32_t *n;           /* [walks][3] */
    int32_t *m;           /* [walks] current rank */
    uint64_t *fac;        /* [walks][3][cap] */
    uint64_t *sgn;        /* ZT and ZB, else NULL */
    uint8_t *valid;       /* ZT only, else NULL */
    int32_t *list_size;   /* [walks][3] */
    uint32_t *list_pairs; /* [walks][3][500] */
    int32_t *flips;       /* [walks] flips since the last rank drop */
    int32_t *best_rank;   /* [walks] */
    int32_t *best_m;      /* [walks] */
    uint64_t *best_fac;   /* [walks][3][cap] */
    uint64_t *best_sgn;   /* ZT and ZB */
    uint8_t *best_valid;  /* ZT only */
    int64_t *rng_pos;     /* [walks] draws consumed since seeding */
    int32_t *status;      /* [walks] FG_WALK_* bits */
    int32_t *best_n;      /* [walks][3] sizes of the best scheme (resizing; NULL = n) */
    uint64_t *fac2;       /* ZB only: [walks][3][cap] entries with |c| = 2; for ZB, fac marks the
                             nonzero entries and sgn the negative ones (valid unused) */
    uint64_t *best_fac2;  /* ZB only */
} fg_records;

typedef struct {
    uint64_t flips;            /* accepted flips in the call, all walks */
    uint64_t verified_flips;   /* flips of walks whose scheme passed the exact Brent check */
    int32_t walks_valid;       /* walks whose current scheme verified */
    int32_t walks_failed;      /* walks with a nonzero status */
    int32_t min_rank;          /* lowest current rank */
    int32_t min_best_rank;     /* lowest best rank */
    float kernel_ms;           /* device time of the walk kernel(s), CUDA events */
    float verify_ms;           /* device time of the verification kernel */
} fg_stats;

#define FG_LIST_CAP 500   /* FlipSet capacity, config.cuh:14 */
#define FG_MAX_RANK 350   /* config.cuh:10 */

typedef struct fg_handle fg_handle;

/* Allocates device state for cfg->walks walks and seeds their streams
 * (replaces FlipGraph's constructor: cudaMallocManaged x5 and
 * initializeRandomStatesKernel, flip_graph.cu:4-188,445-451). */
fg_status fg_create(const fg_config *cfg, fg_handle **out);
fg_status fg_destroy(fg_handle *h);

/* Every walk := naive n1 x n2 x n3 scheme, best := current, best_rank :=
 * n1*n2*n3, flips := 0 (initializeNaiveKernel + initializeSchemesKernel,
 * flip_graph.cu:453-457,510-518). */
fg_status fg_init_naive(fg_handle *h, int n1, int n2, int n3);

/* Per-walk shapes: walk w := naive shapes[w][0] x shapes[w][1] x shapes[w][2]
 * scheme (the batched uneven search: many shapes in one launch).  The
 * reference can only do this through --input-path with one scheme per shape
 * replicated idx % count (flip_graph.cu:459-470). */
fg_status fg_init_naive_shapes(fg_handle *h, const int32_t *shapes);

/* Copies host records into the handle (FlipGraph::initializeFromFile +
 * initializeCopyKernel, flip_graph.cu:201-224,459-470, after the host has
 * parsed and replicated the schemes).  rng_pos is not read: streams keep
 * their position.  The fast and learned modes keep no lists: list_size and
 * list_pairs may be NULL there and are not copied.  Before anything is
 * copied every walk is checked: sizes positive with n1*n2, n2*n3, n3*n1 <= 64
 * (best_n too when resizing), m and best_m in [0, cap], and in the list modes
 * list sizes in [0, 500] with every pair two distinct slots below m.  A
 * failing record returns FG_ERR_ARG / FG_ERR_CAPACITY naming the walk, and
 * the handle keeps its state. */
fg_status fg_set_records(fg_handle *h, const fg_records *rec);

/* Copies the handle's records to host buffers (the reference reads managed
 * memory in place, flip_graph.cu:253-265,303-380).  NULL fields are skipped;
 * in the fast and learned modes list_pairs, when given, reads as zero. */
fg_status fg_get_records(fg_handle *h, fg_records *rec);

/* Runs `launches` launches of the walk (randomWalkKernel, flip_graph.cu:520-573,
 * each move gated by its probability in the config) on every walk, then
 * verifies every walk's scheme exactly (flip_graph.cu:571-572).  Stats
 * cover this call. */
fg_status fg_run(fg_handle *h, int launches, fg_stats *stats);

/* One launch of the complexity minimizer's flip walk (minimizeKernel,
 * complexity_minimizer.cu:190-214): checkReduce=false flips; best_* records
 * receive the lowest-complexity scheme seen.  best_complexity [walks] is
 * read (the running bests) and written.  List modes: the reference's walk
 * (one warp per walk); Z2 fast mode: the fast walk's stream and pair order,
 * one thread per walk. */
fg_status fg_minimize(fg_handle *h, int32_t *best_complexity);

/* Exact Brent-equation check of every walk's current (best=0) or best
 * (best=1) scheme; out [walks] = 1 when valid (Scheme::validate,
 * scheme_z2.cu:20-29, scheme_integer.cu:20-38). */
fg_status fg_validate(fg_handle *h, int best, uint8_t *out);

/* Records `draws` cuRAND XORWOW outputs of walks [first_walk, first_walk+count)
 * from curand_init(seed, walk, 0): out_draws[w][q] = q-th curand() value,
 * out_uniforms[w][q] = q-th curand_uniform() value.  Test support: lets a
 * CPU checker replay the reference's stream. */
fg_status fg_xorwow_tape(uint64_t seed, int first_walk, int count, int draws, int device,
                         uint32_t *out_draws, float *out_uniforms);

/* Philox4x32-10 blocks computed on the device (test support):
 * out[q] = Philox(ctr[q], key) for q < count, ctr [count][4], out [count][4]. */
fg_status fg_philox_blocks(const uint32_t *ctr, int count, uint32_t key0, uint32_t key1, int device,
                           uint32_t *out);

/* Per-walk counters without copying records (any pointer may be NULL), each
 * [walks]: current rank m, best rank, rank of the stored best scheme, flips
 * since the last rank drop, flips accepted in the last launch, and the result
 * of the last verification. */
fg_status fg_get_counters(fg_handle *h, int32_t *m, int32_t *best_rank, int32_t *best_m, int32_t *flips_since_drop,
                          uint64_t *flips_last_launch, uint8_t *valid);

/* One walk's current (best=0) or best (best=1) scheme: n [3], m, factors
 * [3][cap] (fac; sgn and valid for ZT, else may be NULL). */
fg_status fg_get_scheme(fg_handle *h, int walk, int best, int32_t *n, int32_t *m, uint64_t *fac, uint64_t *sgn,
                        uint8_t *valid);
/* ZB walks: as fg_get_scheme with the sign-magnitude masks (fac nonzero, sgn
 * negative, fac2 |c| = 2).  No reference counterpart. */
fg_status fg_get_scheme_zb(fg_handle *h, int walk, int best, int32_t *n, int32_t *m, uint64_t *fac, uint64_t *sgn,
                           uint64_t *fac2);

/* Fast mode runs each shape segment either one thread per walk or one warp
 * per walk; both kernels give identical results, the choice only sets speed.
 * -1 (the default) chooses per segment from its slot count and walk count;
 * n >= 0 forces one thread per walk for segments of at most n slots and one
 * warp per walk above (0 = always warp, a large n = always thread). */
fg_status fg_set_fast_split(fg_handle *h, int simt_max_cap);

/* Resizing (resize_p > 0): fg_run performs, per launch, the walk launch, the
 * resize step and the per-size best-rank update.  A caller that interleaves
 * its own reporting (as the flip_graph executable mirrors FlipGraph::run,
 * flip_graph.cu:286-299) drives the steps itself instead:
 *   fg_run_walks      walk launches only (random step counts, verification);
 *   fg_resize         the resize step of every walk (resizeKernel);
 *   fg_get_sizes      current and best-scheme sizes, [walks][3] each;
 *   fg_copy_to_best   the current schemes of `walks` become their best ones;
 *   fg_set_best_ranks every walk's best rank (the per-size table's value). */
fg_status fg_run_walks(fg_handle *h, int launches, fg_stats *stats);
fg_status fg_resize(fg_handle *h);
fg_status fg_get_sizes(fg_handle *h, int32_t *n, int32_t *best_n);
fg_status fg_copy_to_best(fg_handle *h, const int32_t *walks, int count);
fg_status fg_set_best_ranks(fg_handle *h, const int32_t *ranks);

/* List modes: rebuilds every walk's three FlipSet lists from its current
 * factors in the reference's initFlips order (scheme_z2.cu:166-175) -- for
 * records set with empty lists.  A no-op in the fast and learned modes. */
fg_status fg_rebuild_lists(fg_handle *h);

/* Fast mode kernel for every segment, overriding the automatic choice:
 * FG_FAST_THREAD (one thread per walk), FG_FAST_GROUP (`lanes` = 4, 8, 16 or 32
 * lanes per walk; 0 = by slot count, widened when the slots need it),
 * FG_FAST_WARP (one warp per walk); -1 restores the automatic choice.  All
 * three give identical results. */
enum { FG_FAST_THREAD = 0, FG_FAST_GROUP = 1, FG_FAST_WARP = 2 };
fg_status fg_set_fast_kernel(fg_handle *h, int kernel, int lanes);

/* List modes (reference stream and philox lists) on the Z2 ring: the kernel that
 * runs randomWalkKernel's loop (flip_graph.cu:520-573).  FG_LIST_WARP = one warp
 * per walk (every option, including resizing, sandwiching, basis changes and the
 * Gauss reduction); FG_LIST_THREAD = one thread per walk with the FlipSet lists
 * in a device scratch of 3,024 bytes per walk, allocated on first use (only
 * with sandwiching, basis changes and the Gauss reduction off, for slots up to
 * 256, and on ZT for factors of at most 31 entries, every input factor valid
 * above 16; with resizing the segments follow the sizes after every resize,
 * and a launch whose sizes do not fit takes the warp kernel);
 * -1 = automatic (thread per walk where it applies, resizing is off and the
 * batch has enough walks to fill the GPU).  Both give identical results.  FG_LIST_THREAD on a
 * configuration it does not cover returns FG_ERR_ARG. */
enum { FG_LIST_WARP = 0, FG_LIST_THREAD = 1 };
fg_status fg_set_list_kernel(fg_handle *h, int kernel);

/* Z2 fast mode: chooses each shape segment's kernel (thread per walk with 2, 4
 * or 8 warps per block; 8, 16 or 32 lanes per walk); list modes on the
 * thread-per-walk list kernel: each segment's warps per block (2, 4, 6 or 8,
 * kinds 0, lanes 0).  Both by timing the step's concurrent launches of all
 * segments for `iterations` steps: from the static choice, first one warps-per-
 * block value for every thread-per-walk segment, then each segment in turn; a
 * candidate replaces the configuration in place only when, timed in the order
 * in place, candidate, candidate, in place, it is more than 3 % faster.
 * Each trial starts from a snapshot of the records, which is put back
 * afterwards, so tuning changes no trajectory and no stream position.  The
 * choice holds until the records are replaced (fg_set_records, fg_init_naive*)
 * and yields to fg_set_fast_kernel.  kinds / lanes / warps (fg_segment_count
 * entries each, may be NULL) receive the choices (warps: warps per block of
 * the thread-per-walk kernel, else 0).  No reference counterpart. */
fg_status fg_autotune(fg_handle *h, int iterations, int32_t *kinds, int32_t *lanes, int32_t *warps);
int fg_segment_count(fg_handle *h);

/* Tensor-core (tcgen05) bf16 GEMM of the learned proposal's MLP, on host
 * buffers (test and support entry; no reference counterpart):
 *   D[M][N] = A[M][K] * B[N][K]^T, A and B bf16 bit patterns, row-major;
 *   mode 0: outF (fp32) = D, or outF += D when `accumulate`;
 *   mode 1: outH (bf16) = relu(D + bias) (bias [N] or NULL);
 *   mode 2: outH (bf16) = D where mask[M][N] > 0, else 0.
 * M % 128 == 0, K % 64 == 0, N % 64 == 0. */
fg_status fg_gemm_bf16(const uint16_t *A, const uint16_t *B, const float *bias, const uint16_t *mask, int M, int N,
                       int K, int mode, int accumulate, float *outF, uint16_t *outH, int device);

/* ------------------------------------------------------------------------
 * Learned flip proposal: the scoring network (no reference counterpart).
 * A candidate flip is described by 192 binary features packed in three
 * uint64 words (bit q of word w = feature 64w + q).  The network is
 * 192 -> 256 -> 256 -> 1 with ReLU, bf16 weights and activations, fp32
 * accumulation on the tensor cores; its score is the logit of "the rank drops
 * within the next 1000 flips".  Parameters are one fp32 block of
 * fg_mlp_param_count() floats: W1 [256][192], b1 [256], W2 [256][256],
 * b2 [256], w3 [256], b3.
 * ------------------------------------------------------------------------ */
typedef struct fg_mlp fg_mlp;

int fg_mlp_param_count(void);
/* He-uniform weights from `seed`, zero biases. */
fg_status fg_mlp_create(int device, uint64_t seed, fg_mlp **out);
fg_status fg_mlp_destroy(fg_mlp *m);
fg_status fg_mlp_set_params(fg_mlp *m, const float *params);
fg_status fg_mlp_get_params(fg_mlp *m, float *params);
/* Mean binary cross-entropy of one batch (labels 0/1) and its gradient
 * (same layout as the parameters); no update. */
fg_status fg_mlp_gradients(fg_mlp *m, const uint64_t *features, const float *labels, int rows, float *loss,
                           float *grads);
fg_status fg_mlp_score(fg_mlp *m, const uint64_t *features, int rows, float *scores);
/* Adam (lr, betas 0.9/0.999) over shuffled mini-batches (`batch` a multiple
 * of 128) for `epochs` passes; *last_loss = mean loss of the last pass. */
fg_status fg_mlp_train(fg_mlp *m, const uint64_t *features, const float *labels, int64_t n, int batch, int epochs,
                       float lr, uint64_t seed, float *last_loss);

/* FG_MODE_LEARNED: proposal of the following launches.  `mlp` NULL = uniform
 * choice among the candidates; candidates in [1, 16]; the sampling
 * distribution is softmax(score / temperature), replaced by a uniform choice
 * when its entropy (nats) is below min_entropy.  The network is borrowed
 * (not owned) and must outlive its use. */
fg_status fg_set_proposal(fg_handle *h, fg_mlp *mlp, int candidates, float temperature, float min_entropy);

/* FG_MODE_LEARNED with one candidate: runs `launches` launches of plain
 * (uniform-proposal) walks and logs every `every`-th accepted flip of each
 * walk as a training record -- its 192 features and label 1 if the walk's
 * rank dropped at that flip or within the next `horizon` accepted flips, else
 * 0.  Records whose outcome the run did not see are dropped.  At most
 * `capacity` records are logged; *count receives how many were written to
 * features [count][3] and labels [count]. */
fg_status fg_collect_records(fg_handle *h, int every, int horizon, int launches, int64_t capacity, uint64_t *features,
                             float *labels, int64_t *count);

/* Page-locked host buffers for fast record transfers (cudaHostAlloc). */
fg_status fg_host_alloc(uint64_t bytes, void **out);
fg_status fg_host_free(void *p);

/* ------------------------------------------------------------------------
 * Additions reducer (greedy / randomised common-subexpression elimination),
 * the reference's SchemeAdditionsReducer (scheme_additions_reducer.cu) with
 * runReducersKernel (scheme_additions_reducer.cu:494-540) on the GPU.
 * Reducer r uses cuRAND XORWOW seeded curand_init(seed, r, 0)
 * (scheme_additions_reducer.cu:445); its stream persists across runs.
 * ------------------------------------------------------------------------ */
typedef struct {
    int32_t count;    /* --count: parallel reducers */
    int32_t schemes;  /* --schemes-count: reducer r reduces scheme r % schemes */
    uint64_t seed;    /* --seed */
    int32_t device;
    int32_t threads;  /* threads per reducer block: 0 = 128; wider helps when few reducers (one
                         scheme, large pair tables) leave the SMs half idle, results unchanged */
} fg_reducer_config;

typedef struct fg_reducer fg_reducer;

/* coef [schemes][3][m][64] int8 in {-1,0,1}: row t of U (nn0 entries), of V
 * (nn1), of W (nn2 entries, W stored transposed as in the scheme files). */
fg_status fg_reducer_create(const fg_reducer_config *cfg, int n1, int n2, int n3, int m, const int8_t *coef,
                            fg_reducer **out);

/* One runReducersKernel launch.  best_fresh [3] and best_vars [3][500][2] are
 * the incumbent's fresh variables per component (partial initialisation);
 * independent = 1 when --max-flips is 0 (scheme_additions_reducer.cu:604).
 * out_counts [count][13] = per component (U, V, W) four ints: additions, fresh
 * variables, naive additions, selection mode; then the number of draws the
 * reducer consumed in this run.  out_scale [count][3]; out_vars [count][3][500][2]
 * the fresh variables (pairs of signed variable ids; zero past each
 * component's fresh count).  Either of the last two may be NULL. */
fg_status fg_reducer_run(fg_reducer *h, int independent, const int32_t *best_fresh, const int32_t *best_vars,
                         int32_t *out_counts, float *out_scale, int32_t *out_vars);

/* The flip pass of --max-flips > 0 (flipSchemesKernel, scheme_additions_reducer.cu:
 * 448-460, run before every reduction after the first, reduceIteration
 * scheme_additions_reducer.cu:172-176): each scheme s in [1, schemes) becomes
 * scheme 0 after curand() % (max_flips + 1) ternary flips (SchemeInteger::tryFlip
 * with reductions, scheme_integer.cu:907-975; the first flip that finds no pair
 * ends it), drawn from reducer s's stream, which the next fg_reducer_run
 * continues.  A flip that reduces leaves scheme s with a lower rank; the
 * reducers then use it (fewer U and V expressions, fewer W variables).  Needs
 * schemes <= count and scheme 0 ternary.  ranks_out [schemes] and coef_out
 * [schemes][3][m][64] (rows past a scheme's rank zero) may be NULL.  A scheme
 * whose flips stopped at a retry bound returns FG_ERR_WALK after the pass. */
fg_status fg_reducer_flip(fg_reducer *h, int max_flips, int32_t *ranks_out, int8_t *coef_out);
fg_status fg_reducer_destroy(fg_reducer *h);

/* One reducer pass without any device allocation: the same result as
 * fg_reducer_create + one fg_reducer_run (out_vars omitted) +
 * fg_reducer_destroy, with every device buffer (coefficients, cuRAND states,
 * incumbent variables, outputs) placed in one static scratch array of 4 MiB
 * inside the library.  No counterpart in the reference, whose reducer always
 * allocates managed memory (scheme_additions_reducer.cu:4-29).  Inputs that
 * do not fit return FG_ERR_CAPACITY: count > 1024; schemes * 3 * m * 64
 * coefficient bytes plus the per-reducer buffers above 4 MiB; or pair tables
 * larger than one block's shared memory (dense schemes, e.g. 4x4x4 at rank 51
 * and up), which fg_reducer_create would move to allocated global memory.
 * The scratch array's device address is looked up on every call, so calls
 * may span a cudaDeviceReset.  All calls share the one scratch array: calls
 * that overlap in time race on it, so the caller serialises them. */
fg_status fg_reducer_run_noalloc(const fg_reducer_config *cfg, int n1, int n2, int n3, int m, const int8_t *coef,
                                 int independent, const int32_t *best_fresh, const int32_t *best_vars,
                                 int32_t *out_counts, float *out_scale);

/* Message of the last failing call on this thread ("" when none). */
const char *fg_last_error(void);

/* Library version string. */
const char *fg_version(void);

#ifdef __cplusplus
}
#endif
#endif
