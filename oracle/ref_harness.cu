// Test infrastructure: drives the reference's own, unmodified CUDA kernels and
// dumps their complete state so that golden fixtures can be cut from it.
//
// This file is compiled only against a staged copy of the reference sources
// (oracle/build_ref.sh) and only ever runs to GENERATE fixtures under
// tests/golden/.  Nothing in the product links or runs it.
//
// Commands
//   walk  N1 N2 N3 S ITERS PLUS_ITERS EXPAND_P REDUCE_P SEED LAUNCHES OUT
//       Follows FlipGraph's naive path (flip_graph.cu:185,229,192,236) with
//       --resize-probability 0 (so randomIterations=false, flip_graph.cu:530)
//       and sandwiching/basis probabilities 0.  After every launch of
//       randomWalkKernel (flip_graph.cu:520-573) the full per-walk state is
//       written.  After the last launch the XORWOW draw tape of every walk is
//       written, cut exactly at the number of draws the walk consumed (found
//       by stepping a fresh curand_init(seed, idx, 0) state until it equals
//       the walk's final state).
//   reduce IN COUNT SCHEMES_COUNT SEED OUT [MAX_FLIPS ITERATIONS]
//       Reads one scheme body (n1 n2 n3 m + U,V,W rows) with
//       checkValidity=false, runs initializeKernel and one runReducersKernel
//       (scheme_additions_reducer.cu:433-540) and writes per-reducer
//       additions / fresh-variable counts / modes plus the reducer tapes.
//       With MAX_FLIPS > 0, ITERATIONS iterations of reduceIteration
//       (scheme_additions_reducer.cu:172-182: flipSchemesKernel from the
//       second on, then runReducersKernel with independent=false), each
//       followed by the host's updateBestTogether (:296-339, the index vector
//       kept across iterations as the class keeps it); per iteration the
//       schemes' ranks, every reducer's counts and the chosen top reducer.
//
//   reduce_time IN COUNT SEED LAUNCHES [OUT]
//       Times runReducersKernel (independent, after initializeKernel) on COUNT
//       reducers over the scheme of IN with CUDA events; prints JSON with the
//       reducer runs per second and the addition totals' minimum and sum (the
//       benchmark's reference leg for the additions reducer).
//
//   minimize_time IN COUNT ITERATIONS SEED LAUNCHES [OUT]
//       The complexity minimizer's initializeKernel and LAUNCHES timed
//       minimizeKernel launches (complexity_minimizer.cu:173-214) on COUNT copies
//       of the scheme of IN; prints the mean launch time and the best complexity,
//       and writes every walk's best complexity to OUT (the benchmark's
//       reference leg for the minimizer).
//
//   gauss IN SEED OUT   (Z2 build)
//       Reads schemes in flip_graph's text layout (a count, then per scheme
//       "n1 n2 n3 m" and its rows; checkValidity=false), gives scheme k the
//       stream curand_init(SEED, k, 0) (initializeRandomStatesKernel) and
//       calls SchemeZ2::tryReduceGauss once per scheme (scheme_z2.cu:1156-1163,
//       a function the reference defines but never calls).  Writes the result
//       flag and the scheme after the call, then the draw tapes.
//
// Binary output: little-endian int32 / uint32 / uint64 / float records; the
// layout is documented in tests/golden/make_golden.py which parses it.

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "entities/complexity_minimizer.cuh"
#include "entities/flip_graph.cuh"
#include "entities/scheme_additions_reducer.cuh"

#define HCHECK(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) { \
    fprintf(stderr, "CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); exit(2); } } while (0)

static void put_i32(FILE *f, int32_t v) { fwrite(&v, 4, 1, f); }
static void put_u32(FILE *f, uint32_t v) { fwrite(&v, 4, 1, f); }
static void put_u64(FILE *f, uint64_t v) { fwrite(&v, 8, 1, f); }

#ifdef SCHEME_INTEGER
static const int kRingIsZT = 1;
static void put_factor(FILE *f, const Addition &a) { put_u64(f, a.values); put_u64(f, a.signs); put_i32(f, a.valid ? 1 : 0); }
#else
static const int kRingIsZT = 0;
static void put_factor(FILE *f, const T &a) { put_u64(f, (uint64_t)a); }
#endif

static void put_scheme(FILE *f, const Scheme &s, bool withFlips) {
    for (int i = 0; i < 3; i++) put_i32(f, s.n[i]);
    put_i32(f, s.m);
    for (int c = 0; c < 3; c++)
        for (int t = 0; t < s.m; t++) put_factor(f, s.uvw[c][t]);
    if (withFlips) {
        for (int c = 0; c < 3; c++) {
            put_i32(f, (int32_t)s.flips[c].size);
            for (size_t p = 0; p < s.flips[c].size; p++) put_u32(f, s.flips[c].pairs[p]);
        }
    }
}

// Steps a fresh XORWOW stream (curand_init(seed, idx, 0)) and records every
// draw as (curand() value, curand_uniform() value) until the stream equals the
// walk's final state or maxDraws is reached.  Both values come from cuRAND
// itself: one copy of the state is advanced with curand(), a second copy with
// curand_uniform(); both consume exactly one 32-bit output per call.
__global__ void tapeKernel(const curandState *finalStates, int count, int seed, int maxDraws,
                           uint32_t *draws, float *uniforms, int *consumed) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= count) return;
    curandState a, b;
    curand_init(seed, idx, 0, &a);
    b = a;
    const curandState &fin = finalStates[idx];
    int used = -1;
    for (int n = 0; n <= maxDraws; n++) {
        bool same = a.d == fin.d;
        for (int q = 0; q < 5; q++) same = same && a.v[q] == fin.v[q];
        if (same) { used = n; break; }
        if (n == maxDraws) break;
        draws[(size_t)idx * maxDraws + n] = curand(&a);
        uniforms[(size_t)idx * maxDraws + n] = curand_uniform(&b);
    }
    consumed[idx] = used;
}

static void write_tapes(FILE *f, const curandState *states, int count, int seed, int maxDraws) {
    curandState *dStates; uint32_t *dDraws; float *dUni; int *dUsed;
    HCHECK(cudaMalloc(&dStates, count * sizeof(curandState)));
    HCHECK(cudaMemcpy(dStates, states, count * sizeof(curandState), cudaMemcpyDefault));
    HCHECK(cudaMalloc(&dDraws, (size_t)count * maxDraws * 4));
    HCHECK(cudaMalloc(&dUni, (size_t)count * maxDraws * 4));
    HCHECK(cudaMalloc(&dUsed, count * 4));
    tapeKernel<<<(count + 63) / 64, 64>>>(dStates, count, seed, maxDraws, dDraws, dUni, dUsed);
    HCHECK(cudaGetLastError());
    HCHECK(cudaDeviceSynchronize());
    std::vector<uint32_t> draws((size_t)count * maxDraws);
    std::vector<float> uni((size_t)count * maxDraws);
    std::vector<int> used(count);
    HCHECK(cudaMemcpy(draws.data(), dDraws, draws.size() * 4, cudaMemcpyDeviceToHost));
    HCHECK(cudaMemcpy(uni.data(), dUni, uni.size() * 4, cudaMemcpyDeviceToHost));
    HCHECK(cudaMemcpy(used.data(), dUsed, count * 4, cudaMemcpyDeviceToHost));
    for (int w = 0; w < count; w++) {
        put_i32(f, used[w]);
        int n = used[w] < 0 ? 0 : used[w];
        fwrite(&draws[(size_t)w * maxDraws], 4, n, f);
        fwrite(&uni[(size_t)w * maxDraws], 4, n, f);
    }
    cudaFree(dStates); cudaFree(dDraws); cudaFree(dUni); cudaFree(dUsed);
}

// FlipGraph::updateRanks (flip_graph.cu:249-266) restated over the harness's
// managed arrays: per (sorted) size key the best rank; an improving walk's
// scheme is copied to its best slot; every walk gets its key's best rank.
static void update_ranks(std::unordered_map<std::string, int> &table, Scheme *schemes, Scheme *best, int *bestRanks,
                         int S) {
    std::vector<std::string> keys(S);
    for (int i = 0; i < S; i++) {
        keys[i] = getKey(schemes[i]);
        auto it = table.find(keys[i]);
        if (it == table.end() || schemes[i].m < it->second) {
            table[keys[i]] = schemes[i].m;
            schemes[i].copyTo(best[i]);
        }
    }
    for (int i = 0; i < S; i++) bestRanks[i] = table[keys[i]];
}

static int cmd_walk(int argc, char **argv) {
    if (argc < 13 || argc > 16) { fprintf(stderr, "walk: bad arguments\n"); return 1; }
    // optional arguments: --resize-probability (> 0 runs FlipGraph::run's resize loop),
    // --sandwiching-probability, --basis-probability
    const double resizeP = argc >= 14 ? atof(argv[13]) : 0.0;
    const double sandwichP = argc >= 15 ? atof(argv[14]) : 0.0;
    const double basisP = argc >= 16 ? atof(argv[15]) : 0.0;
    const bool moves = sandwichP > 0 || basisP > 0;
    int n1 = atoi(argv[2]), n2 = atoi(argv[3]), n3 = atoi(argv[4]);
    int S = atoi(argv[5]), iters = atoi(argv[6]), plusIters = atoi(argv[7]);
    double expandP = atof(argv[8]), reduceP = atof(argv[9]);
    int seed = atoi(argv[10]), launches = atoi(argv[11]);
    const char *out = argv[12];
    int blockSize = 32, numBlocks = (S + blockSize - 1) / blockSize;

    Scheme *schemes, *best; int *bestRanks, *flips; curandState *states;
    HCHECK(cudaMallocManaged(&schemes, S * sizeof(Scheme)));
    HCHECK(cudaMallocManaged(&best, S * sizeof(Scheme)));
    HCHECK(cudaMallocManaged(&bestRanks, S * sizeof(int)));
    HCHECK(cudaMallocManaged(&flips, S * sizeof(int)));
    HCHECK(cudaMallocManaged(&states, S * sizeof(curandState)));

    initializeRandomStatesKernel<<<numBlocks, blockSize>>>(states, S, seed);
    HCHECK(cudaDeviceSynchronize());
    initializeNaiveKernel<<<numBlocks, blockSize>>>(schemes, S, n1, n2, n3);
    HCHECK(cudaDeviceSynchronize());
    initializeSchemesKernel<<<numBlocks, blockSize>>>(schemes, best, bestRanks, flips, n1, n2, n3, S);
    HCHECK(cudaDeviceSynchronize());
    std::unordered_map<std::string, int> table;
    if (resizeP > 0) {  // FlipGraph constructor (flip_graph.cu:19) + initialize (190-198)
        table[getKey(n1, n2, n3)] = n1 * n2 * n3;
        update_ranks(table, schemes, best, bestRanks, S);
    }

    FILE *f = fopen(out, "wb");
    if (!f) { fprintf(stderr, "cannot open %s\n", out); return 1; }
    // magic "FGW3" (resize + sandwiching + basis probabilities), "FGW2" (resize) or "FGW1"
    put_i32(f, moves ? 0x46475733 : (resizeP > 0 ? 0x46475732 : 0x46475731));
    put_i32(f, kRingIsZT);
    put_i32(f, n1); put_i32(f, n2); put_i32(f, n3);
    put_i32(f, S); put_i32(f, iters); put_i32(f, plusIters);
    fwrite(&expandP, 8, 1, f); fwrite(&reduceP, 8, 1, f);
    if (resizeP > 0 || moves) fwrite(&resizeP, 8, 1, f);
    if (moves) { fwrite(&sandwichP, 8, 1, f); fwrite(&basisP, 8, 1, f); }
    put_i32(f, seed); put_i32(f, launches);
    for (int w = 0; w < S; w++) put_scheme(f, schemes[w], true);   // initial state

    for (int L = 0; L < launches; L++) {
        randomWalkKernel<<<numBlocks, blockSize>>>(schemes, best, bestRanks, flips, states, S, iters, plusIters,
                                                   reduceP, expandP, sandwichP, basisP, resizeP > 0);
        HCHECK(cudaGetLastError());
        HCHECK(cudaDeviceSynchronize());
        if (resizeP > 0) {  // FlipGraph::run (flip_graph.cu:296-299)
            resizeKernel<<<numBlocks, blockSize>>>(schemes, best, S, states, resizeP);
            HCHECK(cudaGetLastError());
            HCHECK(cudaDeviceSynchronize());
            update_ranks(table, schemes, best, bestRanks, S);
        }
        for (int w = 0; w < S; w++) {
            put_i32(f, flips[w]);
            put_i32(f, bestRanks[w]);
            put_scheme(f, schemes[w], true);
            put_scheme(f, best[w], false);
            put_i32(f, schemes[w].validate() ? 1 : 0);
        }
    }
    // Tape long enough for any walk: bounded by the device buffer size.
    size_t budget = (size_t)1 << 28;  // bytes for draws + uniforms
    size_t perIter = kRingIsZT ? 700 : 40;  // ZT flips draw a permutation of all pairs
    if (getenv("FG_NO_TAPE")) perIter = 0, budget = 0;  // walks run only to produce input schemes
    int maxDraws = (int)std::min<size_t>(budget / (8 * (size_t)S), perIter * iters * launches + 4096);
    write_tapes(f, states, S, seed, maxDraws);
    fclose(f);
    cudaFree(schemes); cudaFree(best); cudaFree(bestRanks); cudaFree(flips); cudaFree(states);
    return 0;
}

static int cmd_reduce_flips(int argc, char **argv);

static int cmd_reduce(int argc, char **argv) {
    if (argc == 9 && atoi(argv[7]) > 0) return cmd_reduce_flips(argc, argv);
    if (argc != 7) { fprintf(stderr, "reduce: bad arguments\n"); return 1; }
    const char *in = argv[2];
    int count = atoi(argv[3]), schemesCount = atoi(argv[4]), seed = atoi(argv[5]);
    const char *out = argv[6];
    typedef AdditionsReducer<MAX_U_EXPRESSIONS, MAX_U_FRESH_VARIABLES, MAX_U_REAL_VARIABLES, MAX_U_SUBEXPRESSIONS> RU;
    typedef AdditionsReducer<MAX_V_EXPRESSIONS, MAX_V_FRESH_VARIABLES, MAX_V_REAL_VARIABLES, MAX_V_SUBEXPRESSIONS> RV;
    typedef AdditionsReducer<MAX_W_EXPRESSIONS, MAX_W_FRESH_VARIABLES, MAX_W_REAL_VARIABLES, MAX_W_SUBEXPRESSIONS> RW;
    RU *ru; RV *rv; RW *rw; SchemeInteger *schemes; curandState *states;
    HCHECK(cudaMallocManaged(&ru, (count + 1) * sizeof(RU)));
    HCHECK(cudaMallocManaged(&rv, (count + 1) * sizeof(RV)));
    HCHECK(cudaMallocManaged(&rw, (count + 1) * sizeof(RW)));
    HCHECK(cudaMallocManaged(&schemes, (count + 1) * sizeof(SchemeInteger)));
    HCHECK(cudaMallocManaged(&states, count * sizeof(curandState)));
    std::ifstream fin(in);
    int n1, n2, n3, m;
    fin >> n1 >> n2 >> n3 >> m;
    if (!schemes[0].read(fin, n1, n2, n3, m, false)) { fprintf(stderr, "read failed\n"); return 1; }
    int blockSize = 32, numBlocks = (count + blockSize - 1) / blockSize;
    initializeKernel<<<numBlocks, blockSize>>>(ru, rv, rw, schemes, states, count, schemesCount, seed);
    HCHECK(cudaGetLastError());
    HCHECK(cudaDeviceSynchronize());
    runReducersKernel<<<numBlocks, blockSize>>>(ru, rv, rw, schemes, states, count, schemesCount, true);
    HCHECK(cudaGetLastError());
    HCHECK(cudaDeviceSynchronize());
    FILE *f = fopen(out, "wb");
    put_i32(f, 0x46475231);  // magic "FGR1"
    put_i32(f, count); put_i32(f, seed);
    for (int r = 0; r <= count; r++) {
        put_i32(f, ru[r].getAdditions()); put_i32(f, ru[r].getFreshVars()); put_i32(f, ru[r].getNaiveAdditions());
        put_i32(f, rv[r].getAdditions()); put_i32(f, rv[r].getFreshVars()); put_i32(f, rv[r].getNaiveAdditions());
        put_i32(f, rw[r].getAdditions()); put_i32(f, rw[r].getFreshVars()); put_i32(f, rw[r].getNaiveAdditions());
        std::string modes = ru[r].getMode() + "," + rv[r].getMode() + "," + rw[r].getMode();
        put_i32(f, (int)modes.size());
        fwrite(modes.data(), 1, modes.size(), f);
    }
    int maxDraws = 1 << 18;
    write_tapes(f, states, count, seed, maxDraws);
    fclose(f);
    return 0;
}

// reduce_time IN COUNT SEED LAUNCHES [OUT]: LAUNCHES times initializeKernel + one timed
// runReducersKernel (independent) of COUNT reducers over the one scheme of IN (read with
// checkValidity=false); prints the mean kernel time, reducer runs per second and the
// per-reducer addition totals' minimum and sum (the same seed every launch).  OUT, when
// given, receives one text line per reducer: U, V, W additions and the three modes.
static int cmd_reduce_time(int argc, char **argv) {
    if (argc != 6 && argc != 7) { fprintf(stderr, "reduce_time: bad arguments\n"); return 1; }
    const char *in = argv[2];
    int count = atoi(argv[3]), seed = atoi(argv[4]), launches = atoi(argv[5]);
    if (count < 1 || launches < 1) { fprintf(stderr, "reduce_time: bad arguments\n"); return 1; }
    typedef AdditionsReducer<MAX_U_EXPRESSIONS, MAX_U_FRESH_VARIABLES, MAX_U_REAL_VARIABLES, MAX_U_SUBEXPRESSIONS> RU;
    typedef AdditionsReducer<MAX_V_EXPRESSIONS, MAX_V_FRESH_VARIABLES, MAX_V_REAL_VARIABLES, MAX_V_SUBEXPRESSIONS> RV;
    typedef AdditionsReducer<MAX_W_EXPRESSIONS, MAX_W_FRESH_VARIABLES, MAX_W_REAL_VARIABLES, MAX_W_SUBEXPRESSIONS> RW;
    RU *ru; RV *rv; RW *rw; SchemeInteger *schemes; curandState *states;
    HCHECK(cudaMallocManaged(&ru, (count + 1) * sizeof(RU)));
    HCHECK(cudaMallocManaged(&rv, (count + 1) * sizeof(RV)));
    HCHECK(cudaMallocManaged(&rw, (count + 1) * sizeof(RW)));
    HCHECK(cudaMallocManaged(&schemes, (count + 1) * sizeof(SchemeInteger)));
    HCHECK(cudaMallocManaged(&states, count * sizeof(curandState)));
    std::ifstream fin(in);
    int n1, n2, n3, m;
    fin >> n1 >> n2 >> n3 >> m;
    if (!schemes[0].read(fin, n1, n2, n3, m, false)) { fprintf(stderr, "read failed\n"); return 1; }
    int blockSize = 32, numBlocks = (count + blockSize - 1) / blockSize;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double total_ms = 0;
    for (int L = 0; L < launches; L++) {
        initializeKernel<<<numBlocks, blockSize>>>(ru, rv, rw, schemes, states, count, 1, seed);
        HCHECK(cudaGetLastError());
        HCHECK(cudaDeviceSynchronize());
        cudaEventRecord(e0);
        runReducersKernel<<<numBlocks, blockSize>>>(ru, rv, rw, schemes, states, count, 1, true);
        cudaEventRecord(e1);
        HCHECK(cudaGetLastError());
        HCHECK(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        total_ms += ms;
        fprintf(stderr, "launch %d: %.3f ms\n", L, ms);
    }
    if (argc == 7) {
        FILE *f = fopen(argv[6], "w");
        if (!f) { fprintf(stderr, "reduce_time: cannot write %s\n", argv[6]); return 1; }
        for (int r = 0; r < count; r++)
            fprintf(f, "%d %d %d %s %s %s\n", ru[r].getAdditions(), rv[r].getAdditions(), rw[r].getAdditions(),
                    ru[r].getMode().c_str(), rv[r].getMode().c_str(), rw[r].getMode().c_str());
        fclose(f);
    }
    long long sum = 0;
    int best = 1 << 30;
    for (int r = 0; r < count; r++) {
        const int a = ru[r].getAdditions() + rv[r].getAdditions() + rw[r].getAdditions();
        sum += a;
        if (a < best) best = a;
    }
    printf("{\"reducers\": %d, \"launches\": %d, \"ms_per_launch\": %.3f, \"runs_per_s\": %.6e, "
           "\"best_additions\": %d, \"sum_additions\": %lld, \"seed\": %d}\n",
           count, launches, total_ms / launches, count / (total_ms / launches / 1000.0), best, sum, seed);
    cudaFree(ru); cudaFree(rv); cudaFree(rw); cudaFree(schemes); cudaFree(states);
    return 0;
}

static int cmd_reduce_flips(int argc, char **argv) {
    const char *in = argv[2];
    int count = atoi(argv[3]), schemesCount = atoi(argv[4]), seed = atoi(argv[5]);
    const char *out = argv[6];
    int maxFlips = atoi(argv[7]), iterations = atoi(argv[8]);
    if (count < 10 || schemesCount > count || iterations < 1) { fprintf(stderr, "reduce: bad flip arguments\n"); return 1; }
    typedef AdditionsReducer<MAX_U_EXPRESSIONS, MAX_U_FRESH_VARIABLES, MAX_U_REAL_VARIABLES, MAX_U_SUBEXPRESSIONS> RU;
    typedef AdditionsReducer<MAX_V_EXPRESSIONS, MAX_V_FRESH_VARIABLES, MAX_V_REAL_VARIABLES, MAX_V_SUBEXPRESSIONS> RV;
    typedef AdditionsReducer<MAX_W_EXPRESSIONS, MAX_W_FRESH_VARIABLES, MAX_W_REAL_VARIABLES, MAX_W_SUBEXPRESSIONS> RW;
    RU *ru; RV *rv; RW *rw; SchemeInteger *schemes; curandState *states;
    HCHECK(cudaMallocManaged(&ru, (count + 1) * sizeof(RU)));
    HCHECK(cudaMallocManaged(&rv, (count + 1) * sizeof(RV)));
    HCHECK(cudaMallocManaged(&rw, (count + 1) * sizeof(RW)));
    HCHECK(cudaMallocManaged(&schemes, (count + 1) * sizeof(SchemeInteger)));
    HCHECK(cudaMallocManaged(&states, count * sizeof(curandState)));
    std::ifstream fin(in);
    int n1, n2, n3, m;
    fin >> n1 >> n2 >> n3 >> m;
    if (!schemes[0].read(fin, n1, n2, n3, m, false)) { fprintf(stderr, "read failed\n"); return 1; }
    int blockSize = 32, numBlocks = (count + blockSize - 1) / blockSize;
    initializeKernel<<<numBlocks, blockSize>>>(ru, rv, rw, schemes, states, count, schemesCount, seed);
    HCHECK(cudaGetLastError());
    HCHECK(cudaDeviceSynchronize());
    // SchemeAdditionsReducer::initialize (scheme_additions_reducer.cu:145-160)
    int reducedAdditions = ru[count].getAdditions() + rv[count].getAdditions() + rw[count].getAdditions();
    int reducedFresh = n1 * n2 * (n1 * n2 - 1) + n2 * n3 * (n2 * n3 - 1) + m * (m - 1);
    std::vector<int> indices(count);
    for (int i = 0; i < count; i++) indices[i] = i;
    FILE *f = fopen(out, "wb");
    put_i32(f, 0x46475232);  // magic "FGR2"
    put_i32(f, count); put_i32(f, seed); put_i32(f, schemesCount); put_i32(f, maxFlips); put_i32(f, iterations);
    for (int it = 1; it <= iterations; it++) {
        if (it > 1) {
            flipSchemesKernel<<<(schemesCount + blockSize - 1) / blockSize, blockSize>>>(schemes, states, schemesCount, maxFlips);
            HCHECK(cudaGetLastError());
            HCHECK(cudaDeviceSynchronize());
        }
        runReducersKernel<<<numBlocks, blockSize>>>(ru, rv, rw, schemes, states, count, schemesCount, false);
        HCHECK(cudaGetLastError());
        HCHECK(cudaDeviceSynchronize());
        for (int s = 0; s < schemesCount; s++) put_i32(f, schemes[s].m);
        for (int r = 0; r < count; r++) {
            put_i32(f, ru[r].getAdditions()); put_i32(f, ru[r].getFreshVars()); put_i32(f, ru[r].getNaiveAdditions());
            put_i32(f, rv[r].getAdditions()); put_i32(f, rv[r].getFreshVars()); put_i32(f, rv[r].getNaiveAdditions());
            put_i32(f, rw[r].getAdditions()); put_i32(f, rw[r].getFreshVars()); put_i32(f, rw[r].getNaiveAdditions());
            std::string modes = ru[r].getMode() + "," + rv[r].getMode() + "," + rw[r].getMode();
            put_i32(f, (int)modes.size());
            fwrite(modes.data(), 1, modes.size(), f);
        }
        // updateBestTogether: reducers ordered by total additions, then total fresh variables
        auto total = [&](int r, bool fresh) {
            return fresh ? ru[r].getFreshVars() + rv[r].getFreshVars() + rw[r].getFreshVars()
                         : ru[r].getAdditions() + rv[r].getAdditions() + rw[r].getAdditions();
        };
        std::partial_sort(indices.begin(), indices.begin() + 10, indices.end(), [&](int a, int b) {
            if (total(a, false) != total(b, false)) return total(a, false) < total(b, false);
            return total(a, true) < total(b, true);
        });
        const int top = indices[0];
        const int additions = total(top, false), fresh = total(top, true);
        const int improved = additions < reducedAdditions || (additions == reducedAdditions && fresh < reducedFresh);
        if (improved) {
            reducedAdditions = additions;
            reducedFresh = fresh;
            ru[count].copyFrom(ru[top]);
            rv[count].copyFrom(rv[top]);
            rw[count].copyFrom(rw[top]);
        }
        put_i32(f, top); put_i32(f, improved);
    }
    write_tapes(f, states, count, seed, 1 << 18);
    fclose(f);
    return 0;
}

// minimize_time IN COUNT ITERATIONS SEED LAUNCHES [OUT]: the complexity minimizer's own
// kernels (complexity_minimizer.cu:173-214): initializeKernel replicates the one scheme of IN
// (read with checkValidity=false) to COUNT walks with streams curand_init(SEED, idx, 0), then
// LAUNCHES timed minimizeKernel launches of ITERATIONS flips each.  Prints the mean launch
// time; OUT, when given, receives each walk's best complexity, one per line.
static int cmd_minimize_time(int argc, char **argv) {
    if (argc != 7 && argc != 8) { fprintf(stderr, "minimize_time: bad arguments\n"); return 1; }
    const char *in = argv[2];
    int count = atoi(argv[3]), iterations = atoi(argv[4]), seed = atoi(argv[5]), launches = atoi(argv[6]);
    if (count < 1 || iterations < 1 || launches < 1) { fprintf(stderr, "minimize_time: bad arguments\n"); return 1; }
    Scheme *schemes, *best;
    int *bestComplexities;
    curandState *states;
    HCHECK(cudaMallocManaged(&schemes, count * sizeof(Scheme)));
    HCHECK(cudaMallocManaged(&best, count * sizeof(Scheme)));
    HCHECK(cudaMallocManaged(&bestComplexities, count * sizeof(int)));
    HCHECK(cudaMallocManaged(&states, count * sizeof(curandState)));
    std::ifstream fin(in);
    int n1, n2, n3, m;
    fin >> n1 >> n2 >> n3 >> m;
    if (!schemes[0].read(fin, n1, n2, n3, m, false)) { fprintf(stderr, "read failed\n"); return 1; }
    const int complexity = schemes[0].getComplexity();
    int blockSize = 32, numBlocks = (count + blockSize - 1) / blockSize;
    initializeKernel<<<numBlocks, blockSize>>>(schemes, best, bestComplexities, states, count, 1, complexity, seed);
    HCHECK(cudaGetLastError());
    HCHECK(cudaDeviceSynchronize());
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double total_ms = 0;
    for (int L = 0; L < launches; L++) {
        cudaEventRecord(e0);
        minimizeKernel<<<numBlocks, blockSize>>>(schemes, best, bestComplexities, states, count, iterations);
        cudaEventRecord(e1);
        HCHECK(cudaGetLastError());
        HCHECK(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        total_ms += ms;
        fprintf(stderr, "launch %d: %.3f ms\n", L, ms);
    }
    int bestAll = 1 << 30;
    for (int w = 0; w < count; w++) bestAll = std::min(bestAll, bestComplexities[w]);
    if (argc == 8) {
        FILE *f = fopen(argv[7], "w");
        if (!f) { fprintf(stderr, "minimize_time: cannot write %s\n", argv[7]); return 1; }
        for (int w = 0; w < count; w++) fprintf(f, "%d\n", bestComplexities[w]);
        fclose(f);
    }
    printf("{\"walks\": %d, \"iterations\": %d, \"launches\": %d, \"ms_per_launch\": %.3f, "
           "\"initial_complexity\": %d, \"best_complexity\": %d, \"seed\": %d}\n",
           count, iterations, launches, total_ms / launches, complexity, bestAll, seed);
    cudaFree(schemes); cudaFree(best); cudaFree(bestComplexities); cudaFree(states);
    return 0;
}

#ifndef SCHEME_INTEGER
__global__ void gaussKernel(Scheme *schemes, curandState *states, int count, int *found) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= count) return;
    found[idx] = schemes[idx].tryReduceGauss(states[idx]) ? 1 : 0;
}

static int cmd_gauss(int argc, char **argv) {
    if (argc != 5) { fprintf(stderr, "gauss: bad arguments\n"); return 1; }
    std::ifstream fin(argv[2]);
    int seed = atoi(argv[3]);
    int count = 0;
    fin >> count;
    if (count <= 0) { fprintf(stderr, "gauss: no schemes\n"); return 1; }
    Scheme *schemes; curandState *states; int *found;
    HCHECK(cudaMallocManaged(&schemes, count * sizeof(Scheme)));
    HCHECK(cudaMallocManaged(&states, count * sizeof(curandState)));
    HCHECK(cudaMallocManaged(&found, count * sizeof(int)));
    for (int k = 0; k < count; k++)
        if (!schemes[k].read(fin, false)) { fprintf(stderr, "gauss: read failed at %d\n", k); return 1; }
    int blockSize = 32, numBlocks = (count + blockSize - 1) / blockSize;
    initializeRandomStatesKernel<<<numBlocks, blockSize>>>(states, count, seed);
    HCHECK(cudaGetLastError());
    HCHECK(cudaDeviceSynchronize());
    gaussKernel<<<numBlocks, blockSize>>>(schemes, states, count, found);
    HCHECK(cudaGetLastError());
    HCHECK(cudaDeviceSynchronize());
    FILE *f = fopen(argv[4], "wb");
    if (!f) { fprintf(stderr, "cannot open %s\n", argv[4]); return 1; }
    put_i32(f, 0x46474731);  // magic "FGG1"
    put_i32(f, count); put_i32(f, seed);
    for (int k = 0; k < count; k++) {
        put_i32(f, found[k]);
        put_scheme(f, schemes[k], false);
    }
    write_tapes(f, states, count, seed, 64);
    fclose(f);
    cudaFree(schemes); cudaFree(states); cudaFree(found);
    return 0;
}
#endif

// Counting twin of randomWalkKernel (flip_graph.cu:520-573, randomIterations
// false): the same loop over the reference's own Scheme operators, taking the
// same draws in the same order, plus one per-walk count of accepted flips
// (tryFlip returned true).  cmd_time runs it on a copy of the state the
// unmodified kernel starts from and checks on the device that both end in
// byte-identical states, so the count is the unmodified kernel's.
__global__ void countingWalkKernel(Scheme *schemes, Scheme *schemesBest, int *bestRanks, int *flips,
                                   curandState *states, int schemesCount, int maxIterations, int plusIterations,
                                   double reduceProbability, double expandProbability, double sandwichingProbability,
                                   double basisProbability, unsigned long long *accepted) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= schemesCount) return;
    Scheme &scheme = schemes[idx];
    curandState &state = states[idx];
    int flipsCount = flips[idx];
    int bestRank = bestRanks[idx];
    unsigned long long count = 0;
    for (int iteration = 0; iteration < maxIterations; iteration++) {
        int rank = scheme.m;
        if (!scheme.tryFlip(state)) {
            scheme.tryExpand(randint(1, 2, state), state);
            continue;
        }
        count++;
        if (scheme.m < rank) flipsCount = 0;
        flipsCount++;
        if (scheme.m < bestRank || (scheme.m == bestRank && curand_uniform(&state) < 0.01)) {
            bestRank = scheme.m;
            scheme.copyTo(schemesBest[idx], false);
        }
        if (curand_uniform(&state) * maxIterations < reduceProbability) scheme.tryReduce();
        if (curand_uniform(&state) * maxIterations < expandProbability && scheme.m <= schemesBest[idx].m + 2) {
            if (scheme.tryExpand(randint(1, 2, state), state)) flipsCount = 0;
        }
        if (curand_uniform(&state) * maxIterations < sandwichingProbability) scheme.sandwiching(state);
        if (curand_uniform(&state) * maxIterations < basisProbability) scheme.swapBasis(state);
        if (flipsCount >= plusIterations && scheme.tryPlus(state)) flipsCount = 0;
    }
    flips[idx] = flipsCount;
    bestRanks[idx] = bestRank;
    accepted[idx] = count;
}

// Per walk: 1 when the two runs' schemes, best schemes, counters and cuRAND
// states differ anywhere (whole structs, word by word); valid = validate().
__global__ void compareWalksKernel(const Scheme *a, const Scheme *b, const Scheme *ab, const Scheme *bb,
                                   const int *ar, const int *br, const int *af, const int *bf,
                                   const curandState *as, const curandState *bs, int S, int *differs, int *valid) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= S) return;
    int d = ar[idx] != br[idx] || af[idx] != bf[idx];
    const uint32_t *x = reinterpret_cast<const uint32_t *>(&a[idx]), *y = reinterpret_cast<const uint32_t *>(&b[idx]);
    for (size_t q = 0; q < sizeof(Scheme) / 4 && !d; q++) d = x[q] != y[q];
    x = reinterpret_cast<const uint32_t *>(&ab[idx]); y = reinterpret_cast<const uint32_t *>(&bb[idx]);
    for (size_t q = 0; q < sizeof(Scheme) / 4 && !d; q++) d = x[q] != y[q];
    x = reinterpret_cast<const uint32_t *>(&as[idx]); y = reinterpret_cast<const uint32_t *>(&bs[idx]);
    for (size_t q = 0; q < sizeof(curandState) / 4 && !d; q++) d = x[q] != y[q];
    differs[idx] = d;
    valid[idx] = a[idx].validate() ? 1 : 0;
}

struct WalkArrays {
    Scheme *schemes = nullptr, *best = nullptr;
    int *bestRanks = nullptr, *flips = nullptr;
    curandState *states = nullptr;
    void alloc(int S) {
        HCHECK(cudaMallocManaged(&schemes, S * sizeof(Scheme)));
        HCHECK(cudaMallocManaged(&best, S * sizeof(Scheme)));
        HCHECK(cudaMallocManaged(&bestRanks, S * sizeof(int)));
        HCHECK(cudaMallocManaged(&flips, S * sizeof(int)));
        HCHECK(cudaMallocManaged(&states, S * sizeof(curandState)));
    }
    void copyFrom(const WalkArrays &o, int S) {
        HCHECK(cudaMemcpy(schemes, o.schemes, S * sizeof(Scheme), cudaMemcpyDefault));
        HCHECK(cudaMemcpy(best, o.best, S * sizeof(Scheme), cudaMemcpyDefault));
        HCHECK(cudaMemcpy(bestRanks, o.bestRanks, S * sizeof(int), cudaMemcpyDefault));
        HCHECK(cudaMemcpy(flips, o.flips, S * sizeof(int), cudaMemcpyDefault));
        HCHECK(cudaMemcpy(states, o.states, S * sizeof(curandState), cudaMemcpyDefault));
    }
    void release() { cudaFree(schemes); cudaFree(best); cudaFree(bestRanks); cudaFree(flips); cudaFree(states); }
};

// time S ITERS LAUNCHES SEED PLUS_ITERS shape... (e.g. 2x2x2 3x3x3)
//   Throughput of the reference's own walk kernel on the batched uneven
//   workload, set up the way the reference runs several shapes: one naive
//   scheme per shape replicated idx % count by initializeCopyKernel
//   (flip_graph.cu:459-470), best ranks per shape as updateRanks leaves them
//   (flip_graph.cu:249-266), resize off.  Each launch of the unmodified
//   randomWalkKernel is timed with CUDA events.  Accepted flips come from the
//   counting twin run on a copy of the same state; after every launch the two
//   runs are compared on the device (twin_mismatches must be 0) and every
//   scheme is validated: verified flips are the accepted flips of walks whose
//   scheme passes validate() after the launch.
static int cmd_time(int argc, char **argv) {
    if (argc < 8) { fprintf(stderr, "time: bad arguments\n"); return 1; }
    int S = atoi(argv[2]), iters = atoi(argv[3]), launches = atoi(argv[4]), seed = atoi(argv[5]);
    int plusIters = atoi(argv[6]);
    int count = argc - 7;
    int blockSize = 32, numBlocks = (S + blockSize - 1) / blockSize;
    WalkArrays A, B;
    A.alloc(S);
    B.alloc(S);
    unsigned long long *accepted; int *differs, *valid;
    HCHECK(cudaMallocManaged(&accepted, S * sizeof(unsigned long long)));
    HCHECK(cudaMallocManaged(&differs, S * sizeof(int)));
    HCHECK(cudaMallocManaged(&valid, S * sizeof(int)));
    for (int i = 0; i < count; i++) {
        int a, b, c;
        if (sscanf(argv[7 + i], "%dx%dx%d", &a, &b, &c) != 3) { fprintf(stderr, "bad shape\n"); return 1; }
        A.schemes[i].initializeNaive(a, b, c);
    }
    initializeRandomStatesKernel<<<numBlocks, blockSize>>>(A.states, S, seed);
    initializeCopyKernel<<<numBlocks, blockSize>>>(A.schemes, S, count);
    HCHECK(cudaDeviceSynchronize());
    initializeSchemesKernel<<<numBlocks, blockSize>>>(A.schemes, A.best, A.bestRanks, A.flips, 1, 1, 1, S);
    HCHECK(cudaDeviceSynchronize());
    for (int w = 0; w < S; w++) A.bestRanks[w] = A.schemes[w].m;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // One untimed launch brings managed memory to the device.
    randomWalkKernel<<<numBlocks, blockSize>>>(A.schemes, A.best, A.bestRanks, A.flips, A.states, S, iters, plusIters,
                                               0.0, 0.01, 0.0, 0.0, false);
    HCHECK(cudaDeviceSynchronize());
    B.copyFrom(A, S);
    double total_ms = 0, acceptedAll = 0, verifiedAll = 0;
    long long mismatches = 0;
    int validLast = 0;
    for (int L = 0; L < launches; L++) {
        cudaEventRecord(e0);
        randomWalkKernel<<<numBlocks, blockSize>>>(A.schemes, A.best, A.bestRanks, A.flips, A.states, S, iters,
                                                   plusIters, 0.0, 0.01, 0.0, 0.0, false);
        cudaEventRecord(e1);
        HCHECK(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        total_ms += ms;
        countingWalkKernel<<<numBlocks, blockSize>>>(B.schemes, B.best, B.bestRanks, B.flips, B.states, S, iters,
                                                     plusIters, 0.0, 0.01, 0.0, 0.0, accepted);
        HCHECK(cudaGetLastError());
        compareWalksKernel<<<numBlocks, blockSize>>>(A.schemes, B.schemes, A.best, B.best, A.bestRanks, B.bestRanks,
                                                     A.flips, B.flips, A.states, B.states, S, differs, valid);
        HCHECK(cudaGetLastError());
        HCHECK(cudaDeviceSynchronize());
        validLast = 0;
        for (int w = 0; w < S; w++) {
            mismatches += differs[w];
            acceptedAll += (double)accepted[w];
            if (valid[w]) verifiedAll += (double)accepted[w];
            validLast += valid[w];
        }
        fprintf(stderr, "launch %d: %.3f ms\n", L, ms);
    }
    int minRank[64];
    for (int i = 0; i < count && i < 64; i++) minRank[i] = 1 << 30;
    for (int w = 0; w < S; w++) {
        int i = w % count;
        if (i < 64 && A.bestRanks[w] < minRank[i]) minRank[i] = A.bestRanks[w];
    }
    double flipsUpper = (double)S * iters * launches;
    printf("{\"walks\": %d, \"iterations\": %d, \"launches\": %d, \"ms_per_launch\": %.3f, "
           "\"accepted_flips\": %.0f, \"verified_flips\": %.0f, \"verified_flips_per_s\": %.6e, "
           "\"flips_per_s_upper_bound\": %.6e, \"twin_mismatches\": %lld, \"valid_walks\": %d, \"ring\": \"%s\", "
           "\"best_ranks\": [",
           S, iters, launches, total_ms / launches, acceptedAll, verifiedAll, verifiedAll / (total_ms / 1000.0),
           flipsUpper / (total_ms / 1000.0), mismatches, validLast, kRingIsZT ? "ZT" : "Z2");
    for (int i = 0; i < count && i < 64; i++) printf("%s%d", i ? ", " : "", minRank[i]);
    printf("]}\n");
    A.release();
    B.release();
    cudaFree(accepted); cudaFree(differs); cudaFree(valid);
    return 0;
}

// ttr N1 N2 N3 S ITERS PLUS_ITERS SEED TARGET MAX_SECONDS
//   Time to target rank of the reference's own walk kernel: naive starts,
//   launches of randomWalkKernel (resize off) until some walk's best rank
//   reaches TARGET or MAX_SECONDS elapse; prints the wall time.
static int cmd_ttr(int argc, char **argv) {
    if (argc != 11) { fprintf(stderr, "ttr: bad arguments\n"); return 1; }
    int n1 = atoi(argv[2]), n2 = atoi(argv[3]), n3 = atoi(argv[4]), S = atoi(argv[5]);
    int iters = atoi(argv[6]), plusIters = atoi(argv[7]), seed = atoi(argv[8]), target = atoi(argv[9]);
    double maxSeconds = atof(argv[10]);
    int blockSize = 32, numBlocks = (S + blockSize - 1) / blockSize;
    Scheme *schemes, *best; int *bestRanks, *flips; curandState *states;
    HCHECK(cudaMallocManaged(&schemes, S * sizeof(Scheme)));
    HCHECK(cudaMallocManaged(&best, S * sizeof(Scheme)));
    HCHECK(cudaMallocManaged(&bestRanks, S * sizeof(int)));
    HCHECK(cudaMallocManaged(&flips, S * sizeof(int)));
    HCHECK(cudaMallocManaged(&states, S * sizeof(curandState)));
    auto t0 = std::chrono::steady_clock::now();
    initializeRandomStatesKernel<<<numBlocks, blockSize>>>(states, S, seed);
    initializeNaiveKernel<<<numBlocks, blockSize>>>(schemes, S, n1, n2, n3);
    initializeSchemesKernel<<<numBlocks, blockSize>>>(schemes, best, bestRanks, flips, n1, n2, n3, S);
    HCHECK(cudaDeviceSynchronize());
    int launches = 0, reached = 0, bestSeen = n1 * n2 * n3;
    double secs = 0;
    while (!reached && secs < maxSeconds) {
        randomWalkKernel<<<numBlocks, blockSize>>>(schemes, best, bestRanks, flips, states, S, iters, plusIters, 0.0,
                                                   0.01, 0.0, 0.0, false);
        HCHECK(cudaDeviceSynchronize());
        launches++;
        for (int w = 0; w < S; w++) {
            if (bestRanks[w] < bestSeen) bestSeen = bestRanks[w];
            if (bestRanks[w] <= target && best[w].validate()) reached = 1;
        }
        secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    printf("{\"reached\": %d, \"seconds\": %.3f, \"launches\": %d, \"steps_per_walk\": %lld, \"best_rank\": %d}\n",
           reached, secs, launches, (long long)launches * iters, bestSeen);
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 2) { fprintf(stderr, "usage: ref_harness walk|reduce|reduce_time|minimize_time|time|ttr ...\n"); return 1; }
    if (std::string(argv[1]) == "ttr") return cmd_ttr(argc, argv);
    std::string cmd = argv[1];
    if (cmd == "walk") return cmd_walk(argc, argv);
    if (cmd == "reduce") return cmd_reduce(argc, argv);
    if (cmd == "reduce_time") return cmd_reduce_time(argc, argv);
    if (cmd == "minimize_time") return cmd_minimize_time(argc, argv);
    if (cmd == "time") return cmd_time(argc, argv);
#ifndef SCHEME_INTEGER
    if (cmd == "gauss") return cmd_gauss(argc, argv);
#endif
    fprintf(stderr, "unknown command %s\n", argv[1]);
    return 1;
}
