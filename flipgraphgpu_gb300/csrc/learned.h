// Learned-proposal walk (learned.cu): Z2 walks stepped in lockstep so that the
// candidate flips of all walks are scored by the MLP on the tensor cores
// between steps.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "fg_device.cuh"

struct fg_mlp;

namespace fg {

struct LearnedConfig {
    int K = 1;               // candidates drawn per step
    float invTemp = 1.0f;    // softmax of score / temperature
    float minEntropy = 0.0f; // below this (nats) the step falls back to a uniform pick
    int recordEvery = 0;     // > 0: log every recordEvery-th accepted flip as a training record
};

// Per-walk step state kept between kernel launches.
struct LWalk {
    int m, P0, P1, P2, status, flips, bestRank, bestM;
    int it, pending, copied, ndrops;
    unsigned long long draws, accepted, total;
};

struct LearnedBuffers {
    int S = 0, Spad = 0, sh = 0, scap = 0, K = 0;
    uint32_t *words = nullptr;   // word (c, t, walk) at ((c * scap + t) << sh) + walk
    LWalk *lw = nullptr;
    uint32_t *cand = nullptr;    // [S][K] packed candidate: c | o << 2 | a << 3 | b << 12
    uint64_t *feat = nullptr;    // [S][K][3] feature words
    float *scores = nullptr;     // [S][K]
    // training records
    long long recCap = 0;
    uint64_t *recFeat = nullptr; // [recCap][3]
    uint32_t *recWalk = nullptr, *recFlip = nullptr;
    unsigned long long *recCount = nullptr;
    int dropCap = 0;
    uint32_t *drops = nullptr;   // [S][dropCap] accepted-flip indices at which the rank dropped
};

// The step loop of a launch (step kernels and the network's scoring between them) as a CUDA
// graph: captured on the second launch with the same arguments (the first one runs directly
// and sets the kernels' attributes and the network's workspace), then replayed.
struct LearnedGraph {
    cudaGraphExec_t exec = nullptr;
    std::vector<unsigned char> key;  // the launch arguments the graph was captured with
    bool primed = false, failed = false;
    void reset() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        key.clear();
        primed = failed = false;
    }
};

cudaError_t learned_alloc(LearnedBuffers &L, int S, int scap, int K);
cudaError_t learned_alloc_records(LearnedBuffers &L, long long recCap, int dropCap);
void learned_free(LearnedBuffers &L);
// One launch (P.iterations steps per walk) over the batch records in B.
cudaError_t learned_launch(LearnedBuffers &L, const DevBatch &B, const WalkParams &P, const LearnedConfig &C,
                           fg_mlp *mlp, cudaStream_t s, LearnedGraph *G = nullptr);
// Labels of the logged records: 1 if the walk's rank dropped at or within
// `horizon` accepted flips after the record's flip, 0 if it did not; records
// whose outcome is unknown (walk ended or drop log full) are dropped.
cudaError_t learned_take_records(LearnedBuffers &L, int horizon, std::vector<uint64_t> &feat, std::vector<float> &label,
                                 cudaStream_t s);

}  // namespace fg
