// The learned flip proposal's network on the GPU (mlp.cu): a 192 -> 256 -> 256
// -> 1 MLP with bf16 weights and activations, fp32 accumulation on the tensor
// cores, trained with binary cross-entropy and Adam.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

struct fg_mlp;

namespace fg {

constexpr int kMlpIn = 192;      // input features (three 64-bit words)
constexpr int kMlpHidden = 256;  // width of both hidden layers

// Parameter block offsets (floats) inside one contiguous fp32 buffer.
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpHidden * kMlpIn;
constexpr int kOffW2 = kOffB1 + kMlpHidden;
constexpr int kOffB2 = kOffW2 + kMlpHidden * kMlpHidden;
constexpr int kOffW3 = kOffB2 + kMlpHidden;
constexpr int kOffB3 = kOffW3 + kMlpHidden;
constexpr int kMlpParams = kOffB3 + 1;

// Scores `rows` rows of feature words ([rows][3] uint64, device) into
// scores[rows] (device) on stream s; the network's device must be current.
cudaError_t mlp_score_device(fg_mlp *m, const uint64_t *features, int rows, float *scores, cudaStream_t s);
// Counts the reallocations of the network's workspace (0 for no network): a graph that
// captured the scoring is valid only while this is unchanged.
unsigned long long mlp_workspace_epoch(const fg_mlp *m);

}  // namespace fg
