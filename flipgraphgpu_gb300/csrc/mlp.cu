// Learned flip proposal network: forward, backward and Adam on the GPU.
//
//   X  [R][192]  bf16 0/1 features, expanded from three 64-bit words per row
//   H1 = relu(X W1^T + b1)         tcgen05 GEMM, bias+ReLU epilogue -> bf16
//   H2 = relu(H1 W2^T + b2)        tcgen05 GEMM, bias+ReLU epilogue -> bf16
//   s  = H2 w3 + b3                one warp per row
// Backward of the mean binary cross-entropy of sigmoid(s):
//   dZ2 = bf16(ds w3 * [H2 > 0]);  dZ1 = bf16((dZ2 W2) * [H1 > 0])  (GEMM, mask epilogue)
//   gW2 = dZ2^T H1,  gW1 = dZ1^T X  (GEMMs over the batch: K = R, operands transposed)
// The CPU oracle restates the same arithmetic (oracle/mlp_oracle.py).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

#include "../../include/flipgraph.h"
#include "launch.h"
#include "mlp.h"
#include "tc_gemm.h"

using bf16 = __nv_bfloat16;

struct fg_mlp {
    int dev = 0;
    cudaStream_t stream = nullptr;
    float *P = nullptr, *G = nullptr, *Am = nullptr, *Av = nullptr;  // params, grads, Adam moments
    bf16 *W1h = nullptr, *W2h = nullptr, *W2th = nullptr;            // bf16 copies (W2th = W2^T)
    int cap = 0;                                                     // workspace rows
    bf16 *X = nullptr, *H1 = nullptr, *H2 = nullptr, *dZ2 = nullptr, *dZ1 = nullptr;
    bf16 *XT = nullptr, *H1T = nullptr, *dZ2T = nullptr, *dZ1T = nullptr;
    float *scores = nullptr, *ds = nullptr, *lab = nullptr, *loss = nullptr;
    int *err = nullptr;
    int adamStep = 0;
    unsigned long long epoch = 0;  // bumped whenever the workspace is reallocated (captured graphs name its buffers)
};

namespace fg {
namespace {

__global__ void k_expand(const uint64_t *F, const int *idx, int first, int rows, int rowsPad, bf16 *X) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;  // (row, 8-feature chunk)
    if (q >= rowsPad * 24) return;
    const int row = q / 24, ch = q % 24;
    uint32_t byte = 0;
    if (row < rows) {
        const long r = idx ? idx[first + row] : (long)first + row;
        byte = (uint32_t)(F[r * 3 + ch / 8] >> ((ch % 8) * 8)) & 0xFFu;
    }
    __align__(16) bf16 v[8];
#pragma unroll
    for (int b = 0; b < 8; b++) v[b] = __float2bfloat16_rn((float)((byte >> b) & 1u));
    *reinterpret_cast<uint4 *>(X + (size_t)row * kMlpIn + ch * 8) = *reinterpret_cast<const uint4 *>(v);
}

__global__ void k_labels(const float *L, const int *idx, int first, int rows, int rowsPad, float *out) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= rowsPad) return;
    out[row] = row < rows ? L[idx ? idx[first + row] : first + row] : -1.0f;  // -1: padding row
}

// One warp per row: score, and with labels the loss, ds and dZ2.
__global__ void k_head(const bf16 *H2, const float *P, const float *lab, int rowsPad, float invB, float *scores,
                       float *ds, bf16 *dZ2, float *loss) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= rowsPad) return;
    const int row = warp;
    const uint4 raw = *reinterpret_cast<const uint4 *>(H2 + (size_t)row * kMlpHidden + lane * 8);
    const bf16 *h = reinterpret_cast<const bf16 *>(&raw);
    const float *w3 = P + kOffW3 + lane * 8;
    float hv[8], acc = 0.0f;
#pragma unroll
    for (int q = 0; q < 8; q++) {
        hv[q] = __bfloat162float(h[q]);
        acc = fmaf(hv[q], w3[q], acc);
    }
#pragma unroll
    for (int d = 16; d; d >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, d);
    const float s = acc + P[kOffB3];
    if (lane == 0) scores[row] = s;
    if (!lab) return;
    const float y = lab[row];
    float d = 0.0f;
    if (y >= 0.0f) {
        const float p = 1.0f / (1.0f + expf(-s));
        d = (p - y) * invB;
        if (lane == 0) atomicAdd(loss, fmaxf(s, 0.0f) + log1pf(expf(-fabsf(s))) - y * s);
    }
    if (lane == 0) ds[row] = d;
    __align__(16) bf16 g[8];
#pragma unroll
    for (int q = 0; q < 8; q++) g[q] = __float2bfloat16_rn(hv[q] > 0.0f ? d * w3[q] : 0.0f);
    *reinterpret_cast<uint4 *>(dZ2 + (size_t)row * kMlpHidden + lane * 8) = *reinterpret_cast<const uint4 *>(g);
}

// out[c][r] = in[r][c]; R, C multiples of 32.
__global__ void k_transpose(const bf16 *in, int R, int C, bf16 *out) {
    __shared__ bf16 t[32][33];
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += blockDim.y) t[y][threadIdx.x] = in[(size_t)(r0 + y) * C + c0 + threadIdx.x];
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += blockDim.y) out[(size_t)(c0 + y) * R + r0 + threadIdx.x] = t[threadIdx.x][y];
}

// out[r] = sum_c in[r][c] (one warp per row).
__global__ void k_rowsum(const bf16 *in, int rows, int cols, float *out) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= rows) return;
    float acc = 0.0f;
    for (int c = lane; c < cols; c += 32) acc += __bfloat162float(in[(size_t)warp * cols + c]);
#pragma unroll
    for (int d = 16; d; d >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, d);
    if (lane == 0) out[warp] = acc;
}

// gw3[j] += sum_r H2[r][j] ds[r] over this block's 128 rows; gb3 += sum_r ds[r].
__global__ void k_head_grads(const bf16 *H2, const float *ds, int rowsPad, float *gw3, float *gb3) {
    const int j = threadIdx.x, r0 = blockIdx.x * 128;
    float acc = 0.0f, sacc = 0.0f;
    for (int r = r0; r < r0 + 128 && r < rowsPad; r++) {
        const float d = ds[r];
        acc = fmaf(__bfloat162float(H2[(size_t)r * kMlpHidden + j]), d, acc);
        sacc += d;
    }
    atomicAdd(&gw3[j], acc);
    if (j == 0) atomicAdd(gb3, sacc);
}

__global__ void k_adam(float *P, const float *G, float *m, float *v, int n, float lr, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float g = G[i];
    const float mi = 0.9f * m[i] + 0.1f * g, vi = 0.999f * v[i] + 0.001f * g * g;
    m[i] = mi;
    v[i] = vi;
    P[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + 1e-8f);
}

__global__ void k_refresh(const float *P, bf16 *W1h, bf16 *W2h, bf16 *W2th) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kMlpHidden * kMlpIn) W1h[i] = __float2bfloat16_rn(P[kOffW1 + i]);
    if (i < kMlpHidden * kMlpHidden) {
        const int r = i / kMlpHidden, c = i % kMlpHidden;
        W2h[i] = __float2bfloat16_rn(P[kOffW2 + i]);
        W2th[(size_t)c * kMlpHidden + r] = __float2bfloat16_rn(P[kOffW2 + i]);
    }
}

cudaError_t refresh(fg_mlp *m) {
    k_refresh<<<(kMlpHidden * kMlpHidden + 255) / 256, 256, 0, m->stream>>>(m->P, m->W1h, m->W2h, m->W2th);
    return cudaGetLastError();
}

template <class T> cudaError_t dalloc(T **p, size_t n) { return cudaMalloc(reinterpret_cast<void **>(p), n * sizeof(T)); }

void free_workspace(fg_mlp *m) {
    void *ps[] = {m->X, m->H1, m->H2, m->dZ2, m->dZ1, m->XT, m->H1T, m->dZ2T, m->dZ1T, m->scores, m->ds, m->lab};
    for (void *p : ps)
        if (p) cudaFree(p);
    m->X = m->H1 = m->H2 = m->dZ2 = m->dZ1 = m->XT = m->H1T = m->dZ2T = m->dZ1T = nullptr;
    m->scores = m->ds = m->lab = nullptr;
    m->cap = 0;
}

cudaError_t ensure_workspace(fg_mlp *m, int rowsPad) {
    if (rowsPad <= m->cap) return cudaSuccess;
    cudaError_t e = cudaStreamSynchronize(m->stream);
    if (e != cudaSuccess) return e;
    free_workspace(m);
    const size_t R = (size_t)rowsPad;
    if ((e = dalloc(&m->X, R * kMlpIn)) || (e = dalloc(&m->H1, R * kMlpHidden)) || (e = dalloc(&m->H2, R * kMlpHidden)) ||
        (e = dalloc(&m->dZ2, R * kMlpHidden)) || (e = dalloc(&m->dZ1, R * kMlpHidden)) ||
        (e = dalloc(&m->XT, R * kMlpIn)) || (e = dalloc(&m->H1T, R * kMlpHidden)) ||
        (e = dalloc(&m->dZ2T, R * kMlpHidden)) || (e = dalloc(&m->dZ1T, R * kMlpHidden)) ||
        (e = dalloc(&m->scores, R)) || (e = dalloc(&m->ds, R)) || (e = dalloc(&m->lab, R))) {
        free_workspace(m);
        return e;
    }
    m->cap = rowsPad;
    m->epoch++;
    return cudaSuccess;
}

GemmEpilogue epi(int mode, int M, int ldo) {
    GemmEpilogue E{};
    E.mode = mode;
    E.M = M;
    E.ldo = ldo;
    return E;
}

// Forward to H2 for rows [first, first + rows) of F (optionally through idx); X, H1, H2 filled.
cudaError_t forward(fg_mlp *m, const uint64_t *F, const int *idx, int first, int rows, int rowsPad) {
    cudaStream_t s = m->stream;
    k_expand<<<(rowsPad * 24 + 255) / 256, 256, 0, s>>>(F, idx, first, rows, rowsPad, m->X);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    GemmEpilogue E1 = epi(EPI_BIAS_RELU_BF16, rowsPad, kMlpHidden);
    E1.bias = m->P + kOffB1;
    E1.outH = m->H1;
    E1.err = m->err;
    if ((e = gemm_bf16_tn(m->X, m->W1h, rowsPad, kMlpHidden, kMlpIn, E1, s))) return e;
    GemmEpilogue E2 = E1;
    E2.bias = m->P + kOffB2;
    E2.outH = m->H2;
    return gemm_bf16_tn(m->H1, m->W2h, rowsPad, kMlpHidden, kMlpHidden, E2, s);
}

// Loss and gradients (into m->G) of one padded batch; the loss sum is added to *m->loss.
cudaError_t batch_gradients(fg_mlp *m, const uint64_t *F, const float *L, const int *idx, int first, int rows,
                            int rowsPad) {
    cudaStream_t s = m->stream;
    cudaError_t e = forward(m, F, idx, first, rows, rowsPad);
    if (e) return e;
    k_labels<<<(rowsPad + 255) / 256, 256, 0, s>>>(L, idx, first, rows, rowsPad, m->lab);
    if ((e = cudaMemsetAsync(m->G, 0, sizeof(float) * kMlpParams, s))) return e;
    k_head<<<(rowsPad * 32 + 255) / 256, 256, 0, s>>>(m->H2, m->P, m->lab, rowsPad, 1.0f / (float)rows, m->scores,
                                                      m->ds, m->dZ2, m->loss);
    k_head_grads<<<rowsPad / 128, kMlpHidden, 0, s>>>(m->H2, m->ds, rowsPad, m->G + kOffW3, m->G + kOffB3);
    // dZ1 = (dZ2 W2) masked by H1 > 0
    GemmEpilogue E3 = epi(EPI_MASK_BF16, rowsPad, kMlpHidden);
    E3.mask = m->H1;
    E3.outH = m->dZ1;
    E3.err = m->err;
    if ((e = gemm_bf16_tn(m->dZ2, m->W2th, rowsPad, kMlpHidden, kMlpHidden, E3, s))) return e;
    const dim3 tb(32, 8);
    k_transpose<<<dim3(kMlpHidden / 32, rowsPad / 32), tb, 0, s>>>(m->dZ2, rowsPad, kMlpHidden, m->dZ2T);
    k_transpose<<<dim3(kMlpHidden / 32, rowsPad / 32), tb, 0, s>>>(m->H1, rowsPad, kMlpHidden, m->H1T);
    k_transpose<<<dim3(kMlpHidden / 32, rowsPad / 32), tb, 0, s>>>(m->dZ1, rowsPad, kMlpHidden, m->dZ1T);
    k_transpose<<<dim3(kMlpIn / 32, rowsPad / 32), tb, 0, s>>>(m->X, rowsPad, kMlpIn, m->XT);
    if ((e = cudaGetLastError())) return e;
    GemmEpilogue E4 = epi(EPI_F32, kMlpHidden, kMlpHidden);
    E4.outF = m->G + kOffW2;
    E4.err = m->err;
    if ((e = gemm_bf16_tn(m->dZ2T, m->H1T, kMlpHidden, kMlpHidden, rowsPad, E4, s))) return e;
    GemmEpilogue E5 = epi(EPI_F32, kMlpHidden, kMlpIn);
    E5.outF = m->G + kOffW1;
    E5.err = m->err;
    if ((e = gemm_bf16_tn(m->dZ1T, m->XT, kMlpHidden, kMlpIn, rowsPad, E5, s))) return e;
    k_rowsum<<<kMlpHidden * 32 / 256, 256, 0, s>>>(m->dZ2T, kMlpHidden, rowsPad, m->G + kOffB2);
    k_rowsum<<<kMlpHidden * 32 / 256, 256, 0, s>>>(m->dZ1T, kMlpHidden, rowsPad, m->G + kOffB1);
    return cudaGetLastError();
}

cudaError_t adam_step(fg_mlp *m, float lr) {
    m->adamStep++;
    const float c1 = 1.0f / (1.0f - powf(0.9f, (float)m->adamStep)), c2 = 1.0f / (1.0f - powf(0.999f, (float)m->adamStep));
    k_adam<<<(kMlpParams + 255) / 256, 256, 0, m->stream>>>(m->P, m->G, m->Am, m->Av, kMlpParams, lr, c1, c2);
    cudaError_t e = cudaGetLastError();
    return e ? e : refresh(m);
}

fg_status mfail(fg_status s, const char *msg) {
    last_error() = msg;
    return s;
}
#define MCUDA(call)                                                             \
    do {                                                                        \
        cudaError_t e_ = (call);                                                \
        if (e_ != cudaSuccess) return mfail(FG_ERR_CUDA, cudaGetErrorString(e_)); \
    } while (0)

fg_status check_err(fg_mlp *m) {
    int err = 0;
    MCUDA(cudaMemcpyAsync(&err, m->err, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
    MCUDA(cudaStreamSynchronize(m->stream));
    if (err) return mfail(FG_ERR_CUDA, "tensor-core GEMM timed out waiting on a barrier");
    return FG_OK;
}

}  // namespace

unsigned long long mlp_workspace_epoch(const fg_mlp *m) { return m ? m->epoch : 0ull; }

cudaError_t mlp_score_device(fg_mlp *m, const uint64_t *features, int rows, float *scores, cudaStream_t s) {
    const int rowsPad = (rows + 127) / 128 * 128;
    cudaStream_t keep = m->stream;
    cudaError_t e = ensure_workspace(m, rowsPad);
    if (e) return e;
    m->stream = s;
    e = forward(m, features, nullptr, 0, rows, rowsPad);
    if (!e) {
        k_head<<<(rowsPad * 32 + 255) / 256, 256, 0, s>>>(m->H2, m->P, nullptr, rowsPad, 0.0f, m->scores, nullptr,
                                                          nullptr, nullptr);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemcpyAsync(scores, m->scores, sizeof(float) * rows, cudaMemcpyDeviceToDevice, s);
    m->stream = keep;
    return e;
}

}  // namespace fg

using namespace fg;

extern "C" {

fg_status fg_mlp_create(int device, uint64_t seed, fg_mlp **out) {
    if (!out) return mfail(FG_ERR_ARG, "null argument");
    *out = nullptr;
    MCUDA(cudaSetDevice(device));
    fg_mlp *m = new fg_mlp;
    m->dev = device;
    cudaError_t e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    if (!e) e = dalloc(&m->P, kMlpParams);
    if (!e) e = dalloc(&m->G, kMlpParams);
    if (!e) e = dalloc(&m->Am, kMlpParams);
    if (!e) e = dalloc(&m->Av, kMlpParams);
    if (!e) e = dalloc(&m->W1h, (size_t)kMlpHidden * kMlpIn);
    if (!e) e = dalloc(&m->W2h, (size_t)kMlpHidden * kMlpHidden);
    if (!e) e = dalloc(&m->W2th, (size_t)kMlpHidden * kMlpHidden);
    if (!e) e = dalloc(&m->loss, 1);
    if (!e) e = dalloc(&m->err, 1);
    if (!e) e = cudaMemset(m->err, 0, sizeof(int));
    if (!e) e = cudaMemset(m->Am, 0, sizeof(float) * kMlpParams);
    if (!e) e = cudaMemset(m->Av, 0, sizeof(float) * kMlpParams);
    if (e) {
        fg_mlp_destroy(m);
        return mfail(FG_ERR_CUDA, cudaGetErrorString(e));
    }
    // He-uniform initialisation from a seeded generator; biases zero.
    std::vector<float> p(kMlpParams, 0.0f);
    std::mt19937_64 g(seed);
    std::uniform_real_distribution<float> u(-1.0f, 1.0f);
    for (int i = 0; i < kMlpHidden * kMlpIn; i++) p[kOffW1 + i] = u(g) * sqrtf(6.0f / kMlpIn);
    for (int i = 0; i < kMlpHidden * kMlpHidden; i++) p[kOffW2 + i] = u(g) * sqrtf(6.0f / kMlpHidden);
    for (int i = 0; i < kMlpHidden; i++) p[kOffW3 + i] = u(g) * sqrtf(3.0f / kMlpHidden);
    e = cudaMemcpy(m->P, p.data(), sizeof(float) * kMlpParams, cudaMemcpyHostToDevice);
    if (!e) e = refresh(m);
    if (!e) e = cudaStreamSynchronize(m->stream);
    if (e) {
        fg_mlp_destroy(m);
        return mfail(FG_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = m;
    return FG_OK;
}

fg_status fg_mlp_destroy(fg_mlp *m) {
    if (!m) return FG_OK;
    cudaSetDevice(m->dev);
    if (m->stream) cudaStreamSynchronize(m->stream);
    free_workspace(m);
    void *ps[] = {m->P, m->G, m->Am, m->Av, m->W1h, m->W2h, m->W2th, m->loss, m->err};
    for (void *p : ps)
        if (p) cudaFree(p);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return FG_OK;
}

fg_status fg_mlp_set_params(fg_mlp *m, const float *params) {
    if (!m || !params) return mfail(FG_ERR_ARG, "null argument");
    MCUDA(cudaSetDevice(m->dev));
    MCUDA(cudaMemcpyAsync(m->P, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, m->stream));
    MCUDA(refresh(m));
    MCUDA(cudaStreamSynchronize(m->stream));
    return FG_OK;
}

fg_status fg_mlp_get_params(fg_mlp *m, float *params) {
    if (!m || !params) return mfail(FG_ERR_ARG, "null argument");
    MCUDA(cudaSetDevice(m->dev));
    MCUDA(cudaMemcpyAsync(params, m->P, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, m->stream));
    MCUDA(cudaStreamSynchronize(m->stream));
    return FG_OK;
}

int fg_mlp_param_count(void) { return kMlpParams; }

fg_status fg_mlp_gradients(fg_mlp *m, const uint64_t *features, const float *labels, int rows, float *loss,
                           float *grads) {
    if (!m || !features || !labels || !grads || rows <= 0) return mfail(FG_ERR_ARG, "bad argument");
    MCUDA(cudaSetDevice(m->dev));
    const int rowsPad = (rows + 127) / 128 * 128;
    MCUDA(ensure_workspace(m, rowsPad));
    uint64_t *dF = nullptr;
    float *dL = nullptr;
    MCUDA(dalloc(&dF, (size_t)rows * 3));
    cudaError_t e = dalloc(&dL, (size_t)rows);
    if (!e) e = cudaMemcpyAsync(dF, features, sizeof(uint64_t) * 3 * rows, cudaMemcpyHostToDevice, m->stream);
    if (!e) e = cudaMemcpyAsync(dL, labels, sizeof(float) * rows, cudaMemcpyHostToDevice, m->stream);
    if (!e) e = cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream);
    if (!e) e = batch_gradients(m, dF, dL, nullptr, 0, rows, rowsPad);
    float lsum = 0.0f;
    if (!e) e = cudaMemcpyAsync(grads, m->G, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, m->stream);
    if (!e) e = cudaMemcpyAsync(&lsum, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
    if (!e) e = cudaStreamSynchronize(m->stream);
    cudaFree(dF);
    if (dL) cudaFree(dL);
    if (e) return mfail(FG_ERR_CUDA, cudaGetErrorString(e));
    if (loss) *loss = lsum / (float)rows;
    return check_err(m);
}

fg_status fg_mlp_score(fg_mlp *m, const uint64_t *features, int rows, float *scores) {
    if (!m || !features || !scores || rows <= 0) return mfail(FG_ERR_ARG, "bad argument");
    MCUDA(cudaSetDevice(m->dev));
    uint64_t *dF = nullptr;
    float *dS = nullptr;
    MCUDA(dalloc(&dF, (size_t)rows * 3));
    cudaError_t e = dalloc(&dS, (size_t)rows);
    if (!e) e = cudaMemcpyAsync(dF, features, sizeof(uint64_t) * 3 * rows, cudaMemcpyHostToDevice, m->stream);
    if (!e) e = mlp_score_device(m, dF, rows, dS, m->stream);
    if (!e) e = cudaMemcpyAsync(scores, dS, sizeof(float) * rows, cudaMemcpyDeviceToHost, m->stream);
    if (!e) e = cudaStreamSynchronize(m->stream);
    cudaFree(dF);
    if (dS) cudaFree(dS);
    if (e) return mfail(FG_ERR_CUDA, cudaGetErrorString(e));
    return check_err(m);
}

fg_status fg_mlp_train(fg_mlp *m, const uint64_t *features, const float *labels, int64_t n, int batch, int epochs,
                       float lr, uint64_t seed, float *last_loss) {
    if (!m || !features || !labels || n <= 0 || batch <= 0 || batch % 128 || epochs <= 0 || !(lr > 0.0f))
        return mfail(FG_ERR_ARG, "bad argument (batch must be a positive multiple of 128)");
    if (n > (int64_t)0x7FFFFFFF) return mfail(FG_ERR_CAPACITY, "too many records");
    MCUDA(cudaSetDevice(m->dev));
    MCUDA(ensure_workspace(m, batch));
    uint64_t *dF = nullptr;
    float *dL = nullptr;
    int *dIdx = nullptr;
    MCUDA(dalloc(&dF, (size_t)n * 3));
    cudaError_t e = dalloc(&dL, (size_t)n);
    if (!e) e = dalloc(&dIdx, (size_t)n);
    if (!e) e = cudaMemcpyAsync(dF, features, sizeof(uint64_t) * 3 * n, cudaMemcpyHostToDevice, m->stream);
    if (!e) e = cudaMemcpyAsync(dL, labels, sizeof(float) * n, cudaMemcpyHostToDevice, m->stream);
    std::vector<int> perm((size_t)n);
    std::mt19937_64 g(seed);
    float lastLoss = 0.0f;
    for (int ep = 0; ep < epochs && !e; ep++) {
        for (int64_t i = 0; i < n; i++) perm[i] = (int)i;
        std::shuffle(perm.begin(), perm.end(), g);
        e = cudaMemcpyAsync(dIdx, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, m->stream);
        if (!e) e = cudaMemsetAsync(m->loss, 0, sizeof(float), m->stream);
        for (int64_t first = 0; first < n && !e; first += batch) {
            const int rows = (int)std::min<int64_t>(batch, n - first);
            const int rowsPad = (rows + 127) / 128 * 128;
            e = batch_gradients(m, dF, dL, dIdx, (int)first, rows, rowsPad);
            if (!e) e = adam_step(m, lr);
        }
        if (!e) e = cudaMemcpyAsync(&lastLoss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->stream);
        if (!e) e = cudaStreamSynchronize(m->stream);
    }
    cudaFree(dF);
    if (dL) cudaFree(dL);
    if (dIdx) cudaFree(dIdx);
    if (e) return mfail(FG_ERR_CUDA, cudaGetErrorString(e));
    if (last_loss) *last_loss = lastLoss / (float)n;
    return check_err(m);
}

}  // extern "C"
