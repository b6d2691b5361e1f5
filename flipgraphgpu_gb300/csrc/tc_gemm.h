// Host interface of the tcgen05 GEMM (tc_gemm.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace fg {

enum { EPI_F32 = 0, EPI_BIAS_RELU_BF16 = 1, EPI_MASK_BF16 = 2 };

struct GemmEpilogue {
    int mode;     // EPI_*
    int M;        // rows actually stored (<= the padded M)
    int ldo;      // row stride of the output (and of mask), elements
    int beta;     // EPI_F32: 1 = add into outF
    const float *bias;           // EPI_BIAS_RELU_BF16: [N] or null
    const __nv_bfloat16 *mask;   // EPI_MASK_BF16: [M][ldo], zero where the output is zeroed
    float *outF;                 // EPI_F32 output
    __nv_bfloat16 *outH;         // bf16 outputs
    int *err;                    // set to 1 if a barrier wait ran out (may be null)
};

// D = A[M][K] * B[N][K]^T on the tensor cores; A, B bf16 row-major, 16-byte
// aligned; M % 128 == 0, K % 64 == 0, N % 64 == 0.
cudaError_t gemm_bf16_tn(const void *A, const void *B, int M, int N, int K, const GemmEpilogue &E, cudaStream_t s);

}  // namespace fg
