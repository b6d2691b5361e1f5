// Dense bf16 GEMM on the 5th-generation tensor cores (tcgen05), the building
// block of the learned flip proposal's MLP (forward, backward, scoring):
//
//   D[M][N] = A[M][K] * B[N][K]^T      A, B bf16 row-major (K contiguous)
//
// One CTA per 128 x BN tile, 128 threads: thread 0 streams K-blocks of 64 with
// TMA (128-byte swizzle) through a 4-stage mbarrier ring, thread 32 issues
// tcgen05.mma (M=128, N=BN, K=16) into a TMEM accumulator, and the four warps
// read it back (warp w owns TMEM lanes 32w..32w+31 = tile rows) for the fused
// epilogue: fp32 store (optionally accumulating), bias + ReLU to bf16, or a
// ReLU-derivative mask to bf16.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/flipgraph.h"
#include "launch.h"
#include "tc_gemm.cuh"
#include "tc_gemm.h"

namespace fg {

namespace {

constexpr int BM = 128, BK = 64, STAGES = 4;

template <int BN>
constexpr size_t gemm_smem_bytes() {
    return 1024 /* alignment slack */ + (size_t)STAGES * (BM + BN) * BK * 2 + 256;
}

template <int BN>
__global__ void __launch_bounds__(128, 1)
    k_gemm_tn(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, GemmEpilogue E, int K) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    __nv_bfloat16 *sa = reinterpret_cast<__nv_bfloat16 *>(base);
    __nv_bfloat16 *sb = sa + (size_t)STAGES * BM * BK;
    uint64_t *full = reinterpret_cast<uint64_t *>(sb + (size_t)STAGES * BN * BK);
    uint64_t *empty = full + STAGES;
    uint64_t *done = empty + STAGES;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
    volatile int *abort = reinterpret_cast<volatile int *>(tslot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int nk = K / BK;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(done, 1);
        *abort = 0;
        tc::fence_mbar_init();
    }
    if (warp == 0) tc::tmem_alloc(tslot, BN);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot;

    if (threadIdx.x == 0) {
        // TMA producer
        int issued = 0;
        for (int kb = 0; kb < nk; kb++) {
            const int s = kb % STAGES;
            if (kb >= STAGES && !tc::mbar_wait(&empty[s], ((kb / STAGES) - 1) & 1, abort)) break;
            tc::mbar_expect_tx(&full[s], (uint32_t)(BM + BN) * BK * 2);
            tc::tma_load_2d(sa + (size_t)s * BM * BK, &tmA, kb * BK, m0, &full[s]);
            tc::tma_load_2d(sb + (size_t)s * BN * BK, &tmB, kb * BK, n0, &full[s]);
            issued = kb + 1;
        }
        if (*abort) {
            // let the copies still in flight land before the CTA exits
            for (int kb = issued - STAGES < 0 ? 0 : issued - STAGES; kb < issued; kb++)
                for (uint32_t i = 0; i < tc::kSpinLimit && !tc::mbar_try_wait(&full[kb % STAGES], (kb / STAGES) & 1); i++) {
                }
        }
    } else if (threadIdx.x == 32) {
        // MMA issuer
        constexpr uint32_t idesc = tc::idesc_bf16_f32(BM, BN);
        for (int kb = 0; kb < nk; kb++) {
            const int s = kb % STAGES;
            if (!tc::mbar_wait(&full[s], (kb / STAGES) & 1, abort)) break;
            tc::fence_after();
            const uint64_t ad = tc::desc_sw128(tc::smem_u32(sa + (size_t)s * BM * BK));
            const uint64_t bd = tc::desc_sw128(tc::smem_u32(sb + (size_t)s * BN * BK));
#pragma unroll
            for (int k = 0; k < BK / 16; k++)  // 16 bf16 = 32 B further along the swizzled row
                tc::mma_bf16(tmem, ad + 2 * k, bd + 2 * k, idesc, (kb > 0 || k > 0) ? 1u : 0u);
            tc::mma_commit(&empty[s]);
        }
        tc::mma_commit(done);  // arrives once every MMA issued above has completed
    }
    __syncwarp();
    // Epilogue: every thread waits for the accumulator (bounded even after an abort,
    // so that no MMA is still writing TMEM when it is freed).
    bool ok = false;
    for (uint32_t i = 0; i < tc::kSpinLimit; i++)
        if (tc::mbar_try_wait(done, 0)) { ok = true; break; }
    if (!ok) *abort = 1;
    __syncthreads();  // after this no thread writes *abort: every warp takes the same branch below
    tc::fence_after();
    const bool aborted = *abort != 0;
    if (!aborted) {
        const int row = m0 + 32 * warp + lane;
        const uint32_t tl = tmem + ((uint32_t)(32 * warp) << 16);
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            float v[16];
            tc::tmem_ld16(tl + (uint32_t)c0, v);
            const int col = n0 + c0;
            if (row >= E.M) continue;
            if (E.mode == EPI_F32) {
                float *dst = E.outF + (size_t)row * E.ldo + col;
                if (E.beta) {
#pragma unroll
                    for (int q = 0; q < 16; q++) v[q] += dst[q];
                }
#pragma unroll
                for (int q = 0; q < 16; q += 4) *reinterpret_cast<float4 *>(dst + q) = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
            } else {
                if (E.mode == EPI_BIAS_RELU_BF16) {
#pragma unroll
                    for (int q = 0; q < 16; q++) v[q] = fmaxf(v[q] + (E.bias ? E.bias[col + q] : 0.0f), 0.0f);
                } else {  // EPI_MASK_BF16: keep where the mask (a ReLU output) is positive
                    const __nv_bfloat16 *mk = E.mask + (size_t)row * E.ldo + col;
#pragma unroll
                    for (int q = 0; q < 16; q++) v[q] = __bfloat162float(mk[q]) > 0.0f ? v[q] : 0.0f;
                }
                __align__(16) __nv_bfloat16 h[16];
#pragma unroll
                for (int q = 0; q < 16; q++) h[q] = __float2bfloat16_rn(v[q]);
                uint4 *dst = reinterpret_cast<uint4 *>(E.outH + (size_t)row * E.ldo + col);
                dst[0] = reinterpret_cast<const uint4 *>(h)[0];
                dst[1] = reinterpret_cast<const uint4 *>(h)[1];
            }
        }
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_free(tmem, BN);
    if (threadIdx.x == 0 && aborted && E.err) atomicExch(E.err, 1);
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// Row-major bf16 [rows][cols] matrix, box = 64 columns x box_rows rows, 128-byte swizzle.
bool make_map(CUtensorMap *m, const void *ptr, int rows, int cols, int box_rows) {
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
    cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
cudaError_t gemm_t(const void *A, const void *B, int M, int N, int K, const GemmEpilogue &E, cudaStream_t s) {
    CUtensorMap ta, tb;
    if (!make_map(&ta, A, M, K, BM) || !make_map(&tb, B, N, K, BN)) return cudaErrorInvalidValue;
    const size_t smem = gemm_smem_bytes<BN>();
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_gemm_tn<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    dim3 grid(M / BM, N / BN);
    k_gemm_tn<BN><<<grid, 128, smem, s>>>(ta, tb, E, K);
    return cudaGetLastError();
}

}  // namespace

cudaError_t gemm_bf16_tn(const void *A, const void *B, int M, int N, int K, const GemmEpilogue &E, cudaStream_t s) {
    if (M <= 0 || N <= 0 || K <= 0 || M % BM || K % BK || N % 16) return cudaErrorInvalidValue;
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15) return cudaErrorMisalignedAddress;
    if (E.mode == EPI_F32 ? !E.outF : !E.outH) return cudaErrorInvalidValue;
    if (E.mode == EPI_MASK_BF16 && !E.mask) return cudaErrorInvalidValue;
    if (E.ldo < N || E.ldo % 8) return cudaErrorInvalidValue;
    if (N % 256 == 0) return gemm_t<256>(A, B, M, N, K, E, s);
    if (N % 128 == 0) return gemm_t<128>(A, B, M, N, K, E, s);
    if (N % 64 == 0) return gemm_t<64>(A, B, M, N, K, E, s);
    return cudaErrorInvalidValue;
}

}  // namespace fg

using namespace fg;

extern "C" fg_status fg_gemm_bf16(const uint16_t *A, const uint16_t *B, const float *bias, const uint16_t *mask, int M,
                                  int N, int K, int mode, int accumulate, float *outF, uint16_t *outH, int device) {
    if (!A || !B || M <= 0 || N <= 0 || K <= 0) {
        last_error() = "bad argument";
        return FG_ERR_ARG;
    }
    if (mode < EPI_F32 || mode > EPI_MASK_BF16 || (mode == EPI_F32 ? !outF : !outH) || (mode == EPI_MASK_BF16 && !mask)) {
        last_error() = "bad epilogue arguments";
        return FG_ERR_ARG;
    }
    if (M % 128 || K % 64 || N % 64) {
        last_error() = "M must be a multiple of 128, K of 64, N of 64";
        return FG_ERR_ARG;
    }
    if (cudaSetDevice(device) != cudaSuccess) {
        last_error() = "cudaSetDevice failed";
        return FG_ERR_CUDA;
    }
    void *dA = nullptr, *dB = nullptr, *dBias = nullptr, *dMask = nullptr, *dOut = nullptr;
    int *dErr = nullptr;
    const size_t outBytes = (size_t)M * N * (mode == EPI_F32 ? 4 : 2);
    cudaError_t e = cudaMalloc(&dA, (size_t)M * K * 2);
    if (e == cudaSuccess) e = cudaMalloc(&dB, (size_t)N * K * 2);
    if (e == cudaSuccess) e = cudaMalloc(&dOut, outBytes);
    if (e == cudaSuccess) e = cudaMalloc(&dErr, sizeof(int));
    if (e == cudaSuccess && bias) e = cudaMalloc(&dBias, (size_t)N * 4);
    if (e == cudaSuccess && mask) e = cudaMalloc(&dMask, (size_t)M * N * 2);
    if (e == cudaSuccess) e = cudaMemcpy(dA, A, (size_t)M * K * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dB, B, (size_t)N * K * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && bias) e = cudaMemcpy(dBias, bias, (size_t)N * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && mask) e = cudaMemcpy(dMask, mask, (size_t)M * N * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(dErr, 0, sizeof(int));
    if (e == cudaSuccess && mode == EPI_F32 && accumulate) e = cudaMemcpy(dOut, outF, outBytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        GemmEpilogue E{};
        E.mode = mode;
        E.M = M;
        E.ldo = N;
        E.beta = accumulate;
        E.bias = static_cast<const float *>(dBias);
        E.mask = static_cast<const __nv_bfloat16 *>(dMask);
        E.outF = static_cast<float *>(dOut);
        E.outH = static_cast<__nv_bfloat16 *>(dOut);
        E.err = dErr;
        e = gemm_bf16_tn(dA, dB, M, N, K, E, 0);
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    int err = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&err, dErr, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(mode == EPI_F32 ? (void *)outF : (void *)outH, dOut, outBytes, cudaMemcpyDeviceToHost);
    void *ptrs[] = {dA, dB, dBias, dMask, dOut, dErr};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (e != cudaSuccess) {
        last_error() = cudaGetErrorString(e);
        return FG_ERR_CUDA;
    }
    if (err) {
        last_error() = "tensor-core GEMM timed out waiting on a barrier";
        return FG_ERR_CUDA;
    }
    return FG_OK;
}
