// pt_unet.cu -- learned psi guess (no reference counterpart): BF16 implicit-GEMM convolutions
// on the tcgen05 tensor cores (pt_tc.cuh), their self-check entry point, and the U-Net built on
// them.
#include <cstring>
#include <vector>

#include "pt_internal.h"
#include "pt_tc.cuh"

namespace pt {

// plain GEMM problem: C (M x N, FP32) = A (M x K) * B (N x K)^T, BF16 row-major operands
struct GemmProb {
    int M, N, K;
    const uint16_t* A;
    const uint16_t* B;
    float* C;
    __device__ __forceinline__ uint16_t gather_a(int r, int k) const {
        return (r < M && k < K) ? A[(size_t)r * K + k] : (uint16_t)0;
    }
    __device__ __forceinline__ uint16_t gather_b(int c, int k) const { return k < K ? B[(size_t)c * K + k] : (uint16_t)0; }
    __device__ __forceinline__ void store(int r, int c, float v) const { C[(size_t)r * N + c] = v; }
};

}  // namespace pt

using namespace pt;

extern "C" int pt_tc_gemm_check(const uint16_t* A, const uint16_t* B, float* C, int M, int N, int K) {
    if (!A || !B || !C) return fail(PT_ERR_ARG, "null pointer");
    if (M <= 0 || K <= 0 || N < 16 || N > 256 || N % 16) return fail(PT_ERR_ARG, "pt_tc_gemm_check: N must be 16..256, a multiple of 16");
    uint16_t *dA = nullptr, *dB = nullptr;
    float* dC = nullptr;
    int* derr = nullptr;
    int rc = 0, herr = 0;
    const size_t smem = tc::smem_bytes(N);
    auto cleanup = [&]() {
        if (dA) cudaFree(dA);
        if (dB) cudaFree(dB);
        if (dC) cudaFree(dC);
        if (derr) cudaFree(derr);
    };
    if ((rc = cuda_check(cudaMalloc(&dA, sizeof(uint16_t) * (size_t)M * K), "gemm check")) ||
        (rc = cuda_check(cudaMalloc(&dB, sizeof(uint16_t) * (size_t)N * K), "gemm check")) ||
        (rc = cuda_check(cudaMalloc(&dC, sizeof(float) * (size_t)M * N), "gemm check")) ||
        (rc = cuda_check(cudaMalloc(&derr, sizeof(int)), "gemm check")) ||
        (rc = cuda_check(cudaMemcpy(dA, A, sizeof(uint16_t) * (size_t)M * K, cudaMemcpyHostToDevice), "gemm check")) ||
        (rc = cuda_check(cudaMemcpy(dB, B, sizeof(uint16_t) * (size_t)N * K, cudaMemcpyHostToDevice), "gemm check")) ||
        (rc = cuda_check(cudaMemset(derr, 0, sizeof(int)), "gemm check")) ||
        (rc = cuda_check(cudaFuncSetAttribute(tc::k_tc_gemm<GemmProb>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                         "gemm check"))) {
        cleanup();
        return rc;
    }
    GemmProb p{M, N, K, dA, dB, dC};
    tc::k_tc_gemm<GemmProb><<<(M + tc::kTileM - 1) / tc::kTileM, tc::kThreads, smem>>>(p, derr);
    rc = cuda_check(cudaGetLastError(), "k_tc_gemm launch");
    if (!rc) rc = cuda_check(cudaDeviceSynchronize(), "k_tc_gemm");
    if (!rc) rc = cuda_check(cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost), "gemm check");
    if (!rc) rc = cuda_check(cudaMemcpy(C, dC, sizeof(float) * (size_t)M * N, cudaMemcpyDeviceToHost), "gemm check");
    cleanup();
    if (!rc && herr) rc = fail(PT_ERR_ITER_CAP, "tensor-core GEMM: mbarrier wait gave up");
    return rc;
}
