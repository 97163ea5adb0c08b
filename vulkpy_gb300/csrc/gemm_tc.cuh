// Tensor-core (tcgen05) GEMM for bf16 and split-bf16x3 arithmetic.
#pragma once
#include "common.cuh"
#include "gemm_simt.cuh"

namespace vkc {

// C = act(alpha * op(A) op(B) + beta * C + bias) with fp32 A, B, C in memory
// and bf16 (or hi/lo split bf16) tensor-core products accumulated in fp32.
int gemm_tc(vkc_device_t dev, int precision, bool ta, bool tb, int64_t M, int64_t N, int64_t K, float alpha,
            const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc,
            GemmEpilogue epi);

}  // namespace vkc
