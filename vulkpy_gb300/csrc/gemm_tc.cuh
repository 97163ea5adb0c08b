// Tensor-core (tcgen05) GEMM for bf16 and split-bf16x3 arithmetic.
#pragma once
#include "common.cuh"
#include "gemm_simt.cuh"

#include <cuda_bf16.h>

namespace vkc {

// K-major bf16 rows (pitch ldk elements, a multiple of 64) of a GEMM result,
// hi = bf16(x) and, for the split mode, lo = bf16(x - hi): the form the
// tensor-core GEMM's operand pre-pass writes, so a following GEMM can take
// the result as its op(A) without a pre-pass of its own.
struct SplitOut {
  __nv_bfloat16* hi;
  __nv_bfloat16* lo;  // NULL in bf16 mode
  int64_t ldk;
};

// C = act(alpha * op(A) op(B) + beta * C + bias) with fp32 A, B, C in memory
// and bf16 (or hi/lo split bf16) tensor-core products accumulated in fp32.
int gemm_tc(vkc_device_t dev, int precision, bool ta, bool tb, int64_t M, int64_t N, int64_t K, float alpha,
            const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc,
            GemmEpilogue epi);

// gemm_tc on operands already split ([M][Kp] and [N][Kp] K-major bf16, Kp =
// K rounded up to 64, zero past K); `out` (may be NULL) also receives C in
// that form (pitch out->ldk, zero from N on).  M, N, K > 0.
int gemm_tc_presplit(vkc_device_t dev, int precision, int64_t M, int64_t N, int64_t K, float alpha,
                     const __nv_bfloat16* a_hi, const __nv_bfloat16* a_lo, const __nv_bfloat16* b_hi,
                     const __nv_bfloat16* b_lo, float beta, float* C, int64_t ldc, const GemmEpilogue& epi,
                     const SplitOut* out);

// The operand pre-pass alone: op(A) (M x K, K contiguous iff a_kcontig) and
// op(B)^T (N x K) into K-major bf16 hi (and lo) rows of pitch Kp, one launch.
int tc_split_operands(vkc_device_t dev, const float* A, int64_t M, int64_t lda, bool a_kcontig,
                      __nv_bfloat16* a_hi, __nv_bfloat16* a_lo, const float* B, int64_t N, int64_t ldb,
                      bool b_kcontig, __nv_bfloat16* b_hi, __nv_bfloat16* b_lo, int64_t K, int64_t Kp);

}  // namespace vkc
