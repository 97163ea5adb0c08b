// matmul / gemm entry points: dispatch on the requested arithmetic.
// vkarray.py:585-605 + matmul.comp:23-33 (C[M,N] = A[M,K] B[K,N], fp32).
#include "common.cuh"
#include "gemm_simt.cuh"
#include "gemm_tc.cuh"

VKC_EXPORT int vkc_gemm(vkc_device_t dev, int precision, int trans_a, int trans_b, int64_t m, int64_t n, int64_t k,
                        float alpha, const float* a, int64_t lda, const float* b, int64_t ldb, float beta, float* c,
                        int64_t ldc) {
  VKC_BIND(dev);
  VKC_REQUIRE(m >= 0 && n >= 0 && k >= 0, "negative matmul size");
  if (m == 0 || n == 0) return VKC_OK;
  VKC_REQUIRE(c && (k == 0 || (a && b)), "NULL buffer");
  VKC_REQUIRE(ldc >= n, "ldc < n");
  VKC_REQUIRE(lda >= (trans_a ? m : k) && ldb >= (trans_b ? k : n), "leading dimension too small");
  // vectors (M == 1 or N == 1) in fp32 for every precision: bound by reading the matrix
  if (precision == VKC_MM_FP32 || precision == VKC_MM_BF16 || precision == VKC_MM_BF16X3) {
    const int r = vkc::gemm_as_gemv(dev, trans_a != 0, trans_b != 0, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc,
                                    vkc::GemmEpilogue{});
    if (r >= 0) return r;
  }
  switch (precision) {
    case VKC_MM_FP32:
      return vkc::gemm_simt(dev, trans_a != 0, trans_b != 0, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc,
                            vkc::GemmEpilogue{});
    case VKC_MM_BF16:
    case VKC_MM_BF16X3:
      return vkc::gemm_tc(dev, precision, trans_a != 0, trans_b != 0, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc,
                          vkc::GemmEpilogue{});
    default:
      return vkc::set_error(VKC_ERR_INVALID, "unknown matmul precision %d", precision);
  }
}

VKC_EXPORT int vkc_matmul(vkc_device_t dev, int precision, const float* a, const float* b, float* c, int64_t m,
                          int64_t k, int64_t n) {
  return vkc_gemm(dev, precision, 0, 0, m, n, k, 1.0f, a, k > 0 ? k : 1, b, n, 0.0f, c, n);
}
