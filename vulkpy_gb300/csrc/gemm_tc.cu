// Tensor-core GEMM (tcgen05).  Not built yet: reports an error.
#include "gemm_tc.cuh"

namespace vkc {

int gemm_tc(vkc_device_t, int precision, bool, bool, int64_t, int64_t, int64_t, float, const float*, int64_t,
            const float*, int64_t, float, float*, int64_t, GemmEpilogue) {
  return set_error(VKC_ERR_INVALID, "matmul precision %d (tensor cores) is not available in this build", precision);
}

}  // namespace vkc
