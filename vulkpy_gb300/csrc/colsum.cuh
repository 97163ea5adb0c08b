// Column sums with the arithmetic of a serial loop (rows added in order,
// starting from +0), used for bias gradients (db = sum over the batch of dy,
// the reference's dy.sum(axis=0): sum_axis.comp loops over the axis in order).
//
// One 256-thread block owns 32 columns.  A thread summing its column alone
// has only a few loads in flight and waits on memory latency for every few
// rows; here the block stages 256-row chunks of its 32 columns in shared
// memory (each of the 8 warps loads 32 rows: 32 coalesced 128-byte loads in
// flight per warp) and warp 0 then adds each column from shared memory in
// row order.
#pragma once
#include <cstdint>

namespace vkc {

constexpr int kColsumRows = 256;  // rows staged per chunk
constexpr int kColsumCols = 32;   // columns per block

// Sum of y[r*ld + c0 + lane] over r in [0, rows), returned in warp 0 lane
// `lane` (0 elsewhere; columns at or beyond `cols` read as 0).  All 256
// threads of the block must call it.
__device__ __forceinline__ float colsum32(const float* __restrict__ y, int64_t rows, int64_t cols, int64_t ld,
                                          int64_t c0, float (*tile)[kColsumCols + 1]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const bool in = c0 + lane < cols;
  float s = 0.f;
  for (int64_t r0 = 0; r0 < rows; r0 += kColsumRows) {
    const int n = (int)(rows - r0 < kColsumRows ? rows - r0 : kColsumRows);
    if (n == kColsumRows) {
      // a full chunk: the warp's 32 row loads all in flight at once
      float v[kColsumRows / 8];
#pragma unroll
      for (int q = 0; q < kColsumRows / 8; ++q) v[q] = in ? y[(r0 + w + 8 * q) * ld + c0 + lane] : 0.f;
#pragma unroll
      for (int q = 0; q < kColsumRows / 8; ++q) tile[w + 8 * q][lane] = v[q];
    } else {
#pragma unroll 8
      for (int r = w; r < n; r += 8) tile[r][lane] = in ? y[(r0 + r) * ld + c0 + lane] : 0.f;
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll 32
      for (int r = 0; r < n; ++r) s += tile[r][lane];
    }
    __syncthreads();
  }
  return s;
}

}  // namespace vkc
