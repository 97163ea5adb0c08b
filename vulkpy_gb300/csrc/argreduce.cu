// argmax / argmin over all elements or along one axis (numpy semantics: the
// first index of the extreme value; a NaN counts as the extreme, so the first
// NaN wins; -0.0 and +0.0 compare equal).  The reference lists these as not
// yet implemented (README.md:73, example/02-nn.py:96 falls back to numpy).
//
// Each candidate is one 64-bit key: an order-preserving image of the value in
// the high word and the complement of the index in the low word, so the
// maximum key is the extreme value at the smallest index and every combine is
// a plain integer max -- associative, so any tree order gives the same answer.
#include <algorithm>

#include "common.cuh"

namespace vkc {
namespace {

template <bool MIN>
__device__ __forceinline__ uint32_t order_word(float v) {
  if (v != v) return 0xFFFFFFFFu;  // NaN beats every number
  const uint32_t b = __float_as_uint(v == 0.0f ? 0.0f : v);
  const uint32_t o = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
  return MIN ? ~o : o;  // NaN handled above, so ~o < 0xFFFFFFFF
}

template <bool MIN>
__device__ __forceinline__ uint64_t make_key(float v, uint32_t i) {
  return ((uint64_t)order_word<MIN>(v) << 32) | (uint64_t)(~i);
}

__device__ __forceinline__ uint64_t kmax(uint64_t a, uint64_t b) { return a > b ? a : b; }

__device__ __forceinline__ uint64_t warp_max(uint64_t k) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) k = kmax(k, __shfl_xor_sync(0xFFFFFFFFu, k, o));
  return k;
}

// Block-wide maximum; every thread gets the result.
__device__ __forceinline__ uint64_t block_max(uint64_t k, uint64_t* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  k = warp_max(k);
  if (lane == 0) sh[w] = k;
  __syncthreads();
  k = lane < nw ? sh[lane] : 0;
  k = warp_max(k);
  __syncthreads();
  return k;
}

constexpr int kThreads = 256;

// Pass 1: each block reduces a grid-stride share of a[0..n) to one key.
template <bool MIN>
__global__ void __launch_bounds__(kThreads) k_arg_partials(const float* __restrict__ a, size_t n,
                                                           uint64_t* __restrict__ part) {
  __shared__ uint64_t sh[32];
  uint64_t best = 0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if ((((uintptr_t)a) & 15u) == 0) {
    const size_t n4 = n / 4;
    const float4* a4 = reinterpret_cast<const float4*>(a);
    for (size_t i = t; i < n4; i += 2 * stride) {
      const float4 x = __ldg(a4 + i);
      float4 y = make_float4(0.f, 0.f, 0.f, 0.f);
      const bool two = i + stride < n4;
      if (two) y = __ldg(a4 + i + stride);
      const uint32_t b0 = (uint32_t)(4 * i);
      best = kmax(best, kmax(kmax(make_key<MIN>(x.x, b0), make_key<MIN>(x.y, b0 + 1)),
                             kmax(make_key<MIN>(x.z, b0 + 2), make_key<MIN>(x.w, b0 + 3))));
      if (two) {
        const uint32_t b1 = (uint32_t)(4 * (i + stride));
        best = kmax(best, kmax(kmax(make_key<MIN>(y.x, b1), make_key<MIN>(y.y, b1 + 1)),
                               kmax(make_key<MIN>(y.z, b1 + 2), make_key<MIN>(y.w, b1 + 3))));
      }
    }
    for (size_t i = 4 * n4 + t; i < n; i += stride) best = kmax(best, make_key<MIN>(a[i], (uint32_t)i));
  } else {
    for (size_t i = t; i < n; i += stride) best = kmax(best, make_key<MIN>(__ldg(a + i), (uint32_t)i));
  }
  best = block_max(best, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = best;
}

// Pass 2: one block reduces the partial keys and writes the index.
__global__ void __launch_bounds__(1024) k_arg_final(const uint64_t* __restrict__ part, int m,
                                                   uint32_t* __restrict__ out) {
  __shared__ uint64_t sh[32];
  uint64_t best = 0;
  for (int i = threadIdx.x; i < m; i += blockDim.x) best = kmax(best, part[i]);
  best = block_max(best, sh);
  if (threadIdx.x == 0) out[0] = ~(uint32_t)best;
}

// Along a contiguous axis (post == 1): one warp per row.
template <bool MIN>
__global__ void __launch_bounds__(kThreads) k_arg_rows_warp(const float* __restrict__ a, size_t rows,
                                                            size_t len, uint32_t* __restrict__ out) {
  const size_t warps = (size_t)gridDim.x * (blockDim.x >> 5);
  const int lane = threadIdx.x & 31;
  for (size_t r = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < rows; r += warps) {
    const float* row = a + r * len;
    uint64_t best = 0;
    for (size_t k = lane; k < len; k += 32) best = kmax(best, make_key<MIN>(__ldg(row + k), (uint32_t)k));
    best = warp_max(best);
    if (lane == 0) out[r] = ~(uint32_t)best;
  }
}

// Along a long contiguous axis: one block per row.
template <bool MIN>
__global__ void __launch_bounds__(kThreads) k_arg_rows_block(const float* __restrict__ a, size_t rows,
                                                             size_t len, uint32_t* __restrict__ out) {
  __shared__ uint64_t sh[32];
  for (size_t r = blockIdx.x; r < rows; r += gridDim.x) {
    const float* row = a + r * len;
    uint64_t best = 0;
    for (size_t k = threadIdx.x; k < len; k += blockDim.x)
      best = kmax(best, make_key<MIN>(__ldg(row + k), (uint32_t)k));
    best = block_max(best, sh);
    if (threadIdx.x == 0) out[r] = ~(uint32_t)best;
  }
}

// Strided axis (post > 1): a block covers 32 adjacent columns q of one p and
// splits the axis across its 8 warps-rows; the 8 keys per column are merged
// in shared memory.  Loads are 128-byte coalesced along q.
constexpr int kColsX = 32, kColsY = 8;

template <bool MIN>
__global__ void __launch_bounds__(kColsX* kColsY) k_arg_cols(const float* __restrict__ a, size_t prev,
                                                            size_t len, size_t post,
                                                            uint32_t* __restrict__ out) {
  __shared__ uint64_t sh[kColsY][kColsX];
  const size_t qblocks = (post + kColsX - 1) / kColsX;
  for (size_t b = blockIdx.x; b < prev * qblocks; b += gridDim.x) {
    const size_t p = b / qblocks;
    const size_t q = (b % qblocks) * kColsX + threadIdx.x;
    uint64_t best = 0;
    if (q < post) {
      const float* base = a + p * len * post + q;
      for (size_t k = threadIdx.y; k < len; k += kColsY)
        best = kmax(best, make_key<MIN>(__ldg(base + k * post), (uint32_t)k));
    }
    sh[threadIdx.y][threadIdx.x] = best;
    __syncthreads();
    if (threadIdx.y == 0 && q < post) {
#pragma unroll
      for (int y = 1; y < kColsY; ++y) best = kmax(best, sh[y][threadIdx.x]);
      out[p * post + q] = ~(uint32_t)best;
    }
    __syncthreads();
  }
}

template <bool MIN>
int arg_all(vkc_device_t dev, const float* a, size_t n, uint32_t* out) {
  const unsigned g = stream_grid(dev, (n + 7) / 8, kThreads, 4);
  void* part = nullptr;
  int r = scratch_alloc(dev, (size_t)g * sizeof(uint64_t), &part);
  if (r != VKC_OK) return r;
  k_arg_partials<MIN><<<g, kThreads, 0, dev->stream>>>(a, n, static_cast<uint64_t*>(part));
  r = check_launch("argreduce partials");
  if (r == VKC_OK) {
    k_arg_final<<<1, 1024, 0, dev->stream>>>(static_cast<const uint64_t*>(part), (int)g, out);
    r = check_launch("argreduce final");
  }
  scratch_free(dev, part);
  return r;
}

template <bool MIN>
int arg_axis(vkc_device_t dev, const float* a, size_t prev, size_t len, size_t post, uint32_t* out) {
  if (post == 1) {
    if (len >= 2048) {
      const unsigned g = (unsigned)std::min<size_t>(prev, (size_t)dev->sm_count * 16);
      k_arg_rows_block<MIN><<<g, kThreads, 0, dev->stream>>>(a, prev, len, out);
    } else {
      k_arg_rows_warp<MIN><<<stream_grid(dev, prev * 32, kThreads, 8), kThreads, 0, dev->stream>>>(a, prev, len,
                                                                                                    out);
    }
    return check_launch("argreduce rows");
  }
  const size_t blocks = prev * ((post + kColsX - 1) / kColsX);
  const unsigned g = (unsigned)std::min<size_t>(blocks, (size_t)dev->sm_count * 8);
  k_arg_cols<MIN><<<g, dim3(kColsX, kColsY), 0, dev->stream>>>(a, prev, len, post, out);
  return check_launch("argreduce cols");
}

}  // namespace
}  // namespace vkc

VKC_EXPORT int vkc_arg_reduce_all(vkc_device_t dev, int op, const float* a, size_t n, uint32_t* out) {
  VKC_BIND(dev);
  VKC_REQUIRE(op == VKC_ARGMAX || op == VKC_ARGMIN, "unknown arg-reduction %d", op);
  VKC_REQUIRE(n > 0, "arg-reduction of an empty array");
  VKC_REQUIRE(n <= 0xFFFFFFFFull, "arg-reduction indices are uint32: n must be < 2^32");
  VKC_REQUIRE(a && out, "NULL buffer");
  return op == VKC_ARGMAX ? vkc::arg_all<false>(dev, a, n, out) : vkc::arg_all<true>(dev, a, n, out);
}

VKC_EXPORT int vkc_arg_reduce_axis(vkc_device_t dev, int op, const float* a, size_t prev, size_t axis, size_t post,
                                   uint32_t* out) {
  VKC_BIND(dev);
  VKC_REQUIRE(op == VKC_ARGMAX || op == VKC_ARGMIN, "unknown arg-reduction %d", op);
  VKC_REQUIRE(axis > 0, "arg-reduction along an empty axis");
  VKC_REQUIRE(axis <= 0xFFFFFFFFull, "arg-reduction indices are uint32: the axis must be < 2^32");
  if (prev == 0 || post == 0) return VKC_OK;
  VKC_REQUIRE(a && out, "NULL buffer");
  return op == VKC_ARGMAX ? vkc::arg_axis<false>(dev, a, prev, axis, post, out)
                          : vkc::arg_axis<true>(dev, a, prev, axis, post, out);
}
