// gather: flat (gather.comp:21-26) and along an axis (gather_axis.comp:24-43).
//
// Flat gather is random 4-byte reads: each index pulls a 32-byte sector, so
// the kernel is bound by sector traffic, not by the 12 algorithmic bytes per
// index.  Indices are read as uint4 and outputs written as float4.  An index
// past the end writes NaN and raises bit0 of the device error word instead
// of reading out of bounds (the shader has no check).
//
// Axis gather copies whole rows of `post` floats: output [n_idx, prev, post]
// (the reference's layout, vkarray.py:1509-1511), row (k, i) =
// a[i, idx[k], :].  The shader clamps the index to [0, axis_size], one past
// the last row (gather_axis.comp:32); here it is clamped to axis_size - 1.
#include "common.cuh"

#include <algorithm>

namespace {

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads)
k_gather(const float* a, size_t n_a, const uint32_t* idx, size_t n_idx, float* c, uint32_t* err) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t nvec = n_idx >> 2;
  const uint4* i4 = reinterpret_cast<const uint4*>(idx);
  float4* c4 = reinterpret_cast<float4*>(c);
  bool bad = false;
  auto load = [&](uint32_t j) -> float {
    if ((size_t)j < n_a) return __ldg(a + j);
    bad = true;
    return __int_as_float(0x7fc00000);
  };
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  // two index vectors per iteration: 8 independent random reads in flight
  for (; i + stride < nvec; i += 2 * stride) {
    const uint4 j0 = i4[i], j1 = i4[i + stride];
    float4 v0, v1;
    v0.x = load(j0.x);
    v0.y = load(j0.y);
    v0.z = load(j0.z);
    v0.w = load(j0.w);
    v1.x = load(j1.x);
    v1.y = load(j1.y);
    v1.z = load(j1.z);
    v1.w = load(j1.w);
    c4[i] = v0;
    c4[i + stride] = v1;
  }
  for (; i < nvec; i += stride) {
    const uint4 j = i4[i];
    float4 v;
    v.x = load(j.x);
    v.y = load(j.y);
    v.z = load(j.z);
    v.w = load(j.w);
    c4[i] = v;
  }
  size_t t = (nvec << 2) + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n_idx) c[t] = load(idx[t]);
  if (bad) atomicOr(err, 1u);
}

__global__ void __launch_bounds__(kThreads)
k_gather_scalar(const float* a, size_t n_a, const uint32_t* idx, size_t n_idx, float* c, uint32_t* err) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  bool bad = false;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_idx; i += stride) {
    uint32_t j = idx[i];
    if ((size_t)j < n_a) {
      c[i] = a[j];
    } else {
      c[i] = __int_as_float(0x7fc00000);
      bad = true;
    }
  }
  if (bad) atomicOr(err, 1u);
}

// One block-row unit per (k, i); `post` floats copied with float4 when aligned.
template <bool VEC>
__global__ void __launch_bounds__(kThreads)
k_gather_axis(const float* a, size_t prev, size_t axis, size_t post, const uint32_t* idx, size_t n_idx,
              float* c) {
  const size_t rows = n_idx * prev;
  for (size_t u = blockIdx.x; u < rows; u += gridDim.x) {
    const size_t k = u / prev, i = u % prev;
    uint32_t j = idx[k];
    size_t jj = (size_t)j < axis ? (size_t)j : axis - 1;
    const float* src = a + (i * axis + jj) * post;
    float* dst = c + (k * prev + i) * post;
    if (VEC) {
      const float4* s4 = reinterpret_cast<const float4*>(src);
      float4* d4 = reinterpret_cast<float4*>(dst);
      for (size_t t = threadIdx.x; t < (post >> 2); t += kThreads) d4[t] = s4[t];
    } else {
      for (size_t t = threadIdx.x; t < post; t += kThreads) dst[t] = src[t];
    }
  }
}

// Small rows: one element per thread.
__global__ void __launch_bounds__(kThreads)
k_gather_axis_elem(const float* a, size_t prev, size_t axis, size_t post, const uint32_t* idx, size_t n_idx,
                   float* c) {
  const size_t total = n_idx * prev * post;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
    size_t j = e % post;
    size_t r = e / post;
    size_t i = r % prev, k = r / prev;
    uint32_t q = idx[k];
    size_t qq = (size_t)q < axis ? (size_t)q : axis - 1;
    c[e] = a[(i * axis + qq) * post + j];
  }
}

}  // namespace

VKC_EXPORT int vkc_gather(vkc_device_t dev, const float* a, size_t n_a, const uint32_t* idx, size_t n_idx,
                          float* c) {
  VKC_BIND(dev);
  if (n_idx == 0) return VKC_OK;
  VKC_REQUIRE(a && idx && c, "NULL buffer");
  const bool vec = ((((uintptr_t)idx) | ((uintptr_t)c)) & 15u) == 0;
  if (vec) {
    unsigned grid = vkc::wave_grid(dev, k_gather, (n_idx >> 3) + 1, kThreads);
    k_gather<<<grid, kThreads, 0, dev->stream>>>(a, n_a, idx, n_idx, c, dev->err_word);
  } else {
    unsigned grid = vkc::wave_grid(dev, k_gather_scalar, n_idx, kThreads);
    k_gather_scalar<<<grid, kThreads, 0, dev->stream>>>(a, n_a, idx, n_idx, c, dev->err_word);
  }
  return vkc::check_launch("gather");
}

VKC_EXPORT int vkc_gather_axis(vkc_device_t dev, const float* a, size_t prev, size_t axis, size_t post,
                               const uint32_t* idx, size_t n_idx, float* c) {
  VKC_BIND(dev);
  if (n_idx == 0 || prev == 0 || post == 0) return VKC_OK;
  VKC_REQUIRE(a && idx && c, "NULL buffer");
  VKC_REQUIRE(axis > 0, "gather along an empty axis");
  if (post >= 64) {
    const bool vec = (post % 4 == 0) && ((((uintptr_t)a) | ((uintptr_t)c)) & 15u) == 0;
    size_t rows = n_idx * prev;
    unsigned grid = (unsigned)std::min<size_t>(rows, (size_t)dev->sm_count * 16);
    if (vec) k_gather_axis<true><<<grid, kThreads, 0, dev->stream>>>(a, prev, axis, post, idx, n_idx, c);
    else k_gather_axis<false><<<grid, kThreads, 0, dev->stream>>>(a, prev, axis, post, idx, n_idx, c);
  } else {
    unsigned grid = vkc::stream_grid(dev, n_idx * prev * post, kThreads);
    k_gather_axis_elem<<<grid, kThreads, 0, dev->stream>>>(a, prev, axis, post, idx, n_idx, c);
  }
  return vkc::check_launch("gather_axis");
}
