// Accumulators shared by the reduction kernels (reduce.cu) and the kernels
// that fold a reduction into another op (nn.cu's fused softmax cross
// entropy): the same float32 operations wherever they run, so a fused
// kernel reproduces the separate reduction's result bit for bit.
// Internal linkage: each translation unit gets its own copy.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include "../../include/vulkpy_gb300.h"

namespace {

template <int OP>
__device__ __forceinline__ float identity() {
  if constexpr (OP == VKC_SUM) return 0.f;
  else if constexpr (OP == VKC_PROD) return 1.f;
  else if constexpr (OP == VKC_MAXIMUM) return -INFINITY;
  else return INFINITY;
}

template <int OP>
__device__ __forceinline__ float combine(float a, float b) {
  if constexpr (OP == VKC_SUM) return a + b;
  else if constexpr (OP == VKC_PROD) return a * b;
  else if constexpr (OP == VKC_MAXIMUM) return fmaxf(a, b);
  else return fminf(a, b);
}

template <int OP>
__device__ __forceinline__ double combine_d(double a, double b) {
  if constexpr (OP == VKC_SUM) return a + b;
  else if constexpr (OP == VKC_PROD) return a * b;
  else if constexpr (OP == VKC_MAXIMUM) return fmax(a, b);
  else return fmin(a, b);
}

// Accumulator: value s plus (for compensated sums) a running error term c.
template <int OP, bool COMP>
struct Acc {
  float s, c;
  __device__ __forceinline__ void init() { s = identity<OP>(); c = 0.f; }
  __device__ __forceinline__ void push(float x) {
    if constexpr (OP == VKC_SUM && COMP) {
      // Neumaier's improvement of Kahan summation.
      float t = s + x;
      c += (fabsf(s) >= fabsf(x)) ? ((s - t) + x) : ((x - t) + s);
      s = t;
    } else if constexpr (OP == VKC_PROD && COMP) {
      // Compensated product (Graillat): the exact rounding error of s*x is
      // fma(s, x, -p); c carries the accumulated error of the product.
      float p = s * x;
      float e = fmaf(s, x, -p);
      c = fmaf(c, x, e);
      s = p;
    } else {
      s = combine<OP>(s, x);
    }
  }
  __device__ __forceinline__ void merge(float os, float oc) {
    if constexpr (OP == VKC_SUM && COMP) {
      // TwoSum of the leading parts; errors add into c.
      float t = s + os;
      float bp = t - s;
      float err = (s - (t - bp)) + (os - bp);
      s = t;
      c = c + oc + err;
    } else if constexpr (OP == VKC_PROD && COMP) {
      // (s + c)(os + oc) ~ s*os + [err(s*os) + s*oc + c*os], then
      // renormalise (Fast2Sum) so |c| stays below an ulp of s and the
      // dropped c*oc term is negligible in long merge trees.
      float p = s * os;
      float e = fmaf(s, os, -p);
      float cc = fmaf(s, oc, fmaf(c, os, e));
      float t = p + cc;
      c = cc - (t - p);
      s = t;
    } else {
      s = combine<OP>(s, os);
    }
  }
  __device__ __forceinline__ float value() const { return COMP ? s + c : s; }
};

template <int OP, bool COMP>
__device__ __forceinline__ void warp_reduce(Acc<OP, COMP>& a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float os = __shfl_down_sync(0xffffffffu, a.s, o);
    float oc = COMP ? __shfl_down_sync(0xffffffffu, a.c, o) : 0.f;
    a.merge(os, oc);
  }
}

}  // namespace
