// Scalar op bodies shared by the elementwise, broadcast and nn kernels.
// Each is the float32 math of one vulkpy GLSL shader main(), written with
// CUDA's math library (no fast-math): e.g. add.comp:25, pow.comp, sign.comp.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include "../../include/vulkpy_gb300.h"

namespace vkc {

template <int OP>
__device__ __forceinline__ float binop(float a, float b) {
  if constexpr (OP == VKC_ADD) return a + b;
  else if constexpr (OP == VKC_SUB) return a - b;
  else if constexpr (OP == VKC_MUL) return a * b;
  else if constexpr (OP == VKC_DIV) return a / b;           // IEEE division (prec-div)
  else if constexpr (OP == VKC_POW) return powf(a, b);
  else if constexpr (OP == VKC_MAX) return fmaxf(a, b);
  else if constexpr (OP == VKC_MIN) return fminf(a, b);
  else if constexpr (OP == VKC_RSUB) return b - a;
  else if constexpr (OP == VKC_RDIV) return b / a;
  else if constexpr (OP == VKC_RPOW) return powf(b, a);
  else return a;
}

// Square used for x ** 2.0 (exact, numpy's fast path for a scalar exponent of 2).
__device__ __forceinline__ float square(float a) { return a * a; }

template <int OP>
__device__ __forceinline__ float unop(float x) {
  if constexpr (OP == VKC_ABS) return fabsf(x);
  else if constexpr (OP == VKC_SIGN) return x > 0.f ? 1.f : (x < 0.f ? -1.f : x);  // keeps +-0 and NaN
  else if constexpr (OP == VKC_SIN) return sinf(x);
  else if constexpr (OP == VKC_COS) return cosf(x);
  else if constexpr (OP == VKC_TAN) return tanf(x);
  else if constexpr (OP == VKC_ASIN) return asinf(x);
  else if constexpr (OP == VKC_ACOS) return acosf(x);
  else if constexpr (OP == VKC_ATAN) return atanf(x);
  else if constexpr (OP == VKC_SINH) return sinhf(x);
  else if constexpr (OP == VKC_COSH) return coshf(x);
  else if constexpr (OP == VKC_TANH) return tanhf(x);
  else if constexpr (OP == VKC_ASINH) return asinhf(x);
  else if constexpr (OP == VKC_ACOSH) return acoshf(x);
  else if constexpr (OP == VKC_ATANH) return atanhf(x);
  else if constexpr (OP == VKC_EXP) return expf(x);
  else if constexpr (OP == VKC_LOG) return logf(x);
  else if constexpr (OP == VKC_EXP2) return exp2f(x);
  else if constexpr (OP == VKC_LOG2) return log2f(x);
  else if constexpr (OP == VKC_SQRT) return sqrtf(x);        // IEEE sqrt (prec-sqrt)
  else if constexpr (OP == VKC_INVSQRT) return 1.0f / sqrtf(x);
  else return x;                                             // VKC_COPY
}

// clamp(x, lo, hi) as GLSL defines it: min(max(x, lo), hi).
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

}  // namespace vkc

// Expand F(OP) for every binary op code; used to turn a runtime op into a
// template argument.
#define VKC_DISPATCH_BINARY(op, F)                 \
  switch (op) {                                    \
    case VKC_ADD: F(VKC_ADD); break;               \
    case VKC_SUB: F(VKC_SUB); break;               \
    case VKC_MUL: F(VKC_MUL); break;               \
    case VKC_DIV: F(VKC_DIV); break;               \
    case VKC_POW: F(VKC_POW); break;               \
    case VKC_MAX: F(VKC_MAX); break;               \
    case VKC_MIN: F(VKC_MIN); break;               \
    case VKC_RSUB: F(VKC_RSUB); break;             \
    case VKC_RDIV: F(VKC_RDIV); break;             \
    case VKC_RPOW: F(VKC_RPOW); break;             \
    default: return vkc::set_error(VKC_ERR_INVALID, "unknown binary op %d", op); \
  }

#define VKC_DISPATCH_UNARY(op, F)                  \
  switch (op) {                                    \
    case VKC_ABS: F(VKC_ABS); break;               \
    case VKC_SIGN: F(VKC_SIGN); break;             \
    case VKC_SIN: F(VKC_SIN); break;               \
    case VKC_COS: F(VKC_COS); break;               \
    case VKC_TAN: F(VKC_TAN); break;               \
    case VKC_ASIN: F(VKC_ASIN); break;             \
    case VKC_ACOS: F(VKC_ACOS); break;             \
    case VKC_ATAN: F(VKC_ATAN); break;             \
    case VKC_SINH: F(VKC_SINH); break;             \
    case VKC_COSH: F(VKC_COSH); break;             \
    case VKC_TANH: F(VKC_TANH); break;             \
    case VKC_ASINH: F(VKC_ASINH); break;           \
    case VKC_ACOSH: F(VKC_ACOSH); break;           \
    case VKC_ATANH: F(VKC_ATANH); break;           \
    case VKC_EXP: F(VKC_EXP); break;               \
    case VKC_LOG: F(VKC_LOG); break;               \
    case VKC_EXP2: F(VKC_EXP2); break;             \
    case VKC_LOG2: F(VKC_LOG2); break;             \
    case VKC_SQRT: F(VKC_SQRT); break;             \
    case VKC_INVSQRT: F(VKC_INVSQRT); break;       \
    case VKC_COPY: F(VKC_COPY); break;             \
    default: return vkc::set_error(VKC_ERR_INVALID, "unknown unary op %d", op); \
  }
