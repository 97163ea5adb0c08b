// Same-shape elementwise kernels: binary, scalar, unary, clamp and fills.
// Replaces the one-float-per-invocation shaders (add.comp:20-26,
// add_scalar.comp:19-24, exp.comp:18-23, clamp*.comp, ...) with 128-bit
// vector loads/stores in a grid-stride loop sized to the SM count, two
// float4 per thread per iteration to keep enough bytes in flight for HBM3e.
#include "common.cuh"
#include "ops.cuh"

namespace {

constexpr int kThreads = 256;

// Generic elementwise map over up to three float inputs.  `out` may alias
// any input: every element is read and written by the same thread.
template <int NIN, class Op>
__global__ void __launch_bounds__(kThreads)
k_map(const float* in0, const float* in1, const float* in2, float* out, size_t n, Op op) {
  const size_t nvec = n >> 2;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const float4* a4 = reinterpret_cast<const float4*>(in0);
  const float4* b4 = reinterpret_cast<const float4*>(in1);
  const float4* c4 = reinterpret_cast<const float4*>(in2);
  float4* o4 = reinterpret_cast<float4*>(out);
  auto apply = [&](float4 x, float4 y, float4 z) {
    float4 r;
    r.x = op(x.x, y.x, z.x);
    r.y = op(x.y, y.y, z.y);
    r.z = op(x.z, y.z, z.z);
    r.w = op(x.w, y.w, z.w);
    return r;
  };
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  for (; i + stride < nvec; i += 2 * stride) {
    float4 x0 = a4[i], x1 = a4[i + stride];
    float4 y0 = zero, y1 = zero, z0 = zero, z1 = zero;
    if (NIN > 1) { y0 = b4[i]; y1 = b4[i + stride]; }
    if (NIN > 2) { z0 = c4[i]; z1 = c4[i + stride]; }
    o4[i] = apply(x0, y0, z0);
    o4[i + stride] = apply(x1, y1, z1);
  }
  for (; i < nvec; i += stride) {
    float4 x0 = a4[i], y0 = zero, z0 = zero;
    if (NIN > 1) y0 = b4[i];
    if (NIN > 2) z0 = c4[i];
    o4[i] = apply(x0, y0, z0);
  }
  // scalar tail (n % 4 elements)
  size_t t = (nvec << 2) + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) {
    out[t] = op(in0[t], NIN > 1 ? in1[t] : 0.f, NIN > 2 ? in2[t] : 0.f);
  }
}

// Unaligned fallback (pointers not 16-byte aligned).
template <int NIN, class Op>
__global__ void __launch_bounds__(kThreads)
k_map_scalar(const float* in0, const float* in1, const float* in2, float* out, size_t n, Op op) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    out[i] = op(in0[i], NIN > 1 ? in1[i] : 0.f, NIN > 2 ? in2[i] : 0.f);
}

template <int OP>
struct BinOp {
  __device__ float operator()(float a, float b, float) const { return vkc::binop<OP>(a, b); }
};
template <int OP>
struct ScalarOp {
  float s;
  __device__ float operator()(float a, float, float) const { return vkc::binop<OP>(a, s); }
};
struct SquareOp {
  __device__ float operator()(float a, float, float) const { return vkc::square(a); }
};
template <int OP>
struct UnOp {
  __device__ float operator()(float a, float, float) const { return vkc::unop<OP>(a); }
};
template <bool LO_ARR, bool HI_ARR>
struct ClampOp {
  float lo, hi;
  __device__ float operator()(float a, float l, float h) const {
    return vkc::clampf(a, LO_ARR ? l : lo, HI_ARR ? h : hi);
  }
};
// clamp with only an upper array bound passes it in the second slot.
struct ClampHiOnly {
  float lo;
  __device__ float operator()(float a, float h, float) const { return vkc::clampf(a, lo, h); }
};

inline bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

template <int NIN, class Op>
int launch_map(vkc_device_t dev, const float* a, const float* b, const float* c, float* out,
               size_t n, Op op, const char* what) {
  if (n == 0) return VKC_OK;
  bool vec = aligned16(a) && aligned16(out) && (NIN < 2 || aligned16(b)) && (NIN < 3 || aligned16(c));
  if (vec) {
    size_t items = (n >> 2) / 2 + 1;
    unsigned grid = vkc::wave_grid(dev, k_map<NIN, Op>, items, kThreads);
    k_map<NIN><<<grid, kThreads, 0, dev->stream>>>(a, b, c, out, n, op);
  } else {
    unsigned grid = vkc::wave_grid(dev, k_map_scalar<NIN, Op>, n, kThreads);
    k_map_scalar<NIN><<<grid, kThreads, 0, dev->stream>>>(a, b, c, out, n, op);
  }
  return vkc::check_launch(what);
}

template <class T>
__global__ void k_fill(T* p, size_t n, T v) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) p[i] = v;
}

template <class T>
__global__ void k_fill4(T* p, size_t n, T v) {
  // 16-byte stores; T is 4 bytes wide.
  const size_t nvec = n >> 2;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  uint4* p4 = reinterpret_cast<uint4*>(p);
  uint32_t u;
  memcpy(&u, &v, 4);
  const uint4 w = make_uint4(u, u, u, u);
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i < nvec; i += stride) p4[i] = w;
  size_t t = (nvec << 2) + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) p[t] = v;
}

template <class T>
int launch_fill(vkc_device_t dev, T* p, size_t n, T v) {
  if (n == 0) return VKC_OK;
  if (aligned16(p)) {
    unsigned grid = vkc::wave_grid(dev, k_fill4<T>, (n >> 2) + 1, kThreads);
    k_fill4<T><<<grid, kThreads, 0, dev->stream>>>(p, n, v);
  } else {
    unsigned grid = vkc::wave_grid(dev, k_fill<T>, n, kThreads);
    k_fill<T><<<grid, kThreads, 0, dev->stream>>>(p, n, v);
  }
  return vkc::check_launch("fill");
}

}  // namespace

VKC_EXPORT int vkc_binary(vkc_device_t dev, int op, const float* a, const float* b, float* c, size_t n) {
  VKC_BIND(dev);
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(a && b && c, "NULL buffer");
  VKC_REQUIRE(op >= VKC_ADD && op <= VKC_MIN, "binary op %d needs two arrays of one shape", op);
#define F(OP) return launch_map<2>(dev, a, b, nullptr, c, n, BinOp<OP>{}, "binary")
  VKC_DISPATCH_BINARY(op, F);
#undef F
  return VKC_OK;
}

VKC_EXPORT int vkc_binary_scalar(vkc_device_t dev, int op, const float* a, float s, float* c, size_t n) {
  VKC_BIND(dev);
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(a && c, "NULL buffer");
  if (op == VKC_POW && s == 2.0f)
    return launch_map<1>(dev, a, nullptr, nullptr, c, n, SquareOp{}, "square");
#define F(OP) return launch_map<1>(dev, a, nullptr, nullptr, c, n, ScalarOp<OP>{s}, "binary_scalar")
  VKC_DISPATCH_BINARY(op, F);
#undef F
  return VKC_OK;
}

VKC_EXPORT int vkc_unary(vkc_device_t dev, int op, const float* a, float* c, size_t n) {
  VKC_BIND(dev);
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(a && c, "NULL buffer");
#define F(OP) return launch_map<1>(dev, a, nullptr, nullptr, c, n, UnOp<OP>{}, "unary")
  VKC_DISPATCH_UNARY(op, F);
#undef F
  return VKC_OK;
}

VKC_EXPORT int vkc_clamp(vkc_device_t dev, const float* a, const float* lo_arr, const float* hi_arr,
                         float lo, float hi, float* d, size_t n) {
  VKC_BIND(dev);
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(a && d, "NULL buffer");
  if (lo_arr && hi_arr) return launch_map<3>(dev, a, lo_arr, hi_arr, d, n, ClampOp<true, true>{lo, hi}, "clamp");
  if (lo_arr) return launch_map<2>(dev, a, lo_arr, nullptr, d, n, ClampOp<true, false>{lo, hi}, "clamp_vs");
  if (hi_arr) return launch_map<2>(dev, a, hi_arr, nullptr, d, n, ClampHiOnly{lo}, "clamp_sv");
  return launch_map<1>(dev, a, nullptr, nullptr, d, n, ClampOp<false, false>{lo, hi}, "clamp_ss");
}

VKC_EXPORT int vkc_fill_f32(vkc_device_t dev, float* dst, size_t n, float v) {
  VKC_BIND(dev);
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(dst, "NULL buffer");
  return launch_fill<float>(dev, dst, n, v);
}

VKC_EXPORT int vkc_fill_u32(vkc_device_t dev, uint32_t* dst, size_t n, uint32_t v) {
  VKC_BIND(dev);
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(dst, "NULL buffer");
  return launch_fill<uint32_t>(dev, dst, n, v);
}
