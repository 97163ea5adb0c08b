// numpy broadcasting for binary ops, clamp and broadcast_to.
//
// The reference passes all three shapes in a uint buffer and every
// invocation walks ndim dims with a div/mod each (add_broadcast.comp:25-45,
// broadcast.comp:25-44).  Here the host first computes element strides
// (0 on broadcast dims), drops unit dims and merges adjacent dims that are
// contiguous for every operand, which turns most cases into one or two
// dims.  The kernel then works on rows of the innermost dim: the per-row
// operand offsets are computed once per 4096-element chunk and the inner
// loop is a plain 128-bit stream with a stride of 1 (or 0: a per-row scalar).
#include "common.cuh"
#include "ops.cuh"

#include <algorithm>

namespace {

constexpr int kThreads = 256;
constexpr int kMaxDims = 16;
constexpr int kMaxIn = 3;
constexpr int kChunkVec = 4;  // float4 per thread per unit in the 128-bit row kernel

struct Geom {
  int nd = 0;                      // collapsed dims, innermost last
  int64_t shape[kMaxDims];
  int64_t stride[kMaxIn][kMaxDims];
};

// Build collapsed geometry.  Returns VKC_OK or VKC_ERR_INVALID.
int make_geom(int ndim, const int64_t* c_shape, int nin, const int64_t* const* in_shape, Geom& g) {
  VKC_REQUIRE(ndim >= 0 && ndim <= 64, "ndim %d out of range", ndim);
  int64_t st[kMaxIn][64];
  for (int k = 0; k < nin; ++k) {
    int64_t run = 1;
    for (int d = ndim - 1; d >= 0; --d) {
      int64_t s = in_shape[k][d];
      VKC_REQUIRE(s >= 1 && (s == c_shape[d] || s == 1),
                  "operand %d dim %d (size %lld) cannot broadcast to %lld", k, d, (long long)s,
                  (long long)c_shape[d]);
      st[k][d] = (s == 1) ? 0 : run;
      run *= s;
    }
  }
  // keep non-unit output dims
  int64_t sh[64];
  int64_t s2[kMaxIn][64];
  int m = 0;
  for (int d = 0; d < ndim; ++d) {
    VKC_REQUIRE(c_shape[d] >= 0, "negative dim");
    if (c_shape[d] == 1) continue;
    sh[m] = c_shape[d];
    for (int k = 0; k < nin; ++k) s2[k][m] = st[k][d];
    ++m;
  }
  if (m == 0) {  // scalar-shaped output
    sh[0] = 1;
    for (int k = 0; k < nin; ++k) s2[k][0] = 0;
    m = 1;
  }
  // merge from the innermost dim outwards
  int64_t osh[64];
  int64_t ost[kMaxIn][64];
  int o = 0;
  osh[0] = sh[m - 1];
  for (int k = 0; k < nin; ++k) ost[k][0] = s2[k][m - 1];
  for (int d = m - 2; d >= 0; --d) {
    bool ok = true;
    for (int k = 0; k < nin; ++k)
      if (s2[k][d] != ost[k][o] * osh[o]) ok = false;
    if (ok) {
      osh[o] *= sh[d];
    } else {
      ++o;
      osh[o] = sh[d];
      for (int k = 0; k < nin; ++k) ost[k][o] = s2[k][d];
    }
  }
  int nd = o + 1;
  VKC_REQUIRE(nd <= kMaxDims, "broadcast needs %d distinct dims (max %d)", nd, kMaxDims);
  g.nd = nd;
  for (int d = 0; d < nd; ++d) {  // reverse into outermost-first order
    g.shape[d] = osh[nd - 1 - d];
    for (int k = 0; k < kMaxIn; ++k) g.stride[k][d] = (k < nin) ? ost[k][nd - 1 - d] : 0;
  }
  return VKC_OK;
}

template <int NIN>
__device__ __forceinline__ void row_offsets(const Geom& g, int64_t row, int64_t (&off)[kMaxIn]) {
#pragma unroll
  for (int k = 0; k < kMaxIn; ++k) off[k] = 0;
  for (int d = g.nd - 2; d >= 0; --d) {
    int64_t n = g.shape[d];
    int64_t idx = row % n;
    row /= n;
#pragma unroll
    for (int k = 0; k < NIN; ++k) off[k] += idx * g.stride[k][d];
  }
}

template <int OP>
struct BinOp;

// float4 loads per thread issued ahead of their stores in the 128-bit row
// kernel: the long ops (IEEE division, powf) need more bytes in flight per
// thread to keep HBM busy (X / row on 8192 x 32768: 394 -> 333 us); the
// one-instruction ops stream fastest with one (more resident warps).
template <class Op>
struct LoadGroup {
  static constexpr int value = 1;
};
template <>
struct LoadGroup<BinOp<VKC_DIV>> {
  static constexpr int value = kChunkVec;
};
template <>
struct LoadGroup<BinOp<VKC_POW>> {
  static constexpr int value = kChunkVec;
};
template <>
struct LoadGroup<BinOp<VKC_RDIV>> {
  static constexpr int value = kChunkVec;
};
template <>
struct LoadGroup<BinOp<VKC_RPOW>> {
  static constexpr int value = kChunkVec;
};

// Rows of the innermost dim; VEC: inner % 4 == 0, 128-bit loads/stores.
template <int NIN, bool VEC, class Op>
__global__ void __launch_bounds__(kThreads)
k_bcast_rows(Geom g, const float* in0, const float* in1, const float* in2, float* out, int64_t rows,
             int64_t inner, int64_t chunk, int64_t chunks_per_row, Op op) {
  const float* in[kMaxIn] = {in0, in1, in2};
  const int64_t units = rows * chunks_per_row;
  bool inner_bc[kMaxIn];
#pragma unroll
  for (int k = 0; k < kMaxIn; ++k) inner_bc[k] = (g.stride[k][g.nd - 1] == 0);
  for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
    const int64_t row = u / chunks_per_row;
    const int64_t j0 = (u % chunks_per_row) * chunk;
    const int64_t j1 = min(j0 + chunk, inner);
    int64_t off[kMaxIn];
    row_offsets<NIN>(g, row, off);
    float* o = out + row * inner;
    if (VEC) {
      float s[kMaxIn] = {0.f, 0.f, 0.f};
#pragma unroll
      for (int k = 0; k < NIN; ++k)
        if (inner_bc[k]) s[k] = in[k][off[k]];
      constexpr int G = LoadGroup<Op>::value;
      if (G > 1 && j1 - j0 == kChunkVec * 4 * kThreads) {
        // a full chunk in groups of G float4 per thread, each group's loads
        // issued before its stores (the output may be one of the inputs,
        // element for element, so the compiler cannot hoist them itself)
#pragma unroll
        for (int g0 = 0; g0 < kChunkVec; g0 += G) {
          float4 v[G][kMaxIn];
#pragma unroll
          for (int q = 0; q < G; ++q) {
            const int64_t j = j0 + 4 * threadIdx.x + (g0 + q) * 4 * kThreads;
#pragma unroll
            for (int k = 0; k < kMaxIn; ++k) {
              if (k < NIN && !inner_bc[k]) v[q][k] = *reinterpret_cast<const float4*>(in[k] + off[k] + j);
              else v[q][k] = make_float4(s[k], s[k], s[k], s[k]);
            }
          }
#pragma unroll
          for (int q = 0; q < G; ++q) {
            const int64_t j = j0 + 4 * threadIdx.x + (g0 + q) * 4 * kThreads;
            float4 r;
            r.x = op(v[q][0].x, v[q][1].x, v[q][2].x);
            r.y = op(v[q][0].y, v[q][1].y, v[q][2].y);
            r.z = op(v[q][0].z, v[q][1].z, v[q][2].z);
            r.w = op(v[q][0].w, v[q][1].w, v[q][2].w);
            __stcs(reinterpret_cast<float4*>(o + j), r);
          }
        }
        continue;
      }
      // results are stored with the streaming hint (evict first): an output
      // larger than L2 is not read again while it is still there
      for (int64_t j = j0 + 4 * threadIdx.x; j < j1; j += 4 * kThreads) {
        float4 v[kMaxIn];
#pragma unroll
        for (int k = 0; k < kMaxIn; ++k) {
          if (k < NIN && !inner_bc[k]) v[k] = *reinterpret_cast<const float4*>(in[k] + off[k] + j);
          else v[k] = make_float4(s[k], s[k], s[k], s[k]);
        }
        float4 r;
        r.x = op(v[0].x, v[1].x, v[2].x);
        r.y = op(v[0].y, v[1].y, v[2].y);
        r.z = op(v[0].z, v[1].z, v[2].z);
        r.w = op(v[0].w, v[1].w, v[2].w);
        __stcs(reinterpret_cast<float4*>(o + j), r);
      }
    } else {
      for (int64_t j = j0 + threadIdx.x; j < j1; j += kThreads) {
        float v[kMaxIn] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int k = 0; k < NIN; ++k) v[k] = in[k][off[k] + (inner_bc[k] ? 0 : j)];
        o[j] = op(v[0], v[1], v[2]);
      }
    }
  }
}

// Small inner dim: one element per thread, full index decomposition.
template <int NIN, class Op>
__global__ void __launch_bounds__(kThreads)
k_bcast_elem(Geom g, const float* in0, const float* in1, const float* in2, float* out, int64_t total, Op op) {
  const float* in[kMaxIn] = {in0, in1, in2};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
    int64_t r = i;
    int64_t off[kMaxIn] = {0, 0, 0};
    for (int d = g.nd - 1; d >= 0; --d) {
      int64_t n = g.shape[d];
      int64_t idx = r % n;
      r /= n;
#pragma unroll
      for (int k = 0; k < NIN; ++k) off[k] += idx * g.stride[k][d];
    }
    float v[kMaxIn] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < NIN; ++k) v[k] = in[k][off[k]];
    out[i] = op(v[0], v[1], v[2]);
  }
}

template <int OP>
struct BinOp {
  __device__ float operator()(float a, float b, float) const { return vkc::binop<OP>(a, b); }
};
struct CopyOp {
  __device__ float operator()(float a, float, float) const { return a; }
};
struct ClampOp3 {
  __device__ float operator()(float a, float lo, float hi) const { return vkc::clampf(a, lo, hi); }
};

template <int NIN, class Op>
int launch_bcast(vkc_device_t dev, const Geom& g, const float* a, const float* b, const float* c, float* out,
                 Op op) {
  int64_t inner = g.shape[g.nd - 1];
  int64_t total = inner;
  for (int d = 0; d < g.nd - 1; ++d) total *= g.shape[d];
  if (total == 0) return VKC_OK;
  int64_t rows = total / inner;
  // Only operands streamed along the inner dim need 16-byte alignment; a
  // per-row scalar operand (inner stride 0) is read with a scalar load.
  uintptr_t bits = (uintptr_t)out;
  const float* ins[kMaxIn] = {a, b, c};
  for (int k = 0; k < NIN; ++k)
    if (g.stride[k][g.nd - 1] != 0) bits |= (uintptr_t)ins[k];
  const bool aligned = (bits & 15u) == 0;
  if (inner >= 64) {
    bool vec = (inner % 4 == 0) && aligned;
    int64_t chunk = vec ? kChunkVec * 4 * kThreads : kThreads * 8;
    int64_t cpr = (inner + chunk - 1) / chunk;
    // one unit (chunk) per block at a time: the grid is the units, capped at
    // one wave of resident blocks
    const size_t units = (size_t)(rows * cpr);
    if (vec) {
      unsigned grid = vkc::wave_grid(dev, k_bcast_rows<NIN, true, Op>, units * kThreads, kThreads);
      k_bcast_rows<NIN, true><<<grid, kThreads, 0, dev->stream>>>(g, a, b, c, out, rows, inner, chunk, cpr, op);
    } else {
      unsigned grid = vkc::wave_grid(dev, k_bcast_rows<NIN, false, Op>, units * kThreads, kThreads);
      k_bcast_rows<NIN, false><<<grid, kThreads, 0, dev->stream>>>(g, a, b, c, out, rows, inner, chunk, cpr, op);
    }
  } else {
    unsigned grid = vkc::wave_grid(dev, k_bcast_elem<NIN, Op>, (size_t)total, kThreads);
    k_bcast_elem<NIN><<<grid, kThreads, 0, dev->stream>>>(g, a, b, c, out, total, op);
  }
  return vkc::check_launch("broadcast");
}

}  // namespace

VKC_EXPORT int vkc_broadcast_binary(vkc_device_t dev, int op, const float* a, const int64_t* a_shape,
                                    const float* b, const int64_t* b_shape, float* c,
                                    const int64_t* c_shape, int ndim) {
  VKC_BIND(dev);
  VKC_REQUIRE(a && b && c && a_shape && b_shape && c_shape, "NULL argument");
  VKC_REQUIRE(op >= VKC_ADD && op <= VKC_MIN, "broadcast op %d not supported", op);
  const int64_t* shapes[2] = {a_shape, b_shape};
  Geom g;
  int r = make_geom(ndim, c_shape, 2, shapes, g);
  if (r != VKC_OK) return r;
#define F(OP) return launch_bcast<2>(dev, g, a, b, nullptr, c, BinOp<OP>{})
  VKC_DISPATCH_BINARY(op, F);
#undef F
  return VKC_OK;
}

VKC_EXPORT int vkc_broadcast_clamp(vkc_device_t dev, const float* a, const int64_t* a_shape,
                                   const float* lo, const int64_t* lo_shape, float lo_s,
                                   const float* hi, const int64_t* hi_shape, float hi_s,
                                   float* c, const int64_t* c_shape, int ndim) {
  VKC_BIND(dev);
  VKC_REQUIRE(a && c && a_shape && c_shape, "NULL argument");
  VKC_REQUIRE((!lo || lo_shape) && (!hi || hi_shape), "array bound without a shape");
  // Scalars become 1-element device-free operands: use a shape of all ones
  // and point at a device constant written here.
  float* consts = nullptr;
  if (!lo || !hi) {
    int r = vkc::scratch_alloc(dev, 2 * sizeof(float), (void**)&consts);
    if (r != VKC_OK) return r;
    float hv[2] = {lo_s, hi_s};
    cudaError_t e = cudaMemcpyAsync(consts, hv, sizeof(hv), cudaMemcpyHostToDevice, dev->stream);
    if (e != cudaSuccess) {
      vkc::scratch_free(dev, consts);
      return vkc::set_error(VKC_ERR_CUDA, "clamp constants: %s", cudaGetErrorString(e));
    }
  }
  int64_t ones[64];
  for (int d = 0; d < 64; ++d) ones[d] = 1;
  const int64_t* shapes[3] = {a_shape, lo ? lo_shape : ones, hi ? hi_shape : ones};
  Geom g;
  int r = make_geom(ndim, c_shape, 3, shapes, g);
  if (r == VKC_OK)
    r = launch_bcast<3>(dev, g, a, lo ? lo : consts, hi ? hi : consts + 1, c, ClampOp3{});
  vkc::scratch_free(dev, consts);
  return r;
}

VKC_EXPORT int vkc_broadcast_to(vkc_device_t dev, const float* a, const int64_t* a_shape, float* c,
                                const int64_t* c_shape, int ndim) {
  VKC_BIND(dev);
  VKC_REQUIRE(a && c && a_shape && c_shape, "NULL argument");
  const int64_t* shapes[1] = {a_shape};
  Geom g;
  int r = make_geom(ndim, c_shape, 1, shapes, g);
  if (r != VKC_OK) return r;
  return launch_bcast<1>(dev, g, a, nullptr, nullptr, c, CopyOp{});
}
