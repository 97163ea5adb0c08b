// Matrix-vector products: the M == 1 or N == 1 cases of the GEMM
// (vkarray.py:585-605 with a 1-D operand; matmul.comp:23-33 computes them
// with one invocation per output looping over K).
//
// These are bound by reading the matrix once (4 bytes per element), not by
// arithmetic, so they run in fp32 FMA for every requested precision: a
// bf16 operand pre-pass would read and write the matrix again, and a
// 128 x 128 tile GEMM would keep 127 of every 128 rows idle.
//   y[j] = act(alpha * sum_k Mat(j, k) vec[k] + beta * y[j] + bias)
// Mat is either K-contiguous (Mat(j, k) = P[j*ld + k]: one warp per output,
// 16-byte loads along k, shuffle reduction) or J-contiguous (Mat(j, k) =
// P[k*ld + j]: four outputs per thread, K split across blocks, partial sums
// added in split order by a second kernel).  Both orders are fixed, so
// results are reproducible.
#include "common.cuh"
#include "gemm_simt.cuh"

namespace vkc {
namespace {

__device__ __forceinline__ float gemv_epilogue(float s, float alpha, float beta, const float* y, bool has_bias,
                                               float b, int act) {
  float v = alpha * s;
  if (beta != 0.f) v += beta * *y;
  if (has_bias) v += b;
  if (act == VKC_ACT_RELU) v = fmaxf(v, 0.f);
  else if (act == VKC_ACT_SIGMOID) v = 1.0f / (1.0f + expf(0.0f - v));
  return v;
}

// One warp per output j; lanes stride over k.
template <bool VEC>
__global__ void __launch_bounds__(256)
k_gemv_kcontig(int64_t J, int64_t K, float alpha, const float* __restrict__ P, int64_t ld,
               const float* __restrict__ vec, int64_t vs, float beta, float* y, int64_t ys,
               const float* __restrict__ bias, int64_t bias_stride, int act) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t j = warp; j < J; j += nwarps) {
    const float* row = P + j * ld;
    float s = 0.f;
    if (VEC) {
      const int64_t k4 = K / 4;
      float4 a[4];
      int64_t q = lane;
      for (; q + 96 < k4; q += 128) {  // four 16-byte loads in flight per lane
#pragma unroll
        for (int u = 0; u < 4; ++u) a[u] = *(reinterpret_cast<const float4*>(row) + q + 32 * u);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const float4 v = *(reinterpret_cast<const float4*>(vec) + q + 32 * u);
          s = fmaf(a[u].x, v.x, s);
          s = fmaf(a[u].y, v.y, s);
          s = fmaf(a[u].z, v.z, s);
          s = fmaf(a[u].w, v.w, s);
        }
      }
      for (; q < k4; q += 32) {
        const float4 m = *(reinterpret_cast<const float4*>(row) + q);
        const float4 v = *(reinterpret_cast<const float4*>(vec) + q);
        s = fmaf(m.x, v.x, s);
        s = fmaf(m.y, v.y, s);
        s = fmaf(m.z, v.z, s);
        s = fmaf(m.w, v.w, s);
      }
      for (int64_t k = k4 * 4 + lane; k < K; k += 32) s = fmaf(row[k], vec[k], s);
    } else {
      for (int64_t k = lane; k < K; k += 32) s = fmaf(row[k], vec[k * vs], s);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
      float* out = y + j * ys;
      *out = gemv_epilogue(s, alpha, beta, out, bias != nullptr, bias ? bias[j * bias_stride] : 0.f, act);
    }
  }
}

// Four outputs per thread, rows [k0, k1) of split blockIdx.y; with one split
// the epilogue is applied here, else the raw sums go to partial[split][J].
__global__ void __launch_bounds__(256)
k_gemv_jcontig(int64_t J, int64_t K, float alpha, const float* __restrict__ P, int64_t ld,
               const float* __restrict__ vec, int64_t vs, float beta, float* y, const float* __restrict__ bias,
               int64_t bias_stride, int act, float* __restrict__ partial, int64_t span) {
  const int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 4;
  if (j >= J) return;
  const int64_t k0 = (int64_t)blockIdx.y * span, k1 = min(K, k0 + span);
  const bool full = j + 4 <= J && ((ld & 3) == 0) && ((reinterpret_cast<uintptr_t>(P) & 15u) == 0);
  float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
  if (full) {
    int64_t k = k0;
    for (; k + 7 < k1; k += 8) {  // eight rows' loads in flight
      float4 m[8];
      float v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        m[u] = *(reinterpret_cast<const float4*>(P + (k + u) * ld + j));
        v[u] = vec[(k + u) * vs];
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        s0 = fmaf(m[u].x, v[u], s0);
        s1 = fmaf(m[u].y, v[u], s1);
        s2 = fmaf(m[u].z, v[u], s2);
        s3 = fmaf(m[u].w, v[u], s3);
      }
    }
    for (; k < k1; ++k) {
      const float4 m = *(reinterpret_cast<const float4*>(P + k * ld + j));
      const float v = vec[k * vs];
      s0 = fmaf(m.x, v, s0);
      s1 = fmaf(m.y, v, s1);
      s2 = fmaf(m.z, v, s2);
      s3 = fmaf(m.w, v, s3);
    }
  } else {
    for (int64_t k = k0; k < k1; ++k) {
      const float v = vec[k * vs];
      const float* r = P + k * ld + j;
      s0 = fmaf(r[0], v, s0);
      if (j + 1 < J) s1 = fmaf(r[1], v, s1);
      if (j + 2 < J) s2 = fmaf(r[2], v, s2);
      if (j + 3 < J) s3 = fmaf(r[3], v, s3);
    }
  }
  const float s[4] = {s0, s1, s2, s3};
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    if (j + t >= J) break;
    if (partial) {
      partial[(int64_t)blockIdx.y * J + j + t] = s[t];
    } else {
      float* out = y + j + t;
      *out = gemv_epilogue(s[t], alpha, beta, out, bias != nullptr, bias ? bias[(j + t) * bias_stride] : 0.f, act);
    }
  }
}

// Aligned J-contiguous case (ld % 4 == 0, J % 4 == 0, 16-byte aligned P):
// a block owns 128 columns (lane = four columns) and rows [k0, k1) of split
// blockIdx.y, divided among its 8 warps in 8 contiguous slices; the warps'
// sums are added in warp order through shared memory.  Few splits, so the
// combine pass adds few partials.
__global__ void __launch_bounds__(256)
k_gemv_jcontig8(int64_t J, int64_t K, float alpha, const float* __restrict__ P, int64_t ld,
                const float* __restrict__ vec, int64_t vs, float beta, float* y, const float* __restrict__ bias,
                int64_t bias_stride, int act, float* __restrict__ partial, int64_t span) {
  __shared__ float4 part[8][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t j = ((int64_t)blockIdx.x * 32 + lane) * 4;
  const int64_t k0 = (int64_t)blockIdx.y * span, k1 = min(K, k0 + span);
  const int64_t sub = (k1 - k0 + 7) / 8;
  const int64_t a0 = k0 + w * sub, a1 = min(k1, a0 + sub);
  float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
  if (j < J) {
    int64_t k = a0;
    for (; k + 7 < a1; k += 8) {  // eight rows' loads in flight
      float4 m[8];
      float v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        m[u] = *(reinterpret_cast<const float4*>(P + (k + u) * ld + j));
        v[u] = vec[(k + u) * vs];
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        s.x = fmaf(m[u].x, v[u], s.x);
        s.y = fmaf(m[u].y, v[u], s.y);
        s.z = fmaf(m[u].z, v[u], s.z);
        s.w = fmaf(m[u].w, v[u], s.w);
      }
    }
    for (; k < a1; ++k) {
      const float4 m = *(reinterpret_cast<const float4*>(P + k * ld + j));
      const float v = vec[k * vs];
      s.x = fmaf(m.x, v, s.x);
      s.y = fmaf(m.y, v, s.y);
      s.z = fmaf(m.z, v, s.z);
      s.w = fmaf(m.w, v, s.w);
    }
  }
  part[w][lane] = s;
  __syncthreads();
  if (w != 0 || j >= J) return;
  float4 t = part[0][lane];
#pragma unroll
  for (int q = 1; q < 8; ++q) {
    const float4 p = part[q][lane];
    t.x += p.x;
    t.y += p.y;
    t.z += p.z;
    t.w += p.w;
  }
  if (partial) {
    *reinterpret_cast<float4*>(partial + (int64_t)blockIdx.y * J + j) = t;
  } else {
    const float r[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      float* out = y + j + q;
      *out = gemv_epilogue(r[q], alpha, beta, out, bias != nullptr, bias ? bias[(j + q) * bias_stride] : 0.f, act);
    }
  }
}

// y[j] = epilogue(sum over splits in order of partial[s][j]).
__global__ void __launch_bounds__(256)
k_gemv_combine(const float* __restrict__ partial, int splits, int64_t J, float alpha, float beta, float* y,
               const float* __restrict__ bias, int64_t bias_stride, int act) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= J) return;
  float s = 0.f;
  for (int s0 = 0; s0 < splits; s0 += 16) {  // 16 loads in flight, added in split order
    float p[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) p[t] = s0 + t < splits ? partial[(int64_t)(s0 + t) * J + j] : 0.f;
#pragma unroll
    for (int t = 0; t < 16; ++t)
      if (s0 + t < splits) s += p[t];
  }
  float* out = y + j;
  *out = gemv_epilogue(s, alpha, beta, out, bias != nullptr, bias ? bias[j * bias_stride] : 0.f, act);
}

}  // namespace

int gemv(vkc_device_t dev, bool kcontig, int64_t J, int64_t K, float alpha, const float* P, int64_t ld,
         const float* vec, int64_t vs, float beta, float* y, int64_t ys, const float* bias, int64_t bias_stride,
         int act) {
  if (J == 0) return VKC_OK;
  if (kcontig) {
    const bool vec16 = vs == 1 && ld % 4 == 0 && ((reinterpret_cast<uintptr_t>(P) | reinterpret_cast<uintptr_t>(vec)) & 15u) == 0;
    if (vec16) {
      const unsigned grid = wave_grid(dev, k_gemv_kcontig<true>, (size_t)J * 32, 256);
      k_gemv_kcontig<true><<<grid, 256, 0, dev->stream>>>(J, K, alpha, P, ld, vec, vs, beta, y, ys, bias, bias_stride,
                                                           act);
    } else {
      const unsigned grid = wave_grid(dev, k_gemv_kcontig<false>, (size_t)J * 32, 256);
      k_gemv_kcontig<false><<<grid, 256, 0, dev->stream>>>(J, K, alpha, P, ld, vec, vs, beta, y, ys, bias,
                                                            bias_stride, act);
    }
    return check_launch("gemv");
  }
  VKC_REQUIRE(ys == 1, "gemv: strided output with a J-contiguous matrix");
  if (J % 4 == 0 && ld % 4 == 0 && (reinterpret_cast<uintptr_t>(P) & 15u) == 0) {
    const int64_t blocks_x = (J + 127) / 128;
    const int64_t per_sm = resident_blocks((const void*)k_gemv_jcontig8, 256);
    int64_t splits = std::max<int64_t>(1, std::min<int64_t>((int64_t)dev->sm_count * per_sm / blocks_x, K / 64));
    splits = std::min<int64_t>(splits, 65535);
    const int64_t span = (K + splits - 1) / splits;
    splits = std::max<int64_t>(1, (K + span - 1) / span);
    float* partial = nullptr;
    if (splits > 1) {
      int r = scratch_alloc(dev, sizeof(float) * (size_t)splits * J, (void**)&partial);
      if (r != VKC_OK) return r;
    }
    k_gemv_jcontig8<<<dim3((unsigned)blocks_x, (unsigned)splits), 256, 0, dev->stream>>>(
        J, K, alpha, P, ld, vec, vs, beta, y, bias, bias_stride, act, partial, span);
    int r = check_launch("gemv");
    if (r == VKC_OK && partial) {
      k_gemv_combine<<<(unsigned)((J + 255) / 256), 256, 0, dev->stream>>>(partial, (int)splits, J, alpha, beta, y,
                                                                           bias, bias_stride, act);
      r = check_launch("gemv combine");
    }
    scratch_free(dev, partial);
    return r;
  }
  const int64_t threads = (J + 3) / 4;
  const int64_t blocks_x = (threads + 255) / 256;
  // about four 256-thread blocks per SM: each thread keeps 128 bytes of
  // loads in flight, and fewer splits leave less for the combine to add
  const int64_t want = (int64_t)dev->sm_count * 1024 / std::max<int64_t>(1, threads);
  int64_t splits = std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(want, K / 32), 65535));
  const int64_t span = (K + splits - 1) / splits;
  splits = std::max<int64_t>(1, (K + span - 1) / span);
  float* partial = nullptr;
  if (splits > 1) {
    int r = scratch_alloc(dev, sizeof(float) * (size_t)splits * J, (void**)&partial);
    if (r != VKC_OK) return r;
  }
  dim3 grid((unsigned)blocks_x, (unsigned)splits);
  k_gemv_jcontig<<<grid, 256, 0, dev->stream>>>(J, K, alpha, P, ld, vec, vs, beta, y, bias, bias_stride, act,
                                                partial, span);
  int r = check_launch("gemv");
  if (r == VKC_OK && partial) {
    k_gemv_combine<<<(unsigned)((J + 255) / 256), 256, 0, dev->stream>>>(partial, (int)splits, J, alpha, beta, y, bias,
                                                                         bias_stride, act);
    r = check_launch("gemv combine");
  }
  scratch_free(dev, partial);
  return r;
}

}  // namespace vkc
