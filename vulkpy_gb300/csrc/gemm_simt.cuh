// FP32 SIMT GEMM: C = act(alpha * op(A) op(B) + beta * C + bias[n]).
//
// The plain-precision path of matmul.comp:23-33 (one invocation per output
// with a serial K loop and uncoalesced B reads).  128x128 block tile, K
// steps of 16, 256 threads each owning an 8x8 register tile split 4+4 in both
// directions so shared-memory reads are conflict-free float4s; the next
// K-step is prefetched into registers while the current one is multiplied
// out of a double-buffered shared tile.  Within one output the K terms are
// accumulated in order (k = 0, 1, 2, ...) with FMA.
#pragma once
#include "common.cuh"

namespace vkc {

constexpr int kGemmBM = 128, kGemmBN = 128, kGemmBK = 16, kGemmThreads = 256;

struct GemmEpilogue {
  const float* bias = nullptr;  // per output column, may be NULL
  int act = VKC_ACT_NONE;
  // then v *= act'(dmask) for dact RELU / SIGMOID (dmask: the activation's
  // output, C's layout): the backward of the activation below a Dense layer
  // fused into the GEMM that computes its input gradient
  const float* dmask = nullptr;
  int dact = VKC_ACT_NONE;
};

struct SimtSmem {
  float As[2][kGemmBK][kGemmBM];
  float Bs[2][kGemmBK][kGemmBN];
};

// ReLU backward applied to a GEMM result as the separate activation-backward
// kernel does it: v * max(sign(y), 0), one float32 multiply.
__device__ __forceinline__ float relu_mask(float v, float y) {
  float s = y > 0.f ? 1.f : (y < 0.f ? -1.f : y);
  s = fmaxf(s, 0.f);
  return __fmul_rn(s, v);
}

// v times the derivative of the activation (ReLU or sigmoid) whose output is
// y, in the float32 operations of the separate activation-backward kernel:
// ReLU as relu_mask, sigmoid (1 - y) * y * v.
__device__ __forceinline__ float act_deriv(float v, float y, int act) {
  if (act == VKC_ACT_RELU) return relu_mask(v, y);
  return __fmul_rn(__fmul_rn(__fsub_rn(1.0f, y), y), v);
}

// One 128 x 128 output tile at (m0, n0).  `mask` (may be NULL, same layout
// as C) multiplies the result by the ReLU derivative of mask[m, n].  The
// caller synchronises the block before reusing `sm` for another tile.
template <bool TA, bool TB>
__device__ __forceinline__ void simt_tile(int64_t M, int64_t N, int64_t K, float alpha, const float* __restrict__ A,
                                          int64_t lda, const float* __restrict__ B, int64_t ldb, float beta, float* C,
                                          int64_t ldc, GemmEpilogue epi, const float* __restrict__ mask, int64_t m0,
                                          int64_t n0, SimtSmem& sm) {
  auto& As = sm.As;
  auto& Bs = sm.Bs;
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;

  // Per K step each thread loads 8 elements of the A tile and 8 of the B
  // tile as two runs of 4 along the operand's contiguous index (one 16-byte
  // load each when the run is inside the matrix and aligned).
  // op(A)(m,k) = TA ? A[k*lda + m] : A[m*lda + k]; op(B)(k,n) = TB ? B[n*ldb + k] : B[k*ldb + n].
  const bool a_vec = (lda & 3) == 0 && (reinterpret_cast<uintptr_t>(A) & 15u) == 0;
  const bool b_vec = (ldb & 3) == 0 && (reinterpret_cast<uintptr_t>(B) & 15u) == 0;
  float4 ra[2], rb[2];
  // run c of 512: contiguous along k -> (row c >> 2, k 4 (c & 3)); along m/n -> (4 (c & 31), k c >> 5)
  auto load_run = [&](const float* P, int64_t ld, bool vec, bool kcontig, int64_t r0, int64_t R, int64_t k0,
                      int c) -> float4 {
    int64_t r, k;
    if (kcontig) { r = r0 + (c >> 2); k = k0 + (c & 3) * 4; }
    else { r = r0 + (c & 31) * 4; k = k0 + (c >> 5); }
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    float* pv = &v.x;
    if (kcontig) {  // P[r*ld + k .. k+3]
      if (r < R) {
        if (vec && k + 3 < K) v = *reinterpret_cast<const float4*>(P + r * ld + k);
        else
#pragma unroll
          for (int t = 0; t < 4; ++t) pv[t] = (k + t < K) ? P[r * ld + k + t] : 0.f;
      }
    } else {        // P[k*ld + r .. r+3]
      if (k < K) {
        if (vec && r + 3 < R) v = *reinterpret_cast<const float4*>(P + k * ld + r);
        else
#pragma unroll
          for (int t = 0; t < 4; ++t) pv[t] = (r + t < R) ? P[k * ld + r + t] : 0.f;
      }
    }
    return v;
  };
  auto load_a = [&](int64_t k0) {
#pragma unroll
    for (int i = 0; i < 2; ++i) ra[i] = load_run(A, lda, a_vec, !TA, m0, M, k0, tid + i * kGemmThreads);
  };
  auto load_b = [&](int64_t k0) {
#pragma unroll
    for (int i = 0; i < 2; ++i) rb[i] = load_run(B, ldb, b_vec, TB, n0, N, k0, tid + i * kGemmThreads);
  };
  auto store = [&](int buf) {
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int c = tid + i * kGemmThreads;
      if (!TA) {
        const int mm = c >> 2, kq = (c & 3) * 4;
        As[buf][kq][mm] = ra[i].x;
        As[buf][kq + 1][mm] = ra[i].y;
        As[buf][kq + 2][mm] = ra[i].z;
        As[buf][kq + 3][mm] = ra[i].w;
      } else {
        *reinterpret_cast<float4*>(&As[buf][c >> 5][(c & 31) * 4]) = ra[i];
      }
      if (TB) {
        const int nn = c >> 2, kq = (c & 3) * 4;
        Bs[buf][kq][nn] = rb[i].x;
        Bs[buf][kq + 1][nn] = rb[i].y;
        Bs[buf][kq + 2][nn] = rb[i].z;
        Bs[buf][kq + 3][nn] = rb[i].w;
      } else {
        *reinterpret_cast<float4*>(&Bs[buf][c >> 5][(c & 31) * 4]) = rb[i];
      }
    }
  };

  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;

  const int64_t ksteps = (K + kGemmBK - 1) / kGemmBK;
  load_a(0);
  load_b(0);
  store(0);
  __syncthreads();
  for (int64_t ks = 0; ks < ksteps; ++ks) {
    const int buf = ks & 1;
    if (ks + 1 < ksteps) {
      load_a((ks + 1) * kGemmBK);
      load_b((ks + 1) * kGemmBK);
    }
#pragma unroll
    for (int kk = 0; kk < kGemmBK; ++kk) {
      float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 4]);
      float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 4 + 64]);
      float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
      float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4 + 64]);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    if (ks + 1 < ksteps) {
      store(buf ^ 1);
      __syncthreads();
    }
  }

#pragma unroll
  for (int i = 0; i < 8; ++i) {
    int64_t gm = m0 + ty * 4 + (i & 3) + (i >> 2) * 64;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      int64_t gn = n0 + tx * 4 + (j & 3) + (j >> 2) * 64;
      if (gn >= N) continue;
      float v = alpha * acc[i][j];
      if (beta != 0.f) v += beta * C[gm * ldc + gn];
      if (epi.bias) v += epi.bias[gn];
      if (epi.act == VKC_ACT_RELU) v = fmaxf(v, 0.f);
      else if (epi.act == VKC_ACT_SIGMOID) v = 1.0f / (1.0f + expf(0.0f - v));
      if (mask) v = relu_mask(v, mask[gm * ldc + gn]);
      C[gm * ldc + gn] = v;
    }
  }
}

// Split-K support (gemm_tc.cu): the fp32 split count from the tuning table
// or heuristic, and the ordered reduction of the partial tiles with the
// epilogue.
int simt_splits(vkc_device_t dev, int64_t M, int64_t N, int64_t K);
int gemm_splitk_reduce(vkc_device_t dev, const float* partial, int splits, int64_t M, int64_t N, float alpha,
                       float beta, float* C, int64_t ldc, const GemmEpilogue& epi);

// K range blockIdx.z of `span` into partial[z] (M x N, raw sums).
template <bool TA, bool TB>
__global__ void __launch_bounds__(kGemmThreads, 2)
k_gemm_simt_split(int64_t M, int64_t N, int64_t K, const float* __restrict__ A, int64_t lda,
                  const float* __restrict__ B, int64_t ldb, float* partial, int64_t span) {
  __shared__ __align__(16) SimtSmem sm;
  const int64_t k0 = (int64_t)blockIdx.z * span, kk = (K - k0 < span ? K - k0 : span);
  const float* Az = A + (TA ? k0 * lda : k0);
  const float* Bz = B + (TB ? k0 : k0 * ldb);
  simt_tile<TA, TB>(M, N, kk, 1.0f, Az, lda, Bz, ldb, 0.0f, partial + (int64_t)blockIdx.z * M * N, N,
                    GemmEpilogue{}, nullptr, (int64_t)blockIdx.y * kGemmBM, (int64_t)blockIdx.x * kGemmBN, sm);
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(kGemmThreads, 2)
k_gemm_simt(int64_t M, int64_t N, int64_t K, float alpha, const float* __restrict__ A, int64_t lda,
            const float* __restrict__ B, int64_t ldb, float beta, float* C, int64_t ldc, GemmEpilogue epi) {
  __shared__ __align__(16) SimtSmem sm;
  simt_tile<TA, TB>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, epi, nullptr, (int64_t)blockIdx.y * kGemmBM,
                    (int64_t)blockIdx.x * kGemmBN, sm);
}

// Matrix-vector product (gemv.cu): y[j] = act(alpha * sum_k Mat(j, k) vec[k]
// + beta * y[j] + bias[j * bias_stride]); Mat(j, k) = P[j*ld + k] when
// `kcontig`, else P[k*ld + j]; vec[k] at vec[k * vs]; y[j] at y[j * ys].
int gemv(vkc_device_t dev, bool kcontig, int64_t J, int64_t K, float alpha, const float* P, int64_t ld,
         const float* vec, int64_t vs, float beta, float* y, int64_t ys, const float* bias, int64_t bias_stride,
         int act);

// A GEMM with M == 1 or N == 1 as a matrix-vector product; returns -1 when
// the operands do not fit gemv (the caller then runs the tiled GEMM).
inline int gemm_as_gemv(vkc_device_t dev, bool ta, bool tb, int64_t M, int64_t N, int64_t K, float alpha,
                        const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc,
                        const GemmEpilogue& epi) {
  if (K == 0 || (M != 1 && N != 1)) return -1;
  if (M == 1) {
    // y[n] = sum_k op(A)(0, k) op(B)(k, n); op(B)(k, n) = tb ? B[n*ldb + k] : B[k*ldb + n]
    return gemv(dev, tb, N, K, alpha, B, ldb, A, ta ? lda : 1, beta, C, 1, epi.bias, 1, epi.act);
  }
  // N == 1: y[m] = sum_k op(A)(m, k) op(B)(k, 0); op(A)(m, k) = ta ? A[k*lda + m] : A[m*lda + k]
  if (ta && ldc != 1) return -1;
  return gemv(dev, !ta, M, K, alpha, A, lda, B, tb ? 1 : ldb, beta, C, ldc, epi.bias, 0, epi.act);
}

inline int gemm_simt(vkc_device_t dev, bool ta, bool tb, int64_t M, int64_t N, int64_t K, float alpha,
                     const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc,
                     GemmEpilogue epi) {
  if (M == 0 || N == 0) return VKC_OK;
  dim3 grid((unsigned)((N + kGemmBN - 1) / kGemmBN), (unsigned)((M + kGemmBM - 1) / kGemmBM));
  VKC_REQUIRE(grid.y <= 65535, "matmul: M too large for the SIMT grid");
  int splits = K > 0 ? simt_splits(dev, M, N, K) : 1;
  if (splits > 1) {
    // split K when the tiles cannot fill the GPU; partials added in split order
    const int64_t span = (K + splits - 1) / splits;
    splits = (int)((K + span - 1) / span);
    float* partial = nullptr;
    int r = scratch_alloc(dev, sizeof(float) * (size_t)splits * M * N, (void**)&partial);
    if (r != VKC_OK) return r;
    dim3 g3(grid.x, grid.y, (unsigned)splits);
    if (!ta && !tb) k_gemm_simt_split<false, false><<<g3, kGemmThreads, 0, dev->stream>>>(M, N, K, A, lda, B, ldb, partial, span);
    else if (ta && !tb) k_gemm_simt_split<true, false><<<g3, kGemmThreads, 0, dev->stream>>>(M, N, K, A, lda, B, ldb, partial, span);
    else if (!ta && tb) k_gemm_simt_split<false, true><<<g3, kGemmThreads, 0, dev->stream>>>(M, N, K, A, lda, B, ldb, partial, span);
    else k_gemm_simt_split<true, true><<<g3, kGemmThreads, 0, dev->stream>>>(M, N, K, A, lda, B, ldb, partial, span);
    r = check_launch("gemm_simt split");
    if (r == VKC_OK) r = gemm_splitk_reduce(dev, partial, splits, M, N, alpha, beta, C, ldc, epi);
    scratch_free(dev, partial);
    return r;
  }
  if (!ta && !tb) k_gemm_simt<false, false><<<grid, kGemmThreads, 0, dev->stream>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, epi);
  else if (ta && !tb) k_gemm_simt<true, false><<<grid, kGemmThreads, 0, dev->stream>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, epi);
  else if (!ta && tb) k_gemm_simt<false, true><<<grid, kGemmThreads, 0, dev->stream>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, epi);
  else k_gemm_simt<true, true><<<grid, kGemmThreads, 0, dev->stream>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, epi);
  return check_launch("gemm_simt");
}

}  // namespace vkc
