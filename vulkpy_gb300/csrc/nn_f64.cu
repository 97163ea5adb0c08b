// Float64 versions of the Dense / activation / softmax-cross-entropy kernels.
//
// They exist for gradient checking: the same hand-written forward and
// backward math as nn.cu, in double, so autograd gradients can be compared
// with float64 central finite differences at 1e-6 relative without float32
// rounding dominating the comparison.  Not tuned for speed (GB300's fp64
// rate is a small fraction of its fp32 rate).
#include "common.cuh"

namespace {

constexpr int kT = 256;
constexpr int kTile = 64, kKs = 8;

// C[M,N] = op(A) op(B) (+ beta C) (+ bias) then activation; 64x64 tiles,
// each of 256 threads owns a 4x4 block.
template <bool TA, bool TB>
__global__ void __launch_bounds__(kT)
k_gemm_f64(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda, const double* B, int64_t ldb, double beta,
           double* C, int64_t ldc, const double* bias, int act) {
  __shared__ double As[kKs][kTile];
  __shared__ double Bs[kKs][kTile];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t m0 = (int64_t)blockIdx.y * kTile, n0 = (int64_t)blockIdx.x * kTile;
  double acc[4][4] = {};
  for (int64_t k0 = 0; k0 < K; k0 += kKs) {
    for (int e = threadIdx.x; e < kKs * kTile; e += kT) {
      const int kk = e / kTile, mm = e % kTile;
      const int64_t gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? (TA ? A[gk * lda + gm] : A[gm * lda + gk]) : 0.0;
      const int64_t gn = n0 + mm;
      Bs[kk][mm] = (gn < N && gk < K) ? (TB ? B[gn * ldb + gk] : B[gk * ldb + gn]) : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kKs; ++kk)
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(As[kk][ty * 4 + i], Bs[kk][tx * 4 + j], acc[i][j]);
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t gn = n0 + tx * 4 + j;
      if (gn >= N) continue;
      double v = acc[i][j];
      if (beta != 0.0) v += beta * C[gm * ldc + gn];
      if (bias) v += bias[gn];
      if (act == VKC_ACT_RELU) v = fmax(v, 0.0);
      else if (act == VKC_ACT_SIGMOID) v = 1.0 / (1.0 + exp(0.0 - v));
      C[gm * ldc + gn] = v;
    }
  }
}

int gemm_f64(vkc_device_t dev, bool ta, bool tb, int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
             const double* B, int64_t ldb, double beta, double* C, int64_t ldc, const double* bias, int act) {
  dim3 grid((unsigned)((N + kTile - 1) / kTile), (unsigned)((M + kTile - 1) / kTile));
  if (!ta && !tb) k_gemm_f64<false, false><<<grid, kT, 0, dev->stream>>>(M, N, K, A, lda, B, ldb, beta, C, ldc, bias, act);
  else if (ta && !tb) k_gemm_f64<true, false><<<grid, kT, 0, dev->stream>>>(M, N, K, A, lda, B, ldb, beta, C, ldc, bias, act);
  else if (!ta && tb) k_gemm_f64<false, true><<<grid, kT, 0, dev->stream>>>(M, N, K, A, lda, B, ldb, beta, C, ldc, bias, act);
  else k_gemm_f64<true, true><<<grid, kT, 0, dev->stream>>>(M, N, K, A, lda, B, ldb, beta, C, ldc, bias, act);
  return vkc::check_launch("gemm_f64");
}

__global__ void k_colsum_acc_f64(const double* dy, int64_t batch, int64_t out_dim, double* db) {
  int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= out_dim) return;
  double s = 0.0;
  for (int64_t b = 0; b < batch; ++b) s += dy[b * out_dim + o];
  db[o] += s;
}

template <int ACT>
__global__ void k_act_backward_f64(const double* y, const double* dy, double* dx, size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const double yi = y[i];
    if (ACT == VKC_ACT_RELU) {
      double s = yi > 0.0 ? 1.0 : (yi < 0.0 ? -1.0 : yi);
      dx[i] = fmax(s, 0.0) * dy[i];
    } else {
      dx[i] = ((1.0 - yi) * yi) * dy[i];
    }
  }
}

__global__ void k_cross_entropy_f64(const double* x, const double* y, double* loss_rows, double* p_out, int64_t rows,
                                    int64_t cols, int softmax) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  const double* xr = x + r * cols;
  const double* yr = y + r * cols;
  double m = 0.0, s = 1.0;
  if (softmax) {
    m = -INFINITY;
    for (int64_t c = 0; c < cols; ++c) m = fmax(m, xr[c]);
    s = 0.0;
    for (int64_t c = 0; c < cols; ++c) s += exp(xr[c] - m);
  }
  double L = 0.0;
  for (int64_t c = 0; c < cols; ++c) {
    const double p = softmax ? exp(xr[c] - m) / s : xr[c];
    if (p_out) p_out[r * cols + c] = p;
    L += (-yr[c]) * log(p + 1e-8);
  }
  loss_rows[r] = L;
}

__global__ void k_sce_backward_f64(const double* p, const double* y, double* dx, size_t n, double scale) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dx[i] = (p[i] - y[i]) * scale;
}

}  // namespace

VKC_EXPORT int vkc_dense_forward_f64(vkc_device_t dev, const double* x, const double* w, const double* bias, double* y,
                                     int64_t batch, int64_t in_dim, int64_t out_dim, int act) {
  VKC_BIND(dev);
  if (batch <= 0 || out_dim <= 0) return VKC_OK;
  VKC_REQUIRE(x && w && y, "NULL buffer");
  return gemm_f64(dev, false, true, batch, out_dim, in_dim, x, in_dim, w, in_dim, 0.0, y, out_dim, bias, act);
}

VKC_EXPORT int vkc_dense_backward_f64(vkc_device_t dev, const double* x, const double* w, const double* dy, double* dx,
                                      double* dw, double* db, int64_t batch, int64_t in_dim, int64_t out_dim) {
  VKC_BIND(dev);
  if (batch <= 0) return VKC_OK;
  VKC_REQUIRE(x && w && dy, "NULL buffer");
  int r = VKC_OK;
  if (db) {
    k_colsum_acc_f64<<<(unsigned)((out_dim + kT - 1) / kT), kT, 0, dev->stream>>>(dy, batch, out_dim, db);
    r = vkc::check_launch("dense_backward_f64 db");
    if (r != VKC_OK) return r;
  }
  if (dw) r = gemm_f64(dev, true, false, out_dim, in_dim, batch, dy, out_dim, x, in_dim, 1.0, dw, in_dim, nullptr, 0);
  if (r == VKC_OK && dx)
    r = gemm_f64(dev, false, false, batch, in_dim, out_dim, dy, out_dim, w, in_dim, 0.0, dx, in_dim, nullptr, 0);
  return r;
}

VKC_EXPORT int vkc_activation_backward_f64(vkc_device_t dev, int act, const double* y, const double* dy, double* dx,
                                           size_t n) {
  VKC_BIND(dev);
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(y && dy && dx, "NULL buffer");
  unsigned grid = vkc::stream_grid(dev, n, kT);
  if (act == VKC_ACT_RELU) k_act_backward_f64<VKC_ACT_RELU><<<grid, kT, 0, dev->stream>>>(y, dy, dx, n);
  else if (act == VKC_ACT_SIGMOID) k_act_backward_f64<VKC_ACT_SIGMOID><<<grid, kT, 0, dev->stream>>>(y, dy, dx, n);
  else return vkc::set_error(VKC_ERR_INVALID, "activation %d has no backward kernel", act);
  return vkc::check_launch("activation_backward_f64");
}

VKC_EXPORT int vkc_cross_entropy_f64(vkc_device_t dev, const double* x, const double* y, double* loss_rows,
                                     double* p_out, int64_t rows, int64_t cols, int softmax) {
  VKC_BIND(dev);
  if (rows <= 0) return VKC_OK;
  VKC_REQUIRE(x && y && loss_rows, "NULL buffer");
  k_cross_entropy_f64<<<(unsigned)((rows + 127) / 128), 128, 0, dev->stream>>>(x, y, loss_rows, p_out, rows, cols,
                                                                               softmax);
  return vkc::check_launch("cross_entropy_f64");
}

VKC_EXPORT int vkc_softmax_ce_backward_f64(vkc_device_t dev, const double* p, const double* y, double* dx, size_t n,
                                           double scale) {
  VKC_BIND(dev);
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(p && y && dx, "NULL buffer");
  unsigned grid = vkc::stream_grid(dev, n, kT);
  k_sce_backward_f64<<<grid, kT, 0, dev->stream>>>(p, y, dx, n, scale);
  return vkc::check_launch("softmax_ce_backward_f64");
}
