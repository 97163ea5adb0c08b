// Fused kernels for the nn layers, losses and optimizers.
//
//   Dense forward  (nn/layers.py:94-102, batch_affine.comp:25-39): a GEMM
//     x W^T with bias (and optional activation) applied in the epilogue.
//   Dense backward (nn/layers.py:104-141): dW += dy^T x and dx = dy W as two
//     GEMMs; the reference materialises dy[:,:,None]*x[:,None,:] (B*out*in
//     floats, 1 GiB at 256x1024x1024) and sums it over the batch.
//   Softmax / cross entropy (layers.py:297-300, losses.py:113-149,
//     nn_cross_entropy.comp:21-26): one warp per row.
//   Optimizers (optimizers.py:39-52, 120-139, 221-253): one pass over the
//     parameters, reproducing the reference's sequence of float32 array ops
//     (each intermediate rounded, no FMA contraction), so the update is
//     bit-identical to the unfused chain.
#include "common.cuh"
#include "gemm_simt.cuh"
#include "gemm_tc.cuh"
#include "colsum.cuh"
#include "reduce_acc.cuh"

namespace {

constexpr int kThreads = 256;

template <int ACT>
__device__ __forceinline__ float act_bwd(float yi, float dyi);

template <int ACT>
__global__ void __launch_bounds__(kThreads) k_act_backward(const float* y, const float* dy, float* dx, size_t n);

// C *= act'(epi.dmask) elementwise after a GEMM that could not apply it in
// its epilogue (C contiguous: ldc == N); in place, the separate
// activation-backward kernel's arithmetic.
int act_deriv_after(vkc_device_t dev, const vkc::GemmEpilogue& epi, float* C, int64_t M, int64_t N, int64_t ldc) {
  if (epi.dact == VKC_ACT_NONE || M == 0 || N == 0) return VKC_OK;
  VKC_REQUIRE(ldc == N, "activation derivative after a GEMM needs a contiguous C");
  const size_t n = (size_t)(M * N);
  const unsigned grid = vkc::stream_grid(dev, n, kThreads);
  if (epi.dact == VKC_ACT_RELU)
    k_act_backward<VKC_ACT_RELU><<<grid, kThreads, 0, dev->stream>>>(epi.dmask, C, C, n);
  else
    k_act_backward<VKC_ACT_SIGMOID><<<grid, kThreads, 0, dev->stream>>>(epi.dmask, C, C, n);
  return vkc::check_launch("gemm activation derivative");
}

// The tensor-core GEMM applies epi.dmask/dact in its epilogue (or split-K
// reduction); the GEMV and SIMT paths run the derivative as one more launch.
int gemm_any(vkc_device_t dev, int precision, bool ta, bool tb, int64_t M, int64_t N, int64_t K, float alpha,
             const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc,
             vkc::GemmEpilogue epi) {
  vkc::GemmEpilogue plain = epi;
  plain.dmask = nullptr;
  plain.dact = VKC_ACT_NONE;
  if (precision == VKC_MM_FP32 || precision == VKC_MM_BF16 || precision == VKC_MM_BF16X3) {
    const int r = vkc::gemm_as_gemv(dev, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, plain);
    if (r >= 0) return r == VKC_OK ? act_deriv_after(dev, epi, C, M, N, ldc) : r;
  }
  if (precision == VKC_MM_FP32 || ((precision == VKC_MM_BF16 || precision == VKC_MM_BF16X3) && K == 0)) {
    const int r = vkc::gemm_simt(dev, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, plain);
    return r == VKC_OK ? act_deriv_after(dev, epi, C, M, N, ldc) : r;
  }
  if (precision == VKC_MM_BF16 || precision == VKC_MM_BF16X3)
    return vkc::gemm_tc(dev, precision, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, epi);
  return vkc::set_error(VKC_ERR_INVALID, "unknown matmul precision %d", precision);
}

// db[o] += sum_b dy[b, o], b in order (one block per 32 columns);
// `overwrite`: db[o] = the sum, the value adding it to a zeroed gradient
// gives (the sum starts at +0, so it is never -0).
__global__ void __launch_bounds__(256) k_colsum_acc(const float* dy, int64_t batch, int64_t out_dim, float* db,
                                                    int overwrite) {
  __shared__ float tile[vkc::kColsumRows][vkc::kColsumCols + 1];
  vkc::pdl_wait();
  vkc::pdl_trigger();
  const int64_t c0 = (int64_t)blockIdx.x * vkc::kColsumCols;
  const float s = vkc::colsum32(dy, batch, out_dim, out_dim, c0, tile);
  const int64_t o = c0 + threadIdx.x;
  if (threadIdx.x < 32 && o < out_dim) db[o] = overwrite ? s : db[o] + s;
}

// db[o] += sum_b dy[b, o], dW[out,in] += dy[B,out]^T @ x[B,in] and
// dx[B,in] = dy[B,out] @ W[out,in] (any may be NULL).  With dW and dx, the
// bias sum and the weight GEMM run on the device's side stream, forked from
// the current stream and joined back before returning, so the two
// independent GEMMs (and their operand splits and split-K reductions)
// overlap; with dW and db only, the bias sum runs there beside the weight
// GEMM.  Inside a graph capture these become parallel branches.  Each
// kernel's own arithmetic is unchanged, so results are too.
// Only from the device's own stream: on a branch's or a caller's stream the
// one side stream would tie independent branches together.
int colsum_into(vkc_device_t dev, const float* dy, float* db, int64_t batch, int64_t out_dim, int overwrite) {
  if (!db || out_dim <= 0) return VKC_OK;
  const unsigned grid = (unsigned)((out_dim + vkc::kColsumCols - 1) / vkc::kColsumCols);
  const cudaError_t e = vkc::launch_pdl(k_colsum_acc, dim3(grid), dim3(256), 0, dev->stream, dy, batch, out_dim, db,
                                        overwrite);
  if (e != cudaSuccess) return vkc::set_error(VKC_ERR_CUDA, "dense_backward db launch: %s", cudaGetErrorString(e));
  return vkc::check_launch("dense_backward db");
}

// `accumulate` = 0: dW and db are overwritten (beta = 0 for the weight GEMM)
// instead of added to; the same values as adding into zeroed gradients,
// without the zeroing pass.
int dense_backward_gemms(vkc_device_t dev, int precision, const float* x, const float* w, const float* dy, float* dx,
                         float* dw, float* db, int64_t batch, int64_t in_dim, int64_t out_dim, int accumulate = 1,
                         const float* dx_y = nullptr, int dx_act = VKC_ACT_NONE) {
  vkc::GemmEpilogue dx_epi;
  dx_epi.dmask = dx_y;
  dx_epi.dact = dx_act;
  const float wbeta = accumulate ? 1.0f : 0.0f;
  const int overwrite = accumulate ? 0 : 1;
  if (dw && (dx || db) && dev->side_stream && dev->stream == dev->own_stream) {
    cudaStream_t main = dev->stream;
    VKC_CUDA(cudaEventRecord(dev->side_fork, main));
    VKC_CUDA(cudaStreamWaitEvent(dev->side_stream, dev->side_fork, 0));
    VKC_CUDA(cudaStreamWaitEvent(dev->bias_stream, dev->side_fork, 0));
    // bias stream: the bias sum; side stream: the weight GEMM when dx is
    // wanted; main: dx, or the weight GEMM (the first layer has no dx)
    dev->stream = dev->bias_stream;
    int r = colsum_into(dev, dy, db, batch, out_dim, overwrite);
    dev->stream = dev->side_stream;
    if (r == VKC_OK && dx)
      r = gemm_any(dev, precision, true, false, out_dim, in_dim, batch, 1.0f, dy, out_dim, x, in_dim, wbeta, dw,
                   in_dim, vkc::GemmEpilogue{});
    dev->stream = main;
    if (r == VKC_OK && dx)
      r = gemm_any(dev, precision, false, false, batch, in_dim, out_dim, 1.0f, dy, out_dim, w, in_dim, 0.0f, dx,
                   in_dim, dx_epi);
    else if (r == VKC_OK)
      r = gemm_any(dev, precision, true, false, out_dim, in_dim, batch, 1.0f, dy, out_dim, x, in_dim, wbeta, dw,
                   in_dim, vkc::GemmEpilogue{});
    // joined back now, or (vkc_side_defer) when the caller ends the deferral,
    // so the branches of several layers overlap the input-gradient chain; the
    // join is recorded even after an error, so a capture stays joined
    dev->side_pending = 1;
    if (!dev->side_defer) {
      const int rj = vkc_side_defer(dev, 0);
      if (r == VKC_OK) r = rj;
    }
    return r;
  }
  int r = colsum_into(dev, dy, db, batch, out_dim, overwrite);
  if (r != VKC_OK) return r;
  if (dw) {
    r = gemm_any(dev, precision, true, false, out_dim, in_dim, batch, 1.0f, dy, out_dim, x, in_dim, wbeta, dw, in_dim,
                 vkc::GemmEpilogue{});
    if (r != VKC_OK) return r;
  }
  if (dx) {
    r = gemm_any(dev, precision, false, false, batch, in_dim, out_dim, 1.0f, dy, out_dim, w, in_dim, 0.0f, dx, in_dim,
                 dx_epi);
  }
  return r;
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// y = exp(x - max) / sum(exp(x - max)) per row, as layers.py:297-300 orders it.
__global__ void __launch_bounds__(kThreads)
k_softmax(const float* x, float* y, int64_t rows, int64_t cols) {
  const int lane = threadIdx.x & 31;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= rows) return;
  const float* xr = x + r * cols;
  float* yr = y + r * cols;
  float m = -INFINITY;
  for (int64_t c = lane; c < cols; c += 32) m = fmaxf(m, xr[c]);
  m = warp_max(m);
  float s = 0.f;
  for (int64_t c = lane; c < cols; c += 32) s += expf(xr[c] - m);
  s = warp_sum(s);
  for (int64_t c = lane; c < cols; c += 32) yr[c] = expf(xr[c] - m) / s;
}

// One row of cross entropy, called by one whole warp: returns (in every
// lane) sum_c -y * log(p + 1e-8) with p = softmax(x) (or x), storing p and,
// when dx is given, the softmax-cross-entropy gradient (p - y) * gscale.
__device__ __forceinline__ float ce_row(const float* xr, const float* yr, float* pr, float* dxr, int64_t cols,
                                        int softmax, float gscale) {
  const int lane = threadIdx.x & 31;
  float m = 0.f, s = 1.f;
  if (softmax) {
    m = -INFINITY;
    for (int64_t c = lane; c < cols; c += 32) m = fmaxf(m, xr[c]);
    m = warp_max(m);
    s = 0.f;
    for (int64_t c = lane; c < cols; c += 32) s += expf(xr[c] - m);
    s = warp_sum(s);
  }
  float L = 0.f;
  for (int64_t c = lane; c < cols; c += 32) {
    float p = softmax ? expf(xr[c] - m) / s : xr[c];
    if (pr) pr[c] = p;
    if (dxr) dxr[c] = __fmul_rn(__fsub_rn(p, yr[c]), gscale);
    L += (-yr[c]) * logf(p + 1e-8f);
  }
  return warp_sum(L);
}

// loss_rows[r] = sum_c -y * log(p + 1e-8), p = softmax(x) or x (stored in
// p_out when given); with dx, also the softmax-cross-entropy gradient
// (p - y) * gscale.  One warp per row.
__global__ void __launch_bounds__(kThreads)
k_cross_entropy(const float* x, const float* y, float* loss_rows, float* p_out, float* dx, int64_t rows,
                int64_t cols, int softmax, float gscale) {
  vkc::pdl_wait();
  vkc::pdl_trigger();
  const int lane = threadIdx.x & 31;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= rows) return;
  const float L = ce_row(x + r * cols, y + r * cols, p_out ? p_out + r * cols : nullptr, dx ? dx + r * cols : nullptr,
                         cols, softmax, gscale);
  if (lane == 0) loss_rows[r] = L;
}

// The batch reduction of the row losses with the arithmetic of the axis
// reduction that ReduceLoss would launch for them (a (rows,) vector reduced
// over axis 0: one thread in order up to 16 rows, one warp above, both
// compensated sums), scaled by lscale.  One warp; rows <= kFusedCeMaxRows.
constexpr int kFusedCeMaxRows = 2048;

__device__ __forceinline__ void ce_batch_sum_warp(const float* row_loss, float* loss, int64_t rows, float lscale) {
  const int lane = threadIdx.x & 31;
  Acc<VKC_SUM, true> acc;
  acc.init();
  if (rows <= 16) {
    if (lane == 0) {
      for (int64_t k = 0; k < rows; ++k) acc.push(__ldcg(row_loss + k));
      loss[0] = acc.value() * lscale;
    }
    return;
  }
  for (int64_t k = lane; k < rows; k += 32) acc.push(__ldcg(row_loss + k));
  warp_reduce(acc);
  float v = __shfl_sync(0xffffffffu, acc.value(), 0);
  v *= lscale;
  if (lane == 0) loss[0] = v;
}

// k_cross_entropy and then the batch sum in the same launch: every block
// stores its rows' losses and counts itself in `done`; the block that comes
// last (it sees every other block's stores) runs the batch sum on its first
// warp and puts `done` back to zero for the next launch.
__global__ void __launch_bounds__(kThreads)
k_cross_entropy_total(const float* x, const float* y, float* loss_rows, float* p_out, float* dx, int64_t rows,
                      int64_t cols, float gscale, float* loss, float lscale, uint32_t* done) {
  __shared__ uint32_t last;
  vkc::pdl_wait();
  vkc::pdl_trigger();
  const int lane = threadIdx.x & 31;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r < rows) {
    const float L = ce_row(x + r * cols, y + r * cols, p_out + r * cols, dx + r * cols, cols, 1, gscale);
    if (lane == 0) loss_rows[r] = L;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1 ? 1u : 0u;
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (threadIdx.x < 32) ce_batch_sum_warp(loss_rows, loss, rows, lscale);
  if (threadIdx.x == 0) *done = 0u;
}

// The reference's Adam chain (optimizers.py:235-253), one element per step:
//   m *= b1; m += c1*g; v *= b2; v += c2*g^2;
//   mhat = m/d1; vhat = sqrt(v/d2) + eps; mhat *= -lr; mhat /= vhat; value += mhat
__global__ void __launch_bounds__(kThreads)
k_adam(float* value, const float* grad, float* m, float* v, size_t n, float b1, float c1, float b2, float c2,
       float d1, float d2, float eps, float nlr) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float g = grad[i];
    float mi = __fadd_rn(__fmul_rn(m[i], b1), __fmul_rn(c1, g));
    float vi = __fadd_rn(__fmul_rn(v[i], b2), __fmul_rn(c2, __fmul_rn(g, g)));
    m[i] = mi;
    v[i] = vi;
    float mhat = __fdiv_rn(mi, d1);
    float vhat = __fadd_rn(__fsqrt_rn(__fdiv_rn(vi, d2)), eps);
    mhat = __fmul_rn(mhat, nlr);
    mhat = __fdiv_rn(mhat, vhat);
    value[i] = __fadd_rn(value[i], mhat);
  }
}

// SGD (optimizers.py:39-52): diff = (-lr) * g; value += diff.
__global__ void __launch_bounds__(kThreads) k_sgd(float* value, const float* grad, size_t n, float nlr) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    value[i] = __fadd_rn(value[i], __fmul_rn(nlr, grad[i]));
}

// AdaGrad (optimizers.py:120-139): h += g^2; r = g / (sqrt(h) + eps); r *= -lr; value += r.
__global__ void __launch_bounds__(kThreads)
k_adagrad(float* value, const float* grad, float* h, size_t n, float nlr, float eps) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float g = grad[i];
    float hi = __fadd_rn(h[i], __fmul_rn(g, g));
    h[i] = hi;
    float r = __fdiv_rn(g, __fadd_rn(__fsqrt_rn(hi), eps));
    r = __fmul_rn(r, nlr);
    value[i] = __fadd_rn(value[i], r);
  }
}

// Running powers for the device-resident Adam variant: p *= beta, in double
// exactly like the Python floats of AdamState (optimizers.py:241-242).
// Adam step with the running powers on the device: every thread advances
// beta^t from the stored value (the same double product on every thread);
// the last block to finish stores the advanced powers and resets the
// completion counter in powers[2], so one launch both uses and advances them.
__global__ void __launch_bounds__(kThreads)
k_adam_dev(float* value, const float* grad, float* m, float* v, size_t n, float b1, float c1, float b2, float c2,
           double* powers, double beta1, double beta2, float eps, float nlr) {
  const double p1 = powers[0] * beta1, p2 = powers[1] * beta2;
  const float d1 = (float)(1.0 - p1), d2 = (float)(1.0 - p2);
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const float g = grad[i];
    float mi = __fadd_rn(__fmul_rn(m[i], b1), __fmul_rn(c1, g));
    float vi = __fadd_rn(__fmul_rn(v[i], b2), __fmul_rn(c2, __fmul_rn(g, g)));
    m[i] = mi;
    v[i] = vi;
    float mhat = __fdiv_rn(mi, d1);
    float vhat = __fadd_rn(__fsqrt_rn(__fdiv_rn(vi, d2)), eps);
    mhat = __fmul_rn(mhat, nlr);
    mhat = __fdiv_rn(mhat, vhat);
    value[i] = __fadd_rn(value[i], mhat);
  }
  __syncthreads();  // this block has read powers[0..1]
  if (threadIdx.x == 0) {
    unsigned int* done = reinterpret_cast<unsigned int*>(powers + 2);
    __threadfence();
    if (atomicAdd(done, 1u) == gridDim.x - 1) {  // every block has read the old powers
      powers[0] = p1;
      powers[1] = p2;
      *done = 0u;
      __threadfence();
    }
  }
}

// ReLU: dx = max(sign(y), 0) * dy; Sigmoid / Softmax diagonal: ((1 - y) * y) * dy.
template <int ACT>
__device__ __forceinline__ float act_bwd(float yi, float dyi) {
  if (ACT == VKC_ACT_RELU) {
    float s = yi > 0.f ? 1.f : (yi < 0.f ? -1.f : yi);
    s = fmaxf(s, 0.f);
    return __fmul_rn(s, dyi);
  } else {
    return __fmul_rn(__fmul_rn(__fsub_rn(1.0f, yi), yi), dyi);
  }
}

template <int ACT>
__global__ void __launch_bounds__(kThreads)
k_act_backward(const float* y, const float* dy, float* dx, size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) dx[i] = act_bwd<ACT>(y[i], dy[i]);
}

// An activation's backward fused with the next Dense layer's bias gradient:
// dy = act'(y) * dy_act (k_act_backward's float32 operations) is stored for
// the weight and input GEMMs and, in the same block, summed over the batch
// in row order (k_colsum_acc's arithmetic): one launch instead of two, and dy
// is not read back for db.  One block per 32 columns, 256-row chunks staged
// in shared memory; each thread issues its 2 x 32 loads before its stores.
template <int ACT>
__global__ void __launch_bounds__(256) k_act_colsum(const float* y, const float* dy_act, float* dy, int64_t batch,
                                                    int64_t out_dim, float* db, int overwrite) {
  __shared__ float tile[vkc::kColsumRows][vkc::kColsumCols + 1];
  vkc::pdl_wait();
  vkc::pdl_trigger();
  constexpr int kQ = vkc::kColsumRows / 8;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t c = (int64_t)blockIdx.x * vkc::kColsumCols + lane;
  const bool in = c < out_dim;
  float s = 0.f;
  for (int64_t r0 = 0; r0 < batch; r0 += vkc::kColsumRows) {
    const int n = (int)(batch - r0 < vkc::kColsumRows ? batch - r0 : vkc::kColsumRows);
    float yv[kQ], gv[kQ];
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
      const int r = w + 8 * q;
      const bool ok = in && r < n;
      const int64_t off = (r0 + r) * out_dim + c;
      yv[q] = ok ? y[off] : 0.f;
      gv[q] = ok ? dy_act[off] : 0.f;
    }
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
      const int r = w + 8 * q;
      if (r < n) {
        const float v = act_bwd<ACT>(yv[q], gv[q]);
        if (in) dy[(r0 + r) * out_dim + c] = v;
        tile[r][lane] = v;
      }
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll 32
      for (int r = 0; r < n; ++r) s += tile[r][lane];
    }
    __syncthreads();
  }
  if (db && w == 0 && in) db[c] = overwrite ? s : db[c] + s;
}

__global__ void __launch_bounds__(kThreads)
k_sce_backward(const float* p, const float* y, float* dx, size_t n, float scale) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    dx[i] = __fmul_rn(__fsub_rn(p[i], y[i]), scale);
}

}  // namespace

VKC_EXPORT int vkc_adam_update_dev(vkc_device_t dev, float* value, const float* grad, float* m, float* v, size_t n,
                                   double lr, double beta1, double beta2, double eps, double* powers) {
  VKC_BIND(dev);
  VKC_REQUIRE(value && grad && m && v && powers, "NULL buffer");
  unsigned grid = vkc::wave_grid(dev, k_adam_dev, n, kThreads);
  k_adam_dev<<<grid, kThreads, 0, dev->stream>>>(value, grad, m, v, n, (float)beta1, (float)(1.0 - beta1),
                                                 (float)beta2, (float)(1.0 - beta2), powers, beta1, beta2,
                                                 (float)eps, (float)(-lr));
  return vkc::check_launch("adam_dev");
}

VKC_EXPORT int vkc_activation_backward(vkc_device_t dev, int act, const float* y, const float* dy, float* dx,
                                       size_t n) {
  VKC_BIND(dev);
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(y && dy && dx, "NULL buffer");
  unsigned grid = vkc::stream_grid(dev, n, kThreads);
  if (act == VKC_ACT_RELU) k_act_backward<VKC_ACT_RELU><<<grid, kThreads, 0, dev->stream>>>(y, dy, dx, n);
  else if (act == VKC_ACT_SIGMOID) k_act_backward<VKC_ACT_SIGMOID><<<grid, kThreads, 0, dev->stream>>>(y, dy, dx, n);
  else return vkc::set_error(VKC_ERR_INVALID, "activation %d has no backward kernel", act);
  return vkc::check_launch("activation_backward");
}

VKC_EXPORT int vkc_softmax_ce_backward(vkc_device_t dev, const float* p, const float* y, float* dx, size_t n,
                                       float scale) {
  VKC_BIND(dev);
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(p && y && dx, "NULL buffer");
  unsigned grid = vkc::wave_grid(dev, k_sce_backward, n, kThreads);
  k_sce_backward<<<grid, kThreads, 0, dev->stream>>>(p, y, dx, n, scale);
  return vkc::check_launch("softmax_ce_backward");
}

VKC_EXPORT int vkc_dense_forward(vkc_device_t dev, int precision, const float* x, const float* w, const float* bias,
                                 float* y, int64_t batch, int64_t in_dim, int64_t out_dim, int act) {
  VKC_BIND(dev);
  VKC_REQUIRE(batch >= 0 && in_dim >= 0 && out_dim >= 0, "negative size");
  if (batch == 0 || out_dim == 0) return VKC_OK;
  VKC_REQUIRE(x && w && y, "NULL buffer");
  VKC_REQUIRE(act >= VKC_ACT_NONE && act <= VKC_ACT_SIGMOID, "unknown activation %d", act);
  vkc::GemmEpilogue epi;
  epi.bias = bias;
  epi.act = act;
  // y[B,out] = x[B,in] @ W[out,in]^T
  return gemm_any(dev, precision, false, true, batch, out_dim, in_dim, 1.0f, x, in_dim, w, in_dim, 0.0f, y, out_dim,
                  epi);
}

VKC_EXPORT int vkc_dense_stack_forward(vkc_device_t dev, int precision, int layers, const float* x, int64_t batch,
                                       const int64_t* dims, const float* const* w, const float* const* bias,
                                       const int* act, float* const* y) {
  VKC_BIND(dev);
  VKC_REQUIRE(layers >= 1 && x && dims && w && bias && act && y, "NULL argument");
  VKC_REQUIRE(batch >= 0, "negative size");
  for (int l = 0; l <= layers; ++l) VKC_REQUIRE(dims[l] >= 0, "negative size");
  for (int l = 0; l < layers; ++l) {
    VKC_REQUIRE(act[l] >= VKC_ACT_NONE && act[l] <= VKC_ACT_SIGMOID, "unknown activation %d", act[l]);
    VKC_REQUIRE(w[l] && y[l], "NULL buffer");
  }
  if (batch == 0) return VKC_OK;
  // The chained form needs every product on the tensor-core path (the
  // layer-by-layer calls would take it too): M > 1, N > 1, K > 0.
  bool chain = (precision == VKC_MM_BF16 || precision == VKC_MM_BF16X3) && layers >= 2 && batch > 1 &&
               batch < (1ll << 31) && (batch + 127) / 128 <= 65535;
  for (int l = 0; l < layers && chain; ++l)
    chain = dims[l] > 0 && dims[l] < (1ll << 31) && dims[l + 1] > 1 && dims[l + 1] < (1ll << 31);
  if (!chain) {
    const float* in = x;
    for (int l = 0; l < layers; ++l) {
      const int r = vkc_dense_forward(dev, precision, in, w[l], bias[l], y[l], batch, dims[l], dims[l + 1], act[l]);
      if (r != VKC_OK) return r;
      in = y[l];
    }
    return VKC_OK;
  }
  const bool x3 = precision == VKC_MM_BF16X3;
  const int parts = x3 ? 2 : 1;
  std::vector<int64_t> kp((size_t)layers);
  size_t elems = 0;
  for (int l = 0; l < layers; ++l) {
    kp[(size_t)l] = (dims[l] + 63) / 64 * 64;
    elems += (size_t)(batch + dims[l + 1]) * (size_t)kp[(size_t)l] * (size_t)parts;
  }
  void* scratch = nullptr;
  int r = vkc::scratch_alloc(dev, elems * sizeof(__nv_bfloat16), &scratch);
  if (r != VKC_OK) return r;
  // per layer: its input [batch][Kp] and its weight [out][Kp], hi then lo
  std::vector<__nv_bfloat16*> a_hi((size_t)layers), a_lo((size_t)layers), w_hi((size_t)layers), w_lo((size_t)layers);
  __nv_bfloat16* p = static_cast<__nv_bfloat16*>(scratch);
  for (int l = 0; l < layers; ++l) {
    const size_t an = (size_t)batch * (size_t)kp[(size_t)l], wn = (size_t)dims[l + 1] * (size_t)kp[(size_t)l];
    a_hi[(size_t)l] = p;
    p += an;
    a_lo[(size_t)l] = x3 ? p : nullptr;
    p += x3 ? an : 0;
    w_hi[(size_t)l] = p;
    p += wn;
    w_lo[(size_t)l] = x3 ? p : nullptr;
    p += x3 ? wn : 0;
  }
  // The weights of layers 1.. are split on the side stream (they do not
  // depend on the chain), the input and layer 0's weight on the main one.
  const bool fork = dev->side_stream && dev->stream == dev->own_stream;
  cudaStream_t main = dev->stream;
  if (fork) {
    VKC_CUDA(cudaEventRecord(dev->side_fork, main));
    VKC_CUDA(cudaStreamWaitEvent(dev->side_stream, dev->side_fork, 0));
    dev->stream = dev->side_stream;
  }
  for (int l = 1; l < layers && r == VKC_OK; ++l)
    r = vkc::tc_split_operands(dev, w[l], dims[l + 1], dims[l], true, w_hi[(size_t)l], w_lo[(size_t)l], nullptr, 0, 0,
                               true, nullptr, nullptr, dims[l], kp[(size_t)l]);
  cudaError_t ej = cudaSuccess;
  if (fork) {
    dev->stream = main;
    ej = cudaEventRecord(dev->side_join, dev->side_stream);  // recorded even after an error: a capture stays joined
  }
  if (r == VKC_OK)
    r = vkc::tc_split_operands(dev, x, batch, dims[0], true, a_hi[0], a_lo[0], w[0], dims[1], dims[0], true, w_hi[0],
                               w_lo[0], dims[0], kp[0]);
  // each layer's reduction (or epilogue pre-pass) writes the next layer's input split
  for (int l = 0; l < layers; ++l) {
    if (l == 1 && fork) {
      const cudaError_t e = ej == cudaSuccess ? cudaStreamWaitEvent(main, dev->side_join, 0) : ej;
      if (e != cudaSuccess && r == VKC_OK) r = vkc::set_error(VKC_ERR_CUDA, "side stream join: %s", cudaGetErrorString(e));
    }
    if (r != VKC_OK) continue;
    vkc::GemmEpilogue epi;
    epi.bias = bias[l];
    epi.act = act[l];
    vkc::SplitOut out{l + 1 < layers ? a_hi[(size_t)l + 1] : nullptr, l + 1 < layers ? a_lo[(size_t)l + 1] : nullptr,
                      l + 1 < layers ? kp[(size_t)l + 1] : 0};
    r = vkc::gemm_tc_presplit(dev, precision, batch, dims[l + 1], dims[l], 1.0f, a_hi[(size_t)l], a_lo[(size_t)l],
                              w_hi[(size_t)l], w_lo[(size_t)l], 0.0f, y[l], dims[l + 1], epi,
                              l + 1 < layers ? &out : nullptr);
  }
  vkc::scratch_free(dev, scratch);
  return r;
}

VKC_EXPORT int vkc_dense_backward(vkc_device_t dev, int precision, const float* x, const float* w, const float* dy,
                                  float* dx, float* dw, float* db, int64_t batch, int64_t in_dim, int64_t out_dim) {
  VKC_BIND(dev);
  VKC_REQUIRE(batch >= 0 && in_dim >= 0 && out_dim >= 0, "negative size");
  if (batch == 0) return VKC_OK;
  VKC_REQUIRE(x && w && dy, "NULL buffer");
  return dense_backward_gemms(dev, precision, x, w, dy, dx, dw, db, batch, in_dim, out_dim);
}

namespace {
int dense_backward_act_any(vkc_device_t dev, int precision, const float* x, const float* w, const float* dy_act,
                           const float* y, int act, float* dy, float* dx, float* dw, float* db, int64_t batch,
                           int64_t in_dim, int64_t out_dim, int accumulate) {
  VKC_BIND(dev);
  VKC_REQUIRE(batch >= 0 && in_dim >= 0 && out_dim >= 0, "negative size");
  if (batch == 0) return VKC_OK;
  VKC_REQUIRE(x && w && dy_act && y && dy, "NULL buffer");
  VKC_REQUIRE(act == VKC_ACT_RELU || act == VKC_ACT_SIGMOID, "activation %d has no backward kernel", act);
  if (out_dim > 0) {
    const unsigned grid = (unsigned)((out_dim + vkc::kColsumCols - 1) / vkc::kColsumCols);
    const int ow = accumulate ? 0 : 1;
    const cudaError_t e =
        act == VKC_ACT_RELU
            ? vkc::launch_pdl(k_act_colsum<VKC_ACT_RELU>, dim3(grid), dim3(256), 0, dev->stream, y, dy_act, dy, batch,
                              out_dim, db, ow)
            : vkc::launch_pdl(k_act_colsum<VKC_ACT_SIGMOID>, dim3(grid), dim3(256), 0, dev->stream, y, dy_act, dy,
                              batch, out_dim, db, ow);
    if (e != cudaSuccess)
      return vkc::set_error(VKC_ERR_CUDA, "dense_backward_act launch: %s", cudaGetErrorString(e));
    const int r = vkc::check_launch("dense_backward_act dy, db");
    if (r != VKC_OK) return r;
  }
  return dense_backward_gemms(dev, precision, x, w, dy, dx, dw, nullptr, batch, in_dim, out_dim, accumulate);
}
}  // namespace

VKC_EXPORT int vkc_dense_backward_act(vkc_device_t dev, int precision, const float* x, const float* w,
                                      const float* dy_act, const float* y, int act, float* dy, float* dx, float* dw,
                                      float* db, int64_t batch, int64_t in_dim, int64_t out_dim) {
  return dense_backward_act_any(dev, precision, x, w, dy_act, y, act, dy, dx, dw, db, batch, in_dim, out_dim, 1);
}

VKC_EXPORT int vkc_dense_backward_ex(vkc_device_t dev, int precision, const float* x, const float* w,
                                     const float* dy_act, const float* y, int act, float* dy, float* dx, float* dw,
                                     float* db, int64_t batch, int64_t in_dim, int64_t out_dim, int accumulate) {
  if (act != VKC_ACT_NONE)
    return dense_backward_act_any(dev, precision, x, w, dy_act, y, act, dy, dx, dw, db, batch, in_dim, out_dim,
                                  accumulate);
  VKC_BIND(dev);
  VKC_REQUIRE(batch >= 0 && in_dim >= 0 && out_dim >= 0, "negative size");
  if (batch == 0) return VKC_OK;
  VKC_REQUIRE(x && w && dy_act, "NULL buffer");
  return dense_backward_gemms(dev, precision, x, w, dy_act, dx, dw, db, batch, in_dim, out_dim, accumulate);
}

VKC_EXPORT int vkc_dense_backward_chain(vkc_device_t dev, int precision, const float* x, const float* w,
                                        const float* dy, const float* dx_y, int dx_act, float* dx, float* dw,
                                        float* db, int64_t batch, int64_t in_dim, int64_t out_dim, int accumulate) {
  VKC_BIND(dev);
  VKC_REQUIRE(batch >= 0 && in_dim >= 0 && out_dim >= 0, "negative size");
  VKC_REQUIRE(dx_act == VKC_ACT_NONE || dx_act == VKC_ACT_RELU || dx_act == VKC_ACT_SIGMOID,
              "activation %d has no backward kernel", dx_act);
  if (batch == 0) return VKC_OK;
  VKC_REQUIRE(x && w && dy, "NULL buffer");
  VKC_REQUIRE(dx_act == VKC_ACT_NONE || (dx && dx_y), "dx and its activation output are needed");
  return dense_backward_gemms(dev, precision, x, w, dy, dx, dw, db, batch, in_dim, out_dim, accumulate, dx_y,
                              dx_act);
}

VKC_EXPORT int vkc_softmax(vkc_device_t dev, const float* x, float* y, int64_t rows, int64_t cols) {
  VKC_BIND(dev);
  if (rows <= 0 || cols <= 0) return VKC_OK;
  VKC_REQUIRE(x && y, "NULL buffer");
  unsigned grid = (unsigned)((rows * 32 + kThreads - 1) / kThreads);
  k_softmax<<<grid, kThreads, 0, dev->stream>>>(x, y, rows, cols);
  return vkc::check_launch("softmax");
}

VKC_EXPORT int vkc_cross_entropy(vkc_device_t dev, const float* x, const float* y, float* loss_rows, float* p_out,
                                 int64_t rows, int64_t cols, int softmax) {
  VKC_BIND(dev);
  if (rows <= 0) return VKC_OK;
  VKC_REQUIRE(x && y && loss_rows, "NULL buffer");
  unsigned grid = (unsigned)((rows * 32 + kThreads - 1) / kThreads);
  k_cross_entropy<<<grid, kThreads, 0, dev->stream>>>(x, y, loss_rows, p_out, nullptr, rows, cols, softmax, 1.f);
  return vkc::check_launch("cross_entropy");
}

VKC_EXPORT int vkc_softmax_ce_fused(vkc_device_t dev, const float* x, const float* y, float* p_out, float* dx,
                                    float* loss, int64_t rows, int64_t cols, float loss_scale, float grad_scale) {
  VKC_BIND(dev);
  VKC_REQUIRE(rows >= 1 && rows <= kFusedCeMaxRows, "fused softmax cross entropy takes 1 to %d rows",
              kFusedCeMaxRows);
  VKC_REQUIRE(cols >= 1, "no classes");
  VKC_REQUIRE(x && y && p_out && dx && loss, "NULL buffer");
  float* row_loss = nullptr;
  int r = vkc::scratch_alloc(dev, sizeof(float) * (size_t)rows, (void**)&row_loss);
  if (r != VKC_OK) return r;
  const unsigned grid = (unsigned)((rows * 32 + kThreads - 1) / kThreads);
  cudaError_t e = vkc::launch_pdl(k_cross_entropy_total, dim3(grid), dim3(kThreads), 0, dev->stream, x, y, row_loss,
                                  p_out, dx, rows, cols, grad_scale, loss, loss_scale, dev->done_ctr);
  r = e == cudaSuccess ? vkc::check_launch("softmax_ce_fused")
                       : vkc::set_error(VKC_ERR_CUDA, "softmax_ce_fused launch: %s", cudaGetErrorString(e));
  vkc::scratch_free(dev, row_loss);
  return r;
}

VKC_EXPORT int vkc_adam_update(vkc_device_t dev, float* value, const float* grad, float* m, float* v, size_t n,
                               double lr, double beta1, double beta2, double eps, double beta1t, double beta2t) {
  VKC_BIND(dev);
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(value && grad && m && v, "NULL buffer");
  // Scalars as the reference forms them: Python doubles rounded to float32
  // at the array op that consumes them (optimizers.py:235-251).
  const float b1 = (float)beta1, b2 = (float)beta2;
  const float c1 = (float)(1.0 - beta1), c2 = (float)(1.0 - beta2);
  const float d1 = (float)(1.0 - beta1t), d2 = (float)(1.0 - beta2t);
  unsigned grid = vkc::wave_grid(dev, k_adam, n, kThreads);
  k_adam<<<grid, kThreads, 0, dev->stream>>>(value, grad, m, v, n, b1, c1, b2, c2, d1, d2, (float)eps, (float)(-lr));
  return vkc::check_launch("adam");
}

VKC_EXPORT int vkc_sgd_update(vkc_device_t dev, float* value, const float* grad, size_t n, double lr) {
  VKC_BIND(dev);
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(value && grad, "NULL buffer");
  unsigned grid = vkc::wave_grid(dev, k_sgd, n, kThreads);
  k_sgd<<<grid, kThreads, 0, dev->stream>>>(value, grad, n, (float)(-lr));
  return vkc::check_launch("sgd");
}

VKC_EXPORT int vkc_adagrad_update(vkc_device_t dev, float* value, const float* grad, float* h, size_t n, double lr,
                                  double eps) {
  VKC_BIND(dev);
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(value && grad && h, "NULL buffer");
  unsigned grid = vkc::wave_grid(dev, k_adagrad, n, kThreads);
  k_adagrad<<<grid, kThreads, 0, dev->stream>>>(value, grad, h, n, (float)(-lr), (float)eps);
  return vkc::check_launch("adagrad");
}
