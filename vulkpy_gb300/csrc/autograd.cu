// Kernels behind the torch.autograd.Function wrappers (vulkpy_gb300/autograd.py):
// the losses' per-row forward and fused backward, the standalone Softmax /
// ReLU / Sigmoid layers, each in float32 (the training arithmetic) and
// float64 (the same math in double, so gradients can be checked against
// float64 central finite differences).
//
// Losses (vulkpy/nn/losses.py): cross entropy -y log(x + 1e-8)
// (nn_cross_entropy.comp:21-26, backward nn_cross_entropy_backward.comp:
// -y / (x + 1e-8)); softmax cross entropy (losses.py:179-249, backward
// p - y); MSE (y - x)^2 (losses.py:252-320, backward 2 (x - y)); Huber
// 0.5 min(|y - x|, (y - x)^2) (losses.py:323-393); MixLoss, a weighted sum
// of losses (losses.py:396-458).  ReduceLoss scales each loss's gradient by
// 1/batch for a mean (losses.py:70-86).
//
// The float32 backward follows the reference's float32 operations in its
// order (each intermediate rounded, no FMA contraction), so for the
// reference-compatible variants the gradient equals the drop-in nn path bit
// for bit.  Two gradients of the reference are not the derivative of its
// forward, and each has an exact variant here as well:
//   * Softmax backward is dy * y (1 - y), the Jacobian's diagonal only
//     (layers.py:302-323); the exact form is y * (dy - sum(dy * y)).
//   * Huber backward is clamp(x - y, -1, 1) (losses.py:376-393), while the
//     forward 0.5 min(|d|, d^2) has derivative d for |d| <= 1 and
//     0.5 sign(d) beyond.
#include "common.cuh"

#include <math.h>

namespace {

constexpr int kThreads = 256;

template <class T>
__device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <class T>
__device__ __forceinline__ T warp_max_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// IEEE operations written out, so float and double take the same path and
// no FMA is contracted.
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float log_t(float x) { return logf(x); }
__device__ __forceinline__ double log_t(double x) { return log(x); }
__device__ __forceinline__ float exp_t(float x) { return expf(x); }
__device__ __forceinline__ double exp_t(double x) { return exp(x); }

template <class T>
__device__ __forceinline__ T ce_eps() {
  return (T)1e-8f;  // the shader's float literal 1e-8, widened for double
}

// One loss term of one element.
template <class T>
__device__ __forceinline__ T loss_term(int kind, T x, T y) {
  if (kind == VKC_LOSS_CE) {
    return mul_rn(-y, log_t(add_rn(x, ce_eps<T>())));
  } else if (kind == VKC_LOSS_MSE) {
    const T d = sub_rn(y, x);
    return mul_rn(d, d);
  } else {  // VKC_LOSS_HUBER
    const T a = fabs(sub_rn(y, x));
    return mul_rn(fmin(a, mul_rn(a, a)), (T)0.5);
  }
}

// rows[r] = sum_c term(x[r, c], y[r, c]); one warp per row.
template <class T>
__global__ void __launch_bounds__(kThreads)
k_loss_rows(int kind, const T* __restrict__ x, const T* __restrict__ y, T* __restrict__ rows, int64_t R, int64_t C) {
  const int lane = threadIdx.x & 31;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= R) return;
  T s = 0;
  for (int64_t c = lane; c < C; c += 32) s += loss_term<T>(kind, x[r * C + c], y[r * C + c]);
  s = warp_sum_t(s);
  if (lane == 0) rows[r] = s;
}

// Softmax cross entropy rows in double (the float32 kernel is
// k_cross_entropy in nn.cu): p = softmax(x) stored, rows[r] = sum -y log(p + eps).
__global__ void __launch_bounds__(kThreads)
k_sce_rows_f64(const double* __restrict__ x, const double* __restrict__ y, double* __restrict__ rows,
               double* __restrict__ p, int64_t R, int64_t C) {
  const int lane = threadIdx.x & 31;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= R) return;
  const double* xr = x + r * C;
  double m = -INFINITY;
  for (int64_t c = lane; c < C; c += 32) m = fmax(m, xr[c]);
  m = warp_max_t(m);
  double s = 0.0;
  for (int64_t c = lane; c < C; c += 32) s += exp(xr[c] - m);
  s = warp_sum_t(s);
  double L = 0.0;
  for (int64_t c = lane; c < C; c += 32) {
    const double pv = exp(xr[c] - m) / s;
    if (p) p[r * C + c] = pv;
    L += (-y[r * C + c]) * log(pv + ce_eps<double>());
  }
  L = warp_sum_t(L);
  if (lane == 0) rows[r] = L;
}

// Softmax forward in double (float32: k_softmax in nn.cu).
__global__ void __launch_bounds__(kThreads)
k_softmax_f64(const double* __restrict__ x, double* __restrict__ y, int64_t R, int64_t C) {
  const int lane = threadIdx.x & 31;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= R) return;
  const double* xr = x + r * C;
  double m = -INFINITY;
  for (int64_t c = lane; c < C; c += 32) m = fmax(m, xr[c]);
  m = warp_max_t(m);
  double s = 0.0;
  for (int64_t c = lane; c < C; c += 32) s += exp(xr[c] - m);
  s = warp_sum_t(s);
  for (int64_t c = lane; c < C; c += 32) y[r * C + c] = exp(xr[c] - m) / s;
}

// Softmax backward, the exact Jacobian-vector product:
// dx = y * (dy - sum_c dy y), one warp per row.
template <class T>
__global__ void __launch_bounds__(kThreads)
k_softmax_jvp(const T* __restrict__ y, const T* __restrict__ dy, T* __restrict__ dx, int64_t R, int64_t C) {
  const int lane = threadIdx.x & 31;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= R) return;
  T s = 0;
  for (int64_t c = lane; c < C; c += 32) s += dy[r * C + c] * y[r * C + c];
  s = warp_sum_t(s);
  for (int64_t c = lane; c < C; c += 32) {
    const int64_t i = r * C + c;
    dx[i] = mul_rn(y[i], sub_rn(dy[i], s));
  }
}

// ReLU max(x, 0) (relu: x.max(0.0), layers.py:185) and Sigmoid
// 1 / (1 + exp(0 - x)) in the reference's four array operations
// (layers.py:240-244).
template <class T>
__global__ void __launch_bounds__(kThreads)
k_act_forward(int act, const T* __restrict__ x, T* __restrict__ y, size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const T v = x[i];
    if (act == VKC_ACT_RELU) {
      y[i] = fmax(v, (T)0);
    } else {
      const T e = exp_t(sub_rn((T)0, v));
      y[i] = div_rn((T)1, add_rn(e, (T)1));
    }
  }
}

// Up to kMaxTerms weighted loss gradients summed per element:
//   g = c0 * (grad0 * s0); g += c1 * (grad1 * s1); ...
// (MixLoss._sum, losses.py:449-458, with each loss's ReduceLoss scaling s).
constexpr int kMaxTerms = 8;

template <class T>
struct LossTerms {
  int count;
  int huber_exact;
  int kind[kMaxTerms];
  T coeff[kMaxTerms];
  T scale[kMaxTerms];
};

template <class T>
__device__ __forceinline__ T grad_term(int kind, int huber_exact, T x, T y, T p) {
  if (kind == VKC_LOSS_CE) {
    return -div_rn(y, add_rn(x, ce_eps<T>()));
  } else if (kind == VKC_LOSS_SCE) {
    return sub_rn(p, y);
  } else if (kind == VKC_LOSS_MSE) {
    return mul_rn(sub_rn(x, y), (T)2);
  } else {  // VKC_LOSS_HUBER
    const T d = sub_rn(x, y);
    if (huber_exact) return fabs(d) <= (T)1 ? d : (d > (T)0 ? (T)0.5 : (d < (T)0 ? (T)-0.5 : d));
    return fmin(fmax(d, (T)-1), (T)1);
  }
}

template <class T>
__global__ void __launch_bounds__(kThreads)
k_loss_grad(const __grid_constant__ LossTerms<T> t, const T* __restrict__ x, const T* __restrict__ y,
            const T* __restrict__ p, T* __restrict__ dx, size_t n) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const T xi = x[i], yi = y[i];
    const T pi = p ? p[i] : (T)0;
    T g = 0;
    for (int j = 0; j < t.count; ++j) {
      const T gj = mul_rn(mul_rn(grad_term<T>(t.kind[j], t.huber_exact, xi, yi, pi), t.scale[j]), t.coeff[j]);
      g = j == 0 ? gj : add_rn(g, gj);
    }
    dx[i] = g;
  }
}

unsigned row_grid(int64_t rows) { return (unsigned)((rows * 32 + kThreads - 1) / kThreads); }

template <class T>
int loss_rows_impl(vkc_device_t dev, int kind, const T* x, const T* y, T* rows, T* p_out, int64_t R, int64_t C);

template <>
int loss_rows_impl<float>(vkc_device_t dev, int kind, const float* x, const float* y, float* rows, float* p_out,
                          int64_t R, int64_t C) {
  if (kind == VKC_LOSS_SCE) return vkc_cross_entropy(dev, x, y, rows, p_out, R, C, 1);
  if (kind == VKC_LOSS_CE) return vkc_cross_entropy(dev, x, y, rows, nullptr, R, C, 0);
  k_loss_rows<float><<<row_grid(R), kThreads, 0, dev->stream>>>(kind, x, y, rows, R, C);
  return vkc::check_launch("loss_rows");
}

template <>
int loss_rows_impl<double>(vkc_device_t dev, int kind, const double* x, const double* y, double* rows,
                           double* p_out, int64_t R, int64_t C) {
  if (kind == VKC_LOSS_SCE) {
    k_sce_rows_f64<<<row_grid(R), kThreads, 0, dev->stream>>>(x, y, rows, p_out, R, C);
  } else {
    k_loss_rows<double><<<row_grid(R), kThreads, 0, dev->stream>>>(kind, x, y, rows, R, C);
  }
  return vkc::check_launch("loss_rows_f64");
}

template <class T>
int loss_rows_any(vkc_device_t dev, int kind, const T* x, const T* y, T* rows, T* p_out, int64_t R, int64_t C) {
  VKC_BIND(dev);
  VKC_REQUIRE(kind >= VKC_LOSS_CE && kind <= VKC_LOSS_HUBER, "unknown loss %d", kind);
  VKC_REQUIRE(R >= 0 && C >= 0, "negative size");
  if (R == 0) return VKC_OK;
  VKC_REQUIRE(x && y && rows, "NULL buffer");
  return loss_rows_impl<T>(dev, kind, x, y, rows, p_out, R, C);
}

template <class T>
int loss_backward(vkc_device_t dev, int nterms, const int* kinds, const double* coeffs, const double* scales,
                  int huber_exact, const T* x, const T* y, const T* p, T* dx, size_t n) {
  VKC_BIND(dev);
  VKC_REQUIRE(nterms >= 1 && nterms <= kMaxTerms, "1 to %d loss terms", kMaxTerms);
  VKC_REQUIRE(kinds && coeffs && scales, "NULL term table");
  LossTerms<T> t{};
  t.count = nterms;
  t.huber_exact = huber_exact ? 1 : 0;
  bool need_p = false;
  for (int j = 0; j < nterms; ++j) {
    VKC_REQUIRE(kinds[j] >= VKC_LOSS_CE && kinds[j] <= VKC_LOSS_HUBER, "unknown loss %d", kinds[j]);
    need_p |= kinds[j] == VKC_LOSS_SCE;
    t.kind[j] = kinds[j];
    t.coeff[j] = (T)coeffs[j];  // a Python float as the float32 array op receives it
    t.scale[j] = (T)scales[j];
  }
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(x && y && dx, "NULL buffer");
  VKC_REQUIRE(p || !need_p, "softmax cross entropy needs the softmax output p");
  const unsigned grid = vkc::wave_grid(dev, k_loss_grad<T>, n, kThreads);
  k_loss_grad<T><<<grid, kThreads, 0, dev->stream>>>(t, x, y, p, dx, n);
  return vkc::check_launch("loss_backward");
}

template <class T>
int softmax_backward(vkc_device_t dev, const T* y, const T* dy, T* dx, int64_t R, int64_t C) {
  VKC_BIND(dev);
  VKC_REQUIRE(R >= 0 && C >= 0, "negative size");
  if (R == 0 || C == 0) return VKC_OK;
  VKC_REQUIRE(y && dy && dx, "NULL buffer");
  k_softmax_jvp<T><<<row_grid(R), kThreads, 0, dev->stream>>>(y, dy, dx, R, C);
  return vkc::check_launch("softmax_backward");
}

template <class T>
int activation_forward(vkc_device_t dev, int act, const T* x, T* y, size_t n) {
  VKC_BIND(dev);
  VKC_REQUIRE(act == VKC_ACT_RELU || act == VKC_ACT_SIGMOID, "activation %d has no forward kernel", act);
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(x && y, "NULL buffer");
  const unsigned grid = vkc::wave_grid(dev, k_act_forward<T>, n, kThreads);
  k_act_forward<T><<<grid, kThreads, 0, dev->stream>>>(act, x, y, n);
  return vkc::check_launch("activation_forward");
}

}  // namespace

VKC_EXPORT int vkc_loss_rows(vkc_device_t dev, int kind, const float* x, const float* y, float* loss_rows,
                             float* p_out, int64_t rows, int64_t cols) {
  return loss_rows_any<float>(dev, kind, x, y, loss_rows, p_out, rows, cols);
}

VKC_EXPORT int vkc_loss_rows_f64(vkc_device_t dev, int kind, const double* x, const double* y, double* loss_rows,
                                 double* p_out, int64_t rows, int64_t cols) {
  return loss_rows_any<double>(dev, kind, x, y, loss_rows, p_out, rows, cols);
}

VKC_EXPORT int vkc_loss_backward(vkc_device_t dev, int nterms, const int* kinds, const double* coeffs,
                                 const double* scales, int huber_exact, const float* x, const float* y,
                                 const float* p, float* dx, size_t n) {
  return loss_backward<float>(dev, nterms, kinds, coeffs, scales, huber_exact, x, y, p, dx, n);
}

VKC_EXPORT int vkc_loss_backward_f64(vkc_device_t dev, int nterms, const int* kinds, const double* coeffs,
                                     const double* scales, int huber_exact, const double* x, const double* y,
                                     const double* p, double* dx, size_t n) {
  return loss_backward<double>(dev, nterms, kinds, coeffs, scales, huber_exact, x, y, p, dx, n);
}

VKC_EXPORT int vkc_softmax_backward(vkc_device_t dev, const float* y, const float* dy, float* dx, int64_t rows,
                                    int64_t cols) {
  return softmax_backward<float>(dev, y, dy, dx, rows, cols);
}

VKC_EXPORT int vkc_softmax_backward_f64(vkc_device_t dev, const double* y, const double* dy, double* dx,
                                        int64_t rows, int64_t cols) {
  return softmax_backward<double>(dev, y, dy, dx, rows, cols);
}

VKC_EXPORT int vkc_softmax_f64(vkc_device_t dev, const double* x, double* y, int64_t rows, int64_t cols) {
  VKC_BIND(dev);
  if (rows <= 0 || cols <= 0) return VKC_OK;
  VKC_REQUIRE(x && y, "NULL buffer");
  k_softmax_f64<<<row_grid(rows), kThreads, 0, dev->stream>>>(x, y, rows, cols);
  return vkc::check_launch("softmax_f64");
}

VKC_EXPORT int vkc_activation_forward(vkc_device_t dev, int act, const float* x, float* y, size_t n) {
  return activation_forward<float>(dev, act, x, y, n);
}

VKC_EXPORT int vkc_activation_forward_f64(vkc_device_t dev, int act, const double* x, double* y, size_t n) {
  return activation_forward<double>(dev, act, x, y, n);
}
