// Reductions: sum / prod / maximum / minimum over all elements or one axis.
//
// Reference: vkarray.py:1194-1276 drives sum.comp (strided partials from a
// single 64-thread dispatch, sum.comp:18-30), sum_v1.3.comp (subgroupAdd
// per 64 elements) and *_axis{,_rebroadcast}.comp (one invocation per output
// with a serial loop over the axis, sum_axis.comp:20-32).  Here:
//   * axis=None: grid-stride 128-bit loads into per-thread accumulators,
//     warp-shuffle + shared-memory tree per block, then one block combines
//     the block partials (in fp64 for sum/prod once n >= 2^24).
//   * axis: [prev, axis, post] view.  post == 1 -> a warp or block per row;
//     post > 1 -> threads own 4 consecutive columns (coalesced) and walk the
//     axis; when prev*post is too small to fill 152 SMs the axis is split
//     into slices whose partials a second kernel combines.
// Sums are compensated by default (Neumaier per thread, TwoSum when
// merging) and so are products (FMA-based error term: float32 products of
// values near 1 otherwise drift by ~0.1 ulp per factor); plain and pairwise
// modes exist for the precision study.
#include "common.cuh"
#include "reduce_acc.cuh"

#include <algorithm>
#include <cfloat>

namespace {

constexpr int kThreads = 256;

// Block-wide reduction; result valid in thread 0.
template <int OP, bool COMP>
__device__ __forceinline__ void block_reduce(Acc<OP, COMP>& a) {
  __shared__ float sh_s[32], sh_c[32];
  warp_reduce(a);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { sh_s[wid] = a.s; sh_c[wid] = a.c; }
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  if (wid == 0) {
    if (lane < nw) { a.s = sh_s[lane]; a.c = sh_c[lane]; }
    else a.init();
    warp_reduce(a);
  }
  __syncthreads();
}

// ---------------------------------------------------------------- axis=None

// NACC accumulators per thread (1: plain / compensated, 16: pairwise).
template <int OP, bool COMP, int NACC>
__device__ __forceinline__ Acc<OP, COMP> thread_accumulate(const float* a, size_t n, size_t tid, size_t nthreads) {
  Acc<OP, COMP> acc[NACC];
#pragma unroll
  for (int k = 0; k < NACC; ++k) acc[k].init();
  const size_t nvec = n >> 2;
  const float4* a4 = reinterpret_cast<const float4*>(a);
  size_t i = tid;
  if constexpr (NACC >= 4) {
    constexpr int U = NACC / 4;
    for (; i + (U - 1) * nthreads < nvec; i += U * nthreads) {
      float4 v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) v[u] = a4[i + u * nthreads];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        acc[4 * u + 0].push(v[u].x);
        acc[4 * u + 1].push(v[u].y);
        acc[4 * u + 2].push(v[u].z);
        acc[4 * u + 3].push(v[u].w);
      }
    }
  } else {
    for (; i + nthreads < nvec; i += 2 * nthreads) {
      float4 v0 = a4[i], v1 = a4[i + nthreads];
      acc[0].push(v0.x); acc[0].push(v0.y); acc[0].push(v0.z); acc[0].push(v0.w);
      acc[0].push(v1.x); acc[0].push(v1.y); acc[0].push(v1.z); acc[0].push(v1.w);
    }
  }
  for (; i < nvec; i += nthreads) {
    float4 v = a4[i];
    acc[0].push(v.x); acc[0].push(v.y); acc[0].push(v.z); acc[0].push(v.w);
  }
  size_t t = (nvec << 2) + tid;
  if (t < n) acc[0].push(a[t]);
  // pairwise fold of the accumulators
#pragma unroll
  for (int w = NACC / 2; w >= 1; w >>= 1) {
#pragma unroll
    for (int k = 0; k < w; ++k) acc[k].merge(acc[k + w].s, acc[k + w].c);
  }
  return acc[0];
}

// Stage 1: per-block partial (as double) or, with one block, the final value.
template <int OP, bool COMP, int NACC>
__global__ void __launch_bounds__(kThreads)
k_reduce_all(const float* a, size_t n, double* partials, float* out, float scale) {
  const size_t nthreads = (size_t)gridDim.x * blockDim.x;
  const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  Acc<OP, COMP> acc = thread_accumulate<OP, COMP, NACC>(a, n, tid, nthreads);
  block_reduce(acc);
  if (threadIdx.x == 0) {
    if (gridDim.x == 1) {
      float v = acc.value();
      out[0] = (OP == VKC_SUM || OP == VKC_PROD) ? v * scale : v;
    } else {
      partials[2 * blockIdx.x] = (double)acc.s;
      partials[2 * blockIdx.x + 1] = (double)acc.c;
    }
  }
}

// Stage 2: one block combines the partials; fp64 combine when FP64 != 0.
template <int OP, bool COMP, bool FP64>
__global__ void __launch_bounds__(1024)
k_reduce_partials(const double* partials, int np, float* out, float scale) {
  if constexpr (FP64) {
    __shared__ double sh[32];
    double v = (OP == VKC_SUM) ? 0.0 : (OP == VKC_PROD ? 1.0 : (double)identity<OP>());
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
      double p = partials[2 * i] + partials[2 * i + 1];
      v = combine_d<OP>(v, p);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = combine_d<OP>(v, __shfl_down_sync(0xffffffffu, v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (wid == 0) {
      const int nw = (blockDim.x + 31) >> 5;
      v = lane < nw ? sh[lane] : ((OP == VKC_SUM) ? 0.0 : (OP == VKC_PROD ? 1.0 : (double)identity<OP>()));
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v = combine_d<OP>(v, __shfl_down_sync(0xffffffffu, v, o));
      if (lane == 0) {
        float f = (float)v;
        out[0] = (OP == VKC_SUM || OP == VKC_PROD) ? f * scale : f;
      }
    }
  } else {
    Acc<OP, COMP> acc;
    acc.init();
    for (int i = threadIdx.x; i < np; i += blockDim.x) acc.merge((float)partials[2 * i], (float)partials[2 * i + 1]);
    block_reduce(acc);
    if (threadIdx.x == 0) {
      float f = acc.value();
      out[0] = (OP == VKC_SUM || OP == VKC_PROD) ? f * scale : f;
    }
  }
}

template <int OP, bool COMP, int NACC>
int reduce_all_impl(vkc_device_t dev, const float* a, size_t n, float* out, float scale) {
  const bool aligned = ((uintptr_t)a & 15u) == 0;
  if (!aligned) return vkc::set_error(VKC_ERR_INVALID, "reduce: input must be 16-byte aligned");
  const size_t per_block = (size_t)kThreads * 4 * 8;  // >= 8 float4 per thread
  size_t want = (n + per_block - 1) / per_block;
  unsigned grid = (unsigned)std::min<size_t>(std::max<size_t>(want, 1), (size_t)dev->sm_count * 8);
  if (grid == 1) {
    k_reduce_all<OP, COMP, NACC><<<1, kThreads, 0, dev->stream>>>(a, n, nullptr, out, scale);
    return vkc::check_launch("reduce_all");
  }
  double* partials = nullptr;
  int r = vkc::scratch_alloc(dev, sizeof(double) * 2 * grid, (void**)&partials);
  if (r != VKC_OK) return r;
  k_reduce_all<OP, COMP, NACC><<<grid, kThreads, 0, dev->stream>>>(a, n, partials, out, scale);
  r = vkc::check_launch("reduce_all");
  if (r == VKC_OK) {
    const bool fp64 = (OP == VKC_SUM || OP == VKC_PROD) && n >= (size_t(1) << 24);
    if (fp64) k_reduce_partials<OP, COMP, true><<<1, 1024, 0, dev->stream>>>(partials, (int)grid, out, scale);
    else k_reduce_partials<OP, COMP, false><<<1, 1024, 0, dev->stream>>>(partials, (int)grid, out, scale);
    r = vkc::check_launch("reduce_partials");
  }
  vkc::scratch_free(dev, partials);
  return r;
}

// ------------------------------------------------------------------- axis

// post == 1, short rows: one thread per row.
template <int OP, bool COMP>
__global__ void k_rows_thread(const float* a, size_t prev, size_t axis, float* out, int rebroadcast, float scale) {
  size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= prev) return;
  const float* row = a + r * axis;
  Acc<OP, COMP> acc;
  acc.init();
  for (size_t k = 0; k < axis; ++k) acc.push(row[k]);
  float v = acc.value();
  if (OP == VKC_SUM || OP == VKC_PROD) v *= scale;
  if (rebroadcast) {
    for (size_t k = 0; k < axis; ++k) out[r * axis + k] = v;
  } else {
    out[r] = v;
  }
}

// post == 1: one warp per row (rows up to a few thousand elements).
template <int OP, bool COMP>
__global__ void __launch_bounds__(kThreads)
k_rows_warp(const float* a, size_t prev, size_t axis, float* out, int rebroadcast, float scale) {
  const int lane = threadIdx.x & 31;
  size_t r = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= prev) return;
  const float* row = a + r * axis;
  Acc<OP, COMP> acc;
  acc.init();
  for (size_t k = lane; k < axis; k += 32) acc.push(row[k]);
  warp_reduce(acc);
  float v = __shfl_sync(0xffffffffu, acc.value(), 0);
  if (OP == VKC_SUM || OP == VKC_PROD) v *= scale;
  if (rebroadcast) {
    for (size_t k = lane; k < axis; k += 32) out[r * axis + k] = v;
  } else if (lane == 0) {
    out[r] = v;
  }
}

// post == 1: `splits` blocks per row (splits == 1 -> writes the result).
template <int OP, bool COMP>
__global__ void __launch_bounds__(kThreads)
k_rows_block(const float* a, size_t prev, size_t axis, int splits, float* out, double* partials,
             int rebroadcast, float scale) {
  const size_t r = blockIdx.x / splits;
  const int sp = blockIdx.x % splits;
  const float* row = a + r * axis;
  // slice length rounded up to a multiple of 4 so every slice starts on a float4
  const size_t span = (((axis + splits - 1) / splits) + 3) & ~size_t(3);
  size_t k0 = std::min(axis, (size_t)sp * span), k1 = std::min(axis, k0 + span);
  Acc<OP, COMP> acc;
  acc.init();
  const bool vec = ((((uintptr_t)row) | (k0 * 4)) & 15u) == 0;
  if (vec && k1 > k0) {
    size_t nv = (k1 - k0) >> 2;
    const float4* r4 = reinterpret_cast<const float4*>(row + k0);
    for (size_t i = threadIdx.x; i < nv; i += kThreads) {
      float4 v = r4[i];
      acc.push(v.x); acc.push(v.y); acc.push(v.z); acc.push(v.w);
    }
    for (size_t k = k0 + (nv << 2) + threadIdx.x; k < k1; k += kThreads) acc.push(row[k]);
  } else {
    for (size_t k = k0 + threadIdx.x; k < k1; k += kThreads) acc.push(row[k]);
  }
  block_reduce(acc);
  __shared__ float result;
  if (threadIdx.x == 0) {
    if (splits == 1) {
      float v = acc.value();
      if (OP == VKC_SUM || OP == VKC_PROD) v *= scale;
      result = v;
      if (!rebroadcast) out[r] = v;
    } else {
      partials[2 * blockIdx.x] = acc.s;
      partials[2 * blockIdx.x + 1] = acc.c;
    }
  }
  if (splits == 1 && rebroadcast) {
    __syncthreads();
    float v = result;
    for (size_t k = threadIdx.x; k < axis; k += kThreads) out[r * axis + k] = v;
  }
}

// Combine `splits` partials per output; writes out[i*post + j] (or the
// rebroadcast row/column).  Layout of partials: [prev][splits][post] pairs.
template <int OP, bool COMP>
__global__ void k_combine_splits(const double* partials, size_t prev, size_t axis, size_t post, int splits,
                                 float* out, int rebroadcast, float scale) {
  size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= prev * post) return;
  size_t i = idx / post, j = idx % post;
  Acc<OP, COMP> acc;
  acc.init();
  // eight splits' partials loaded ahead of their (ordered) merges: one
  // memory wait per eight instead of one per split
  for (int s0 = 0; s0 < splits; s0 += 8) {
    double pv[8], pc[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const size_t p = (i * splits + s0 + t) * post + j;
      pv[t] = s0 + t < splits ? partials[2 * p] : 0.0;
      pc[t] = s0 + t < splits ? partials[2 * p + 1] : 0.0;
    }
#pragma unroll
    for (int t = 0; t < 8; ++t)
      if (s0 + t < splits) acc.merge((float)pv[t], (float)pc[t]);
  }
  float v = acc.value();
  if (OP == VKC_SUM || OP == VKC_PROD) v *= scale;
  if (rebroadcast) {
    for (size_t k = 0; k < axis; ++k) out[(i * axis + k) * post + j] = v;
  } else {
    out[i * post + j] = v;
  }
}

// post > 1: each thread owns VW consecutive columns (VW = 4 -> float4) of
// one (prev, slice) and walks its slice of the axis.
template <int OP, bool COMP, int VW>
__global__ void __launch_bounds__(kThreads)
k_cols(const float* a, size_t prev, size_t axis, size_t post, int splits, float* out, double* partials,
       int rebroadcast, float scale) {
  const size_t ncolv = post / VW;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= prev * ncolv) return;
  const size_t i = t / ncolv;
  const size_t j = (t % ncolv) * VW;
  const int sp = blockIdx.y;
  const size_t span = (axis + splits - 1) / splits;
  const size_t k0 = (size_t)sp * span, k1 = std::min(axis, k0 + span);
  Acc<OP, COMP> acc[VW];
#pragma unroll
  for (int w = 0; w < VW; ++w) acc[w].init();
  const float* base = a + i * axis * post + j;
  size_t k = k0;
  if constexpr (VW == 4) {
    // eight rows per iteration: 128 bytes of independent loads in flight per
    // thread (four rows left HBM ~30% idle), applied in row order
    for (; k + 7 < k1; k += 8) {
      float4 v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) v[u] = __ldcs(reinterpret_cast<const float4*>(base + (k + u) * post));
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        acc[0].push(v[u].x); acc[1].push(v[u].y); acc[2].push(v[u].z); acc[3].push(v[u].w);
      }
    }
  }
  for (; k < k1; ++k) {
    if constexpr (VW == 4) {
      float4 v = *reinterpret_cast<const float4*>(base + k * post);
      acc[0].push(v.x); acc[1].push(v.y); acc[2].push(v.z); acc[3].push(v.w);
    } else {
      acc[0].push(base[k * post]);
    }
  }
  if (splits > 1) {
#pragma unroll
    for (int w = 0; w < VW; ++w) {
      size_t p = (i * splits + sp) * post + j + w;
      partials[2 * p] = acc[w].s;
      partials[2 * p + 1] = acc[w].c;
    }
    return;
  }
#pragma unroll
  for (int w = 0; w < VW; ++w) {
    float v = acc[w].value();
    if (OP == VKC_SUM || OP == VKC_PROD) v *= scale;
    if (rebroadcast) {
      for (size_t k = 0; k < axis; ++k) out[(i * axis + k) * post + j + w] = v;
    } else {
      out[i * post + j + w] = v;
    }
  }
}

// post > 1, small inputs: one kernel instead of k_cols with axis slices
// plus k_combine_splits (and their scratch).  A block of 32 warps owns
// 32 x VW columns of one `prev` index; warp w walks axis slice w (the slices
// k_cols would use with 32 splits), and the slices are merged in order
// through shared memory, so the result equals that two-kernel path.
constexpr int kColsBlockWarps = 32;
// inputs up to 16 MiB take k_cols_block; larger ones stream through k_cols
constexpr size_t kColsBlockMaxElems = size_t(1) << 22;

template <int OP, bool COMP, int VW>
__global__ void __launch_bounds__(kColsBlockWarps * 32)
k_cols_block(const float* a, size_t prev, size_t axis, size_t post, float* out, int rebroadcast, float scale) {
  __shared__ float sh_s[kColsBlockWarps][32 * VW], sh_c[kColsBlockWarps][32 * VW];
  __shared__ float res[32 * VW];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const size_t ngroups = (post + 32 * VW - 1) / (32 * VW);
  const size_t i = blockIdx.x / ngroups;
  const size_t j = (blockIdx.x % ngroups) * 32 * VW + (size_t)lane * VW;
  const bool cin = j < post;  // VW == 4 only when post % 4 == 0
  const size_t span = (axis + kColsBlockWarps - 1) / kColsBlockWarps;
  const size_t k0 = std::min(axis, (size_t)w * span), k1 = std::min(axis, k0 + span);
  Acc<OP, COMP> acc[VW];
#pragma unroll
  for (int v = 0; v < VW; ++v) acc[v].init();
  if (cin) {
    const float* base = a + i * axis * post + j;
    size_t k = k0;
    if constexpr (VW == 4) {
      for (; k + 7 < k1; k += 8) {
        float4 x[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) x[u] = *reinterpret_cast<const float4*>(base + (k + u) * post);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          acc[0].push(x[u].x); acc[1].push(x[u].y); acc[2].push(x[u].z); acc[3].push(x[u].w);
        }
      }
      for (; k < k1; ++k) {
        const float4 x = *reinterpret_cast<const float4*>(base + k * post);
        acc[0].push(x.x); acc[1].push(x.y); acc[2].push(x.z); acc[3].push(x.w);
      }
    } else {
      for (; k + 7 < k1; k += 8) {
        float x[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) x[u] = base[(k + u) * post];
#pragma unroll
        for (int u = 0; u < 8; ++u) acc[0].push(x[u]);
      }
      for (; k < k1; ++k) acc[0].push(base[k * post]);
    }
  }
#pragma unroll
  for (int v = 0; v < VW; ++v) {
    sh_s[w][lane * VW + v] = acc[v].s;
    sh_c[w][lane * VW + v] = acc[v].c;
  }
  __syncthreads();
  // warp v < VW merges column v of every lane, slices in order
  if (w < VW) {
    const int col = lane * VW + w;
    Acc<OP, COMP> r;
    r.init();
    for (int ww = 0; ww < kColsBlockWarps; ++ww) r.merge(sh_s[ww][col], sh_c[ww][col]);
    float val = r.value();
    if (OP == VKC_SUM || OP == VKC_PROD) val *= scale;
    res[col] = val;
  }
  __syncthreads();
  if (!cin) return;
  if (rebroadcast) {
    for (size_t k = w; k < axis; k += kColsBlockWarps)
#pragma unroll
      for (int v = 0; v < VW; ++v) out[(i * axis + k) * post + j + v] = res[lane * VW + v];
  } else if (w == 0) {
#pragma unroll
    for (int v = 0; v < VW; ++v) out[i * post + j + v] = res[lane * VW + v];
  }
}

template <int OP, bool COMP>
int reduce_axis_impl(vkc_device_t dev, const float* a, size_t prev, size_t axis, size_t post, float* out,
                     int rebroadcast, float scale) {
  const size_t target_threads = (size_t)dev->sm_count * 2048;
  if (post == 1) {
    if (axis <= 16) {
      unsigned grid = (unsigned)((prev + kThreads - 1) / kThreads);
      k_rows_thread<OP, COMP><<<grid, kThreads, 0, dev->stream>>>(a, prev, axis, out, rebroadcast, scale);
      return vkc::check_launch("reduce_rows_thread");
    }
    if (axis <= 2048) {
      size_t warps_per_block = kThreads / 32;
      unsigned grid = (unsigned)((prev + warps_per_block - 1) / warps_per_block);
      k_rows_warp<OP, COMP><<<grid, kThreads, 0, dev->stream>>>(a, prev, axis, out, rebroadcast, scale);
      return vkc::check_launch("reduce_rows_warp");
    }
    // long rows: split each row when there are too few rows to fill the GPU
    int splits = 1;
    if (prev < (size_t)dev->sm_count * 8) {
      size_t want = ((size_t)dev->sm_count * 8 + prev - 1) / prev;
      size_t maxs = std::max<size_t>(1, axis / 4096);
      splits = (int)std::min<size_t>(want, maxs);
    }
    if (splits == 1) {
      k_rows_block<OP, COMP><<<(unsigned)prev, kThreads, 0, dev->stream>>>(a, prev, axis, 1, out, nullptr,
                                                                          rebroadcast, scale);
      return vkc::check_launch("reduce_rows_block");
    }
    double* partials = nullptr;
    int r = vkc::scratch_alloc(dev, sizeof(double) * 2 * prev * splits, (void**)&partials);
    if (r != VKC_OK) return r;
    k_rows_block<OP, COMP><<<(unsigned)(prev * splits), kThreads, 0, dev->stream>>>(a, prev, axis, splits, out,
                                                                                  partials, rebroadcast, scale);
    r = vkc::check_launch("reduce_rows_block");
    if (r == VKC_OK) {
      unsigned g2 = (unsigned)((prev + kThreads - 1) / kThreads);
      k_combine_splits<OP, COMP><<<g2, kThreads, 0, dev->stream>>>(partials, prev, axis, 1, splits, out,
                                                                   rebroadcast, scale);
      r = vkc::check_launch("reduce_combine");
    }
    vkc::scratch_free(dev, partials);
    return r;
  }
  // post > 1
  const bool vec = (post % 4 == 0) && (((uintptr_t)a & 15u) == 0);
  const int vw = vec ? 4 : 1;
  const size_t cols_threads = prev * (post / vw);
  int splits = 1;
  if (cols_threads < target_threads) {
    size_t want = (target_threads + cols_threads - 1) / cols_threads;
    size_t maxs = std::max<size_t>(1, axis / 32);
    splits = (int)std::min<size_t>(std::min<size_t>(want, maxs), 65535);
  }
  if (splits > 1 && prev * axis * post <= kColsBlockMaxElems) {
    // 32 columns per block (scalar loads) unless 128-column blocks still
    // cover every SM: the compensated sum's ~8 instructions per element
    // would otherwise pile onto a few SMs
    const bool vec4 = vec && prev * (post / 128) >= (size_t)dev->sm_count;
    const size_t cols = vec4 ? 128 : 32;
    const size_t blocks = prev * ((post + cols - 1) / cols);
    if (vec4)
      k_cols_block<OP, COMP, 4><<<(unsigned)blocks, kColsBlockWarps * 32, 0, dev->stream>>>(a, prev, axis, post, out,
                                                                                        rebroadcast, scale);
    else
      k_cols_block<OP, COMP, 1><<<(unsigned)blocks, kColsBlockWarps * 32, 0, dev->stream>>>(a, prev, axis, post, out,
                                                                                        rebroadcast, scale);
    return vkc::check_launch("reduce_cols_block");
  }
  double* partials = nullptr;
  if (splits > 1) {
    int r = vkc::scratch_alloc(dev, sizeof(double) * 2 * prev * splits * post, (void**)&partials);
    if (r != VKC_OK) return r;
  }
  dim3 grid((unsigned)((cols_threads + kThreads - 1) / kThreads), (unsigned)splits);
  if (vec)
    k_cols<OP, COMP, 4><<<grid, kThreads, 0, dev->stream>>>(a, prev, axis, post, splits, out, partials,
                                                            rebroadcast, scale);
  else
    k_cols<OP, COMP, 1><<<grid, kThreads, 0, dev->stream>>>(a, prev, axis, post, splits, out, partials,
                                                            rebroadcast, scale);
  int r = vkc::check_launch("reduce_cols");
  if (r == VKC_OK && splits > 1) {
    unsigned g2 = (unsigned)((prev * post + kThreads - 1) / kThreads);
    k_combine_splits<OP, COMP><<<g2, kThreads, 0, dev->stream>>>(partials, prev, axis, post, splits, out,
                                                                 rebroadcast, scale);
    r = vkc::check_launch("reduce_combine");
  }
  vkc::scratch_free(dev, partials);
  return r;
}

}  // namespace

VKC_EXPORT int vkc_reduce_all(vkc_device_t dev, int op, int precision, const float* a, size_t n, float* out,
                              float scale) {
  VKC_BIND(dev);
  VKC_REQUIRE(a && out, "NULL buffer");
  VKC_REQUIRE(n > 0, "reduction of an empty array");
  VKC_REQUIRE(precision >= VKC_RED_PLAIN && precision <= VKC_RED_COMPENSATED, "bad precision %d", precision);
  switch (op) {
    case VKC_SUM:
      if (precision == VKC_RED_COMPENSATED) return reduce_all_impl<VKC_SUM, true, 16>(dev, a, n, out, scale);
      if (precision == VKC_RED_PAIRWISE) return reduce_all_impl<VKC_SUM, false, 16>(dev, a, n, out, scale);
      return reduce_all_impl<VKC_SUM, false, 1>(dev, a, n, out, scale);
    case VKC_PROD:
      if (precision == VKC_RED_COMPENSATED) return reduce_all_impl<VKC_PROD, true, 16>(dev, a, n, out, scale);
      if (precision == VKC_RED_PAIRWISE) return reduce_all_impl<VKC_PROD, false, 16>(dev, a, n, out, scale);
      return reduce_all_impl<VKC_PROD, false, 1>(dev, a, n, out, scale);
    case VKC_MAXIMUM: return reduce_all_impl<VKC_MAXIMUM, false, 16>(dev, a, n, out, scale);
    case VKC_MINIMUM: return reduce_all_impl<VKC_MINIMUM, false, 16>(dev, a, n, out, scale);
    default: return vkc::set_error(VKC_ERR_INVALID, "unknown reduce op %d", op);
  }
}

VKC_EXPORT int vkc_reduce_axis(vkc_device_t dev, int op, const float* a, size_t prev, size_t axis, size_t post,
                               float* out, int rebroadcast, float scale) {
  VKC_BIND(dev);
  VKC_REQUIRE(a && out, "NULL buffer");
  VKC_REQUIRE(axis > 0, "reduction over an empty axis");
  if (prev == 0 || post == 0) return VKC_OK;
  switch (op) {
    case VKC_SUM: return reduce_axis_impl<VKC_SUM, true>(dev, a, prev, axis, post, out, rebroadcast, scale);
    case VKC_PROD: return reduce_axis_impl<VKC_PROD, true>(dev, a, prev, axis, post, out, rebroadcast, scale);
    case VKC_MAXIMUM: return reduce_axis_impl<VKC_MAXIMUM, false>(dev, a, prev, axis, post, out, rebroadcast, scale);
    case VKC_MINIMUM: return reduce_axis_impl<VKC_MINIMUM, false>(dev, a, prev, axis, post, out, rebroadcast, scale);
    default: return vkc::set_error(VKC_ERR_INVALID, "unknown reduce op %d", op);
  }
}

// ------------------------------------------------------- allocation-free variant
//
// vkc_reduce_all_noalloc is vkc_reduce_all for callers that cannot allocate
// device memory at call time: hosts that hand the whole device heap to their
// own allocator up front (so a stream-ordered allocation here could fail or
// be refused), and latency-critical paths where an allocation's possible
// synchronisation or failure is not acceptable.  The block partials that
// vkc_reduce_all takes from the memory pool live instead in a file-scope
// device array of fixed size (1 MiB, room for 65536 partials).  A call
// launches the same grid as vkc_reduce_all (one block per 8192 elements, at
// most 8 per SM), so the two entry points return the same bits; one call
// accepts at most 65536 * 8192 = 2^29 elements and rejects larger inputs.
// Every GPU that loads this library holds the array until the process exits.
//
// Set-up: the first call on each device, with that device current, looks up
// the array's device address (cudaGetSymbolAddress) and caches it; make that
// first call before capturing the stream.  All calls on a device share the
// one array and it keeps the previous call's contents: each block overwrites
// its own slot before the combine kernel reads it, so nothing has to start at
// zero, but calls that overlap on the GPU (different streams, or different
// threads without ordering) race on it.
namespace {

constexpr size_t kNoAllocPerBlock = (size_t)kThreads * 4 * 8;  // elements per block partial
constexpr size_t kNoAllocMaxPartials = 65536;
constexpr size_t kNoAllocMaxElements = kNoAllocPerBlock * kNoAllocMaxPartials;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[2 * kNoAllocMaxPartials];

std::mutex g_noalloc_mu;
double* g_noalloc_addr[kNoAllocMaxDevices] = {};

int noalloc_partials(vkc_device_t dev, double** out) {
  VKC_REQUIRE(dev->index >= 0 && dev->index < kNoAllocMaxDevices, "device index %d not supported", dev->index);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev->index]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess || !p)
      return vkc::set_error(VKC_ERR_CUDA, "cudaGetSymbolAddress(no-alloc partials): %s", cudaGetErrorString(e));
    g_noalloc_addr[dev->index] = static_cast<double*>(p);
  }
  *out = g_noalloc_addr[dev->index];
  return VKC_OK;
}

template <int OP, bool COMP, int NACC>
int reduce_all_noalloc_impl(vkc_device_t dev, const float* a, size_t n, float* out, float scale, double* partials) {
  const size_t want = (n + kNoAllocPerBlock - 1) / kNoAllocPerBlock;
  const size_t grid = std::min<size_t>(std::max<size_t>(want, 1), (size_t)dev->sm_count * 8);
  VKC_REQUIRE(grid <= kNoAllocMaxPartials, "vkc_reduce_all_noalloc: %zu partials exceed the scratch", grid);
  if (grid == 1) {
    k_reduce_all<OP, COMP, NACC><<<1, kThreads, 0, dev->stream>>>(a, n, nullptr, out, scale);
    return vkc::check_launch("reduce_all_noalloc");
  }
  k_reduce_all<OP, COMP, NACC><<<(unsigned)grid, kThreads, 0, dev->stream>>>(a, n, partials, out, scale);
  int r = vkc::check_launch("reduce_all_noalloc");
  if (r != VKC_OK) return r;
  const bool fp64 = (OP == VKC_SUM || OP == VKC_PROD) && n >= (size_t(1) << 24);
  if (fp64) k_reduce_partials<OP, COMP, true><<<1, 1024, 0, dev->stream>>>(partials, (int)grid, out, scale);
  else k_reduce_partials<OP, COMP, false><<<1, 1024, 0, dev->stream>>>(partials, (int)grid, out, scale);
  return vkc::check_launch("reduce_partials_noalloc");
}

}  // namespace

VKC_EXPORT int vkc_reduce_all_noalloc(vkc_device_t dev, int op, int precision, const float* a, size_t n, float* out,
                                      float scale) {
  VKC_BIND(dev);
  VKC_REQUIRE(a && out, "NULL buffer");
  VKC_REQUIRE(n > 0, "reduction of an empty array");
  VKC_REQUIRE(n <= kNoAllocMaxElements,
              "vkc_reduce_all_noalloc: %zu elements exceed the maximum of %zu (fixed 1 MiB scratch); "
              "use vkc_reduce_all", n, kNoAllocMaxElements);
  VKC_REQUIRE(((uintptr_t)a & 15u) == 0, "reduce: input must be 16-byte aligned");
  VKC_REQUIRE(precision >= VKC_RED_PLAIN && precision <= VKC_RED_COMPENSATED, "bad precision %d", precision);
  double* partials = nullptr;
  int r = noalloc_partials(dev, &partials);
  if (r != VKC_OK) return r;
  switch (op) {
    case VKC_SUM:
      if (precision == VKC_RED_COMPENSATED) return reduce_all_noalloc_impl<VKC_SUM, true, 16>(dev, a, n, out, scale, partials);
      if (precision == VKC_RED_PAIRWISE) return reduce_all_noalloc_impl<VKC_SUM, false, 16>(dev, a, n, out, scale, partials);
      return reduce_all_noalloc_impl<VKC_SUM, false, 1>(dev, a, n, out, scale, partials);
    case VKC_PROD:
      if (precision == VKC_RED_COMPENSATED) return reduce_all_noalloc_impl<VKC_PROD, true, 16>(dev, a, n, out, scale, partials);
      if (precision == VKC_RED_PAIRWISE) return reduce_all_noalloc_impl<VKC_PROD, false, 16>(dev, a, n, out, scale, partials);
      return reduce_all_noalloc_impl<VKC_PROD, false, 1>(dev, a, n, out, scale, partials);
    case VKC_MAXIMUM: return reduce_all_noalloc_impl<VKC_MAXIMUM, false, 16>(dev, a, n, out, scale, partials);
    case VKC_MINIMUM: return reduce_all_noalloc_impl<VKC_MINIMUM, false, 16>(dev, a, n, out, scale, partials);
    default: return vkc::set_error(VKC_ERR_INVALID, "unknown reduce op %d", op);
  }
}
