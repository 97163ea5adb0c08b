// Tensor-core GEMM for sm_103a: TMA -> 128B-swizzled shared memory ->
// tcgen05.mma (bf16 x bf16, fp32 accumulate in TMEM) -> tcgen05.ld epilogue.
//
// C[M,N] = act(alpha * op(A) op(B) + beta * C + bias), A/B/C fp32 in memory.
// A pre-pass turns op(A) (M x K) and op(B)^T (N x K) into K-major bf16
// copies: x ~ hi = bf16(x) and, for the split mode, lo = bf16(x - hi).  The
// split-bf16x3 product accumulates hi*hi + hi*lo + lo*hi per K step, which
// keeps ~16 significant bits per operand (relative representation error
// <= 2^-17) at three tensor-core products instead of fp32 FMA.
//
// One CTA computes a 128 x BN tile with 6 warps:
//   warp 0 lane 0  TMA producer: STAGES-deep ring of (A, B[, A_lo, B_lo]) tiles
//   warp 1         allocates TMEM; lane 0 issues tcgen05.mma and commits
//   warps 2-5      epilogue: tcgen05.ld 32 columns at a time, alpha/beta/bias/act
// Every mbarrier wait is bounded by a wall-clock limit; on expiry the CTA
// records bit1 in the device error word, drains what it issued and returns.
#include "gemm_tc.cuh"
#include "tc_ptx.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <map>
#include <mutex>

namespace vkc {
namespace {

// ------------------------------------------------------------ the kernel
template <int BN, bool X3, int STAGES>
struct TcCfg {
  static constexpr uint32_t kABytes = kBM * kBK * 2;
  static constexpr uint32_t kBBytes = BN * kBK * 2;
  static constexpr uint32_t kStageBytes = (X3 ? 2u : 1u) * (kABytes + kBBytes);
  static constexpr uint32_t kSmem = STAGES * kStageBytes + 1024 /*align*/ + 256 /*barriers*/;
  static constexpr uint32_t kTmemCols = BN;  // fp32 accumulator: one column per output column
};

template <int BN, bool X3, int STAGES>
__global__ void __launch_bounds__(kThreadsTC, 1)
k_gemm_tc(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
          const __grid_constant__ CUtensorMap map_alo, const __grid_constant__ CUtensorMap map_blo, int M, int N, int K,
          float alpha, float beta, float* __restrict__ C, int64_t ldc, const float* __restrict__ bias, int act,
          uint32_t* err) {
  using Cfg = TcCfg<BN, X3, STAGES>;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint8_t* gbase = smem_raw + (base - raw);
  const uint32_t bars = base + STAGES * Cfg::kStageBytes;
  auto full_bar = [&](int s) { return bars + 8u * s; };
  auto empty_bar = [&](int s) { return bars + 8u * (STAGES + s); };
  const uint32_t acc_bar = bars + 16u * STAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gbase + STAGES * Cfg::kStageBytes + 16 * STAGES + 8);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * BN;
  const int nk = (K + kBK - 1) / kBK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full_bar(s), 1);
      mbar_init(empty_bar(s), 1);
    }
    mbar_init(acc_bar, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(Cfg::kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(tmem_slot);

  auto stage_a = [&](int s) { return base + s * Cfg::kStageBytes; };
  auto stage_b = [&](int s) { return stage_a(s) + Cfg::kABytes; };
  auto stage_alo = [&](int s) { return stage_b(s) + Cfg::kBBytes; };
  auto stage_blo = [&](int s) { return stage_alo(s) + Cfg::kABytes; };

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer
    int issued = 0;
    bool ok = true;
    for (int kb = 0; kb < nk && ok; ++kb) {
      const int s = kb % STAGES;
      const uint32_t ph = (kb / STAGES) & 1;
      if (*abort_flag || !mbar_wait(empty_bar(s), ph ^ 1)) { ok = false; break; }
      mbar_expect_tx(full_bar(s), Cfg::kStageBytes);
      tma_load_2d(stage_a(s), &map_a, full_bar(s), kb * kBK, m0);
      tma_load_2d(stage_b(s), &map_b, full_bar(s), kb * kBK, n0);
      if (X3) {
        tma_load_2d(stage_alo(s), &map_alo, full_bar(s), kb * kBK, m0);
        tma_load_2d(stage_blo(s), &map_blo, full_bar(s), kb * kBK, n0);
      }
      ++issued;
    }
    if (!ok) {
      atomicOr(err, 2u);
      *abort_flag = 1;
      // drain the copies still in flight into this CTA's shared memory
      for (int kb = std::max(0, issued - STAGES); kb < issued; ++kb) mbar_wait(full_bar(kb % STAGES), (kb / STAGES) & 1);
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    constexpr uint32_t idesc = (1u << 4)            // D: fp32
                               | (1u << 7)          // A: bf16
                               | (1u << 10)         // B: bf16
                               | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
    bool ok = true;
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % STAGES;
      const uint32_t ph = (kb / STAGES) & 1;
      if (*abort_flag || !mbar_wait(full_bar(s), ph)) { ok = false; break; }
      tc_fence_after();
#pragma unroll
      for (int k = 0; k < kBK / 16; ++k) {
        const uint64_t a = sw128_desc(stage_a(s) + 32u * k);
        const uint64_t b = sw128_desc(stage_b(s) + 32u * k);
        mma_bf16(tmem, a, b, idesc, (kb | k) != 0);
        if (X3) {
          mma_bf16(tmem, a, sw128_desc(stage_blo(s) + 32u * k), idesc, 1);
          mma_bf16(tmem, sw128_desc(stage_alo(s) + 32u * k), b, idesc, 1);
        }
      }
      mma_commit(empty_bar(s));  // frees the stage once these MMAs have read it
    }
    if (!ok) {
      atomicOr(err, 2u);
      *abort_flag = 1;
    }
    mma_commit(acc_bar);  // fires when every MMA issued above has completed
  } else if (warp >= 2) {
    // ---------------- epilogue: TMEM -> registers -> global
    const bool ok = mbar_wait(acc_bar, 0) && !*abort_flag && nk > 0;
    tc_fence_after();
    const int q = warp & 3;  // TMEM lanes 32q .. 32q+31 belong to this warp
    const int row = m0 + q * 32 + lane;
    if (!ok) {
      if (lane == 0) atomicOr(err, 2u);
    } else {
#pragma unroll 1
      for (int c = 0; c < BN / 32; ++c) {
        uint32_t r[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(c * 32), r);
        if (row < M) {
          float* crow = C + (int64_t)row * ldc;
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int col = n0 + c * 32 + j;
            if (col < N) {
              float v = alpha * __uint_as_float(r[j]);
              if (beta != 0.f) v += beta * crow[col];
              if (bias) v += bias[col];
              if (act == VKC_ACT_RELU) v = fmaxf(v, 0.f);
              else if (act == VKC_ACT_SIGMOID) v = 1.0f / (1.0f + expf(0.0f - v));
              crow[col] = v;
            }
          }
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Cfg::kTmemCols) : "memory");
  }
}

// ------------------------------------------------------------ split-bf16x3
// The tensor core adds each MMA's result into the fp32 TMEM accumulator
// with truncation, so the error of one long accumulation grows with K/16
// (measured: 1.5e-5 relative at K = 4096, 2.9e-5 at 8192).  This kernel
// restarts the accumulation every 64-wide K block in one of kAccBufs TMEM
// buffers and the epilogue warps add each block's partial into fp32
// registers with round-to-nearest, overlapping with the next blocks' MMAs.

// With gridDim.z > 1 the K blocks are split across CTAs (blockIdx.z takes
// blocks [z*kps, (z+1)*kps)) and each CTA writes its raw fp32 partial tile to
// partial[z][M][N]; k_splitk_reduce then adds the partials in z order and
// applies the epilogue, so results do not depend on scheduling.
template <int STAGES>
__global__ void __launch_bounds__(kThreadsTC, 1)
k_gemm_tc_x3(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
             const __grid_constant__ CUtensorMap map_alo, const __grid_constant__ CUtensorMap map_blo, int M, int N,
             int K, float alpha, float beta, float* __restrict__ C, int64_t ldc, const float* __restrict__ bias, int act,
             uint32_t* err, float* __restrict__ partial, int kps) {
  constexpr int BN = 128;
  using Cfg = TcCfg<BN, true, STAGES>;
  constexpr uint32_t kCols = BN * kAccBufs;  // 512: all of TMEM
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint8_t* gbase = smem_raw + (base - raw);
  const uint32_t bars = base + STAGES * Cfg::kStageBytes;
  auto full_bar = [&](int s) { return bars + 8u * s; };
  auto empty_bar = [&](int s) { return bars + 8u * (STAGES + s); };
  auto accf_bar = [&](int b) { return bars + 8u * (2 * STAGES + b); };
  auto acce_bar = [&](int b) { return bars + 8u * (2 * STAGES + kAccBufs + b); };
  const uint32_t drain_bar = bars + 8u * (2 * STAGES + 2 * kAccBufs);
  uint32_t* tmem_slot =
      reinterpret_cast<uint32_t*>(gbase + STAGES * Cfg::kStageBytes + 8 * (2 * STAGES + 2 * kAccBufs + 1));
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * BN;
  const int nk_all = (K + kBK - 1) / kBK;
  const int kb0 = blockIdx.z * kps;
  const int nk = max(0, min(nk_all, kb0 + kps) - kb0);  // K blocks of this CTA

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full_bar(s), 1);
      mbar_init(empty_bar(s), 1);
    }
    for (int b = 0; b < kAccBufs; ++b) {
      mbar_init(accf_bar(b), 1);
      mbar_init(acce_bar(b), 4);  // one arrive per epilogue warp
    }
    mbar_init(drain_bar, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(tmem_slot);

  auto stage_a = [&](int s) { return base + s * Cfg::kStageBytes; };
  auto stage_b = [&](int s) { return stage_a(s) + Cfg::kABytes; };
  auto stage_alo = [&](int s) { return stage_b(s) + Cfg::kBBytes; };
  auto stage_blo = [&](int s) { return stage_alo(s) + Cfg::kABytes; };

  if (warp == 0 && lane == 0) {
    int issued = 0;
    bool ok = true;
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % STAGES;
      if (*abort_flag || !mbar_wait(empty_bar(s), ((kb / STAGES) & 1) ^ 1)) { ok = false; break; }
      mbar_expect_tx(full_bar(s), Cfg::kStageBytes);
      const int kx = (kb0 + kb) * kBK;
      tma_load_2d(stage_a(s), &map_a, full_bar(s), kx, m0);
      tma_load_2d(stage_b(s), &map_b, full_bar(s), kx, n0);
      tma_load_2d(stage_alo(s), &map_alo, full_bar(s), kx, m0);
      tma_load_2d(stage_blo(s), &map_blo, full_bar(s), kx, n0);
      ++issued;
    }
    if (!ok) {
      atomicOr(err, 2u);
      *abort_flag = 1;
      for (int kb = std::max(0, issued - STAGES); kb < issued; ++kb) mbar_wait(full_bar(kb % STAGES), (kb / STAGES) & 1);
    }
  } else if (warp == 1 && lane == 0) {
    constexpr uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                               ((uint32_t)(kBM >> 4) << 24);
    bool ok = true;
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % STAGES, b = kb % kAccBufs;
      if (*abort_flag || !mbar_wait(full_bar(s), (kb / STAGES) & 1) ||
          !mbar_wait(acce_bar(b), ((kb / kAccBufs) & 1) ^ 1)) {
        ok = false;
        break;
      }
      tc_fence_after();
      const uint32_t d = tmem + (uint32_t)(b * BN);
#pragma unroll
      for (int k = 0; k < kBK / 16; ++k) {
        const uint64_t a = sw128_desc(stage_a(s) + 32u * k);
        const uint64_t bb = sw128_desc(stage_b(s) + 32u * k);
        // small cross terms first, the dominant hi*hi term last
        mma_bf16(d, a, sw128_desc(stage_blo(s) + 32u * k), idesc, k != 0);
        mma_bf16(d, sw128_desc(stage_alo(s) + 32u * k), bb, idesc, 1);
        mma_bf16(d, a, bb, idesc, 1);
      }
      mma_commit(empty_bar(s));
      mma_commit(accf_bar(b));
    }
    if (!ok) {
      atomicOr(err, 2u);
      *abort_flag = 1;
    }
  } else if (warp >= 2) {
    const int q = warp & 3;
    const int row = m0 + q * 32 + lane;
    float sum[BN];
#pragma unroll
    for (int j = 0; j < BN; ++j) sum[j] = 0.f;
    bool ok = nk > 0;
    for (int kb = 0; kb < nk && ok; ++kb) {
      const int b = kb % kAccBufs;
      if (*abort_flag || !mbar_wait(accf_bar(b), (kb / kAccBufs) & 1)) { ok = false; break; }
      tc_fence_after();
#pragma unroll
      for (int c = 0; c < BN / 32; ++c) {
        uint32_t r[32];
        tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * BN + c * 32), r);
#pragma unroll
        for (int j = 0; j < 32; ++j) sum[c * 32 + j] += __uint_as_float(r[j]);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acce_bar(b));
    }
    if (!ok) {
      if (lane == 0) atomicOr(err, 2u);
      *abort_flag = 1;
    } else {
      // All MMAs are done, so the operand stages are free: stage this warp's
      // 32 x 128 block in shared memory (row pitch 129 floats: conflict-free
      // both ways) and write it back one coalesced 128-float row at a time.
      float* tile = reinterpret_cast<float*>(gbase) + q * 32 * (BN + 1);
#pragma unroll
      for (int j = 0; j < BN; ++j) tile[lane * (BN + 1) + j] = sum[j];
      __syncwarp();
      for (int rr = 0; rr < 32; ++rr) {
        const int grow = m0 + q * 32 + rr;
        if (grow >= M) break;
        if (partial) {  // split K: raw partial sums, epilogue after the reduction
          float* prow = partial + ((int64_t)blockIdx.z * M + grow) * N;
#pragma unroll
          for (int i = 0; i < BN / 32; ++i) {
            const int j = i * 32 + lane;
            if (n0 + j < N) prow[n0 + j] = tile[rr * (BN + 1) + j];
          }
          continue;
        }
        float* crow = C + (int64_t)grow * ldc;
#pragma unroll
        for (int i = 0; i < BN / 32; ++i) {
          const int j = i * 32 + lane;
          const int col = n0 + j;
          if (col < N) {
            float v = alpha * tile[rr * (BN + 1) + j];
            if (beta != 0.f) v += beta * crow[col];
            if (bias) v += bias[col];
            if (act == VKC_ACT_RELU) v = fmaxf(v, 0.f);
            else if (act == VKC_ACT_SIGMOID) v = 1.0f / (1.0f + expf(0.0f - v));
            crow[col] = v;
          }
        }
      }
      (void)row;
    }
  }

  // Before TMEM is released every MMA must have completed.  On the normal
  // path the epilogue waited for the last block's commit; after an abort the
  // issuer commits once more and waits (bounded) for that.
  if (warp == 1 && lane == 0 && *abort_flag) {
    mma_commit(drain_bar);
    mbar_wait(drain_bar, 0);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols) : "memory");
  }
}

// ------------------------------------------------------------ operand split
// K contiguous in the source: dst[r*Kp + k] from src[r*ld + k]; zero padding k >= K.
__global__ void k_split_kmajor(const float* __restrict__ src, int64_t R, int64_t K, int64_t ld,
                               __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo, int64_t Kp) {
  const int64_t total = R * Kp;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
    const int64_t r = i / Kp, k = i - r * Kp;
    const float x = k < K ? src[r * ld + k] : 0.f;
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    hi[i] = h;
    if (lo) lo[i] = __float2bfloat16_rn(x - __bfloat162float(h));
  }
}

// K is the row index of the source (src[k*ld + r]): 32x32 tiles through
// shared memory so both the read and the write are coalesced.
__global__ void k_split_transpose(const float* __restrict__ src, int64_t R, int64_t K, int64_t ld,
                                  __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo, int64_t Kp) {
  __shared__ float tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.x * 32, k0 = (int64_t)blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int j = ty; j < 32; j += 8) {
    const int64_t k = k0 + j, r = r0 + tx;
    tile[j][tx] = (k < K && r < R) ? src[k * ld + r] : 0.f;
  }
  __syncthreads();
  for (int j = ty; j < 32; j += 8) {
    const int64_t r = r0 + j, k = k0 + tx;
    if (r < R && k < Kp) {
      const float x = tile[tx][j];
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      hi[r * Kp + k] = h;
      if (lo) lo[r * Kp + k] = __float2bfloat16_rn(x - __bfloat162float(h));
    }
  }
}

// Produce K-major bf16 copies of a logical (R x K) operand.  `k_contig`:
// element (r, k) is src[r*ld + k]; otherwise src[k*ld + r].
int split_operand(vkc_device_t dev, const float* src, int64_t R, int64_t K, int64_t ld, bool k_contig,
                  __nv_bfloat16* hi, __nv_bfloat16* lo, int64_t Kp) {
  if (k_contig) {
    unsigned grid = stream_grid(dev, (size_t)(R * Kp), 256);
    k_split_kmajor<<<grid, 256, 0, dev->stream>>>(src, R, K, ld, hi, lo, Kp);
  } else {
    dim3 grid((unsigned)((R + 31) / 32), (unsigned)((Kp + 31) / 32));
    if (grid.y > 65535) return set_error(VKC_ERR_INVALID, "matmul: K too large for the transpose pre-pass");
    k_split_transpose<<<grid, dim3(32, 8), 0, dev->stream>>>(src, R, K, ld, hi, lo, Kp);
  }
  return check_launch("split_operand");
}

// ------------------------------------------------------------ host side
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    cudaGetLastError();
  });
  return fn;
}

// 2-D bf16 map over [rows][Kp] with a (64 x box_rows) box and 128B swizzle.
int make_map(CUtensorMap* map, const void* ptr, int64_t rows, int64_t Kp, int box_rows) {
  auto fn = encode_fn();
  if (!fn) return set_error(VKC_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(Kp * 2)};
  cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(VKC_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return VKC_OK;
}

template <int BN, bool X3, int STAGES>
int launch_tc(vkc_device_t dev, const CUtensorMap& ma, const CUtensorMap& mb, const CUtensorMap& malo,
              const CUtensorMap& mblo, int64_t M, int64_t N, int64_t K, float alpha, float beta, float* C, int64_t ldc,
              const GemmEpilogue& epi) {
  using Cfg = TcCfg<BN, X3, STAGES>;
  auto kern = k_gemm_tc<BN, X3, STAGES>;
  static bool attr_set = false;
  if (!attr_set) {
    VKC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::kSmem));
    attr_set = true;
  }
  dim3 grid((unsigned)((N + BN - 1) / BN), (unsigned)((M + kBM - 1) / kBM));
  kern<<<grid, kThreadsTC, Cfg::kSmem, dev->stream>>>(ma, mb, malo, mblo, (int)M, (int)N, (int)K, alpha, beta, C, ldc,
                                                      epi.bias, epi.act, dev->err_word);
  return check_launch("gemm_tc");
}

// ---- split-K tuning table: (precision, log2 buckets of M, N, K) -> splits.
// Filled from the autotuner's table at import (vkc_gemm_tune_set); shapes
// without an entry use the occupancy heuristic below.
std::mutex g_tune_mu;
std::map<uint64_t, int> g_tune;

inline int bucket(int64_t x) {
  int b = 0;
  while ((int64_t(1) << b) < x) ++b;
  return b;
}
inline uint64_t tune_key(int precision, int mb, int nb, int kb) {
  return ((uint64_t)precision << 24) | ((uint64_t)mb << 16) | ((uint64_t)nb << 8) | (uint64_t)kb;
}

int heuristic_splits(vkc_device_t dev, int64_t tiles, int nk) {
  int splits = 1;
  if (tiles * 2 <= dev->sm_count && nk >= 4) {
    splits = (int)std::min<int64_t>((dev->sm_count + tiles - 1) / tiles, nk / 2);
    splits = std::max(1, std::min(splits, 16));
  }
  return splits;
}

int choose_splits(vkc_device_t dev, int precision, int64_t M, int64_t N, int64_t K, int64_t tiles, int nk) {
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(tune_key(precision, bucket(M), bucket(N), bucket(K)));
    if (it != g_tune.end()) return std::max(1, std::min(it->second, std::max(1, nk)));
  }
  return heuristic_splits(dev, tiles, nk);
}

// C = act(alpha * sum_z partial[z] + beta * C + bias), z in order.
__global__ void __launch_bounds__(256)
k_splitk_reduce(const float* __restrict__ partial, int splits, int64_t M, int64_t N, float alpha, float beta,
                float* __restrict__ C, int64_t ldc, const float* __restrict__ bias, int act) {
  const int64_t total = M * N;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
    float s = partial[i];
    for (int z = 1; z < splits; ++z) s += partial[(int64_t)z * total + i];
    const int64_t r = i / N, col = i - r * N;
    float* c = C + r * ldc + col;
    float v = alpha * s;
    if (beta != 0.f) v += beta * *c;
    if (bias) v += bias[col];
    if (act == VKC_ACT_RELU) v = fmaxf(v, 0.f);
    else if (act == VKC_ACT_SIGMOID) v = 1.0f / (1.0f + expf(0.0f - v));
    *c = v;
  }
}

template <int STAGES>
int launch_tc_x3(vkc_device_t dev, const CUtensorMap& ma, const CUtensorMap& mb, const CUtensorMap& malo,
                 const CUtensorMap& mblo, int64_t M, int64_t N, int64_t K, float alpha, float beta, float* C,
                 int64_t ldc, const GemmEpilogue& epi) {
  using Cfg = TcCfg<128, true, STAGES>;
  auto kern = k_gemm_tc_x3<STAGES>;
  static bool attr_set = false;
  if (!attr_set) {
    VKC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::kSmem));
    attr_set = true;
  }
  const int64_t tiles = ((N + 127) / 128) * ((M + kBM - 1) / kBM);
  const int nk = (int)((K + kBK - 1) / kBK);
  // Split K when the tiles alone would leave most SMs idle (tuning table
  // first, then the occupancy heuristic); no empty split.
  int splits = choose_splits(dev, VKC_MM_BF16X3, M, N, K, tiles, nk);
  const int kps = (nk + splits - 1) / splits;
  splits = (nk + kps - 1) / kps;
  float* partial = nullptr;
  if (splits > 1) {
    int r = scratch_alloc(dev, sizeof(float) * (size_t)splits * M * N, (void**)&partial);
    if (r != VKC_OK) return r;
  }
  dim3 grid((unsigned)((N + 127) / 128), (unsigned)((M + kBM - 1) / kBM), (unsigned)splits);
  kern<<<grid, kThreadsTC, Cfg::kSmem, dev->stream>>>(ma, mb, malo, mblo, (int)M, (int)N, (int)K, alpha, beta, C, ldc,
                                                      epi.bias, epi.act, dev->err_word, partial, kps);
  int r = check_launch("gemm_tc_x3");
  if (r == VKC_OK && splits > 1) {
    unsigned g = stream_grid(dev, (size_t)(M * N), 256);
    k_splitk_reduce<<<g, 256, 0, dev->stream>>>(partial, splits, M, N, alpha, beta, C, ldc, epi.bias, epi.act);
    r = check_launch("splitk_reduce");
  }
  scratch_free(dev, partial);
  return r;
}

}  // namespace

}  // namespace vkc

VKC_EXPORT int vkc_gemm_tune_set(int precision, int64_t m, int64_t n, int64_t k, int splits) {
  VKC_REQUIRE(splits >= 0 && splits <= 64, "splits out of range");
  std::lock_guard<std::mutex> lk(vkc::g_tune_mu);
  auto key = vkc::tune_key(precision, vkc::bucket(m), vkc::bucket(n), vkc::bucket(k));
  if (splits == 0) vkc::g_tune.erase(key);
  else vkc::g_tune[key] = splits;
  return VKC_OK;
}

VKC_EXPORT int vkc_gemm_tune_get(vkc_device_t dev, int precision, int64_t m, int64_t n, int64_t k, int* splits) {
  VKC_REQUIRE(dev && splits, "NULL argument");
  const int64_t tiles = ((n + 127) / 128) * ((m + 127) / 128);
  const int nk = (int)((k + 63) / 64);
  *splits = vkc::choose_splits(dev, precision, m, n, k, tiles, nk);
  return VKC_OK;
}

VKC_EXPORT int vkc_gemm_tune_clear(void) {
  std::lock_guard<std::mutex> lk(vkc::g_tune_mu);
  vkc::g_tune.clear();
  return VKC_OK;
}

namespace vkc {

int gemm_tc(vkc_device_t dev, int precision, bool ta, bool tb, int64_t M, int64_t N, int64_t K, float alpha,
            const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc,
            GemmEpilogue epi) {
  if (M == 0 || N == 0) return VKC_OK;
  if (K == 0) return gemm_simt(dev, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, epi);
  VKC_REQUIRE(M < (1ll << 31) && N < (1ll << 31) && K < (1ll << 31), "matmul dimension too large");
  VKC_REQUIRE((M + kBM - 1) / kBM <= 65535, "matmul: M too large for the tensor-core grid");
  const bool x3 = precision == VKC_MM_BF16X3;
  const int64_t Kp = (K + 7) / 8 * 8;  // 16-byte aligned rows for TMA
  const size_t a_elems = (size_t)M * Kp, b_elems = (size_t)N * Kp;
  const size_t bytes = (a_elems + b_elems) * sizeof(__nv_bfloat16) * (x3 ? 2 : 1);
  void* scratch = nullptr;
  int r = scratch_alloc(dev, bytes, &scratch);
  if (r != VKC_OK) return r;
  auto* a_hi = static_cast<__nv_bfloat16*>(scratch);
  auto* b_hi = a_hi + a_elems;
  __nv_bfloat16* a_lo = x3 ? b_hi + b_elems : nullptr;
  __nv_bfloat16* b_lo = x3 ? a_lo + a_elems : nullptr;
  // op(A)(m,k): ta ? A[k*lda + m] : A[m*lda + k]  -> K contiguous iff !ta
  // op(B)(k,n): tb ? B[n*ldb + k] : B[k*ldb + n]  -> (n,k) K contiguous iff tb
  r = split_operand(dev, A, M, K, lda, !ta, a_hi, a_lo, Kp);
  if (r == VKC_OK) r = split_operand(dev, B, N, K, ldb, tb, b_hi, b_lo, Kp);
  CUtensorMap ma, mb, malo, mblo;
  const int bn = x3 ? 128 : 256;
  if (r == VKC_OK) r = make_map(&ma, a_hi, M, Kp, kBM);
  if (r == VKC_OK) r = make_map(&mb, b_hi, N, Kp, bn);
  if (r == VKC_OK) r = make_map(&malo, x3 ? (const void*)a_lo : (const void*)a_hi, M, Kp, kBM);
  if (r == VKC_OK) r = make_map(&mblo, x3 ? (const void*)b_lo : (const void*)b_hi, N, Kp, bn);
  if (r == VKC_OK) {
    if (x3) r = launch_tc_x3<3>(dev, ma, mb, malo, mblo, M, N, K, alpha, beta, C, ldc, epi);
    else r = launch_tc<256, false, 4>(dev, ma, mb, malo, mblo, M, N, K, alpha, beta, C, ldc, epi);
  }
  scratch_free(dev, scratch);
  return r;
}

}  // namespace vkc
