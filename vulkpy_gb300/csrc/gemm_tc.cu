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
// k_gemm_tcp is persistent (one CTA per SM; each CTA loads every operand tile
// it multiplies into its own shared memory) with two TMEM accumulators, so a
// tile's epilogue overlaps the next tile's MMAs.  Every mbarrier wait is
// bounded by a wall-clock limit; on expiry the CTA records bit1 in the device
// error word, drains what it issued and returns.
#include "gemm_tc.cuh"
#include "tc_ptx.cuh"
#include "tc_epilogue.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <map>
#include <mutex>

namespace vkc {
namespace {

// ------------------------------------------------------------ the kernel
// Persistent tensor-core GEMM.
//
// Work unit: a 128 x BN tile of C over one K range (split K).  CTA b takes
// units b, b + grid, ...; units run through the tiles in raster groups of 16
// tile rows (down a column of tiles first), so the CTAs working at the same
// time multiply the same few op(B) tiles and the repeated reads hit L2.  Each
// CTA TMA-loads its 128 rows of op(A) and the whole op(B) tile into its own
// shared memory (no clusters; CTAs share nothing) and computes its tile with
// single-CTA tcgen05.mma (M=128, N=BN, K=16) into one of two TMEM
// accumulators, so the epilogue of one accumulation overlaps the MMAs of the
// next.
//
// Warps: 0 = TMA producer (lane 0), 1 = TMEM owner + MMA issuer (lane 0),
// 2..9 = epilogue.  Epilogue warp w reads TMEM lanes 32*(w%4).. (the lane
// quarter its warp rank allows) and columns 128*((w-2)/4).. of a buffer.
//
// bf16 mode: one accumulation per unit over the whole K range.
// split mode (hi*hi + hi*lo + lo*hi): one accumulation per DRAIN K blocks;
// the epilogue adds each into fp32 registers with round-to-nearest, so the
// tensor pipe's truncating accumulation spans at most DRAIN*64 of K.
constexpr int kEpiWarps = 8;
constexpr int kThreadsP = 32 * (2 + kEpiWarps);
constexpr int kGroupM = 16;        // tile rows per raster group (L2 reuse)


// BN: columns of C per CTA tile (256 or 128; the autotuner picks per shape).
template <bool X3, int BN, int STAGES>
struct PCfg {
  static constexpr uint32_t kABytes = kBM * kBK * 2;             // 16 KB
  static constexpr uint32_t kBBytes = BN * kBK * 2;
  static constexpr uint32_t kStageBytes = (X3 ? 2u : 1u) * (kABytes + kBBytes);
  static constexpr uint32_t kBarOff = STAGES * kStageBytes;
  // full[S], empty[S], accf[2], acce[2], drain, red[2], epi, then tmem slot
  // + abort flag
  static constexpr uint32_t kSlotOff = kBarOff + 8u * (2 * STAGES + 8);
  static constexpr uint32_t kEpiOff = (kSlotOff + 16 + 127) / 128 * 128;  // per-warp epilogue stages
  static constexpr uint32_t kSmem = kEpiOff + kEpiWarps * kEpiStageBytes + 1024 /*alignment slack*/;
};

struct PUnit {
  int m0, n0, kb0, nkb, z;
};

template <int BN>
__device__ __forceinline__ PUnit unit_of(int u, int splits, int kps, int nk, int m_blocks, int n_blocks) {
  const int tile = u / splits, z = u - tile * splits;
  const int per_group = kGroupM * n_blocks;
  const int g = tile / per_group, first = g * kGroupM;
  const int gsize = min(kGroupM, m_blocks - first);
  const int within = tile - g * per_group;
  const int mb = first + within % gsize, nb = within / gsize;
  PUnit p;
  p.m0 = mb * kBM;
  p.n0 = nb * BN;
  p.kb0 = z * kps;
  p.nkb = max(0, min(nk, p.kb0 + kps) - p.kb0);
  p.z = z;
  return p;
}

// C = act(alpha * sum_z partial[z] + beta * C + bias), z in order.
__device__ __forceinline__ float splitk_epilogue(float s, float alpha, float beta, float c, bool has_bias, float bias,
                                                 int act) {
  float v = alpha * s;
  if (beta != 0.f) v += beta * c;
  if (has_bias) v += bias;
  if (act == VKC_ACT_RELU) v = fmaxf(v, 0.f);
  else if (act == VKC_ACT_SIGMOID) v = 1.0f / (1.0f + expf(0.0f - v));
  return v;
}

// Split-K inside a cluster: the cluster's `splits` CTAs have each stored the
// partial sums of one K range of the tile (m0, n0) into partial[z] (M x N
// planes); this CTA adds up rows [r0, r1) of the tile, z in order, and
// writes them through the epilogue -- the arithmetic of the separate
// reduction launch.  ew: the epilogue warp (0..7).
__device__ __forceinline__ void cluster_reduce_rows(const float* partial, int splits, int M, int N, int m0, int n0,
                                                    int bn, int r0, int r1, float alpha, float beta, float* C,
                                                    int64_t ldc, const float* bias, int act, const float* dmask,
                                                    int dact, int ew, int lane) {
  const int64_t plane = (int64_t)M * N;
  const int cols = min(bn, N - n0);
  for (int r = r0 + ew; r < r1; r += kEpiWarps) {
    const int64_t row = (int64_t)(m0 + r);
    for (int c = lane; c < cols; c += 32) {
      const int64_t off = row * N + n0 + c;
      float t[8];
#pragma unroll
      for (int z = 0; z < 8; ++z) t[z] = z < splits ? __ldcg(partial + z * plane + off) : 0.f;
      float s = t[0];
#pragma unroll
      for (int z = 1; z < 8; ++z)
        if (z < splits) s += t[z];
      float* cp = C + row * ldc + n0 + c;
      float v = splitk_epilogue(s, alpha, beta, beta != 0.f ? *cp : 0.f, bias != nullptr, bias ? bias[n0 + c] : 0.f, act);
      if (dmask) v = act_deriv(v, dmask[row * ldc + n0 + c], dact);
      *cp = v;
    }
  }
}

// cl_reduce: the grid is made of clusters of `splits` CTAs (one per K range
// of a tile) that reduce their partial sums themselves (no separate launch).
template <bool X3, int BN, int STAGES, int DRAIN>
__global__ void __launch_bounds__(kThreadsP, 1)
k_gemm_tcp(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
           const __grid_constant__ CUtensorMap map_alo, const __grid_constant__ CUtensorMap map_blo, int M, int N,
           int K, float alpha, float beta, float* __restrict__ C, int64_t ldc, const float* __restrict__ bias, int act,
           uint32_t* err, float* __restrict__ partial, int splits, int kps, int m_blocks, int n_blocks,
           int cl_reduce, const float* __restrict__ dmask, int dact) {
  using Cfg = PCfg<X3, BN, STAGES>;
  constexpr uint32_t kCols = 2 * BN;  // two accumulators
  constexpr int CW = BN / 2;          // columns per epilogue warp
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint8_t* gbase = smem_raw + (base - raw);
  const uint32_t bars = base + Cfg::kBarOff;
  auto full_bar = [&](int s) { return bars + 8u * s; };
  auto empty_bar = [&](int s) { return bars + 8u * (STAGES + s); };
  auto accf_bar = [&](int b) { return bars + 8u * (2 * STAGES + b); };
  auto acce_bar = [&](int b) { return bars + 8u * (2 * STAGES + 2 + b); };
  const uint32_t drain_bar = bars + 8u * (2 * STAGES + 4);
  // red[u & 1]: all partials of the cluster's u-th tile stored (two, used in
  // turn: a peer already on the next tile arrives on the other one, so it
  // cannot complete a phase early); epi: this CTA's epilogue warps stored
  auto red_bar = [&](int u) { return bars + 8u * (2 * STAGES + 5 + (u & 1)); };
  const uint32_t epi_bar = bars + 8u * (2 * STAGES + 7);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gbase + Cfg::kSlotOff);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  const int nk = (K + kBK - 1) / kBK;
  const int units = m_blocks * n_blocks * splits;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full_bar(s), 1);
      mbar_init(empty_bar(s), 1);  // the MMA issuer's commit
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accf_bar(b), 1);
      mbar_init(acce_bar(b), kEpiWarps);
    }
    mbar_init(drain_bar, 1);
    if (cl_reduce) {
      mbar_init(red_bar(0), (uint32_t)splits);  // one arrival from each CTA of the cluster
      mbar_init(red_bar(1), (uint32_t)splits);
      mbar_init(epi_bar, kEpiWarps);
    }
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
  // peers arrive on this CTA's red_bar only after every CTA has initialised it
  if (cl_reduce) cluster_sync_all();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(tmem_slot);
  // the set-up above overlaps the previous kernel's tail; operands and C below
  pdl_wait();
  pdl_trigger();

  auto stage_a = [&](int s) { return base + s * Cfg::kStageBytes; };
  auto stage_b = [&](int s) { return stage_a(s) + Cfg::kABytes; };
  auto stage_alo = [&](int s) { return stage_b(s) + Cfg::kBBytes; };
  auto stage_blo = [&](int s) { return stage_alo(s) + Cfg::kABytes; };

  if (warp == 0 && lane == 0) {
    // ---------------- TMA producer
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&map_a)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&map_b)) : "memory");
    if (X3) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&map_alo)) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&map_blo)) : "memory");
    }
    int it = 0;
    bool ok = true;
    for (int u = (int)blockIdx.x; u < units && ok; u += (int)gridDim.x) {
      const PUnit p = unit_of<BN>(u, splits, kps, nk, m_blocks, n_blocks);
      for (int kb = 0; kb < p.nkb; ++kb, ++it) {
        const int s = it % STAGES;
        if (*abort_flag || !mbar_wait(empty_bar(s), ((it / STAGES) & 1) ^ 1)) { ok = false; break; }
        mbar_expect_tx(full_bar(s), Cfg::kStageBytes);
        const int kx = (p.kb0 + kb) * kBK;
        tma_load_2d(stage_a(s), &map_a, full_bar(s), kx, p.m0);
        tma_load_2d(stage_b(s), &map_b, full_bar(s), kx, p.n0);
        if (X3) {
          tma_load_2d(stage_alo(s), &map_alo, full_bar(s), kx, p.m0);
          tma_load_2d(stage_blo(s), &map_blo, full_bar(s), kx, p.n0);
        }
      }
    }
    if (!ok) {
      atomicOr(err, 2u);
      *abort_flag = 1;
    }
    // Tail: wait until the MMAs have released every stage, so no copy or
    // commit is still in flight at exit.
    for (int t = 0; t < STAGES && it - STAGES + t >= 0; ++t) {
      const int j = it - STAGES + t;
      if (!mbar_wait(empty_bar(j % STAGES), (j / STAGES) & 1)) {
        atomicOr(err, 2u);
        break;
      }
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    constexpr uint32_t idesc = (1u << 4)            // D: fp32
                               | (1u << 7)          // A: bf16
                               | (1u << 10)         // B: bf16
                               | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
    int it = 0, acc_it = 0;
    bool ok = true;
    for (int u = (int)blockIdx.x; u < units && ok; u += (int)gridDim.x) {
      const PUnit p = unit_of<BN>(u, splits, kps, nk, m_blocks, n_blocks);
      const int span = X3 ? DRAIN : p.nkb;  // K blocks per accumulation
      for (int g0 = 0; g0 < p.nkb && ok; g0 += span, ++acc_it) {
        const int b = acc_it & 1;
        if (*abort_flag || !mbar_wait(acce_bar(b), ((acc_it >> 1) & 1) ^ 1)) { ok = false; break; }
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(b * BN);
        const int g1 = min(p.nkb, g0 + span);
        for (int kb = g0; kb < g1; ++kb, ++it) {
          const int s = it % STAGES;
          if (*abort_flag || !mbar_wait(full_bar(s), (it / STAGES) & 1)) { ok = false; break; }
          tc_fence_after();
#pragma unroll
          for (int k = 0; k < kBK / 16; ++k) {
            const uint64_t a = sw128_desc(stage_a(s) + 32u * k);
            const uint64_t bb = sw128_desc(stage_b(s) + 32u * k);
            const uint32_t first = (kb == g0 && k == 0) ? 0u : 1u;
            if (X3) {
              // small cross terms first, the dominant hi*hi term last
              mma_bf16(d, a, sw128_desc(stage_blo(s) + 32u * k), idesc, first);
              mma_bf16(d, sw128_desc(stage_alo(s) + 32u * k), bb, idesc, 1);
              mma_bf16(d, a, bb, idesc, 1);
            } else {
              mma_bf16(d, a, bb, idesc, first);
            }
          }
          mma_commit(empty_bar(s));  // frees stage s once read
        }
        if (!ok) break;
        mma_commit(accf_bar(b));
      }
    }
    if (!ok) {
      atomicOr(err, 2u);
      *abort_flag = 1;
    }
  } else if (warp >= 2) {
    // ---------------- epilogue: TMEM -> fp32 registers -> global
    // The store loop runs over 32-column chunks read back from TMEM (not
    // unrolled), so the alpha/beta/bias/activation code exists once: with a
    // fully unrolled 128-column epilogue the kernel spent most of a small
    // launch waiting on instruction fetch.
    const int q = warp & 3;          // TMEM lane quarter
    const int h = (warp - 2) >> 2;   // column half of the tile
    const uint32_t lane_addr = (uint32_t)(q * 32) << 16;
    int acc_it = 0, red_it = 0;
    bool ok = true;
    for (int u = (int)blockIdx.x; u < units && ok; u += (int)gridDim.x) {
      const PUnit p = unit_of<BN>(u, splits, kps, nk, m_blocks, n_blocks);
      const int span = X3 ? DRAIN : p.nkb;
      const int ngroups = (p.nkb + span - 1) / span;
      float acc[X3 ? CW : 1];
      if (X3) {
#pragma unroll
        for (int j = 0; j < (X3 ? CW : 1); ++j) acc[j] = 0.f;
      }
      int b = 0;
      for (int gi = 0; gi < ngroups; ++gi, ++acc_it) {
        b = acc_it & 1;
        if (*abort_flag || !mbar_wait(accf_bar(b), (acc_it >> 1) & 1)) { ok = false; break; }
        tc_fence_after();
        if (X3 && ngroups > 1) {
          // add this accumulation to the fp32 sums; after the last one, put
          // the sums back into the buffer for the store loop below (with a
          // single accumulation the store loop reads it as it is)
          const bool last = gi == ngroups - 1;
#pragma unroll
          for (int c = 0; c < CW / 32; c += 2) {
            const uint32_t ta = tmem + lane_addr + (uint32_t)(b * BN + h * CW + c * 32);
            uint32_t r0[32], r1[32];
            tmem_ld32_nw(ta, r0);
            tmem_ld32_nw(ta + 32, r1);
            tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              acc[(X3 ? c * 32 + j : 0)] += __uint_as_float(r0[j]);
              r0[j] = __float_as_uint(acc[(X3 ? c * 32 + j : 0)]);
              acc[(X3 ? c * 32 + 32 + j : 0)] += __uint_as_float(r1[j]);
              r1[j] = __float_as_uint(acc[(X3 ? c * 32 + 32 + j : 0)]);
            }
            if (last) {
              tmem_st32_nw(ta, r0);
              tmem_st32_nw(ta + 32, r1);
            }
          }
          if (last) tmem_wait_st();
        }
        if (gi + 1 < ngroups) {
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(acce_bar(b));
        }
      }
      if (!ok) break;
      if (ngroups == 0) continue;
      const bool raw_out = partial != nullptr;
      float* cbase = raw_out ? partial + (int64_t)p.z * M * N : C;
      const int64_t ld = raw_out ? (int64_t)N : ldc;
      float* stage = reinterpret_cast<float*>(gbase + Cfg::kEpiOff) + (warp - 2) * (kEpiStageBytes / 4);
#pragma unroll 1
      for (int c = 0; c < CW / 32; ++c) {  // one copy of the epilogue code
        uint32_t r0[32];
        tmem_ld32(tmem + lane_addr + (uint32_t)(b * BN + h * CW + c * 32), r0);
        const int col0 = p.n0 + h * CW + c * 32;
        if (p.m0 + q * 32 < M && col0 < N)
          // (the split kernel with 256-column tiles holds 128 running sums per
          // thread and has no registers to spare for the fixed forms)
          epilogue_tile32<!(X3 && BN == 256)>(r0, stage, cbase, raw_out ? nullptr : dmask, bias, ld, p.m0 + q * 32, M,
                                              col0, N, alpha, beta, act, raw_out, nullptr, 0.f, dact);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acce_bar(b));
      if (cl_reduce) {
        // This warp's partial sums are stored; when all 8 warps' are, one
        // thread tells every CTA of the cluster, and once all `splits` CTAs
        // have, each adds up its share of the tile's rows.  (mbarriers with
        // bounded waits, so a CTA that gave up cannot hang the others.)
        __threadfence();
        __syncwarp();
        if (lane == 0) mbar_arrive(epi_bar);
        if (warp == 2 && lane == 0) {
          if (mbar_wait(epi_bar, red_it & 1)) {
            __threadfence();
            for (int r = 0; r < splits; ++r) mbar_arrive_cluster(red_bar(red_it), (uint32_t)r);
          } else {
            ok = false;
          }
        }
        if (!ok || !mbar_wait_cluster(red_bar(red_it), (red_it >> 1) & 1)) {
          ok = false;
          break;
        }
        ++red_it;
        const int rows = min(kBM, M - p.m0), share = (kBM + splits - 1) / splits;
        const int r0 = min(rows, p.z * share), r1 = min(rows, r0 + share);
        cluster_reduce_rows(partial, splits, M, N, p.m0, p.n0, BN, r0, r1, alpha, beta, C, ldc, bias, act, dmask,
                            dact, warp - 2, lane);
      }
    }
    if (!ok) {
      if (lane == 0) atomicOr(err, 2u);
      *abort_flag = 1;
    }
  }

  // Before TMEM is released every MMA must have completed: on the normal
  // path the epilogue waited for every accumulation's commit; after an abort
  // the issuer commits once more and waits (bounded) for that.
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
  // no CTA leaves while a peer may still arrive on its barriers
  if (cl_reduce) cluster_sync_all();
}

// ------------------------------------------------------------ operand split
__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16& h, __nv_bfloat16& l) {
  h = __float2bfloat16_rn(x);
  l = __float2bfloat16_rn(x - __bfloat162float(h));
}

// K contiguous in the source: dst[r*Kp + k] from src[r*ld + k], zero padding
// k >= K.  8 elements per thread: 2 x float4 in (`vec`: ld % 4 == 0 and a
// 16-byte aligned source; otherwise element loads), one 16-byte store per
// output (Kp % 8 == 0); the chunk that straddles K is read element by
// element, chunks past K are zero.  Blocks `blk` of `nblk` stride over the
// chunks.
__device__ __forceinline__ void split_kmajor8_body(const float* __restrict__ src, int64_t R, int64_t K, int64_t ld,
                                                   __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                                                   int64_t Kp, int64_t blk, int64_t nblk, bool vec = true) {
  const int64_t per_row = Kp / 8, total = R * per_row;
  const int64_t stride = nblk * blockDim.x;
  for (int64_t i = blk * blockDim.x + threadIdx.x; i < total; i += stride) {
    const int64_t r = i / per_row, k = (i - r * per_row) * 8;
    float x[8];
    if (vec && k + 8 <= K) {
      const float4* p = reinterpret_cast<const float4*>(src + r * ld + k);
      const float4 v0 = *p, v1 = *(p + 1);
      x[0] = v0.x, x[1] = v0.y, x[2] = v0.z, x[3] = v0.w, x[4] = v1.x, x[5] = v1.y, x[6] = v1.z, x[7] = v1.w;
    } else {
#pragma unroll
      for (int t = 0; t < 8; ++t) x[t] = k + t < K ? src[r * ld + k + t] : 0.f;
    }
    __align__(16) __nv_bfloat16 h[8], l[8];
#pragma unroll
    for (int t = 0; t < 8; ++t) split_bf16(x[t], h[t], l[t]);
    *reinterpret_cast<uint4*>(hi + r * Kp + k) = *reinterpret_cast<const uint4*>(h);
    if (lo) *reinterpret_cast<uint4*>(lo + r * Kp + k) = *reinterpret_cast<const uint4*>(l);
  }
}

// K is the row index of the source (src[k*ld + r]): 64 (k) x 64 (r) tiles
// through shared memory.  Reads: each thread one float4 of a k row (16 rows
// of 256 bytes per pass; with `vec` false -- ld % 4 != 0 or an unaligned
// source -- four element loads); writes: each thread 8 consecutive k of one
// r as a 16-byte store (8 rows of 128 bytes per pass).  R need not be a
// multiple of 4 (the tail of a row is read element by element).  256
// threads; tile (bx, by) covers rows r in [64 bx, 64 bx + 64), k in
// [64 by, 64 by + 64).
__device__ __forceinline__ void split_transpose_body(const float* __restrict__ src, int64_t R, int64_t K, int64_t ld,
                                                     __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                                                     int64_t Kp, int64_t bx, int64_t by, float (*tile)[65],
                                                     bool vec = true) {
  const int64_t r0 = bx * 64, k0 = by * 64;
  const int t = threadIdx.x;
  {
    const int c4 = (t & 15) * 4, kr = t >> 4;  // 16 float4 per 64-wide row, 16 rows per pass
#pragma unroll
    for (int j = kr; j < 64; j += 16) {
      const int64_t k = k0 + j, r = r0 + c4;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (k < K) {
        const float* p = src + k * ld + r;
        if (vec && r + 3 < R) {
          v = *reinterpret_cast<const float4*>(p);
        } else if (r + 3 < R) {
          v = make_float4(p[0], p[1], p[2], p[3]);
        } else {
          if (r < R) v.x = p[0];
          if (r + 1 < R) v.y = p[1];
          if (r + 2 < R) v.z = p[2];
        }
      }
      tile[j][c4] = v.x;
      tile[j][c4 + 1] = v.y;
      tile[j][c4 + 2] = v.z;
      tile[j][c4 + 3] = v.w;
    }
  }
  __syncthreads();
  const int k8 = (t & 7) * 8, rr = t >> 3;  // 8 threads per 64-wide k row, 32 rows per pass
#pragma unroll
  for (int j = rr; j < 64; j += 32) {
    const int64_t r = r0 + j, k = k0 + k8;
    if (r < R && k < Kp) {  // Kp % 8 == 0, so all 8 are inside the row
      __align__(16) __nv_bfloat16 h[8], l[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) split_bf16(tile[k8 + q][j], h[q], l[q]);
      *reinterpret_cast<uint4*>(hi + r * Kp + k) = *reinterpret_cast<const uint4*>(h);
      if (lo) *reinterpret_cast<uint4*>(lo + r * Kp + k) = *reinterpret_cast<const uint4*>(l);
    }
  }
}

// Both operands of a GEMM in one launch (two launches cost more than the
// conversion itself for the small GEMMs of an MLP step): blocks [0, a.blocks)
// convert op(A), the rest op(B).
struct SplitJob {
  const float* src;
  int64_t R, K, ld, Kp;
  __nv_bfloat16* hi;
  __nv_bfloat16* lo;
  int64_t tiles_x;  // transpose: tiles along R; 0: K contiguous (8 per thread)
  int64_t blocks;
  int vec;          // 16-byte loads allowed (ld % 4 == 0, aligned source)
};

__global__ void __launch_bounds__(256) k_split_pair(const __grid_constant__ SplitJob a,
                                                    const __grid_constant__ SplitJob b) {
  __shared__ float tile[64][65];
  pdl_wait();
  pdl_trigger();
  const bool first = blockIdx.x < a.blocks;
  const SplitJob& j = first ? a : b;
  const int64_t blk = first ? (int64_t)blockIdx.x : (int64_t)blockIdx.x - a.blocks;
  if (j.tiles_x == 0)
    split_kmajor8_body(j.src, j.R, j.K, j.ld, j.hi, j.lo, j.Kp, blk, j.blocks, j.vec != 0);
  else
    split_transpose_body(j.src, j.R, j.K, j.ld, j.hi, j.lo, j.Kp, blk % j.tiles_x, blk / j.tiles_x, tile, j.vec != 0);
}

// Both operands in one k_split_pair launch (16-byte loads where a source
// allows them, element loads where it does not).
int split_operands(vkc_device_t dev, const float* A, int64_t M, int64_t lda, bool a_kcontig, __nv_bfloat16* a_hi,
                   __nv_bfloat16* a_lo, const float* B, int64_t N, int64_t ldb, bool b_kcontig,
                   __nv_bfloat16* b_hi, __nv_bfloat16* b_lo, int64_t K, int64_t Kp) {
  auto aligned = [](const float* p, int64_t ld) { return ld % 4 == 0 && ((uintptr_t)p & 15u) == 0; };
  const int64_t cap = (int64_t)dev->sm_count * resident_blocks((const void*)k_split_pair, 256);
  auto job = [&](const float* src, int64_t R, int64_t ld, bool kcontig, __nv_bfloat16* hi, __nv_bfloat16* lo) {
    SplitJob j{src, R, K, ld, Kp, hi, lo, 0, 0, aligned(src, ld) ? 1 : 0};
    if (kcontig) {
      j.blocks = std::max<int64_t>(1, std::min<int64_t>((R * (Kp / 8) + 255) / 256, cap));
    } else {
      j.tiles_x = (R + 63) / 64;
      j.blocks = j.tiles_x * ((Kp + 63) / 64);
    }
    return j;
  };
  const SplitJob ja = job(A, M, lda, a_kcontig, a_hi, a_lo), jb = job(B, N, ldb, b_kcontig, b_hi, b_lo);
  const int64_t grid = ja.blocks + jb.blocks;
  if (grid > 0x7fffffff) return set_error(VKC_ERR_INVALID, "matmul: operands too large for the pre-pass grid");
  const cudaError_t e = launch_pdl(k_split_pair, dim3((unsigned)grid), dim3(256), 0, dev->stream, ja, jb);
  if (e != cudaSuccess) return set_error(VKC_ERR_CUDA, "split_operands launch: %s", cudaGetErrorString(e));
  return check_launch("split_operands");
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

// ---- tuning table: (precision, log2 buckets of M, N, K) -> (tile width,
// split count), filled from the autotuner's table at import (vkc_gemm_plan_set
// / vkc_gemm_tune_set); shapes without an entry use the occupancy heuristic.
// A value holds splits in the low 16 bits and the tile width (128 or 256;
// 0 = 256) above them.
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

struct TcPlan {
  int bn;      // columns of C per CTA tile
  int splits;  // K ranges
};

// CTA tiles (128 x bn) of an M x N problem.
inline int64_t cta_tiles(int64_t M, int64_t N, int bn) {
  return ((M + kBM - 1) / kBM) * ((N + bn - 1) / bn);
}

TcPlan choose_plan(vkc_device_t dev, int precision, int64_t M, int64_t N, int64_t K) {
  const int nk = (int)std::max<int64_t>(1, (K + kBK - 1) / kBK);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(tune_key(precision, bucket(M), bucket(N), bucket(K)));
    if (it != g_tune.end()) {
      const int bn = (it->second >> 16) == 128 ? 128 : 256;
      return TcPlan{bn, std::max(1, std::min(it->second & 0xffff, nk))};
    }
  }
  return TcPlan{256, heuristic_splits(dev, cta_tiles(M, N, 256), nk)};
}


__device__ __forceinline__ void add4(float4& s, const float4& a) {
  s.x += a.x;
  s.y += a.y;
  s.z += a.z;
  s.w += a.w;
}

// The reduction's results also written as the next GEMM's operand: K-major
// bf16 hi (and lo) rows of pitch ldk (a multiple of 64), the split of
// split_kmajor8_body (same values), with the padding columns [N, ldk) zero.
__device__ __forceinline__ void split_out4(const SplitOut& so, int64_t r, int64_t col, int64_t N, float4 v) {
  __align__(8) __nv_bfloat16 h[4], l[4];
  split_bf16(v.x, h[0], l[0]);
  split_bf16(v.y, h[1], l[1]);
  split_bf16(v.z, h[2], l[2]);
  split_bf16(v.w, h[3], l[3]);
  *reinterpret_cast<uint2*>(so.hi + r * so.ldk + col) = *reinterpret_cast<const uint2*>(h);
  if (so.lo) *reinterpret_cast<uint2*>(so.lo + r * so.ldk + col) = *reinterpret_cast<const uint2*>(l);
  if (col + 4 == N)
    for (int64_t k = N; k < so.ldk; ++k) {
      so.hi[r * so.ldk + k] = __float2bfloat16_rn(0.f);
      if (so.lo) so.lo[r * so.ldk + k] = __float2bfloat16_rn(0.f);
    }
}
__device__ __forceinline__ void split_out1(const SplitOut& so, int64_t r, int64_t col, int64_t N, float v) {
  __nv_bfloat16 h, l;
  split_bf16(v, h, l);
  so.hi[r * so.ldk + col] = h;
  if (so.lo) so.lo[r * so.ldk + col] = l;
  if (col + 1 == N)
    for (int64_t k = N; k < so.ldk; ++k) {
      so.hi[r * so.ldk + k] = __float2bfloat16_rn(0.f);
      if (so.lo) so.lo[r * so.ldk + k] = __float2bfloat16_rn(0.f);
    }
}

// Four columns per thread (N % 4 == 0, ldc % 4 == 0, 16-byte aligned C);
// the split loads are issued four at a time ahead of their (ordered) adds.
__global__ void __launch_bounds__(256)
k_splitk_reduce4(const float* __restrict__ partial, int splits, int64_t M, int64_t N, float alpha, float beta,
                 float* __restrict__ C, int64_t ldc, const float* __restrict__ bias, int act,
                 const float* __restrict__ dmask, int dact, SplitOut so) {
  pdl_wait();
  pdl_trigger();
  const int64_t total = M * N, quads = total / 4;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < quads; q += stride) {
    const int64_t i = q * 4;
    const float4* p = reinterpret_cast<const float4*>(partial + i);
    float4 s = __ldcs(p);
    int z = 1;
    for (; z + 3 < splits; z += 4) {
      const float4 a = __ldcs(p + (int64_t)z * quads), b = __ldcs(p + (int64_t)(z + 1) * quads);
      const float4 c = __ldcs(p + (int64_t)(z + 2) * quads), d = __ldcs(p + (int64_t)(z + 3) * quads);
      add4(s, a);
      add4(s, b);
      add4(s, c);
      add4(s, d);
    }
    for (; z < splits; ++z) add4(s, __ldcs(p + (int64_t)z * quads));
    const int64_t r = i / N, col = i - r * N;
    float4* cp = reinterpret_cast<float4*>(C + r * ldc + col);
    const float4 c0 = beta != 0.f ? *cp : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 b4 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (bias) b4 = make_float4(bias[col], bias[col + 1], bias[col + 2], bias[col + 3]);
    float4 v;
    const bool hb = bias != nullptr;
    v.x = splitk_epilogue(s.x, alpha, beta, c0.x, hb, b4.x, act);
    v.y = splitk_epilogue(s.y, alpha, beta, c0.y, hb, b4.y, act);
    v.z = splitk_epilogue(s.z, alpha, beta, c0.z, hb, b4.z, act);
    v.w = splitk_epilogue(s.w, alpha, beta, c0.w, hb, b4.w, act);
    if (dmask) {
      const float4 y4 = *reinterpret_cast<const float4*>(dmask + r * ldc + col);
      v.x = act_deriv(v.x, y4.x, dact);
      v.y = act_deriv(v.y, y4.y, dact);
      v.z = act_deriv(v.z, y4.z, dact);
      v.w = act_deriv(v.w, y4.w, dact);
    }
    *cp = v;
    if (so.hi) split_out4(so, r, col, N, v);
  }
}

__global__ void __launch_bounds__(256)
k_splitk_reduce(const float* __restrict__ partial, int splits, int64_t M, int64_t N, float alpha, float beta,
                float* __restrict__ C, int64_t ldc, const float* __restrict__ bias, int act,
                const float* __restrict__ dmask, int dact, SplitOut so) {
  pdl_wait();
  pdl_trigger();
  const int64_t total = M * N;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
    float s = partial[i];
    for (int z = 1; z < splits; ++z) s += partial[(int64_t)z * total + i];
    const int64_t r = i / N, col = i - r * N;
    float* c = C + r * ldc + col;
    float v = splitk_epilogue(s, alpha, beta, beta != 0.f ? *c : 0.f, bias != nullptr, bias ? bias[col] : 0.f, act);
    if (dmask) v = act_deriv(v, dmask[r * ldc + col], dact);
    *c = v;
    if (so.hi) split_out1(so, r, col, N, v);
  }
}

int splitk_reduce(vkc_device_t dev, const float* partial, int splits, int64_t M, int64_t N, float alpha, float beta,
                  float* C, int64_t ldc, const GemmEpilogue& epi, const SplitOut* out = nullptr) {
  const SplitOut so = out ? *out : SplitOut{nullptr, nullptr, 0};
  if (N % 4 == 0 && ldc % 4 == 0 && ((uintptr_t)C & 15u) == 0 && ((uintptr_t)epi.dmask & 15u) == 0) {
    unsigned g = wave_grid(dev, k_splitk_reduce4, (size_t)(M * N / 4), 256);
    const cudaError_t e = launch_pdl(k_splitk_reduce4, dim3(g), dim3(256), 0, dev->stream, partial, splits, M, N,
                                     alpha, beta, C, ldc, epi.bias, epi.act, epi.dmask, epi.dact, so);
    if (e != cudaSuccess) return set_error(VKC_ERR_CUDA, "splitk_reduce launch: %s", cudaGetErrorString(e));
  } else {
    unsigned g = stream_grid(dev, (size_t)(M * N), 256);
    const cudaError_t e = launch_pdl(k_splitk_reduce, dim3(g), dim3(256), 0, dev->stream, partial, splits, M, N,
                                     alpha, beta, C, ldc, epi.bias, epi.act, epi.dmask, epi.dact, so);
    if (e != cudaSuccess) return set_error(VKC_ERR_CUDA, "splitk_reduce launch: %s", cudaGetErrorString(e));
  }
  return check_launch("splitk_reduce");
}

// Resident CTAs of this kernel on the device (cached per instantiation).
template <class Kern>
int max_ctas(vkc_device_t dev, Kern kern, uint32_t smem) {
  static int cached = 0;
  if (cached > 0) return cached;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)kern, kThreadsP, smem) != cudaSuccess ||
      per_sm <= 0) {
    cudaGetLastError();
    per_sm = 1;
  }
  cached = per_sm * dev->sm_count;
  return cached;
}

// Clusters of `size` CTAs of this kernel that can be resident at once (0: a
// cluster launch is not possible), cached per instantiation and size.
template <class Kern>
int max_clusters(Kern kern, uint32_t smem, int size) {
  static int cached[9] = {-1, -1, -1, -1, -1, -1, -1, -1, -1};
  if (size < 2 || size > 8) return 0;
  if (cached[size] >= 0) return cached[size];
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)size);
  cfg.blockDim = dim3(kThreadsP);
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)size;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, (const void*)kern, &cfg) != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  cached[size] = n;
  return n;
}

template <bool X3, int BN, int STAGES, int DRAIN>
int launch_tcp(vkc_device_t dev, const CUtensorMap& ma, const CUtensorMap& mb, const CUtensorMap& malo,
               const CUtensorMap& mblo, int64_t M, int64_t N, int64_t K, float alpha, float beta, float* C,
               int64_t ldc, const GemmEpilogue& epi, int splits, const SplitOut* out) {
  using Cfg = PCfg<X3, BN, STAGES>;
  auto kern = k_gemm_tcp<X3, BN, STAGES, DRAIN>;
  static bool attr_set = false;
  if (!attr_set) {
    VKC_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg::kSmem));
    attr_set = true;
  }
  const int64_t m_blocks = (M + kBM - 1) / kBM;
  const int n_blocks = (int)((N + BN - 1) / BN);
  const int64_t tiles = m_blocks * n_blocks;
  const int nk = (int)((K + kBK - 1) / kBK);
  // no empty split
  const int kps = (nk + splits - 1) / splits;
  splits = (nk + kps - 1) / kps;
  float* partial = nullptr;
  if (splits > 1) {
    int r = scratch_alloc(dev, sizeof(float) * (size_t)splits * M * N, (void**)&partial);
    if (r != VKC_OK) return r;
  }
  const int64_t units = tiles * splits;
  if (units >= (int64_t(1) << 31)) {
    scratch_free(dev, partial);
    return set_error(VKC_ERR_INVALID, "matmul: too many output tiles");
  }
  // 2..8 K ranges: the ranges of a tile run as one cluster and reduce in the
  // kernel (units u = tile * splits + z go to CTA u mod grid, and a grid of
  // whole clusters gives the CTAs of a cluster the splits of one tile).
  // Only when switched on (vkc_set_cluster_splitk) and outside a stream
  // capture: it saves a launch's host cost (MLP step eager 6.1k -> 6.4k
  // steps/s) but costs device time -- in a CUDA graph the separate
  // reduction, overlapped with the GEMM's tail by programmatic dependent
  // launch, is faster (10.4k against 8.7k steps/s), and so is an eager
  // 1024^3 bf16 product (0.022 against 0.026 ms).
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(dev->stream, &cap) != cudaSuccess) {
    cudaGetLastError();
    cap = cudaStreamCaptureStatusActive;
  }
  const int clusters = splits > 1 && cap == cudaStreamCaptureStatusNone && !out &&
                               g_cluster_splitk.load(std::memory_order_relaxed)
                           ? max_clusters(kern, Cfg::kSmem, splits)
                           : 0;
  cudaError_t e;
  if (clusters > 0) {
    const int ctas = (int)std::min<int64_t>(tiles, clusters) * splits;
    e = launch_pdl_cluster(kern, dim3((unsigned)ctas), dim3(kThreadsP), Cfg::kSmem, dev->stream, (unsigned)splits, ma,
                           mb, malo, mblo, (int)M, (int)N, (int)K, alpha, beta, C, ldc, epi.bias, epi.act,
                           dev->err_word, partial, splits, kps, (int)m_blocks, n_blocks, 1, epi.dmask, epi.dact);
  } else {
    const int ctas = (int)std::min<int64_t>(units, max_ctas(dev, kern, Cfg::kSmem));
    e = launch_pdl(kern, dim3((unsigned)ctas), dim3(kThreadsP), Cfg::kSmem, dev->stream, ma, mb, malo, mblo, (int)M,
                   (int)N, (int)K, alpha, beta, C, ldc, epi.bias, epi.act, dev->err_word, partial, splits, kps,
                   (int)m_blocks, n_blocks, 0, epi.dmask, epi.dact);
  }
  int r = e == cudaSuccess ? check_launch("gemm_tc")
                           : set_error(VKC_ERR_CUDA, "gemm_tc launch: %s", cudaGetErrorString(e));
  if (r == VKC_OK && splits > 1 && clusters == 0)
    r = splitk_reduce(dev, partial, splits, M, N, alpha, beta, C, ldc, epi, out);
  else if (r == VKC_OK && out)  // no reduction launch to write it: the pre-pass kernel on C
    r = split_operands(dev, C, M, ldc, true, out->hi, out->lo, nullptr, 0, 0, true, nullptr, nullptr, N, out->ldk);
  scratch_free(dev, partial);
  return r;
}

}  // namespace

}  // namespace vkc

namespace vkc {

int gemm_splitk_reduce(vkc_device_t dev, const float* partial, int splits, int64_t M, int64_t N, float alpha,
                       float beta, float* C, int64_t ldc, const GemmEpilogue& epi) {
  return splitk_reduce(dev, partial, splits, M, N, alpha, beta, C, ldc, epi);
}

// Split-K count of the fp32 SIMT GEMM (128 x 128 tiles): the tuning table's
// fp32 entry, else split when the tiles cannot fill half the GPU.
int simt_splits(vkc_device_t dev, int64_t M, int64_t N, int64_t K) {
  const int64_t tiles = ((M + 127) / 128) * ((N + 127) / 128);
  // K ranges of at least one 16-deep K step of the SIMT tile (small GEMMs
  // gain from many splits: 256^3 with 16 ranges 12.3 -> 9.0 us)
  const int cap = (int)std::max<int64_t>(1, (K + kGemmBK - 1) / kGemmBK);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(tune_key(VKC_MM_FP32, bucket(M), bucket(N), bucket(K)));
    if (it != g_tune.end()) return std::max(1, std::min(it->second & 0xffff, cap));
  }
  if (tiles * 2 > dev->sm_count || K < 512) return 1;
  return (int)std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(dev->sm_count / tiles, K / 256), 16));
}

}  // namespace vkc

VKC_EXPORT int vkc_gemm_plan_set(int precision, int64_t m, int64_t n, int64_t k, int splits, int tile_n) {
  VKC_REQUIRE(splits >= 0 && splits <= 64, "splits out of range");
  VKC_REQUIRE(tile_n == 128 || tile_n == 256, "tile width must be 128 or 256");
  std::lock_guard<std::mutex> lk(vkc::g_tune_mu);
  auto key = vkc::tune_key(precision, vkc::bucket(m), vkc::bucket(n), vkc::bucket(k));
  if (splits == 0) vkc::g_tune.erase(key);
  else vkc::g_tune[key] = splits | (tile_n << 16);
  return VKC_OK;
}

VKC_EXPORT int vkc_gemm_tune_set(int precision, int64_t m, int64_t n, int64_t k, int splits) {
  return vkc_gemm_plan_set(precision, m, n, k, splits, 256);
}

VKC_EXPORT int vkc_gemm_plan_get(vkc_device_t dev, int precision, int64_t m, int64_t n, int64_t k, int* splits,
                                 int* tile_n) {
  VKC_REQUIRE(dev && splits, "NULL argument");
  if (precision == VKC_MM_FP32) {
    *splits = vkc::simt_splits(dev, m, n, k);
    if (tile_n) *tile_n = 128;
    return VKC_OK;
  }
  const vkc::TcPlan p = vkc::choose_plan(dev, precision, m, n, k);
  *splits = p.splits;
  if (tile_n) *tile_n = p.bn;
  return VKC_OK;
}

VKC_EXPORT int vkc_gemm_tune_get(vkc_device_t dev, int precision, int64_t m, int64_t n, int64_t k, int* splits) {
  return vkc_gemm_plan_get(dev, precision, m, n, k, splits, nullptr);
}

VKC_EXPORT int vkc_gemm_tune_clear(void) {
  std::lock_guard<std::mutex> lk(vkc::g_tune_mu);
  vkc::g_tune.clear();
  return VKC_OK;
}

namespace vkc {

int tc_split_operands(vkc_device_t dev, const float* A, int64_t M, int64_t lda, bool a_kcontig,
                      __nv_bfloat16* a_hi, __nv_bfloat16* a_lo, const float* B, int64_t N, int64_t ldb,
                      bool b_kcontig, __nv_bfloat16* b_hi, __nv_bfloat16* b_lo, int64_t K, int64_t Kp) {
  return split_operands(dev, A, M, lda, a_kcontig, a_hi, a_lo, B, N, ldb, b_kcontig, b_hi, b_lo, K, Kp);
}

// The GEMM on operands already in K-major bf16 form ([M][Kp] and [N][Kp],
// Kp = K rounded up to 64, zero past K): tensor maps, plan, launch and
// split-K reduction; `out` (may be NULL) also receives C in that form.
int gemm_tc_presplit(vkc_device_t dev, int precision, int64_t M, int64_t N, int64_t K, float alpha,
                     const __nv_bfloat16* a_hi, const __nv_bfloat16* a_lo, const __nv_bfloat16* b_hi,
                     const __nv_bfloat16* b_lo, float beta, float* C, int64_t ldc, const GemmEpilogue& epi,
                     const SplitOut* out) {
  const bool x3 = precision == VKC_MM_BF16X3;
  const int64_t Kp = (K + kBK - 1) / kBK * kBK;
  // boxes are 64 K wide: 128 rows for a CTA's op(A) tile, bn rows for its
  // op(B) tile
  const TcPlan plan = choose_plan(dev, precision, M, N, K);
  CUtensorMap ma, mb, malo, mblo;
  int r = make_map(&ma, a_hi, M, Kp, kBM);
  if (r == VKC_OK) r = make_map(&mb, b_hi, N, Kp, plan.bn);
  if (r == VKC_OK) r = make_map(&malo, x3 ? (const void*)a_lo : (const void*)a_hi, M, Kp, kBM);
  if (r == VKC_OK) r = make_map(&mblo, x3 ? (const void*)b_lo : (const void*)b_hi, N, Kp, plan.bn);
  if (r != VKC_OK) return r;
  // stages fill ~192 KB of shared memory
  if (x3 && plan.bn == 256)
    return launch_tcp<true, 256, 2, kDrainX3>(dev, ma, mb, malo, mblo, M, N, K, alpha, beta, C, ldc, epi, plan.splits,
                                              out);
  if (x3)
    return launch_tcp<true, 128, 3, kDrainX3>(dev, ma, mb, malo, mblo, M, N, K, alpha, beta, C, ldc, epi, plan.splits,
                                              out);
  if (plan.bn == 256)
    return launch_tcp<false, 256, 4, 1>(dev, ma, mb, malo, mblo, M, N, K, alpha, beta, C, ldc, epi, plan.splits, out);
  return launch_tcp<false, 128, 6, 1>(dev, ma, mb, malo, mblo, M, N, K, alpha, beta, C, ldc, epi, plan.splits, out);
}

int gemm_tc(vkc_device_t dev, int precision, bool ta, bool tb, int64_t M, int64_t N, int64_t K, float alpha,
            const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* C, int64_t ldc,
            GemmEpilogue epi) {
  if (M == 0 || N == 0) return VKC_OK;
  if (K == 0) return gemm_simt(dev, ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, epi);
  VKC_REQUIRE(M < (1ll << 31) && N < (1ll << 31) && K < (1ll << 31), "matmul dimension too large");
  VKC_REQUIRE((M + kBM - 1) / kBM <= 65535, "matmul: M too large for the tensor-core grid");
  const bool x3 = precision == VKC_MM_BF16X3;
  // Rows padded with zeros to whole 64-wide K blocks: every TMA box is then
  // inside the operand along K (a box reaching past a short row, e.g. K = 10,
  // made the whole GEMM several times slower).
  const int64_t Kp = (K + kBK - 1) / kBK * kBK;
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
  r = split_operands(dev, A, M, lda, !ta, a_hi, a_lo, B, N, ldb, tb, b_hi, b_lo, K, Kp);
  if (r == VKC_OK) r = gemm_tc_presplit(dev, precision, M, N, K, alpha, a_hi, a_lo, b_hi, b_lo, beta, C, ldc, epi,
                                        nullptr);
  scratch_free(dev, scratch);
  return r;
}

}  // namespace vkc
