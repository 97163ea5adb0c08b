// Grouped GEMM: many independent problems of different shapes in one
// persistent launch, and the grouped element-wise pieces of a batched MLP
// training step (bias-gradient column sums, MSE loss and gradient, SGD).
//
// vulkpy runs every Dense layer of every model as its own job
// (batch_affine.comp, _vkarray.cc:403-438); 64 small models of uneven sizes
// are then bound by per-launch cost and by GEMMs too small to fill 152 SMs.
// Here the output tiles of all problems form one work list, ordered by K
// (longest first), and a persistent grid walks it round-robin.
//
// fp32: each tile is computed by the same code as the single-problem SIMT
// kernel (simt_tile), so results are bit-identical to vkc_gemm.
// bf16 / split-bf16x3: a pre-pass converts every operand into 128 x 64 bf16
// tiles already laid out as the 128-byte-swizzled shared-memory image the
// MMA descriptors expect (tile (r, k): row r's 16-byte chunk c at byte
// r*128 + ((c ^ (r & 7)) << 4)), so one untiled bulk copy per operand tile
// fills a pipeline stage -- no tensor maps, whose per-problem encoding would
// not fit a launch.  The MMA and epilogue follow k_gemm_tcp (split mode: one
// TMEM accumulation per kDrainX3 K blocks, drained into fp32 registers in
// order), so split-bf16x3 results are bit-identical to vkc_gemm when that call
// does not split K.
#include "colsum.cuh"
#include "gemm_simt.cuh"
#include "tc_ptx.cuh"
#include "tc_epilogue.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <numeric>
#include <vector>

namespace vkc {
namespace {

constexpr int kMaxGroup = 128;  // problems per launch (tables travel as kernel parameters)

// ------------------------------------------------------------ fp32 SIMT
struct SimtProb {
  const float* a;
  const float* b;
  float* c;
  const float* bias;
  const float* mask;
  int64_t lda, ldb, ldc;
  int64_t m, n, k;
  float alpha, beta;
  int act, trans;  // trans: bit0 op(A) = A^T, bit1 op(B) = B^T
  int tiles_n, tile0;
};

struct SimtTable {
  int count, total;
  SimtProb p[kMaxGroup];
};

template <class T>
__device__ __forceinline__ int find_problem(const T* p, int count, int t) {
  int lo = 0, hi = count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (p[mid].tile0 <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__global__ void __launch_bounds__(kGemmThreads, 2) k_gemm_simt_grouped(const __grid_constant__ SimtTable tab) {
  __shared__ __align__(16) SimtSmem sm;
  for (int t = blockIdx.x; t < tab.total; t += gridDim.x) {
    const SimtProb& P = tab.p[find_problem(tab.p, tab.count, t)];
    const int local = t - P.tile0;
    const int64_t m0 = (int64_t)(local / P.tiles_n) * kGemmBM;
    const int64_t n0 = (int64_t)(local % P.tiles_n) * kGemmBN;
    GemmEpilogue epi;
    epi.bias = P.bias;
    epi.act = P.act;
    __syncthreads();  // the previous tile's reads of `sm` are done
    switch (P.trans) {
      case 0:
        simt_tile<false, false>(P.m, P.n, P.k, P.alpha, P.a, P.lda, P.b, P.ldb, P.beta, P.c, P.ldc, epi, P.mask, m0,
                                n0, sm);
        break;
      case 1:
        simt_tile<true, false>(P.m, P.n, P.k, P.alpha, P.a, P.lda, P.b, P.ldb, P.beta, P.c, P.ldc, epi, P.mask, m0,
                               n0, sm);
        break;
      case 2:
        simt_tile<false, true>(P.m, P.n, P.k, P.alpha, P.a, P.lda, P.b, P.ldb, P.beta, P.c, P.ldc, epi, P.mask, m0,
                               n0, sm);
        break;
      default:
        simt_tile<true, true>(P.m, P.n, P.k, P.alpha, P.a, P.lda, P.b, P.ldb, P.beta, P.c, P.ldc, epi, P.mask, m0,
                              n0, sm);
        break;
    }
  }
}

// ------------------------------------------------------------ operand tiling
constexpr int kTileRows = 128, kTileK = 64;
constexpr uint32_t kTileBytes = kTileRows * kTileK * 2;  // 16 KB of bf16

struct TileOp {
  const float* src;
  __nv_bfloat16* hi;
  __nv_bfloat16* lo;  // NULL: plain bf16
  int64_t ld;
  int64_t rows, k;    // logical operand: rows x k, element (r, k)
  int k_contig;       // element (r, k) at src[r*ld + k]; else src[k*ld + r]
  int kt;             // K tiles
  int tile0;
};

struct TileTable {
  int count, total;
  TileOp op[2 * kMaxGroup];
};

// One 128 x 64 tile per block iteration: load (coalesced along whichever
// index is contiguous) into shared memory, then write 16-byte chunks of hi
// (and lo = bf16(x - hi)) at their swizzled positions.  Rows >= rows and
// k >= K are written as zeros.
__global__ void __launch_bounds__(256, 3) k_tile_operands(const __grid_constant__ TileTable tab) {
  __shared__ float s[kTileRows][kTileK + 1];
  const int tid = threadIdx.x;
  for (int t = blockIdx.x; t < tab.total; t += gridDim.x) {
    const TileOp& op = tab.op[find_problem(tab.op, tab.count, t)];
    const int local = t - op.tile0;
    const int rt = local / op.kt, kt = local % op.kt;
    const int64_t r0 = (int64_t)rt * kTileRows, k0 = (int64_t)kt * kTileK;
    __syncthreads();
    // all 32 loads of a thread are issued before the shared-memory stores,
    // so a tile waits for memory once
    constexpr int kPer = kTileRows * kTileK / 256;
    float v[kPer];
    if (op.k_contig) {
#pragma unroll
      for (int i = 0; i < kPer; ++i) {
        const int e = i * 256 + tid;
        const int r = e >> 6, k = e & 63;
        const int64_t gr = r0 + r, gk = k0 + k;
        v[i] = (gr < op.rows && gk < op.k) ? __ldg(op.src + gr * op.ld + gk) : 0.f;
      }
#pragma unroll
      for (int i = 0; i < kPer; ++i) {
        const int e = i * 256 + tid;
        s[e >> 6][e & 63] = v[i];
      }
    } else {
#pragma unroll
      for (int i = 0; i < kPer; ++i) {
        const int e = i * 256 + tid;
        const int k = e >> 7, r = e & 127;
        const int64_t gr = r0 + r, gk = k0 + k;
        v[i] = (gr < op.rows && gk < op.k) ? __ldg(op.src + gk * op.ld + gr) : 0.f;
      }
#pragma unroll
      for (int i = 0; i < kPer; ++i) {
        const int e = i * 256 + tid;
        s[e & 127][e >> 7] = v[i];
      }
    }
    __syncthreads();
    const size_t tile_elems = (size_t)local * (kTileRows * kTileK);
    uint8_t* hi = reinterpret_cast<uint8_t*>(op.hi + tile_elems);
    uint8_t* lo = op.lo ? reinterpret_cast<uint8_t*>(op.lo + tile_elems) : nullptr;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int cidx = i * 256 + tid;  // 128 rows x 8 chunks of 8 elements
      const int r = cidx >> 3, c = cidx & 7;
      uint32_t h[4], l[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float x0 = s[r][c * 8 + 2 * j], x1 = s[r][c * 8 + 2 * j + 1];
        const __nv_bfloat16 h0 = __float2bfloat16_rn(x0), h1 = __float2bfloat16_rn(x1);
        const __nv_bfloat16 l0 = __float2bfloat16_rn(x0 - __bfloat162float(h0));
        const __nv_bfloat16 l1 = __float2bfloat16_rn(x1 - __bfloat162float(h1));
        h[j] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
        l[j] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
      }
      const size_t off = (size_t)r * 128 + (size_t)(((c ^ (r & 7)) << 4));
      *reinterpret_cast<uint4*>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
      if (lo) *reinterpret_cast<uint4*>(lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
    }
  }
}

// ------------------------------------------------------------ tensor cores
// One problem as the kernel walks it.  A problem with M <= 64 < N runs
// swapped (C^T = op(B)^T op(A)^T): its small dimension becomes the MMA's N,
// so a tile multiplies 128 x roundup16(M) instead of padding M to 128 rows.
// The kernel's tile grid is mk x nk (mk = M, nk = N, or the reverse when
// swapped); a tile's MMA is 128 x bn with bn the columns left, rounded up to
// 16 (at most 128), and the last K block issues only the 16-wide K steps
// that hold data (the operand tiles are zero past K, so the skipped steps
// would add exact zeros).
struct TcProb {
  const uint8_t* a_hi;  // tiles of the kernel's A side: [mk/128][K/64] x 16 KB
  const uint8_t* a_lo;
  const uint8_t* b_hi;  // tiles of the kernel's B side: [nk/128][K/64] x 16 KB
  const uint8_t* b_lo;
  float* c;
  const float* bias;
  const float* mask;
  int64_t ldc;
  int m, n, kt;  // m x n: C's shape; kt: 64-wide K blocks (>= 1)
  int nk;        // columns of the kernel's tile grid (n, or m when swapped)
  int klast;     // 16-wide K steps in the last K block (1..4)
  int swap;
  float alpha, beta;
  int act, tiles_n, tile0;
  float* upd;  // parameter stepped by upd_scale * C in the epilogue (NULL: none)
  float upd_scale;
};

// L2 prefetch of columns [c0, c1) (at most 64) of row r: the first, the
// 33rd and the last element's lines cover the span at any alignment.
__device__ __forceinline__ void prefetch_seg_l2(const float* base, int64_t ld, int64_t r, int c0, int c1) {
  if (c1 <= c0) return;
  const float* p = base + r * ld;
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p + c0));
  if (c1 - c0 > 32) asm volatile("prefetch.global.L2 [%0];" ::"l"(p + c0 + 32));
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p + c1 - 1));
}

__device__ __forceinline__ int tile_bn(const TcProb& P, int n0) {
  const int left = P.nk - n0;
  return left >= 128 ? 128 : ((left + 15) & ~15);
}

struct TcTable {
  int count, total;
  TcProb p[kMaxGroup];
};

constexpr int kGroupedStages = 3;
// warps: 0 producer, 1 TMEM owner + MMA issuer, 2..9 epilogue (two per TMEM
// lane quarter, 64 columns each: the per-tile epilogue is the critical path
// of the short-K tiles, so it gets eight warps)
constexpr int kGroupedEpiWarps = 8;
constexpr int kThreadsGrouped = 32 * (2 + kGroupedEpiWarps);

template <bool X3>
struct GroupedCfg {
  static constexpr uint32_t kStageBytes = (X3 ? 4u : 2u) * kTileBytes;
  static constexpr uint32_t kBarBytes = 8u * (2 * kGroupedStages + 2 * kAccBufs + 1) + 16;
  static constexpr uint32_t kEpiOff = kGroupedStages * kStageBytes + (kBarBytes + 127) / 128 * 128;
  static constexpr uint32_t kSmem = kEpiOff + kGroupedEpiWarps * kEpiStageBytes + 1024;
};

// One CTA per SM walks the tile list.  The stage ring and the TMEM buffer
// ring continue across tiles (a running K-block counter gives every slot and
// parity), so the next tile's copies and MMAs overlap this tile's epilogue.
template <bool X3>
__global__ void __launch_bounds__(kThreadsGrouped, 1)
k_gemm_tc_grouped(const __grid_constant__ TcTable tab, uint32_t* err) {
  constexpr int BN = 128;
  constexpr int S = kGroupedStages;
  using Cfg = GroupedCfg<X3>;
  constexpr uint32_t kCols = BN * kAccBufs;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  uint8_t* gbase = smem_raw + (base - raw);
  const uint32_t bars = base + S * Cfg::kStageBytes;
  auto full_bar = [&](int s) { return bars + 8u * s; };
  auto empty_bar = [&](int s) { return bars + 8u * (S + s); };
  auto accf_bar = [&](int b) { return bars + 8u * (2 * S + b); };
  auto acce_bar = [&](int b) { return bars + 8u * (2 * S + kAccBufs + b); };
  const uint32_t drain_bar = bars + 8u * (2 * S + 2 * kAccBufs);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gbase + S * Cfg::kStageBytes + 8 * (2 * S + 2 * kAccBufs + 1));
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(full_bar(s), 1);
      mbar_init(empty_bar(s), 1);
    }
    for (int b = 0; b < kAccBufs; ++b) {
      mbar_init(accf_bar(b), 1);
      mbar_init(acce_bar(b), kGroupedEpiWarps);
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

  auto stage = [&](int s, int which) { return base + s * Cfg::kStageBytes + (uint32_t)which * kTileBytes; };

  if (warp == 0 && lane == 0) {
    // ---------------- bulk-copy producer
    uint32_t g = 0, issued_from = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < tab.total && ok; t += gridDim.x) {
      const TcProb& P = tab.p[find_problem(tab.p, tab.count, t)];
      const int local = t - P.tile0;
      const int tn = local % P.tiles_n;
      const size_t a_off = (size_t)(local / P.tiles_n) * P.kt * kTileBytes;
      const size_t b_off = (size_t)tn * P.kt * kTileBytes;
      // only the B tile's first bn rows (bn * 128 contiguous bytes) are used
      const uint32_t b_bytes = (uint32_t)tile_bn(P, tn * BN) * 128u;
      for (int kb = 0; kb < P.kt; ++kb, ++g) {
        const int s = g % S;
        if (*abort_flag || !mbar_wait(empty_bar(s), ((g / S) & 1) ^ 1)) { ok = false; break; }
        mbar_expect_tx(full_bar(s), (X3 ? 2u : 1u) * (kTileBytes + b_bytes));
        const size_t kofs = (size_t)kb * kTileBytes;
        bulk_load(stage(s, 0), P.a_hi + a_off + kofs, kTileBytes, full_bar(s));
        bulk_load(stage(s, 1), P.b_hi + b_off + kofs, b_bytes, full_bar(s));
        if (X3) {
          bulk_load(stage(s, 2), P.a_lo + a_off + kofs, kTileBytes, full_bar(s));
          bulk_load(stage(s, 3), P.b_lo + b_off + kofs, b_bytes, full_bar(s));
        }
      }
    }
    if (!ok) {
      atomicOr(err, 2u);
      *abort_flag = 1;
      // drain the copies still in flight into this CTA's shared memory
      issued_from = g > (uint32_t)S ? g - S : 0;
      for (uint32_t q = issued_from; q < g; ++q) mbar_wait(full_bar(q % S), (q / S) & 1);
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer
    uint32_t g = 0, acc = 0;  // g: K blocks (stage ring), acc: accumulations (TMEM ring)
    bool ok = true;
    for (int t = blockIdx.x; t < tab.total && ok; t += gridDim.x) {
      const TcProb& P = tab.p[find_problem(tab.p, tab.count, t)];
      const int bn = tile_bn(P, ((t - P.tile0) % P.tiles_n) * BN);
      const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(bn >> 3) << 17) |
                             ((uint32_t)(kTileRows >> 4) << 24);
      const int span = X3 ? kDrainX3 : P.kt;  // K blocks per TMEM accumulation
      for (int g0 = 0; g0 < P.kt && ok; g0 += span, ++acc) {
        const int b = acc % kAccBufs;
        if (*abort_flag || !mbar_wait(acce_bar(b), ((acc / kAccBufs) & 1) ^ 1)) { ok = false; break; }
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(b * BN);
        const int g1 = min(P.kt, g0 + span);
        for (int kb = g0; kb < g1; ++kb, ++g) {
          const int s = g % S;
          if (*abort_flag || !mbar_wait(full_bar(s), (g / S) & 1)) { ok = false; break; }
          tc_fence_after();
          const int ksteps = kb == P.kt - 1 ? P.klast : kTileK / 16;
#pragma unroll
          for (int k = 0; k < kTileK / 16; ++k) {
            if (k >= ksteps) break;
            const uint64_t a = sw128_desc(stage(s, 0) + 32u * k);
            const uint64_t bb = sw128_desc(stage(s, 1) + 32u * k);
            const uint32_t first = (kb == g0 && k == 0) ? 0u : 1u;
            if (X3) {
              // the same order of products as k_gemm_tcp: op(A)_hi op(B)_lo,
              // op(A)_lo op(B)_hi, then hi*hi (a swapped problem has op(B)
              // on the A side, so its cross terms come in the other order)
              const uint64_t alo = sw128_desc(stage(s, 2) + 32u * k), blo = sw128_desc(stage(s, 3) + 32u * k);
              if (P.swap) {
                mma_bf16(d, alo, bb, idesc, first);
                mma_bf16(d, a, blo, idesc, 1);
              } else {
                mma_bf16(d, a, blo, idesc, first);
                mma_bf16(d, alo, bb, idesc, 1);
              }
              mma_bf16(d, a, bb, idesc, 1);
            } else {
              mma_bf16(d, a, bb, idesc, first);
            }
          }
          mma_commit(empty_bar(s));
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
    // ---------------- epilogue: accumulations -> fp32 registers -> global
    // The sums go back into the last accumulation's TMEM buffer and the store
    // loop reads them 32 columns at a time (not unrolled), so the epilogue
    // code exists once instead of 128 times (instruction fetch dominated
    // small launches with the unrolled form).
    constexpr int CW = BN / 2;        // columns per epilogue warp
    const int q = warp & 3;           // TMEM lane quarter
    const int hc = (warp - 2) >> 2;   // column half
    const uint32_t lane_addr = ((uint32_t)(q * 32) << 16) + (uint32_t)(hc * CW);
    uint32_t g = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < tab.total && ok; t += gridDim.x) {
      const TcProb& P = tab.p[find_problem(tab.p, tab.count, t)];
      const int local = t - P.tile0;
      // kernel coordinates: rows m0 (TMEM lanes), columns n0 (TMEM columns)
      const int m0 = (local / P.tiles_n) * kTileRows, n0 = (local % P.tiles_n) * BN + hc * CW;
      // The epilogue's second input (ReLU mask or the parameter of a fused
      // update) does not depend on the accumulator: ask L2 for this warp's
      // part of it now, so its loads after the wait find it there.
      if (const float* aux = P.mask ? P.mask : P.upd) {
        if (!P.swap) {
          const int r = m0 + q * 32 + lane;
          if (r < P.m) prefetch_seg_l2(aux, P.ldc, r, n0, min(n0 + CW, P.n));
        } else {
          const int c0 = m0 + q * 32, c1 = min(c0 + 32, P.n);
          for (int r = n0 + lane; r < min(n0 + CW, P.m); r += 32) prefetch_seg_l2(aux, P.ldc, r, c0, c1);
        }
      }
      const int span = X3 ? kDrainX3 : P.kt;
      const int ngroups = (P.kt + span - 1) / span;
      float sum[X3 ? CW : 1];
      if (X3) {
#pragma unroll
        for (int j = 0; j < (X3 ? CW : 1); ++j) sum[j] = 0.f;
      }
      int b = 0;
      for (int gi = 0; gi < ngroups; ++gi, ++g) {
        b = g % kAccBufs;
        if (*abort_flag || !mbar_wait(accf_bar(b), (g / kAccBufs) & 1)) { ok = false; break; }
        tc_fence_after();
        if (X3 && ngroups > 1) {  // one accumulation: the store loop reads it from TMEM as it is
          const bool last = gi == ngroups - 1;
#pragma unroll
          for (int c = 0; c < CW / 32; c += 2) {
            const uint32_t ta = tmem + lane_addr + (uint32_t)(b * BN + c * 32);
            uint32_t r0[32], r1[32];
            tmem_ld32_nw(ta, r0);
            tmem_ld32_nw(ta + 32, r1);
            tmem_wait_ld();
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              sum[(X3 ? c * 32 + j : 0)] += __uint_as_float(r0[j]);
              r0[j] = __float_as_uint(sum[(X3 ? c * 32 + j : 0)]);
              sum[(X3 ? c * 32 + 32 + j : 0)] += __uint_as_float(r1[j]);
              r1[j] = __float_as_uint(sum[(X3 ? c * 32 + 32 + j : 0)]);
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
      float* stage = reinterpret_cast<float*>(gbase + Cfg::kEpiOff) + (warp - 2) * (kEpiStageBytes / 4);
#pragma unroll 1
      for (int c = 0; c < CW / 32; ++c) {  // one copy of the epilogue code
        const int col0 = n0 + c * 32;
        if (col0 >= P.nk) break;
        uint32_t r[32];
        tmem_ld32(tmem + lane_addr + (uint32_t)(b * BN + c * 32), r);
        if (P.swap) {
          // lanes are columns of C (kernel rows), TMEM columns rows of C
          if (m0 + q * 32 < P.n)
            epilogue_tile32_t(r, P.c, P.mask, P.bias, P.ldc, m0 + q * 32, P.n, col0, P.m, P.alpha, P.beta, P.act,
                              P.upd, P.upd_scale);
        } else if (m0 + q * 32 < P.m) {
          epilogue_tile32(r, stage, P.c, P.mask, P.bias, P.ldc, m0 + q * 32, P.m, col0, P.n, P.alpha, P.beta, P.act,
                          false, P.upd, P.upd_scale);
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acce_bar(b));
    }
    if (!ok) {
      if (lane == 0) atomicOr(err, 2u);
      *abort_flag = 1;
    }
  }

  // Every MMA must have completed before TMEM is released: on the normal path
  // the epilogue consumed every commit; after an abort the issuer commits once
  // more and waits (bounded) for it.
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

// ------------------------------------------------------------ MLP pieces
struct ColsumItem {
  const float* dy;
  float* db;
  float* value;  // parameter stepped by scale * db (NULL: none)
  float scale;
  int64_t batch, cols;
  int block0;  // first block of this item (blocks of 32 columns)
};
struct ColsumTable {
  int count, total, overwrite;
  ColsumItem it[kMaxGroup];
};

// db[o] += sum_b dy[b, o], b in order: the arithmetic of the single-layer
// bias-gradient kernel.  `overwrite`: db[o] = the sum, which equals adding it
// to a zeroed gradient (the sum starts at +0, so it is never -0).  With a
// value: value[o] += scale * db[o] (the SGD step's arithmetic).
__global__ void __launch_bounds__(256) k_colsum_grouped(const __grid_constant__ ColsumTable tab) {
  __shared__ float tile[kColsumRows][kColsumCols + 1];
  for (int t = blockIdx.x; t < tab.total; t += gridDim.x) {
    int lo = 0, hi = tab.count - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tab.it[mid].block0 <= t) lo = mid;
      else hi = mid - 1;
    }
    const ColsumItem& I = tab.it[lo];
    const int64_t c0 = (int64_t)(t - I.block0) * kColsumCols;
    const float s = colsum32(I.dy, I.batch, I.cols, I.cols, c0, tile);
    const int64_t o = c0 + threadIdx.x;
    if (threadIdx.x < 32 && o < I.cols) {
      const float d = tab.overwrite ? s : I.db[o] + s;
      I.db[o] = d;
      if (I.value) I.value[o] = __fadd_rn(I.value[o], __fmul_rn(I.scale, d));
    }
  }
}

struct VecItem {
  float* value;        // SGD: parameter; MSE: gradient output
  const float* grad;   // SGD: gradient;  MSE: prediction x
  const float* y;      // MSE target
  int64_t n;
  int64_t cols;        // MSE row length
  float scale;         // SGD: -lr; MSE: float32(1 / batch)
  float* loss;         // MSE: per-row losses (batch floats), may be NULL
  int block0;
};
struct VecTable {
  int count, total;
  VecItem it[2 * kMaxGroup];
};

constexpr int kVecChunk = 4096;  // elements per block iteration

__device__ __forceinline__ int find_vec(const VecTable& tab, int t) {
  int lo = 0, hi = tab.count - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tab.it[mid].block0 <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// value += (-lr) * grad, as the single-tensor SGD kernel computes it; 16-byte
// accesses when both tensors are 16-byte aligned.
__global__ void __launch_bounds__(256) k_sgd_grouped(const __grid_constant__ VecTable tab) {
  for (int t = blockIdx.x; t < tab.total; t += gridDim.x) {
    const VecItem& I = tab.it[find_vec(tab, t)];
    const int64_t i0 = (int64_t)(t - I.block0) * kVecChunk;
    const int64_t i1 = min(i0 + kVecChunk, I.n);
    const bool vec = ((reinterpret_cast<uintptr_t>(I.value) | reinterpret_cast<uintptr_t>(I.grad)) & 15u) == 0;
    if (vec && i1 - i0 == kVecChunk) {  // kVecChunk = 4096 = 256 threads x 4 float4
      float4 vv[4], gg[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t i = i0 + (int64_t)(u * 256 + threadIdx.x) * 4;
        vv[u] = *reinterpret_cast<const float4*>(I.value + i);
        gg[u] = *reinterpret_cast<const float4*>(I.grad + i);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t i = i0 + (int64_t)(u * 256 + threadIdx.x) * 4;
        float4 o;
        o.x = __fadd_rn(vv[u].x, __fmul_rn(I.scale, gg[u].x));
        o.y = __fadd_rn(vv[u].y, __fmul_rn(I.scale, gg[u].y));
        o.z = __fadd_rn(vv[u].z, __fmul_rn(I.scale, gg[u].z));
        o.w = __fadd_rn(vv[u].w, __fmul_rn(I.scale, gg[u].w));
        *reinterpret_cast<float4*>(I.value + i) = o;
      }
    } else {
      for (int64_t i = i0 + threadIdx.x; i < i1; i += 256)
        I.value[i] = __fadd_rn(I.value[i], __fmul_rn(I.scale, I.grad[i]));
    }
  }
}

// dst[i] = v for every tensor (zero_grad of every parameter in one launch).
__global__ void __launch_bounds__(256) k_fill_grouped(const __grid_constant__ VecTable tab) {
  for (int t = blockIdx.x; t < tab.total; t += gridDim.x) {
    const VecItem& I = tab.it[find_vec(tab, t)];
    const int64_t i0 = (int64_t)(t - I.block0) * kVecChunk;
    const int64_t i1 = min(i0 + kVecChunk, I.n);
    if ((reinterpret_cast<uintptr_t>(I.value) & 15u) == 0 && i1 - i0 == kVecChunk) {
      const float4 f = make_float4(I.scale, I.scale, I.scale, I.scale);
#pragma unroll
      for (int u = 0; u < 4; ++u) *reinterpret_cast<float4*>(I.value + i0 + (int64_t)(u * 256 + threadIdx.x) * 4) = f;
    } else {
      for (int64_t i = i0 + threadIdx.x; i < i1; i += 256) I.value[i] = I.scale;
    }
  }
}

// Adam for many tensors in one launch: each tensor's arithmetic is the
// single-tensor kernel's (k_adam_dev in nn.cu), and each keeps its own
// running powers; the last chunk of a tensor to finish stores its advanced
// powers (every chunk has read the old ones by then) and resets the counter.
struct AdamItem {
  float* value;
  const float* grad;
  float* m;
  float* v;
  double* powers;  // beta1^t, beta2^t, completion counter
  int64_t n;
  int block0, chunks;
};
// Adam chunks: 1024 elements (one float4 of each array per thread), so a
// step's ~2M parameters make several blocks per SM whose loads and stores
// overlap (4096-element chunks made one wave of ~3 blocks per SM that all
// loaded, then all computed, then all stored).
constexpr int kAdamChunk = 1024;
struct AdamTable {
  int count, total;
  float b1, c1, b2, c2, eps, nlr;
  double beta1, beta2;
  AdamItem it[kMaxGroup];
};

// One element of the Adam update, the float32 operations of the
// single-tensor kernel in the same order.
__device__ __forceinline__ void adam_elem(const AdamTable& tab, float d1, float d2, float gi, float& mi, float& vi,
                                          float& xi) {
  mi = __fadd_rn(__fmul_rn(mi, tab.b1), __fmul_rn(tab.c1, gi));
  vi = __fadd_rn(__fmul_rn(vi, tab.b2), __fmul_rn(tab.c2, __fmul_rn(gi, gi)));
  float mhat = __fdiv_rn(mi, d1);
  const float vhat = __fadd_rn(__fsqrt_rn(__fdiv_rn(vi, d2)), tab.eps);
  mhat = __fmul_rn(mhat, tab.nlr);
  mhat = __fdiv_rn(mhat, vhat);
  xi = __fadd_rn(xi, mhat);
}

__global__ void __launch_bounds__(256) k_adam_grouped(const __grid_constant__ AdamTable tab) {
  pdl_wait();
  pdl_trigger();
  for (int t = blockIdx.x; t < tab.total; t += gridDim.x) {
    int lo = 0, hi = tab.count - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tab.it[mid].block0 <= t) lo = mid;
      else hi = mid - 1;
    }
    const AdamItem& I = tab.it[lo];
    const double p1 = I.powers[0] * tab.beta1, p2 = I.powers[1] * tab.beta2;
    const float d1 = (float)(1.0 - p1), d2 = (float)(1.0 - p2);
    const int64_t i0 = (int64_t)(t - I.block0) * kAdamChunk;
    const int64_t i1 = min(i0 + kAdamChunk, I.n);
    const bool vec = ((reinterpret_cast<uintptr_t>(I.value) | reinterpret_cast<uintptr_t>(I.grad) |
                       reinterpret_cast<uintptr_t>(I.m) | reinterpret_cast<uintptr_t>(I.v)) & 15u) == 0;
    if (vec && i1 - i0 == kAdamChunk) {
      // a full chunk: a float4 of each array per thread, every load issued
      // before the first store (the four arrays are distinct, but the
      // compiler cannot know it)
      constexpr int kU = kAdamChunk / 1024;
      float4 gg[kU], mm[kU], vv[kU], xx[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int64_t i = i0 + (int64_t)(u * 256 + threadIdx.x) * 4;
        gg[u] = *reinterpret_cast<const float4*>(I.grad + i);
        mm[u] = *reinterpret_cast<const float4*>(I.m + i);
        vv[u] = *reinterpret_cast<const float4*>(I.v + i);
        xx[u] = *reinterpret_cast<const float4*>(I.value + i);
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const int64_t i = i0 + (int64_t)(u * 256 + threadIdx.x) * 4;
        adam_elem(tab, d1, d2, gg[u].x, mm[u].x, vv[u].x, xx[u].x);
        adam_elem(tab, d1, d2, gg[u].y, mm[u].y, vv[u].y, xx[u].y);
        adam_elem(tab, d1, d2, gg[u].z, mm[u].z, vv[u].z, xx[u].z);
        adam_elem(tab, d1, d2, gg[u].w, mm[u].w, vv[u].w, xx[u].w);
        *reinterpret_cast<float4*>(I.m + i) = mm[u];
        *reinterpret_cast<float4*>(I.v + i) = vv[u];
        *reinterpret_cast<float4*>(I.value + i) = xx[u];
      }
    } else {
      for (int64_t i = i0 + threadIdx.x; i < i1; i += 256) {
        float mi = I.m[i], vi = I.v[i], xi = I.value[i];
        adam_elem(tab, d1, d2, I.grad[i], mi, vi, xi);
        I.m[i] = mi;
        I.v[i] = vi;
        I.value[i] = xi;
      }
    }
    __syncthreads();  // this chunk has read the powers
    if (threadIdx.x == 0) {
      unsigned int* done = reinterpret_cast<unsigned int*>(I.powers + 2);
      __threadfence();
      if (atomicAdd(done, 1u) == (unsigned)I.chunks - 1) {
        I.powers[0] = p1;
        I.powers[1] = p2;
        *done = 0u;
        __threadfence();
      }
    }
  }
}

// MSE gradient of the mean-reduced loss: ((x - y) * 2) * float32(1/batch),
// the three float32 operations of MSELoss.backward and ReduceLoss.grad.  A
// thread's 16 elements of a chunk are loaded before any is stored.
__global__ void __launch_bounds__(256) k_mse_grad_grouped(const __grid_constant__ VecTable tab) {
  constexpr int kPer = kVecChunk / 256;
  for (int t = blockIdx.x; t < tab.total; t += gridDim.x) {
    const VecItem& I = tab.it[find_vec(tab, t)];
    const int64_t i0 = (int64_t)(t - I.block0) * kVecChunk;
    const int64_t i1 = min(i0 + kVecChunk, I.n);
    float xv[kPer], yv[kPer];
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int64_t i = i0 + u * 256 + threadIdx.x;
      xv[u] = i < i1 ? I.grad[i] : 0.f;
      yv[u] = i < i1 ? I.y[i] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int64_t i = i0 + u * 256 + threadIdx.x;
      if (i < i1) I.value[i] = __fmul_rn(__fmul_rn(__fsub_rn(xv[u], yv[u]), 2.0f), I.scale);
    }
  }
}

// MSE loss per model: mean over rows of sum over columns of (y - x)^2.  One
// block of 32 warps per model; a warp takes rows w, w + 32, ... with its
// lanes along the columns (four rows' loads in flight), adds each row's
// squares in a fixed shuffle tree, and keeps its rows' sums in order; the
// warps' sums are then added in warp order.  (Not the order of the per-op
// path, whose reduction kernels depend on the shape; the value agrees to
// rounding.)
constexpr int kMseWarps = 32;

__global__ void __launch_bounds__(32 * kMseWarps) k_mse_loss_grouped(const __grid_constant__ VecTable tab, float* out) {
  __shared__ float part[kMseWarps];
  const VecItem& I = tab.it[blockIdx.x];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t rows = I.n / I.cols;
  float acc = 0.f;
  for (int64_t r0 = w; r0 < rows; r0 += 4 * kMseWarps) {
    float s[4] = {0.f, 0.f, 0.f, 0.f};
    for (int64_t c0 = 0; c0 < I.cols; c0 += 32) {
      const int64_t c = c0 + lane;
      float d[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t r = r0 + (int64_t)u * kMseWarps;
        const bool in = r < rows && c < I.cols;
        d[u] = in ? __fsub_rn(I.y[r * I.cols + c], I.grad[r * I.cols + c]) : 0.f;
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) s[u] = __fadd_rn(s[u], __fmul_rn(d[u], d[u]));
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) s[u] += __shfl_xor_sync(0xffffffffu, s[u], o);
      acc += s[u];
    }
  }
  if (lane == 0) part[w] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float tot = 0.f;
    for (int k = 0; k < kMseWarps; ++k) tot += part[k];
    out[blockIdx.x] = tot * I.scale;
  }
}

}  // namespace
}  // namespace vkc

using namespace vkc;

// ------------------------------------------------------------ host side
namespace {

int check_problem(const vkc_gemm_problem& p, int i) {
  if (p.m < 0 || p.n < 0 || p.k < 0) return set_error(VKC_ERR_INVALID, "grouped gemm: problem %d has a negative size", i);
  if (p.m == 0 || p.n == 0) return VKC_OK;
  if (!p.c || (p.k > 0 && (!p.a || !p.b)))
    return set_error(VKC_ERR_INVALID, "grouped gemm: problem %d has a NULL buffer", i);
  if (p.m >= (1ll << 31) || p.n >= (1ll << 31) || p.k >= (1ll << 31))
    return set_error(VKC_ERR_INVALID, "grouped gemm: problem %d dimension too large", i);
  if (p.act != VKC_ACT_NONE && p.act != VKC_ACT_RELU && p.act != VKC_ACT_SIGMOID)
    return set_error(VKC_ERR_INVALID, "grouped gemm: problem %d has unknown activation %d", i, p.act);
  return VKC_OK;
}

// Order (longest K first) of the problems that have work.
std::vector<int> work_order(const vkc_gemm_problem* probs, int count) {
  std::vector<int> idx;
  for (int i = 0; i < count; ++i)
    if (probs[i].m > 0 && probs[i].n > 0) idx.push_back(i);
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return probs[x].k > probs[y].k; });
  return idx;
}

int grouped_simt(vkc_device_t dev, const vkc_gemm_problem* probs, const std::vector<int>& order) {
  for (size_t s = 0; s < order.size(); s += kMaxGroup) {
    SimtTable tab{};
    int total = 0;
    const size_t e = std::min(order.size(), s + kMaxGroup);
    for (size_t j = s; j < e; ++j) {
      const vkc_gemm_problem& q = probs[order[j]];
      SimtProb& P = tab.p[tab.count++];
      P.a = q.a;
      P.b = q.b;
      P.c = q.c;
      P.bias = q.bias;
      P.mask = q.relu_mask;
      P.lda = q.lda;
      P.ldb = q.ldb;
      P.ldc = q.ldc;
      P.m = q.m;
      P.n = q.n;
      P.k = q.k;
      P.alpha = q.alpha;
      P.beta = q.beta;
      P.act = q.act;
      P.trans = (q.ta ? 1 : 0) | (q.tb ? 2 : 0);
      P.tiles_n = (int)((q.n + kGemmBN - 1) / kGemmBN);
      P.tile0 = total;
      const int64_t tiles = ((q.m + kGemmBM - 1) / kGemmBM) * P.tiles_n;
      if (total + tiles >= (1ll << 31)) return set_error(VKC_ERR_INVALID, "grouped gemm: too many tiles");
      total += (int)tiles;
    }
    tab.total = total;
    if (total == 0) continue;
    const unsigned grid = wave_grid(dev, k_gemm_simt_grouped, (size_t)total * kGemmThreads, kGemmThreads);
    k_gemm_simt_grouped<<<grid, kGemmThreads, 0, dev->stream>>>(tab);
    int r = check_launch("gemm_grouped (fp32)");
    if (r != VKC_OK) return r;
  }
  return VKC_OK;
}

int grouped_tc(vkc_device_t dev, bool x3, const vkc_gemm_problem* probs, const vkc_gemm_update* upd,
               const std::vector<int>& order) {
  for (size_t s = 0; s < order.size(); s += kMaxGroup) {
    const size_t e = std::min(order.size(), s + kMaxGroup);
    // operand tile buffers: one allocation for the chunk
    std::vector<size_t> a_off, b_off;
    size_t bytes = 0;
    for (size_t j = s; j < e; ++j) {
      const vkc_gemm_problem& q = probs[order[j]];
      const size_t kt = (size_t)((q.k + kTileK - 1) / kTileK);
      const size_t at = (size_t)((q.m + kTileRows - 1) / kTileRows) * kt;
      const size_t bt = (size_t)((q.n + kTileRows - 1) / kTileRows) * kt;
      a_off.push_back(bytes);
      bytes += at * kTileBytes * (x3 ? 2 : 1);
      b_off.push_back(bytes);
      bytes += bt * kTileBytes * (x3 ? 2 : 1);
    }
    void* scratch = nullptr;
    int r = scratch_alloc(dev, bytes, &scratch);
    if (r != VKC_OK) return r;
    uint8_t* sbase = static_cast<uint8_t*>(scratch);

    TileTable tt{};
    TcTable tab{};
    int ttotal = 0, total = 0;
    for (size_t j = s; j < e; ++j) {
      const vkc_gemm_problem& q = probs[order[j]];
      const int kt = (int)((q.k + kTileK - 1) / kTileK);
      const int mt = (int)((q.m + kTileRows - 1) / kTileRows), nt = (int)((q.n + kTileRows - 1) / kTileRows);
      uint8_t* a_hi = sbase + a_off[j - s];
      uint8_t* a_lo = x3 ? a_hi + (size_t)mt * kt * kTileBytes : nullptr;
      uint8_t* b_hi = sbase + b_off[j - s];
      uint8_t* b_lo = x3 ? b_hi + (size_t)nt * kt * kTileBytes : nullptr;
      // op(A)(m, k): ta ? A[k*lda + m] : A[m*lda + k]  -> K contiguous iff !ta
      TileOp& oa = tt.op[tt.count++];
      oa.src = q.a;
      oa.hi = reinterpret_cast<__nv_bfloat16*>(a_hi);
      oa.lo = reinterpret_cast<__nv_bfloat16*>(a_lo);
      oa.ld = q.lda;
      oa.rows = q.m;
      oa.k = q.k;
      oa.k_contig = q.ta ? 0 : 1;
      oa.kt = kt;
      oa.tile0 = ttotal;
      ttotal += mt * kt;
      // op(B)^T(n, k): tb ? B[n*ldb + k] : B[k*ldb + n]  -> K contiguous iff tb
      TileOp& ob = tt.op[tt.count++];
      ob.src = q.b;
      ob.hi = reinterpret_cast<__nv_bfloat16*>(b_hi);
      ob.lo = reinterpret_cast<__nv_bfloat16*>(b_lo);
      ob.ld = q.ldb;
      ob.rows = q.n;
      ob.k = q.k;
      ob.k_contig = q.tb ? 1 : 0;
      ob.kt = kt;
      ob.tile0 = ttotal;
      ttotal += nt * kt;

      TcProb& P = tab.p[tab.count++];
      const bool swap = q.m <= 64 && q.n > 64;
      P.swap = swap ? 1 : 0;
      P.a_hi = swap ? b_hi : a_hi;
      P.a_lo = swap ? b_lo : a_lo;
      P.b_hi = swap ? a_hi : b_hi;
      P.b_lo = swap ? a_lo : b_lo;
      P.nk = (int)(swap ? q.m : q.n);
      P.klast = (int)(((q.k - (int64_t)(kt - 1) * kTileK) + 15) / 16);
      P.c = q.c;
      P.bias = q.bias;
      P.mask = q.relu_mask;
      P.ldc = q.ldc;
      P.m = (int)q.m;
      P.n = (int)q.n;
      P.kt = kt;
      P.alpha = q.alpha;
      P.beta = q.beta;
      P.act = q.act;
      P.tiles_n = swap ? mt : nt;
      P.tile0 = total;
      P.upd = upd ? upd[order[j]].value : nullptr;
      P.upd_scale = upd ? upd[order[j]].scale : 0.f;
      total += mt * nt;
    }
    tt.total = ttotal;
    tab.total = total;
    const unsigned tgrid = wave_grid(dev, k_tile_operands, (size_t)ttotal * 256, 256);
    k_tile_operands<<<tgrid, 256, 0, dev->stream>>>(tt);
    r = check_launch("gemm_grouped tiling");
    if (r == VKC_OK) {
      const unsigned grid = (unsigned)std::min<int>(total, dev->sm_count);
      if (x3) {
        static bool attr = false;
        if (!attr) {
          cudaFuncSetAttribute(k_gemm_tc_grouped<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               GroupedCfg<true>::kSmem);
          attr = true;
        }
        k_gemm_tc_grouped<true><<<grid, kThreadsGrouped, GroupedCfg<true>::kSmem, dev->stream>>>(tab, dev->err_word);
      } else {
        static bool attr = false;
        if (!attr) {
          cudaFuncSetAttribute(k_gemm_tc_grouped<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               GroupedCfg<false>::kSmem);
          attr = true;
        }
        k_gemm_tc_grouped<false><<<grid, kThreadsGrouped, GroupedCfg<false>::kSmem, dev->stream>>>(tab, dev->err_word);
      }
      r = check_launch("gemm_grouped (tensor cores)");
    }
    scratch_free(dev, scratch);
    if (r != VKC_OK) return r;
  }
  return VKC_OK;
}

}  // namespace

namespace {
int vec_launch(vkc_device_t dev, int kind, float* const* value, const float* const* grad, const float* const* y,
               const int64_t* n, const int64_t* cols, const float* scale, int count, float* loss_out);

int gemm_grouped(vkc_device_t dev, int precision, const vkc_gemm_problem* problems, const vkc_gemm_update* updates,
                 int count) {
  VKC_REQUIRE(count >= 0, "negative problem count");
  if (count == 0) return VKC_OK;
  VKC_REQUIRE(problems, "problems is NULL");
  VKC_REQUIRE(precision == VKC_MM_FP32 || precision == VKC_MM_BF16 || precision == VKC_MM_BF16X3,
              "unknown matmul precision %d", precision);
  for (int i = 0; i < count; ++i) {
    int r = check_problem(problems[i], i);
    if (r != VKC_OK) return r;
    if (updates && updates[i].value) {
      const vkc_gemm_problem& q = problems[i];
      VKC_REQUIRE(q.alpha == 1.f && q.beta == 0.f && !q.bias && q.act == VKC_ACT_NONE && !q.relu_mask,
                  "problem %d: a fused update needs a plain product (alpha 1, beta 0, no bias/act/mask)", i);
      VKC_REQUIRE(q.ldc == q.n, "problem %d: a fused update needs a contiguous C (ldc = n)", i);
      VKC_REQUIRE(updates[i].value != q.c && updates[i].value != q.a && updates[i].value != q.b,
                  "problem %d: the updated value may not be C or an operand of its problem", i);
    }
  }
  std::vector<int> order = work_order(problems, count);
  std::vector<int> tc, simt;
  // K = 0 has no tensor-core work: C = act(beta*C + bias) through the SIMT path
  for (int i : order) (precision != VKC_MM_FP32 && problems[i].k > 0 ? tc : simt).push_back(i);
  // Another problem may read an updated value as its operand (dx = dy W
  // beside dW's step): the tensor-core path reads operands only in its
  // tiling pass before the GEMM, so the step can run in the epilogue when all
  // its problems go in one launch; the SIMT path reads them in the GEMM, so
  // its steps (and those of a tensor-core call of several launches) run as
  // one separate update after every product.
  const bool fuse = updates && tc.size() <= (size_t)kMaxGroup;
  int r = grouped_simt(dev, problems, simt);
  if (r != VKC_OK) return r;
  r = grouped_tc(dev, precision == VKC_MM_BF16X3, problems, fuse ? updates : nullptr, tc);
  if (r != VKC_OK || !updates) return r;
  std::vector<float*> val;
  std::vector<const float*> grad;
  std::vector<int64_t> n;
  std::vector<float> scale;
  auto add = [&](const std::vector<int>& ids) {
    for (int i : ids) {
      if (!updates[i].value) continue;
      val.push_back(updates[i].value);
      grad.push_back(problems[i].c);
      n.push_back(problems[i].m * problems[i].n);
      scale.push_back(updates[i].scale);
    }
  };
  add(simt);
  if (!fuse) add(tc);
  if (val.empty()) return VKC_OK;
  return vec_launch(dev, 0, val.data(), grad.data(), nullptr, n.data(), nullptr, scale.data(), (int)val.size(),
                    nullptr);
}

int colsum_grouped(vkc_device_t dev, const float* const* dy, float* const* db, const int64_t* batch,
                   const int64_t* cols, int count, int overwrite, float* const* value, const float* scale) {
  VKC_REQUIRE(count >= 0, "negative item count");
  if (count == 0) return VKC_OK;
  VKC_REQUIRE(dy && db && batch && cols, "NULL argument");
  VKC_REQUIRE(!value || scale, "value without scale");
  for (int s = 0; s < count; s += kMaxGroup) {
    ColsumTable tab{};
    tab.overwrite = overwrite ? 1 : 0;
    int total = 0;
    for (int i = s; i < std::min(count, s + kMaxGroup); ++i) {
      VKC_REQUIRE(batch[i] >= 0 && cols[i] >= 0, "negative size");
      float* v = value ? value[i] : nullptr;
      if (cols[i] == 0 || (batch[i] == 0 && !overwrite && !v)) continue;
      VKC_REQUIRE((dy[i] || batch[i] == 0) && db[i], "NULL buffer");
      VKC_REQUIRE(v != db[i], "value %d is its own gradient", i);
      ColsumItem& I = tab.it[tab.count++];
      I.dy = dy[i];
      I.db = db[i];
      I.value = v;
      I.scale = v ? scale[i] : 0.f;
      I.batch = batch[i];
      I.cols = cols[i];
      I.block0 = total;
      total += (int)((cols[i] + kColsumCols - 1) / kColsumCols);
    }
    tab.total = total;
    if (total == 0) continue;
    k_colsum_grouped<<<(unsigned)std::min<int>(total, dev->sm_count * 8), 256, 0, dev->stream>>>(tab);
    int r = check_launch("colsum_grouped");
    if (r != VKC_OK) return r;
  }
  return VKC_OK;
}
}  // namespace

VKC_EXPORT int vkc_gemm_grouped(vkc_device_t dev, int precision, const vkc_gemm_problem* problems, int count) {
  VKC_BIND(dev);
  return gemm_grouped(dev, precision, problems, nullptr, count);
}

VKC_EXPORT int vkc_gemm_grouped_update(vkc_device_t dev, int precision, const vkc_gemm_problem* problems,
                                       const vkc_gemm_update* updates, int count) {
  VKC_BIND(dev);
  return gemm_grouped(dev, precision, problems, updates, count);
}

VKC_EXPORT int vkc_colsum_update_grouped(vkc_device_t dev, const float* const* dy, float* const* db,
                                         const int64_t* batch, const int64_t* cols, int count, int overwrite,
                                         float* const* value, const float* scale) {
  VKC_BIND(dev);
  return colsum_grouped(dev, dy, db, batch, cols, count, overwrite, value, scale);
}

VKC_EXPORT int vkc_colsum_grouped(vkc_device_t dev, const float* const* dy, float* const* db, const int64_t* batch,
                                  const int64_t* cols, int count, int overwrite) {
  VKC_BIND(dev);
  return colsum_grouped(dev, dy, db, batch, cols, count, overwrite, nullptr, nullptr);
}

namespace {
int vec_launch(vkc_device_t dev, int kind, float* const* value, const float* const* grad, const float* const* y,
               const int64_t* n, const int64_t* cols, const float* scale, int count, float* loss_out) {
  for (int s = 0; s < count; s += 2 * kMaxGroup) {
    VecTable tab{};
    int total = 0;
    const int e = std::min(count, s + 2 * kMaxGroup);
    for (int i = s; i < e; ++i) {
      VKC_REQUIRE(n[i] >= 0, "negative size");
      if (n[i] == 0 && kind != 2) continue;
      VecItem& I = tab.it[tab.count++];
      I.value = value ? value[i] : nullptr;
      I.grad = grad[i];
      I.y = y ? y[i] : nullptr;
      I.n = n[i];
      I.cols = cols ? cols[i] : 1;
      I.scale = scale[i];
      I.block0 = total;
      total += (int)((n[i] + kVecChunk - 1) / kVecChunk);
    }
    tab.total = total;
    if (tab.count == 0) continue;
    if (kind == 0) {
      k_sgd_grouped<<<(unsigned)std::min<int>(std::max(total, 1), dev->sm_count * 8), 256, 0, dev->stream>>>(tab);
    } else if (kind == 3) {
      if (total == 0) continue;
      k_fill_grouped<<<(unsigned)std::min<int>(total, dev->sm_count * 8), 256, 0, dev->stream>>>(tab);
    } else if (kind == 1) {
      k_mse_grad_grouped<<<(unsigned)std::min<int>(std::max(total, 1), dev->sm_count * 8), 256, 0, dev->stream>>>(tab);
    } else {
      k_mse_loss_grouped<<<(unsigned)tab.count, 32 * kMseWarps, 0, dev->stream>>>(tab, loss_out + s);
    }
    int r = check_launch("grouped vector op");
    if (r != VKC_OK) return r;
  }
  return VKC_OK;
}
}  // namespace

VKC_EXPORT int vkc_sgd_update_grouped(vkc_device_t dev, float* const* value, const float* const* grad,
                                      const int64_t* n, double lr, int count) {
  VKC_BIND(dev);
  VKC_REQUIRE(count >= 0, "negative item count");
  if (count == 0) return VKC_OK;
  VKC_REQUIRE(value && grad && n, "NULL argument");
  for (int i = 0; i < count; ++i) VKC_REQUIRE(n[i] == 0 || (value[i] && grad[i]), "NULL buffer");
  std::vector<float> scale((size_t)count, (float)(-lr));
  return vec_launch(dev, 0, value, grad, nullptr, n, nullptr, scale.data(), count, nullptr);
}

VKC_EXPORT int vkc_fill_f32_grouped(vkc_device_t dev, float* const* dst, const int64_t* n, float v, int count) {
  VKC_BIND(dev);
  VKC_REQUIRE(count >= 0, "negative item count");
  if (count == 0) return VKC_OK;
  VKC_REQUIRE(dst && n, "NULL argument");
  for (int i = 0; i < count; ++i) VKC_REQUIRE(n[i] == 0 || dst[i], "NULL buffer");
  std::vector<float> scale((size_t)count, v);
  return vec_launch(dev, 3, dst, const_cast<const float* const*>(dst), nullptr, n, nullptr, scale.data(), count,
                    nullptr);
}

VKC_EXPORT int vkc_adam_update_grouped(vkc_device_t dev, float* const* value, const float* const* grad,
                                       float* const* m, float* const* v, double* const* powers, const int64_t* n,
                                       int count, double lr, double beta1, double beta2, double eps) {
  VKC_BIND(dev);
  VKC_REQUIRE(count >= 0, "negative item count");
  if (count == 0) return VKC_OK;
  VKC_REQUIRE(value && grad && m && v && powers && n, "NULL argument");
  for (int s = 0; s < count; s += kMaxGroup) {
    AdamTable tab{};
    tab.b1 = (float)beta1;
    tab.c1 = (float)(1.0 - beta1);
    tab.b2 = (float)beta2;
    tab.c2 = (float)(1.0 - beta2);
    tab.eps = (float)eps;
    tab.nlr = (float)(-lr);
    tab.beta1 = beta1;
    tab.beta2 = beta2;
    int total = 0;
    for (int i = s; i < std::min(count, s + kMaxGroup); ++i) {
      VKC_REQUIRE(n[i] >= 0, "negative size");
      VKC_REQUIRE(powers[i] && (n[i] == 0 || (value[i] && grad[i] && m[i] && v[i])), "NULL buffer");
      AdamItem& I = tab.it[tab.count++];
      I = AdamItem{value[i], grad[i], m[i], v[i], powers[i], n[i], total,
                   (int)std::max<int64_t>(1, (n[i] + kAdamChunk - 1) / kAdamChunk)};
      total += I.chunks;  // an empty tensor still gets one chunk: its powers advance
    }
    tab.total = total;
    const cudaError_t e = launch_pdl(k_adam_grouped, dim3((unsigned)std::min<int>(total, dev->sm_count * 8)),
                                     dim3(256), 0, dev->stream, tab);
    int r = e == cudaSuccess ? check_launch("adam_grouped")
                             : set_error(VKC_ERR_CUDA, "adam_grouped launch: %s", cudaGetErrorString(e));
    if (r != VKC_OK) return r;
  }
  return VKC_OK;
}

VKC_EXPORT int vkc_mse_grouped(vkc_device_t dev, const float* const* x, const float* const* y, float* const* dx,
                               const int64_t* batch, const int64_t* cols, float* loss, int count) {
  VKC_BIND(dev);
  VKC_REQUIRE(count >= 0, "negative item count");
  if (count == 0) return VKC_OK;
  VKC_REQUIRE(x && y && batch && cols, "NULL argument");
  VKC_REQUIRE(count <= 2 * kMaxGroup || !loss, "grouped MSE loss: at most %d models per call", 2 * kMaxGroup);
  std::vector<int64_t> n((size_t)count);
  std::vector<float> scale((size_t)count);
  for (int i = 0; i < count; ++i) {
    VKC_REQUIRE(batch[i] > 0 && cols[i] > 0, "grouped MSE: empty model %d", i);
    VKC_REQUIRE(x[i] && y[i], "NULL buffer");
    n[i] = batch[i] * cols[i];
    scale[i] = (float)(1.0 / (double)batch[i]);
  }
  int r = VKC_OK;
  if (dx) {
    for (int i = 0; i < count; ++i) VKC_REQUIRE(dx[i], "NULL buffer");
    r = vec_launch(dev, 1, dx, x, y, n.data(), cols, scale.data(), count, nullptr);
  }
  if (r == VKC_OK && loss) r = vec_launch(dev, 2, nullptr, x, y, n.data(), cols, scale.data(), count, loss);
  return r;
}
