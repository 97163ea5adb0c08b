// Epilogue of the tensor-core GEMMs: one warp's 32 rows x 32 columns.
//
// tcgen05.ld gives each lane one row (32 consecutive columns).  Stored from
// there, every warp store instruction would touch 32 rows (32 partial
// sectors); instead the block goes through a 4 KB per-warp shared-memory
// stage (16-byte chunks XOR-swizzled by row, conflict-free both ways) and
// comes back with lane = column, so each store writes 128 contiguous bytes of
// one row and the bias / C / mask reads are coalesced the same way.
//   v = act(alpha * acc + beta * C + bias), then (grouped backward)
//   v *= ReLU'(mask); `raw` stores acc unchanged (split-K partials).
#pragma once
#include "gemm_simt.cuh"

namespace vkc {
namespace {

constexpr uint32_t kEpiStageBytes = 32 * 32 * 4;  // per epilogue warp

__device__ __forceinline__ float epi_value(float a, float alpha, float beta, float c, bool has_bias, float b, int act,
                                           bool has_mask, float m, int mact = VKC_ACT_RELU) {
  float v = alpha * a;
  if (beta != 0.f) v += beta * c;
  if (has_bias) v += b;
  if (act == VKC_ACT_RELU) v = fmaxf(v, 0.f);
  else if (act == VKC_ACT_SIGMOID) v = 1.0f / (1.0f + expf(0.0f - v));
  if (has_mask) v = act_deriv(v, m, mact);
  return v;
}

// The common epilogues in fixed form: alpha == 1, beta == 0, act none or
// ReLU, v = a (+ bias) (max 0) (* act'(mask), mact: ReLU or sigmoid).  With
// alpha == 1 the product
// alpha * a is exact, so these give epi_value's results bit for bit whatever
// the compiler contracts.  get(j) is this lane's value of row j; the lane
// writes column `col` of rows row0 .. row0+rows-1 (rows <= 32) through a
// pointer stepped by ld, so a value costs a load from the stage, the
// arithmetic and a store (the general form re-derives every offset and
// tests every flag per value).  All 32 mask rows are loaded before the
// first store: one wait for memory per 32 rows.  (Stepped pointers keep
// this within the 168 registers a thread of a 10-warp CTA can have; 32
// offsets computed from the row index did not fit.)
//
// UPD (a parameter update fused into a gradient GEMM): v = a is stored as
// the gradient and then value += scale * v, the SGD step with scale = -lr in
// the arithmetic of the separate SGD kernels; `aux` is then the parameter
// (same shape and leading dimension as C) and `b` the scale.  NR: rows per
// call (the update form goes 16 rows at a time: its parameter rows and the
// pointer to them would not fit the registers for 32).
template <int NR, bool HB, bool RELU, bool HM, bool UPD, typename Get>
__device__ __forceinline__ void epi_rows_fixed(Get get, float* C, const float* aux, float b, int64_t ld,
                                               int64_t row0, int col, int rows, int mact = VKC_ACT_RELU) {
  float* cp = C + row0 * ld + col;
  float m[NR];
  if (HM || UPD) {
    const float* mp = aux + row0 * ld + col;
#pragma unroll
    for (int j = 0; j < NR; ++j) {
      m[j] = j < rows ? *mp : 0.f;
      mp += ld;
    }
  }
  float* up = UPD ? const_cast<float*>(aux) + row0 * ld + col : nullptr;
#pragma unroll
  for (int j = 0; j < NR; ++j) {
    if (j < rows) {
      float v = get(j);
      if (HB) v = v + b;
      if (RELU) v = fmaxf(v, 0.f);
      if (HM) v = act_deriv(v, m[j], mact);
      *cp = v;
      if (UPD) *up = __fadd_rn(m[j], __fmul_rn(b, v));
    }
    cp += ld;
    if (UPD) up += ld;
  }
}

// Picks the fixed form for the flags, or returns false (general form).
// upd: the parameter of a fused update (nullptr: none), upd_scale its scale.
template <typename Get>
__device__ __forceinline__ bool epi_rows_dispatch(Get get, float* C, const float* mask, float b, int64_t ld,
                                                  int64_t row0, int col, int rows, float alpha, float beta, int act,
                                                  bool hb, bool hm, bool raw, float* upd = nullptr,
                                                  float upd_scale = 0.f, int mact = VKC_ACT_RELU) {
  if (raw) {
    epi_rows_fixed<32, false, false, false, false>(get, C, nullptr, 0.f, ld, row0, col, rows);
    return true;
  }
  if (alpha != 1.f || beta != 0.f || (act != VKC_ACT_NONE && act != VKC_ACT_RELU)) return false;
  const bool relu = act == VKC_ACT_RELU;
  if (upd) {  // the host admits updates only on plain products
    epi_rows_fixed<16, false, false, false, true>(get, C, upd, upd_scale, ld, row0, col, rows);
    if (rows > 16) {
      auto get_hi = [&](int j) { return get(j + 16); };
      epi_rows_fixed<16, false, false, false, true>(get_hi, C, upd, upd_scale, ld, row0 + 16, col, rows - 16);
    }
    return true;
  }
  if (!hm) {
    if (!hb && !relu) epi_rows_fixed<32, false, false, false, false>(get, C, nullptr, 0.f, ld, row0, col, rows);
    else if (hb && !relu) epi_rows_fixed<32, true, false, false, false>(get, C, nullptr, b, ld, row0, col, rows);
    else if (hb && relu) epi_rows_fixed<32, true, true, false, false>(get, C, nullptr, b, ld, row0, col, rows);
    else return false;
    return true;
  }
  if (!hb && !relu) {
    epi_rows_fixed<32, false, false, true, false>(get, C, mask, 0.f, ld, row0, col, rows, mact);
    return true;
  }
  return false;
}

// acc: this lane's row (row0 + lane), columns col0 .. col0+31.  C / mask
// point at row 0 of the matrix (leading dimension ld); rows >= M and columns
// >= N are skipped.  All 32 lanes must call it (warp-synchronous).  FIXED:
// use the fixed forms where the flags allow (a kernel short of registers
// keeps only the general form).
template <bool FIXED = true>
__device__ __forceinline__ void epilogue_tile32(const uint32_t (&acc)[32], float* __restrict__ stage, float* C,
                                                const float* mask, const float* __restrict__ bias, int64_t ld,
                                                int row0, int M, int col0, int N, float alpha, float beta, int act,
                                                bool raw, float* upd = nullptr, float upd_scale = 0.f,
                                                int mact = VKC_ACT_RELU) {
  const int lane = threadIdx.x & 31;
  float4* srow = reinterpret_cast<float4*>(stage) + lane * 8;
#pragma unroll
  for (int q = 0; q < 8; ++q)
    srow[q ^ (lane & 7)] = make_float4(__uint_as_float(acc[4 * q]), __uint_as_float(acc[4 * q + 1]),
                                       __uint_as_float(acc[4 * q + 2]), __uint_as_float(acc[4 * q + 3]));
  __syncwarp();
  const int col = col0 + lane;
  const bool cin = col < N;
  const int rows = min(32, M - row0);
  const bool hb = bias != nullptr, hm = mask != nullptr, hc = beta != 0.f && !raw;
  const float b = (hb && cin) ? bias[col] : 0.f;
  // row j of the stage: chunk ((lane >> 2) ^ j) & 7, which repeats every 8 rows
  int so[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) so[q] = ((((lane >> 2) ^ q) & 7) << 2) + (lane & 3);
  auto staged = [&](int j) {
    return FIXED ? stage[j * 32 + so[j & 7]] : stage[j * 32 + ((((lane >> 2) ^ j) & 7) << 2) + (lane & 3)];
  };
  if (FIXED && cin &&
      epi_rows_dispatch(staged, C, mask, b, ld, row0, col, rows, alpha, beta, act, hb, hm, raw, upd, upd_scale,
                        mact)) {
  } else if (cin) {
#pragma unroll 1
    for (int j0 = 0; j0 < rows; j0 += 16) {
      // the group's loads before its stores (a load after a store to C could
      // not be hoisted: the pointers may alias)
      float cv[16], mv[16];
#pragma unroll
      for (int t = 0; t < 16; ++t) {
        const int64_t off = (int64_t)(row0 + j0 + t) * ld + col;
        const bool in = j0 + t < rows;
        cv[t] = (in && hc) ? C[off] : 0.f;
        mv[t] = (in && hm) ? mask[off] : 0.f;
      }
#pragma unroll
      for (int t = 0; t < 16; ++t) {
        if (j0 + t < rows) {
          const float a = staged(j0 + t);
          C[(int64_t)(row0 + j0 + t) * ld + col] =
              raw ? a : epi_value(a, alpha, beta, cv[t], hb, b, act, hm, mv[t], mact);
        }
      }
    }
  }
  __syncwarp();
}

// The same for an accumulator of the transposed product (a swapped
// problem: TMEM lanes are columns of C, TMEM columns are rows of C).  acc:
// this lane's column n0 + lane, rows m0 .. m0+31 of C; each store writes 32
// consecutive columns of one row, so no shared-memory stage is needed.
// Rows >= M and columns >= N are skipped.  All 32 lanes must call it.
__device__ __forceinline__ void epilogue_tile32_t(const uint32_t (&acc)[32], float* C, const float* mask,
                                                  const float* __restrict__ bias, int64_t ld, int n0, int N, int m0,
                                                  int M, float alpha, float beta, int act, float* upd = nullptr,
                                                  float upd_scale = 0.f) {
  const int lane = threadIdx.x & 31;
  const int col = n0 + lane;
  const bool cin = col < N;
  const int rows = min(32, M - m0);
  const bool hb = bias != nullptr, hm = mask != nullptr, hc = beta != 0.f;
  const float b = (hb && cin) ? bias[col] : 0.f;
  auto reg = [&](int j) { return __uint_as_float(acc[j]); };
  if (!cin || epi_rows_dispatch(reg, C, mask, b, ld, m0, col, rows, alpha, beta, act, hb, hm, false, upd, upd_scale))
    return;
#pragma unroll
  for (int j0 = 0; j0 < 32; j0 += 16) {
    if (j0 >= rows) break;
    float cv[16], mv[16];
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      const int64_t off = (int64_t)(m0 + j0 + t) * ld + col;
      const bool in = j0 + t < rows;
      cv[t] = (in && hc) ? C[off] : 0.f;
      mv[t] = (in && hm) ? mask[off] : 0.f;
    }
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      if (j0 + t < rows)
        C[(int64_t)(m0 + j0 + t) * ld + col] =
            epi_value(__uint_as_float(acc[j0 + t]), alpha, beta, cv[t], hb, b, act, hm, mv[t]);
    }
  }
}

}  // namespace
}  // namespace vkc
