// gather: flat (gather.comp:21-26) and along an axis (gather_axis.comp:24-43).
//
// Flat gather is random 4-byte reads: each index pulls a 32-byte sector, so
// the direct kernel is bound by the DRAM's random-access rate, not by the 12
// algorithmic bytes per index.  Indices are read as uint4 and outputs written
// as float4.  An index past the end writes NaN and raises bit0 of the device
// error word instead of reading out of bounds (the shader has no check).
//
// Large tables and many indices take the binned form instead (three
// launches, the same values):
//   1. each chunk of 4096 indices is partitioned in shared memory by table
//      window (2^wbits floats, at most 32 windows, plus one bin for indices
//      out of range); the partitioned indices, their positions in the chunk
//      and each (chunk, window) run's start and length are stored;
//   2. blocks ordered window-major read, for one window, the runs of 16
//      chunks: the blocks resident at one time touch about one window, which
//      stays in L2, so the table comes from DRAM about once, not once per
//      index; each value is stored in its partitioned slot (in the output
//      buffer, contiguous per run);
//   3. each chunk's values are put back in position order through shared
//      memory and stored coalesced.
// No pass writes DRAM at random addresses.
//
// Axis gather copies whole rows of `post` floats: output [n_idx, prev, post]
// (the reference's layout, vkarray.py:1509-1511), row (k, i) =
// a[i, idx[k], :].  The shader clamps the index to [0, axis_size], one past
// the last row (gather_axis.comp:32); here it is clamped to axis_size - 1.
#include "common.cuh"

#include <algorithm>
#include <atomic>

namespace {

constexpr int kThreads = 256;

// 0: binned form for large tables and index counts; 1: never; 2: whenever the
// buffers are 16-byte aligned (vkc_set_gather_bins).
std::atomic<int> g_gather_bins{0};

__global__ void __launch_bounds__(kThreads)
k_gather(const float* a, size_t n_a, const uint32_t* idx, size_t n_idx, float* c, uint32_t* err) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t nvec = n_idx >> 2;
  const uint4* i4 = reinterpret_cast<const uint4*>(idx);
  float4* c4 = reinterpret_cast<float4*>(c);
  bool bad = false;
  auto load = [&](uint32_t j) -> float {
    if ((size_t)j < n_a) return __ldg(a + j);
    bad = true;
    return __int_as_float(0x7fc00000);
  };
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  // two index vectors per iteration: 8 independent random reads in flight
  for (; i + stride < nvec; i += 2 * stride) {
    const uint4 j0 = i4[i], j1 = i4[i + stride];
    float4 v0, v1;
    v0.x = load(j0.x);
    v0.y = load(j0.y);
    v0.z = load(j0.z);
    v0.w = load(j0.w);
    v1.x = load(j1.x);
    v1.y = load(j1.y);
    v1.z = load(j1.z);
    v1.w = load(j1.w);
    c4[i] = v0;
    c4[i + stride] = v1;
  }
  for (; i < nvec; i += stride) {
    const uint4 j = i4[i];
    float4 v;
    v.x = load(j.x);
    v.y = load(j.y);
    v.z = load(j.z);
    v.w = load(j.w);
    c4[i] = v;
  }
  size_t t = (nvec << 2) + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n_idx) c[t] = load(idx[t]);
  if (bad) atomicOr(err, 1u);
}

__global__ void __launch_bounds__(kThreads)
k_gather_scalar(const float* a, size_t n_a, const uint32_t* idx, size_t n_idx, float* c, uint32_t* err) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  bool bad = false;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_idx; i += stride) {
    uint32_t j = idx[i];
    if ((size_t)j < n_a) {
      c[i] = a[j];
    } else {
      c[i] = __int_as_float(0x7fc00000);
      bad = true;
    }
  }
  if (bad) atomicOr(err, 1u);
}

// ---- binned form
constexpr int kBinChunk = 4096;        // indices per chunk (16 per thread in pass 1)
constexpr int kBinChunksPerBlock = 16;  // chunks per pass-2 block (two per warp)
constexpr int kMaxBins = 33;            // 32 windows + out of range

// Pass 1: partition chunk blockIdx.x by window.  runs[c * nb + b] = start |
// count << 16 (both <= 4096) of bin b inside the chunk's slots; slot s of
// the chunk holds index part_idx[base + s] from position part_off[base + s].
__global__ void __launch_bounds__(kThreads)
k_gather_bin(const uint32_t* __restrict__ idx, size_t n_idx, size_t n_a, int wbits, int nb,
             uint32_t* __restrict__ part_idx, uint16_t* __restrict__ part_off, uint32_t* __restrict__ runs) {
  __shared__ uint32_t hist[kMaxBins];
  __shared__ uint32_t start[kMaxBins];
  __shared__ __align__(16) uint32_t s_idx[kBinChunk];
  __shared__ __align__(16) uint16_t s_off[kBinChunk];
  const size_t c = blockIdx.x, base = c * kBinChunk;
  const int len = (int)min((size_t)kBinChunk, n_idx - base);
  const int t = threadIdx.x;
  if (t < kMaxBins) hist[t] = 0u;
  __syncthreads();
  uint32_t iv[16], key[16];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int p = q * 1024 + t * 4;
    if (p + 4 <= len) {
      const uint4 x = *reinterpret_cast<const uint4*>(idx + base + p);
      iv[4 * q] = x.x;
      iv[4 * q + 1] = x.y;
      iv[4 * q + 2] = x.z;
      iv[4 * q + 3] = x.w;
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e) iv[4 * q + e] = p + e < len ? idx[base + p + e] : 0u;
    }
  }
#pragma unroll
  for (int e = 0; e < 16; ++e) {
    const int p = (e >> 2) * 1024 + t * 4 + (e & 3);
    key[e] = 0u;
    if (p < len) {
      const uint32_t i = iv[e];
      const uint32_t b = (size_t)i < n_a ? (i >> wbits) : (uint32_t)(nb - 1);
      key[e] = (b << 16) | atomicAdd(&hist[b], 1u);
    }
  }
  __syncthreads();
  if (t == 0) {
    uint32_t sum = 0u;
    for (int b = 0; b < nb; ++b) {
      start[b] = sum;
      runs[c * nb + b] = sum | (hist[b] << 16);
      sum += hist[b];
    }
  }
  __syncthreads();
#pragma unroll
  for (int e = 0; e < 16; ++e) {
    const int p = (e >> 2) * 1024 + t * 4 + (e & 3);
    if (p < len) {
      const uint32_t slot = start[key[e] >> 16] + (key[e] & 0xffffu);
      s_idx[slot] = iv[e];
      s_off[slot] = (uint16_t)p;
    }
  }
  __syncthreads();
  if (len == kBinChunk) {
    uint4* di = reinterpret_cast<uint4*>(part_idx + base);
    const uint4* si = reinterpret_cast<const uint4*>(s_idx);
    for (int j = t; j < kBinChunk / 4; j += kThreads) di[j] = si[j];
    uint4* dp = reinterpret_cast<uint4*>(part_off + base);
    const uint4* sp = reinterpret_cast<const uint4*>(s_off);
    for (int j = t; j < kBinChunk / 8; j += kThreads) dp[j] = sp[j];
  } else {
    for (int j = t; j < len; j += kThreads) {
      part_idx[base + j] = s_idx[j];
      part_off[base + j] = s_off[j];
    }
  }
}

// Pass 2: block (w, g) -- window-major -- reads window w's run of chunks
// 16g .. 16g + 15 (one warp per chunk, two chunks per warp) and stores each
// value in its slot of vals.  Bin nb - 1 holds the indices out of range:
// NaN, and bit0 of the error word.
__global__ void __launch_bounds__(kThreads)
k_gather_windows(const float* __restrict__ a, const uint32_t* __restrict__ part_idx,
                 const uint32_t* __restrict__ runs, size_t n_chunks, int nb, unsigned groups, float* vals,
                 uint32_t* err) {
  const int w = (int)(blockIdx.x / groups);
  const size_t g = blockIdx.x - (size_t)w * groups;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool oob = w == nb - 1;
  bool bad = false;
  for (int k = warp; k < kBinChunksPerBlock; k += kThreads / 32) {
    const size_t c = g * kBinChunksPerBlock + (size_t)k;
    if (c >= n_chunks) break;
    const uint32_t r = runs[c * nb + w];
    const uint32_t cnt = r >> 16;
    const size_t s0 = c * kBinChunk + (r & 0xffffu);
    if (oob) {
      for (uint32_t j = lane; j < cnt; j += 32) vals[s0 + j] = __int_as_float(0x7fc00000);
      bad = bad || cnt != 0u;
      continue;
    }
    for (uint32_t j = lane; j < cnt; j += 128) {
      uint32_t i[4];
      float v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) i[u] = j + 32u * u < cnt ? part_idx[s0 + j + 32u * u] : 0u;
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = j + 32u * u < cnt ? __ldg(a + i[u]) : 0.f;
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (j + 32u * u < cnt) vals[s0 + j + 32u * u] = v[u];
    }
  }
  if (bad && lane == 0) atomicOr(err, 1u);
}

// Pass 3: chunk blockIdx.x of c holds its values in partitioned order; put
// them back in position order (every read of the chunk before any write).
__global__ void __launch_bounds__(kThreads)
k_gather_unbin(const uint16_t* __restrict__ part_off, size_t n_idx, float* c) {
  __shared__ __align__(16) float s[kBinChunk];
  const size_t base = (size_t)blockIdx.x * kBinChunk;
  const int len = (int)min((size_t)kBinChunk, n_idx - base);
  const int t = threadIdx.x;
  if (len == kBinChunk) {
    const float4* v4 = reinterpret_cast<const float4*>(c + base);
    const ushort4* o4 = reinterpret_cast<const ushort4*>(part_off + base);
    for (int j = t; j < kBinChunk / 4; j += kThreads) {
      const float4 v = v4[j];
      const ushort4 o = o4[j];
      s[o.x] = v.x;
      s[o.y] = v.y;
      s[o.z] = v.z;
      s[o.w] = v.w;
    }
  } else {
    for (int j = t; j < len; j += kThreads) s[part_off[base + j]] = c[base + j];
  }
  __syncthreads();
  if (len == kBinChunk) {
    float4* d4 = reinterpret_cast<float4*>(c + base);
    const float4* s4 = reinterpret_cast<const float4*>(s);
    for (int j = t; j < kBinChunk / 4; j += kThreads) d4[j] = s4[j];
  } else {
    for (int j = t; j < len; j += kThreads) c[base + j] = s[j];
  }
}

// The binned form; returns false (nothing launched) when its scratch cannot
// be had, so the caller can take the direct kernel.
bool gather_binned(vkc_device_t dev, const float* a, size_t n_a, const uint32_t* idx, size_t n_idx, float* c,
                   int* status) {
  const size_t n_chunks = (n_idx + kBinChunk - 1) / kBinChunk;
  const uint64_t span = std::min<uint64_t>((uint64_t)n_a, 1ull << 32);
  int lg = 0;
  while ((1ull << lg) < span) ++lg;
  const int wbits = std::max(20, lg - 5);
  const int nw = (int)((span + (1ull << wbits) - 1) >> wbits);  // <= 32
  const int nb = nw + 1;
  const size_t idx_bytes = n_chunks * kBinChunk * sizeof(uint32_t);
  const size_t off_bytes = n_chunks * kBinChunk * sizeof(uint16_t);
  const size_t run_bytes = n_chunks * (size_t)nb * sizeof(uint32_t);
  void* scratch = nullptr;
  if (vkc::scratch_alloc(dev, idx_bytes + off_bytes + run_bytes, &scratch) != VKC_OK) return false;
  uint32_t* part_idx = static_cast<uint32_t*>(scratch);
  uint16_t* part_off = reinterpret_cast<uint16_t*>(static_cast<uint8_t*>(scratch) + idx_bytes);
  uint32_t* runs = reinterpret_cast<uint32_t*>(static_cast<uint8_t*>(scratch) + idx_bytes + off_bytes);
  const unsigned groups = (unsigned)((n_chunks + kBinChunksPerBlock - 1) / kBinChunksPerBlock);
  k_gather_bin<<<(unsigned)n_chunks, kThreads, 0, dev->stream>>>(idx, n_idx, n_a, wbits, nb, part_idx, part_off,
                                                                  runs);
  k_gather_windows<<<groups * (unsigned)nb, kThreads, 0, dev->stream>>>(a, part_idx, runs, n_chunks, nb, groups, c,
                                                                         dev->err_word);
  k_gather_unbin<<<(unsigned)n_chunks, kThreads, 0, dev->stream>>>(part_off, n_idx, c);
  vkc::scratch_free(dev, scratch);
  *status = vkc::check_launch("gather (binned)");
  return true;
}

// One block-row unit per (k, i); `post` floats copied with float4 when aligned.
template <bool VEC>
__global__ void __launch_bounds__(kThreads)
k_gather_axis(const float* a, size_t prev, size_t axis, size_t post, const uint32_t* idx, size_t n_idx,
              float* c) {
  const size_t rows = n_idx * prev;
  for (size_t u = blockIdx.x; u < rows; u += gridDim.x) {
    const size_t k = u / prev, i = u % prev;
    uint32_t j = idx[k];
    size_t jj = (size_t)j < axis ? (size_t)j : axis - 1;
    const float* src = a + (i * axis + jj) * post;
    float* dst = c + (k * prev + i) * post;
    if (VEC) {
      const float4* s4 = reinterpret_cast<const float4*>(src);
      float4* d4 = reinterpret_cast<float4*>(dst);
      for (size_t t = threadIdx.x; t < (post >> 2); t += kThreads) d4[t] = s4[t];
    } else {
      for (size_t t = threadIdx.x; t < post; t += kThreads) dst[t] = src[t];
    }
  }
}

// Small rows: one element per thread.
__global__ void __launch_bounds__(kThreads)
k_gather_axis_elem(const float* a, size_t prev, size_t axis, size_t post, const uint32_t* idx, size_t n_idx,
                   float* c) {
  const size_t total = n_idx * prev * post;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
    size_t j = e % post;
    size_t r = e / post;
    size_t i = r % prev, k = r / prev;
    uint32_t q = idx[k];
    size_t qq = (size_t)q < axis ? (size_t)q : axis - 1;
    c[e] = a[(i * axis + qq) * post + j];
  }
}

}  // namespace

VKC_EXPORT int vkc_gather(vkc_device_t dev, const float* a, size_t n_a, const uint32_t* idx, size_t n_idx,
                          float* c) {
  VKC_BIND(dev);
  if (n_idx == 0) return VKC_OK;
  VKC_REQUIRE(a && idx && c, "NULL buffer");
  const bool vec = ((((uintptr_t)idx) | ((uintptr_t)c)) & 15u) == 0;
  // binned: tables beyond L2 (>= 2^25 floats) and >= 2^21 indices, or forced
  const int mode = g_gather_bins.load(std::memory_order_relaxed);
  const bool binned = vec && n_idx < (1ull << 32) &&
                      (mode == 2 || (mode == 0 && n_a >= (1ull << 25) && n_idx >= (1ull << 21)));
  int status = VKC_OK;
  if (binned && gather_binned(dev, a, n_a, idx, n_idx, c, &status)) return status;
  if (vec) {
    unsigned grid = vkc::wave_grid(dev, k_gather, (n_idx >> 3) + 1, kThreads);
    k_gather<<<grid, kThreads, 0, dev->stream>>>(a, n_a, idx, n_idx, c, dev->err_word);
  } else {
    unsigned grid = vkc::wave_grid(dev, k_gather_scalar, n_idx, kThreads);
    k_gather_scalar<<<grid, kThreads, 0, dev->stream>>>(a, n_a, idx, n_idx, c, dev->err_word);
  }
  return vkc::check_launch("gather");
}

VKC_EXPORT int vkc_set_gather_bins(int mode) {
  VKC_REQUIRE(mode >= 0 && mode <= 2, "gather bins mode %d (0 auto, 1 never, 2 always)", mode);
  g_gather_bins.store(mode, std::memory_order_relaxed);
  return VKC_OK;
}

VKC_EXPORT int vkc_gather_axis(vkc_device_t dev, const float* a, size_t prev, size_t axis, size_t post,
                               const uint32_t* idx, size_t n_idx, float* c) {
  VKC_BIND(dev);
  if (n_idx == 0 || prev == 0 || post == 0) return VKC_OK;
  VKC_REQUIRE(a && idx && c, "NULL buffer");
  VKC_REQUIRE(axis > 0, "gather along an empty axis");
  if (post >= 64) {
    const bool vec = (post % 4 == 0) && ((((uintptr_t)a) | ((uintptr_t)c)) & 15u) == 0;
    size_t rows = n_idx * prev;
    unsigned grid = (unsigned)std::min<size_t>(rows, (size_t)dev->sm_count * 16);
    if (vec) k_gather_axis<true><<<grid, kThreads, 0, dev->stream>>>(a, prev, axis, post, idx, n_idx, c);
    else k_gather_axis<false><<<grid, kThreads, 0, dev->stream>>>(a, prev, axis, post, idx, n_idx, c);
  } else {
    unsigned grid = vkc::stream_grid(dev, n_idx * prev * post, kThreads);
    k_gather_axis_elem<<<grid, kThreads, 0, dev->stream>>>(a, prev, axis, post, idx, n_idx, c);
  }
  return vkc::check_launch("gather_axis");
}
