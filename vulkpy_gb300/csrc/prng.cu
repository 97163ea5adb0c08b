// xoshiro128++ random numbers, bit-exact with vulkpy's PRNG::Xoshiro128pp.
//
// Seeding (_vkarray.cc:643-675): the first state is four chained splitmix64
// outputs (each output is fed back as the next input, 659-663) truncated to
// 32 bits; state i is the reference's jump() (597-621) applied i times.
// That jump keeps its accumulators across the four JUMP words and writes
// them back after each word, so it is not the published 2^64 jump, but it
// is still linear over GF(2) (xors, shifts and rotations only).  The host
// therefore builds the 128x128 bit matrix J of one jump and its powers
// J^(2^k); the GPU computes every state i = J^i s0 independently instead of
// the reference's serial loop over all states.
//
// Generation (_vkarray.cc:697-717 with prng_xoshiro128pp_*.comp): the
// reference submits one job per chunk of `size` outputs and host-waits
// between chunks; output k comes from state k % size after k / size earlier
// steps.  Here one launch does all chunks: thread t keeps state t in
// registers and writes out[t], out[t+size], ... (coalesced across threads).
#include "common.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

namespace {

constexpr int kThreads = 256;

// ---------------------------------------------------------------- host side
inline uint32_t rotl32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }

// One xoshiro128++ state update (the output is not needed here).
inline void host_step(uint32_t s[4]) {
  const uint32_t t = s[1] << 9;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl32(s[3], 11);
}

// The reference's jump, restated (accumulators never reset, written back
// after each 32-bit word of the jump polynomial).
inline void host_ref_jump(uint32_t s[4]) {
  static const uint32_t kJump[4] = {0x8764000bu, 0xf542d2d3u, 0x6fa035c3u, 0x77f2db5bu};
  uint32_t acc[4] = {0, 0, 0, 0};
  for (uint32_t j : kJump) {
    for (int b = 0; b < 32; ++b) {
      if (j & (1u << b)) {
        acc[0] ^= s[0];
        acc[1] ^= s[1];
        acc[2] ^= s[2];
        acc[3] ^= s[3];
      }
      host_step(s);
    }
    std::memcpy(s, acc, sizeof(acc));
  }
}

inline uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// A GF(2) linear map on 128-bit states, stored as the images of the 128
// unit vectors: col[p] = map(e_p), 4 words each.
struct BitMatrix {
  uint32_t col[128][4];
};

inline void apply(const BitMatrix& m, const uint32_t x[4], uint32_t y[4]) {
  uint32_t r[4] = {0, 0, 0, 0};
  for (int p = 0; p < 128; ++p)
    if ((x[p >> 5] >> (p & 31)) & 1u)
      for (int w = 0; w < 4; ++w) r[w] ^= m.col[p][w];
  std::memcpy(y, r, sizeof(r));
}

template <class F>
BitMatrix matrix_of(F f) {
  BitMatrix m;
  for (int p = 0; p < 128; ++p) {
    uint32_t e[4] = {0, 0, 0, 0};
    e[p >> 5] = 1u << (p & 31);
    f(e);
    std::memcpy(m.col[p], e, sizeof(e));
  }
  return m;
}

inline BitMatrix square(const BitMatrix& m) {
  BitMatrix r;
  for (int p = 0; p < 128; ++p) apply(m, m.col[p], r.col[p]);
  return r;
}

// Powers M^(2^k), k = 0..K-1, laid out [K][128][4] words.
std::vector<uint32_t> powers(BitMatrix m, int K) {
  std::vector<uint32_t> out((size_t)K * 128 * 4);
  for (int k = 0; k < K; ++k) {
    std::memcpy(&out[(size_t)k * 512], m.col, sizeof(m.col));
    m = square(m);
  }
  return out;
}

// Byte tables of the powers for the device: entry [k][p][v] = M^(2^k) applied
// to byte value v placed at byte p of the state (bits 8p .. 8p+7), laid out
// [K][16][256][4] words, so one application is 16 independent table loads
// and xors (instead of one dependent load per set bit of the state).
std::vector<uint32_t> byte_tables(const std::vector<uint32_t>& pows, int K) {
  std::vector<uint32_t> out((size_t)K * 16 * 256 * 4, 0u);
  for (int k = 0; k < K; ++k)
    for (int p = 0; p < 16; ++p)
      for (int v = 1; v < 256; ++v) {
        // entry v = entry (v without its lowest bit) ^ column of that bit
        const int low = __builtin_ctz((unsigned)v);
        const uint32_t* prev = &out[(((size_t)k * 16 + p) * 256 + (v & (v - 1))) * 4];
        const uint32_t* col = &pows[((size_t)k * 128 + p * 8 + low) * 4];
        uint32_t* e = &out[(((size_t)k * 16 + p) * 256 + v) * 4];
        for (int w = 0; w < 4; ++w) e[w] = prev[w] ^ col[w];
      }
  return out;
}
constexpr int kTableWords = 16 * 256 * 4;  // one power's byte tables

constexpr int kJumpPowers = 32;  // states < 2^32

int ensure_jump_powers(vkc_device_t dev) {
  if (dev->xo_jump_pows) return VKC_OK;
  static std::vector<uint32_t> host_pows =
      byte_tables(powers(matrix_of([](uint32_t* s) { host_ref_jump(s); }), kJumpPowers), kJumpPowers);
  uint32_t* d = nullptr;
  VKC_CUDA(cudaMalloc(&d, host_pows.size() * sizeof(uint32_t)));
  cudaError_t e = cudaMemcpy(d, host_pows.data(), host_pows.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(d);
    return vkc::set_error(VKC_ERR_CUDA, "jump powers upload: %s", cudaGetErrorString(e));
  }
  dev->xo_jump_pows = d;
  return VKC_OK;
}

// Powers of the next() map itself, N^(2^k): with few states a state's chain
// of outputs is cut into segments whose start states are N^(g L) s, so the
// segments run in parallel (outputs and final states are those of the
// serial loop).
constexpr int kNextPowers = 48;  // up to 2^48 steps per state
int ensure_next_powers(vkc_device_t dev) {
  if (dev->xo_next_pows) return VKC_OK;
  static std::vector<uint32_t> host_pows =
      byte_tables(powers(matrix_of([](uint32_t* s) { host_step(s); }), kNextPowers), kNextPowers);
  uint32_t* d = nullptr;
  VKC_CUDA(cudaMalloc(&d, host_pows.size() * sizeof(uint32_t)));
  cudaError_t e = cudaMemcpy(d, host_pows.data(), host_pows.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(d);
    return vkc::set_error(VKC_ERR_CUDA, "next powers upload: %s", cudaGetErrorString(e));
  }
  dev->xo_next_pows = d;
  return VKC_OK;
}

// ---------------------------------------------------------------- device side
__device__ __forceinline__ uint32_t rotl(uint32_t x, int k) { return __funnelshift_l(x, x, k); }

// xoshiro128++ next(): returns the output and advances the state.
__device__ __forceinline__ uint32_t next(uint4& s) {
  const uint32_t result = rotl(s.x + s.w, 7) + s.x;
  const uint32_t t = s.y << 9;
  s.z ^= s.x;
  s.w ^= s.y;
  s.y ^= s.z;
  s.x ^= s.w;
  s.z ^= t;
  s.w = rotl(s.w, 11);
  return result;
}

// [0,1) float from the top 23 bits (prng_xoshiro128pp_float.comp:33).
__device__ __forceinline__ float to_unit(uint32_t r) { return __uint_as_float((r >> 9) | 0x3f800000u) - 1.0f; }

// Box-Muller pair (prng_box_muller.comp:26-31).
__device__ __forceinline__ void box_muller(float u0, float u1, float mean, float stddev, float& z0, float& z1) {
  const float r = sqrtf(-2.0f * logf(1.0f - u0)) * stddev;
  const float angle = 6.28318530718f * u1;
  float s, c;
  sincosf(angle, &s, &c);
  z0 = __fmaf_rn(r, s, mean);
  z1 = __fmaf_rn(r, c, mean);
}

// x times one power of a map, from its byte tables (16 x 256 entries).
__device__ __forceinline__ uint4 apply_dev(const uint4* __restrict__ tab, uint4 x) {
  const uint32_t w[4] = {x.x, x.y, x.z, x.w};
  uint4 c[16];
#pragma unroll
  for (int p = 0; p < 16; ++p) c[p] = __ldg(&tab[p * 256 + ((w[p >> 2] >> ((p & 3) * 8)) & 0xffu)]);
  uint4 r = c[0];
#pragma unroll
  for (int p = 1; p < 16; ++p) {
    r.x ^= c[p].x;
    r.y ^= c[p].y;
    r.z ^= c[p].z;
    r.w ^= c[p].w;
  }
  return r;
}

__global__ void __launch_bounds__(kThreads)
k_seed(uint4 s0, const uint4* __restrict__ jump_pows, uint32_t size, uint4* state) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= size) return;
  uint4 x = s0;
  uint32_t e = i;
  int k = 0;
  while (e) {
    if (e & 1u) x = apply_dev(jump_pows + (size_t)k * (kTableWords / 4), x);
    e >>= 1;
    ++k;
  }
  state[i] = x;
}

// s advanced by e steps of next(): N^e s from the powers N^(2^k).
__device__ __forceinline__ uint4 advance(const uint4* __restrict__ pows, uint4 s, uint64_t e) {
  int k = 0;
  while (e) {
    if (e & 1u) s = apply_dev(pows + (size_t)k * (kTableWords / 4), s);
    e >>= 1;
    ++k;
  }
  return s;
}

enum { kOutU32 = 0, kOutF32 = 1, kOutRange = 2 };

template <int MODE>
__device__ __forceinline__ void put(void* out, size_t k, uint32_t r, uint32_t low, uint32_t range) {
  if (MODE == kOutU32) {
    static_cast<uint32_t*>(out)[k] = r;
  } else if (MODE == kOutF32) {
    static_cast<float*>(out)[k] = to_unit(r);
  } else {
    // prng_randrange.comp:26: low + uint(float(range) * u)
    static_cast<uint32_t*>(out)[k] = low + (uint32_t)((float)range * to_unit(r));
  }
}

// Segmented generation: thread (t, g) = (idx % size, idx / size) produces
// steps [g L, (g + 1) L) of state t (out[step * size + t]); the thread
// holding a state's last step stores it to state_out (state_in is read by
// every segment, so it is not overwritten here).
template <int MODE>
__global__ void __launch_bounds__(kThreads)
k_generate_seg(const uint4* __restrict__ state_in, uint4* __restrict__ state_out, uint32_t size, void* out, size_t n,
               uint32_t low, uint32_t range, const uint4* __restrict__ pows, uint64_t L, uint32_t G) {
  const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (uint64_t)size * G) return;
  const uint32_t t = (uint32_t)(idx % size), g = (uint32_t)(idx / size);
  if ((size_t)t >= n) return;
  const uint64_t cnt = (n - t + size - 1) / size;  // steps of state t
  const uint64_t b0 = (uint64_t)g * L;
  if (b0 >= cnt) return;
  const uint64_t b1 = min(cnt, b0 + L);
  uint4 s = advance(pows, state_in[t], b0);
  for (uint64_t step = b0; step < b1; ++step) put<MODE>(out, step * size + t, next(s), low, range);
  if (b1 == cnt) state_out[t] = s;
}

template <int MODE>
__global__ void __launch_bounds__(kThreads)
k_generate(uint4* state, uint32_t size, void* out, size_t n, uint32_t low, uint32_t range) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= size || (size_t)t >= n) return;
  uint4 s = state[t];
  const size_t step = size;
  const size_t cnt = (n - t + step - 1) / step;  // outputs of state t
  size_t k = t, j = 0;
  // four draws, then their four stores
  for (; j + 4 <= cnt; j += 4, k += 4 * step) {
    const uint32_t r0 = next(s), r1 = next(s), r2 = next(s), r3 = next(s);
    put<MODE>(out, k, r0, low, range);
    put<MODE>(out, k + step, r1, low, range);
    put<MODE>(out, k + 2 * step, r2, low, range);
    put<MODE>(out, k + 3 * step, r3, low, range);
  }
  for (; j < cnt; ++j, k += step) put<MODE>(out, k, next(s), low, range);
  state[t] = s;
}

// Normal numbers with an even number of states: thread p owns states 2p and
// 2p+1, which produce both halves of every Box-Muller pair it writes.
// `m` is the length of the uniform stream (n, or n+1 for odd n).
__global__ void __launch_bounds__(kThreads)
k_normal_pairs(uint4* state, uint32_t size, float* out, size_t n, size_t m, float mean, float stddev) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t ta = 2 * p;
  if (ta >= size || (size_t)ta >= m) return;
  uint4 sa = state[ta], sb = state[ta + 1];
  for (size_t k0 = ta; k0 < m; k0 += size) {
    const float u0 = to_unit(next(sa));
    const float u1 = to_unit(next(sb));  // k0 + 1 < m: m is even
    float z0, z1;
    box_muller(u0, u1, mean, stddev, z0, z1);
    out[k0] = z0;
    if (k0 + 1 < n) out[k0 + 1] = z1;
  }
  state[ta] = sa;
  state[ta + 1] = sb;
}

// k_normal_pairs cut into segments of L pair-steps (as k_generate_seg).
__global__ void __launch_bounds__(kThreads)
k_normal_pairs_seg(const uint4* __restrict__ state_in, uint4* __restrict__ state_out, uint32_t size, float* out,
                   size_t n, size_t m, float mean, float stddev, const uint4* __restrict__ pows, uint64_t L,
                   uint32_t G) {
  const uint32_t pairs = size / 2;
  const uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (uint64_t)pairs * G) return;
  const uint32_t p = (uint32_t)(idx % pairs), g = (uint32_t)(idx / pairs);
  const uint32_t ta = 2 * p;
  if ((size_t)ta >= m) return;
  const uint64_t cnt = (m - ta + size - 1) / size;  // pair steps of states ta, ta + 1
  const uint64_t b0 = (uint64_t)g * L;
  if (b0 >= cnt) return;
  const uint64_t b1 = min(cnt, b0 + L);
  uint4 sa = advance(pows, state_in[ta], b0), sb = advance(pows, state_in[ta + 1], b0);
  for (uint64_t step = b0; step < b1; ++step) {
    const size_t k0 = step * size + ta;
    const float u0 = to_unit(next(sa));
    const float u1 = to_unit(next(sb));
    float z0, z1;
    box_muller(u0, u1, mean, stddev, z0, z1);
    out[k0] = z0;
    if (k0 + 1 < n) out[k0 + 1] = z1;
  }
  if (b1 == cnt) {
    state_out[ta] = sa;
    state_out[ta + 1] = sb;
  }
}

__global__ void __launch_bounds__(kThreads)
k_box_muller(const float* u, float* out, size_t n, float mean, float stddev) {
  const size_t pairs = (n + 1) / 2;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < pairs; i += stride) {
    const size_t j = 2 * i;
    float z0, z1;
    box_muller(u[j], u[j + 1], mean, stddev, z0, z1);
    out[j] = z0;
    if (j + 1 < n) out[j + 1] = z1;
  }
}

// Segments per state for `active` states of `steps` outputs each: enough
// threads to fill the GPU, at least `min_len` steps per segment (a segment's
// start costs one application of a power of N, 16 table loads, per set bit
// of its offset, so cheap steps (uniform draws: 256) need longer segments
// than Box-Muller pairs (16); 64 states x 65536 outputs: uniforms 24 -> 9 us,
// normals 60 -> 19 us).  1 = serial chains.
uint32_t segments(vkc_device_t dev, uint64_t active, uint64_t steps, uint64_t min_len) {
  const uint64_t want_threads = (uint64_t)dev->sm_count * 512;
  if (active >= want_threads || steps < 2 * min_len) return 1;
  if (!dev->xo_next_pows) {
    // the powers are uploaded synchronously on first use: not while the
    // stream is being captured (the serial kernel computes the same values)
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(dev->stream, &st) != cudaSuccess || st != cudaStreamCaptureStatusNone) {
      cudaGetLastError();
      return 1;
    }
  }
  const uint64_t g = std::min<uint64_t>((want_threads + active - 1) / active, steps / min_len);
  return (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(g, 1u << 20));
}

// Run a segmented kernel: the final states go to a scratch copy (every
// segment reads the initial ones) and are copied back for the first
// `active` states (the others do not advance).
template <class Launch>
int run_segmented(vkc_device_t dev, uint32_t* state, uint32_t active, Launch launch) {
  {
    std::lock_guard<std::mutex> lk(dev->mu);
    int r = ensure_next_powers(dev);
    if (r != VKC_OK) return r;
  }
  uint4* state_out = nullptr;
  int r = vkc::scratch_alloc(dev, (size_t)active * sizeof(uint4), (void**)&state_out);
  if (r != VKC_OK) return r;
  launch(state_out, reinterpret_cast<const uint4*>(dev->xo_next_pows));
  r = vkc::check_launch("xoshiro (segmented)");
  if (r == VKC_OK) {
    cudaError_t e = cudaMemcpyAsync(state, state_out, (size_t)active * sizeof(uint4), cudaMemcpyDeviceToDevice,
                                    dev->stream);
    if (e != cudaSuccess) r = vkc::set_error(VKC_ERR_CUDA, "xoshiro state copy: %s", cudaGetErrorString(e));
  }
  vkc::scratch_free(dev, state_out);
  return r;
}

template <int MODE>
int generate(vkc_device_t dev, uint32_t* state, uint32_t size, void* out, size_t n, uint32_t low, uint32_t range) {
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(state && out, "NULL buffer");
  VKC_REQUIRE(size > 0, "PRNG has no states");
  VKC_REQUIRE(((uintptr_t)state & 15u) == 0, "state buffer must be 16-byte aligned");
  uint32_t active = (uint32_t)std::min<size_t>(size, n);
  const uint64_t steps = (n + size - 1) / size;
  const uint32_t G = segments(dev, active, steps, 256);
  if (G > 1) {
    const uint64_t L = (steps + G - 1) / G;
    return run_segmented(dev, state, active, [&](uint4* state_out, const uint4* pows) {
      const uint64_t threads = (uint64_t)size * G;
      k_generate_seg<MODE><<<(unsigned)((threads + kThreads - 1) / kThreads), kThreads, 0, dev->stream>>>(
          reinterpret_cast<const uint4*>(state), state_out, size, out, n, low, range, pows, L, G);
    });
  }
  unsigned grid = (active + kThreads - 1) / kThreads;
  k_generate<MODE><<<grid, kThreads, 0, dev->stream>>>(reinterpret_cast<uint4*>(state), size, out, n, low, range);
  return vkc::check_launch("xoshiro");
}

}  // namespace

VKC_EXPORT int vkc_xoshiro_seed(vkc_device_t dev, uint64_t seed, uint32_t size, uint32_t* state) {
  VKC_BIND(dev);
  VKC_REQUIRE(state, "NULL state buffer");
  VKC_REQUIRE(size > 0, "PRNG size must be positive");
  VKC_REQUIRE(((uintptr_t)state & 15u) == 0, "state buffer must be 16-byte aligned");
  uint32_t s0[4];
  for (int i = 0; i < 4; ++i) {
    seed = splitmix64(seed);
    s0[i] = (uint32_t)seed;
  }
  {
    std::lock_guard<std::mutex> lk(dev->mu);
    int r = ensure_jump_powers(dev);
    if (r != VKC_OK) return r;
  }
  unsigned grid = (size + kThreads - 1) / kThreads;
  k_seed<<<grid, kThreads, 0, dev->stream>>>(make_uint4(s0[0], s0[1], s0[2], s0[3]),
                                               reinterpret_cast<const uint4*>(dev->xo_jump_pows), size,
                                               reinterpret_cast<uint4*>(state));
  return vkc::check_launch("xoshiro_seed");
}

VKC_EXPORT int vkc_xoshiro_u32(vkc_device_t dev, uint32_t* state, uint32_t size, uint32_t* out, size_t n) {
  VKC_BIND(dev);
  return generate<kOutU32>(dev, state, size, out, n, 0, 0);
}

VKC_EXPORT int vkc_xoshiro_f32(vkc_device_t dev, uint32_t* state, uint32_t size, float* out, size_t n) {
  VKC_BIND(dev);
  return generate<kOutF32>(dev, state, size, out, n, 0, 0);
}

VKC_EXPORT int vkc_xoshiro_randrange(vkc_device_t dev, uint32_t* state, uint32_t size, uint32_t* out, size_t n,
                                     uint32_t low, uint32_t high_incl) {
  VKC_BIND(dev);
  VKC_REQUIRE(low <= high_incl, "low must not exceed high");
  return generate<kOutRange>(dev, state, size, out, n, low, high_incl - low + 1u);
}

VKC_EXPORT int vkc_box_muller(vkc_device_t dev, const float* u, float* out, size_t n, float mean, float stddev) {
  VKC_BIND(dev);
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(u && out, "NULL buffer");
  unsigned grid = vkc::wave_grid(dev, k_box_muller, (n + 1) / 2, kThreads);
  k_box_muller<<<grid, kThreads, 0, dev->stream>>>(u, out, n, mean, stddev);
  return vkc::check_launch("box_muller");
}

VKC_EXPORT int vkc_xoshiro_normal(vkc_device_t dev, uint32_t* state, uint32_t size, float* out, size_t n,
                                  float mean, float stddev) {
  VKC_BIND(dev);
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(state && out, "NULL buffer");
  VKC_REQUIRE(size > 0, "PRNG has no states");
  VKC_REQUIRE(((uintptr_t)state & 15u) == 0, "state buffer must be 16-byte aligned");
  const size_t m = (n % 2 == 0) ? n : n + 1;  // random.py:116-118 draws 2*(n//2+1) for odd n
  if (size % 2 == 0) {
    uint32_t pairs = (uint32_t)std::min<size_t>(size / 2, m / 2);
    const uint64_t steps = (m + size - 1) / size;
    const uint32_t G = segments(dev, pairs, steps, 16);
    if (G > 1) {
      const uint64_t L = (steps + G - 1) / G;
      return run_segmented(dev, state, (uint32_t)std::min<size_t>(size, m), [&](uint4* state_out, const uint4* pows) {
        const uint64_t threads = (uint64_t)(size / 2) * G;
        k_normal_pairs_seg<<<(unsigned)((threads + kThreads - 1) / kThreads), kThreads, 0, dev->stream>>>(
            reinterpret_cast<const uint4*>(state), state_out, size, out, n, m, mean, stddev, pows, L, G);
      });
    }
    unsigned grid = (pairs + kThreads - 1) / kThreads;
    k_normal_pairs<<<grid, kThreads, 0, dev->stream>>>(reinterpret_cast<uint4*>(state), size, out, n, m, mean,
                                                        stddev);
    return vkc::check_launch("xoshiro_normal");
  }
  // Odd number of states: a pair can straddle two states in different
  // chunks, so draw the uniform stream first, then transform it.
  float* u = out;
  if (m != n) {
    int r = vkc::scratch_alloc(dev, m * sizeof(float), (void**)&u);
    if (r != VKC_OK) return r;
  }
  int r = generate<kOutF32>(dev, state, size, u, m, 0, 0);
  if (r == VKC_OK) {
    unsigned grid = vkc::wave_grid(dev, k_box_muller, m / 2, kThreads);
    k_box_muller<<<grid, kThreads, 0, dev->stream>>>(u, out, n, mean, stddev);
    r = vkc::check_launch("box_muller");
  }
  if (u != out) vkc::scratch_free(dev, u);
  return r;
}
