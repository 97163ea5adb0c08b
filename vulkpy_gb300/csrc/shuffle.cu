// Random permutation of 0..n-1 on the device, for GPU-side shuffling.
//
// The reference shuffles on the host (example/02-nn.py:82, "TODO: Implement
// GPU shuffle()").  A sort of random keys would cost several passes over
// HBM; instead each output index is computed independently: a keyed Feistel
// network is a bijection on [0, 2^d) (d even, the smallest with 2^d >= n),
// and walking its cycle from i until the value falls below n restricts it to
// a bijection on [0, n) (cycle walking).  Since 2^d < 4n, a walk takes fewer
// than 4 steps on average and always ends: the cycle through i returns to i.
//
// Round function: the murmur3 32-bit finaliser (a public-domain mixer) of
// R ^ key[r mod 4] ^ r * 0x9E3779B9, masked to d/2 bits; 6 rounds.  The four
// keys are drawn from the xoshiro128++ stream, so a seeded generator gives a
// reproducible permutation and advances exactly as a 4-value draw would.
#include "common.cuh"

namespace vkc {
namespace {

constexpr int kThreads = 256;
constexpr int kRounds = 6;

__device__ __forceinline__ uint32_t fmix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x85EBCA6Bu;
  x ^= x >> 13;
  x *= 0xC2B2AE35u;
  x ^= x >> 16;
  return x;
}

__device__ __forceinline__ uint64_t feistel(uint64_t x, int h, uint32_t mask, const uint32_t (&key)[4]) {
  uint32_t l = (uint32_t)(x >> h), r = (uint32_t)x & mask;
#pragma unroll
  for (int i = 0; i < kRounds; ++i) {
    const uint32_t f = fmix32(r ^ key[i & 3] ^ ((uint32_t)i * 0x9E3779B9u)) & mask;
    const uint32_t nl = r;
    r = l ^ f;
    l = nl;
  }
  return ((uint64_t)l << h) | r;
}

__global__ void __launch_bounds__(kThreads) k_permutation(const uint32_t* __restrict__ keys, int h,
                                                          uint32_t* __restrict__ out, size_t n) {
  const uint32_t key[4] = {keys[0], keys[1], keys[2], keys[3]};
  const uint32_t mask = (h >= 32) ? 0xFFFFFFFFu : ((1u << h) - 1u);
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    uint64_t x = i;
    do {
      x = feistel(x, h, mask, key);
    } while (x >= n);
    out[i] = (uint32_t)x;
  }
}

// Half-width of the Feistel domain: d = max(2, ceil(log2 n)) rounded up to
// even, h = d / 2.
int half_bits(size_t n) {
  int d = 0;
  while (d < 64 && ((uint64_t)1 << d) < n) ++d;
  if (d < 2) d = 2;
  if (d & 1) ++d;
  return d / 2;
}

}  // namespace
}  // namespace vkc

VKC_EXPORT int vkc_xoshiro_permutation(vkc_device_t dev, uint32_t* state, uint32_t size, uint32_t* out,
                                       size_t n) {
  VKC_BIND(dev);
  VKC_REQUIRE(n <= 0xFFFFFFFFull, "permutation indices are uint32: n must be < 2^32");
  VKC_REQUIRE(state && size > 0, "NULL or empty generator state");
  if (n == 0) return VKC_OK;
  VKC_REQUIRE(out, "NULL buffer");
  void* keys = nullptr;
  int r = vkc::scratch_alloc(dev, 4 * sizeof(uint32_t), &keys);
  if (r != VKC_OK) return r;
  r = vkc_xoshiro_u32(dev, state, size, static_cast<uint32_t*>(keys), 4);
  if (r == VKC_OK) {
    const unsigned g = vkc::stream_grid(dev, n, vkc::kThreads, 8);
    vkc::k_permutation<<<g, vkc::kThreads, 0, dev->stream>>>(static_cast<const uint32_t*>(keys),
                                                             vkc::half_bits(n), out, n);
    r = vkc::check_launch("permutation");
  }
  vkc::scratch_free(dev, keys);
  return r;
}
