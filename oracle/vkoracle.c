/*
 * vkoracle.c -- CPU restatement of vulkpy's algorithms.  TEST INFRASTRUCTURE:
 * this is the checker (and the timed CPU baseline), never the product.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use it.
 *
 * Each function restates one reference routine (paths inside the vulkpy
 * project) in plain C, float32 arithmetic, in the reference's loop order:
 *   xo_seed        PRNG::Xoshiro128pp ctor, _vkarray.cc:643-675 (splitmix64
 *                  589-595, jump 597-621, next 627-641)
 *   xo_generate    Xoshiro128pp::random, _vkarray.cc:697-717 with
 *                  prng_xoshiro128pp_uint32.comp:26-43 / _float.comp:26-44
 *   box_muller     prng_box_muller.comp:19-32 (all n outputs written)
 *   randrange      prng_randrange.comp:20-27
 *   ew_*           add.comp etc. (one element per invocation)
 *   bcast_binary   add_broadcast.comp:25-45 index math
 *   reduce_axis    sum_axis.comp:20-32 (serial loop per output)
 *   reduce_all     numpy-intended full reduction, sequential fp32
 *   matmul         matmul.comp:23-33 (serial K loop per output)
 *   gather         gather.comp:21-26, gather_axis.comp:24-43 (clamped to axis-1)
 * OpenMP parallelises over independent outputs only, so results do not
 * depend on the thread count.
 */
#include <math.h>
#include <stdint.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define EXPORT __attribute__((visibility("default")))

/* ---------------------------------------------------------------- PRNG */
static inline uint32_t rotl32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }

static inline uint32_t xo_next(uint32_t s[4]) {
  const uint32_t result = rotl32(s[0] + s[3], 7) + s[0];
  const uint32_t t = s[1] << 9;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl32(s[3], 11);
  return result;
}

static inline uint64_t splitmix64(uint64_t x) {
  uint64_t z = (x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

/* The reference's jump: accumulators are not reset between the four JUMP
 * words and are written back into the state after every word. */
static void ref_jump(uint32_t s[4]) {
  static const uint32_t JUMP[4] = {0x8764000bu, 0xf542d2d3u, 0x6fa035c3u, 0x77f2db5bu};
  uint32_t s0 = 0, s1 = 0, s2 = 0, s3 = 0;
  for (int w = 0; w < 4; ++w) {
    for (int b = 0; b < 32; ++b) {
      if (JUMP[w] & (1u << b)) {
        s0 ^= s[0];
        s1 ^= s[1];
        s2 ^= s[2];
        s3 ^= s[3];
      }
      xo_next(s);
    }
    s[0] = s0;
    s[1] = s1;
    s[2] = s2;
    s[3] = s3;
  }
}

EXPORT void xo_seed(uint64_t seed, uint32_t size, uint32_t* state) {
  uint32_t s[4];
  for (int i = 0; i < 4; ++i) {
    seed = splitmix64(seed);
    s[i] = (uint32_t)seed;
    state[i] = s[i];
  }
  for (uint32_t i = 1; i < size; ++i) {
    ref_jump(s);
    memcpy(state + 4 * (size_t)i, s, sizeof(s));
  }
}

static inline float to_unit(uint32_t r) {
  uint32_t bits = (r >> 9) | 0x3f800000u;
  float f;
  memcpy(&f, &bits, 4);
  return f - 1.0f;
}

/* mode 0: raw uint32, 1: [0,1) float.  out[k] = next^(k/size)(state[k%size]). */
EXPORT void xo_generate(uint32_t* state, uint32_t size, void* out, uint64_t n, int mode) {
  uint32_t active = (uint64_t)size < n ? size : (uint32_t)n;
#pragma omp parallel for schedule(static)
  for (int64_t t = 0; t < (int64_t)active; ++t) {
    uint32_t s[4];
    memcpy(s, state + 4 * t, sizeof(s));
    for (uint64_t k = (uint64_t)t; k < n; k += size) {
      uint32_t r = xo_next(s);
      if (mode == 0) ((uint32_t*)out)[k] = r;
      else ((float*)out)[k] = to_unit(r);
    }
    memcpy(state + 4 * t, s, sizeof(s));
  }
}

EXPORT void box_muller(const float* u, float* out, uint64_t n, float mean, float stddev) {
  uint64_t pairs = (n + 1) / 2;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)pairs; ++i) {
    uint64_t j = 2 * (uint64_t)i, k = j + 1;
    float r = sqrtf(-2.0f * logf(1.0f - u[j])) * stddev;
    float angle = 6.28318530718f * u[k];
    float a = mean + r * sinf(angle);
    float b = mean + r * cosf(angle);
    out[j] = a;
    if (k < n) out[k] = b;
  }
}

EXPORT void randrange(const float* u, uint32_t* out, uint64_t n, uint32_t low, uint32_t high_incl) {
  const uint32_t range = high_incl - low + 1u;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) out[i] = low + (uint32_t)((float)range * u[i]);
}

/* ----------------------------------------------------------- elementwise */
static inline float binop(int op, float a, float b) {
  switch (op) {
    case 0: return a + b;
    case 1: return a - b;
    case 2: return a * b;
    case 3: return a / b;
    case 4: return powf(a, b);
    case 5: return fmaxf(a, b);
    case 6: return fminf(a, b);
    case 7: return b - a;
    case 8: return b / a;
    case 9: return powf(b, a);
  }
  return a;
}

static inline float unop(int op, float x) {
  switch (op) {
    case 0: return fabsf(x);
    case 1: return x > 0.f ? 1.f : (x < 0.f ? -1.f : x);
    case 2: return sinf(x);
    case 3: return cosf(x);
    case 4: return tanf(x);
    case 5: return asinf(x);
    case 6: return acosf(x);
    case 7: return atanf(x);
    case 8: return sinhf(x);
    case 9: return coshf(x);
    case 10: return tanhf(x);
    case 11: return asinhf(x);
    case 12: return acoshf(x);
    case 13: return atanhf(x);
    case 14: return expf(x);
    case 15: return logf(x);
    case 16: return exp2f(x);
    case 17: return log2f(x);
    case 18: return sqrtf(x);
    case 19: return 1.0f / sqrtf(x);
  }
  return x;
}

EXPORT void ew_binary(int op, const float* a, const float* b, float* c, uint64_t n) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) c[i] = binop(op, a[i], b[i]);
}

EXPORT void ew_scalar(int op, const float* a, float s, float* c, uint64_t n) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) c[i] = (op == 4 && s == 2.0f) ? a[i] * a[i] : binop(op, a[i], s);
}

EXPORT void ew_unary(int op, const float* a, float* c, uint64_t n) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) c[i] = unop(op, a[i]);
}

/* add_broadcast.comp:25-45: shapes padded to ndim; sizes divided down per dim. */
EXPORT void bcast_binary(int op, const float* a, const int64_t* sa, const float* b, const int64_t* sb, float* c,
                         const int64_t* sc, int ndim) {
  int64_t na = 1, nb = 1, nc = 1;
  for (int d = 0; d < ndim; ++d) {
    na *= sa[d];
    nb *= sb[d];
    nc *= sc[d];
  }
#pragma omp parallel for schedule(static)
  for (int64_t ci = 0; ci < nc; ++ci) {
    int64_t size_a = na, size_b = nb, size_c = nc;
    int64_t ai = 0, bi = 0, rem = ci;
    for (int d = 0; d < ndim; ++d) {
      size_a /= sa[d];
      size_b /= sb[d];
      size_c /= sc[d];
      int64_t q = rem / size_c;
      ai += size_a * (q < sa[d] - 1 ? q : sa[d] - 1);
      bi += size_b * (q < sb[d] - 1 ? q : sb[d] - 1);
      rem = rem % size_c;
    }
    c[ci] = binop(op, a[ai], b[bi]);
  }
}

/* ------------------------------------------------------------ reductions */
static inline float red(int op, float acc, float x) {
  switch (op) {
    case 0: return acc + x;
    case 1: return acc * x;
    case 2: return fmaxf(acc, x);
    default: return fminf(acc, x);
  }
}
static inline float red_init(int op) {
  switch (op) {
    case 0: return 0.f;
    case 1: return 1.f;
    case 2: return -INFINITY;
    default: return INFINITY;
  }
}

/* sum_axis.comp:20-32: out[i*post+j] = fold_k a[(i*axis+k)*post + j], in k order. */
EXPORT void reduce_axis(int op, const float* a, uint64_t prev, uint64_t axis, uint64_t post, float* out) {
#pragma omp parallel for schedule(static) collapse(2)
  for (int64_t i = 0; i < (int64_t)prev; ++i) {
    for (int64_t j = 0; j < (int64_t)post; ++j) {
      float acc = red_init(op);
      const float* base = a + (uint64_t)i * axis * post + (uint64_t)j;
      for (uint64_t k = 0; k < axis; ++k) acc = red(op, acc, base[k * post]);
      out[(uint64_t)i * post + (uint64_t)j] = acc;
    }
  }
}

/* Full reduction in one sequential fp32 pass per thread block of 4096, then
 * sequentially over blocks (a fixed order, independent of thread count). */
EXPORT float reduce_all(int op, const float* a, uint64_t n) {
  const uint64_t B = 4096;
  uint64_t nb = (n + B - 1) / B;
  float* parts = (float*)malloc(sizeof(float) * (nb ? nb : 1));
  if (!parts) return NAN;
#pragma omp parallel for schedule(static)
  for (int64_t blk = 0; blk < (int64_t)nb; ++blk) {
    float p = red_init(op);
    uint64_t e = ((uint64_t)blk + 1) * B;
    if (e > n) e = n;
    for (uint64_t i = (uint64_t)blk * B; i < e; ++i) p = red(op, p, a[i]);
    parts[blk] = p;
  }
  float acc = red_init(op);
  for (uint64_t blk = 0; blk < nb; ++blk) acc = red(op, acc, parts[blk]);
  free(parts);
  return acc;
}

/* ------------------------------------------------------------------ matmul */
EXPORT void matmul(const float* a, const float* b, float* c, int64_t M, int64_t K, int64_t N) {
#pragma omp parallel for schedule(static)
  for (int64_t row = 0; row < M; ++row) {
    for (int64_t col = 0; col < N; ++col) {
      float sum = 0.0f;
      for (int64_t s = 0; s < K; ++s) sum += a[row * K + s] * b[s * N + col];
      c[row * N + col] = sum;
    }
  }
}

/* ------------------------------------------------------------------ gather */
EXPORT void gather(const float* a, uint64_t n_a, const uint32_t* idx, uint64_t n_idx, float* c) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n_idx; ++i) c[i] = (uint64_t)idx[i] < n_a ? a[idx[i]] : NAN;
}

EXPORT void gather_axis(const float* a, uint64_t prev, uint64_t axis, uint64_t post, const uint32_t* idx,
                        uint64_t n_idx, float* c) {
#pragma omp parallel for schedule(static) collapse(2)
  for (int64_t k = 0; k < (int64_t)n_idx; ++k) {
    for (int64_t i = 0; i < (int64_t)prev; ++i) {
      uint64_t q = idx[k] < axis ? idx[k] : axis - 1;
      for (uint64_t j = 0; j < post; ++j)
        c[((uint64_t)k * prev + (uint64_t)i) * post + j] = a[((uint64_t)i * axis + q) * post + j];
    }
  }
}

/* ------------------------------------------------------------- permutation
 * No reference kernel (the reference shuffles on the host,
 * example/02-nn.py:82).  Restates the library's keyed Feistel permutation:
 * 6 rounds of murmur3's fmix32 on R ^ key[r % 4] ^ r * 0x9E3779B9 over d/2-bit
 * halves, d = max(2, ceil(log2 n)) rounded up to even, cycle-walked into
 * [0, n). */
static inline uint32_t fmix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x85EBCA6Bu;
  x ^= x >> 13;
  x *= 0xC2B2AE35u;
  x ^= x >> 16;
  return x;
}

EXPORT void permutation(const uint32_t* key, uint32_t* out, uint64_t n) {
  int d = 0;
  while (d < 64 && ((uint64_t)1 << d) < n) ++d;
  if (d < 2) d = 2;
  if (d & 1) ++d;
  const int h = d / 2;
  const uint32_t mask = h >= 32 ? 0xFFFFFFFFu : ((1u << h) - 1u);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < (int64_t)n; ++i) {
    uint64_t x = (uint64_t)i;
    do {
      uint32_t l = (uint32_t)(x >> h), r = (uint32_t)x & mask;
      for (uint32_t k = 0; k < 6; ++k) {
        uint32_t f = fmix32(r ^ key[k & 3] ^ (k * 0x9E3779B9u)) & mask;
        uint32_t nl = r;
        r = l ^ f;
        l = nl;
      }
      x = ((uint64_t)l << h) | r;
    } while (x >= n);
    out[i] = (uint32_t)x;
  }
}

EXPORT int oracle_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
