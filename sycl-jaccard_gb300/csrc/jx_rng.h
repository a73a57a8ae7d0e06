/*
 * Counter-based random numbers shared by the host graph generator and the device generator.
 *
 * Every random draw is a pure function of (seed, stream, counter), so a graph is the same
 * whether it is generated on the host (any architecture, any thread count) or on the GPU.
 * Only integer arithmetic is used: no libm, no floating-point rounding that could differ
 * between x86_64 and aarch64.
 *
 * The mixer is the SplitMix64 finaliser (Steele, Lea, Flood, "Fast splittable pseudorandom
 * number generators", OOPSLA 2014), applied twice to fold three 64-bit words together.
 */
#ifndef JX_RNG_H
#define JX_RNG_H

#include <stdint.h>

#if defined(__CUDACC__)
#define JX_HD __host__ __device__ __forceinline__
#else
#define JX_HD static inline
#endif

JX_HD uint64_t jx_mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* One 64-bit draw for (seed, stream, counter). */
JX_HD uint64_t jx_draw(uint64_t seed, uint64_t stream, uint64_t counter) {
  return jx_mix64(jx_mix64(seed * 0xD1B54A32D192ED03ull + stream) ^ counter);
}

/* Uniform integer in [0, n) from the high 32 bits of a draw (multiply-shift range reduction). */
JX_HD uint32_t jx_bounded32(uint64_t draw, uint32_t n) {
  return (uint32_t)(((draw >> 32) * (uint64_t)n) >> 32);
}

/*
 * R-MAT quadrant choice for one recursion level from a 32-bit uniform u.
 * t0 < t1 < t2 are the cumulative thresholds a, a+b, a+b+c scaled by 2^32.
 * Returns the (row bit, col bit) pair packed as (row << 1) | col.
 */
JX_HD uint32_t jx_rmat_quadrant(uint32_t u, uint32_t t0, uint32_t t1, uint32_t t2) {
  return u < t0 ? 0u : (u < t1 ? 1u : (u < t2 ? 2u : 3u));
}

/*
 * One R-MAT edge sample: `scale` recursion levels, two levels per 64-bit draw.
 * Level 0 decides the most significant bit of both endpoints.
 */
JX_HD void jx_rmat_sample(uint64_t seed, uint64_t sample, int scale, uint32_t t0, uint32_t t1,
                          uint32_t t2, uint32_t *src, uint32_t *dst) {
  uint32_t r = 0, c = 0;
  uint64_t d = 0;
  for (int l = 0; l < scale; ++l) {
    uint32_t u;
    if ((l & 1) == 0) {
      d = jx_draw(seed, sample, (uint64_t)(l >> 1));
      u = (uint32_t)(d >> 32);
    } else {
      u = (uint32_t)d;
    }
    uint32_t q = jx_rmat_quadrant(u, t0, t1, t2);
    r = (r << 1) | (q >> 1);
    c = (c << 1) | (q & 1u);
  }
  *src = r;
  *dst = c;
}

/*
 * A seeded bijection of [0, 2^bits) (1 <= bits <= 32) for relabelling vertex ids: four rounds
 * of (multiply by an odd key, xor with the upper half shifted down, add a key), each step a
 * bijection modulo 2^bits.
 */
JX_HD uint32_t jx_permute_bits(uint32_t x, int bits, uint64_t seed) {
  const uint32_t mask = bits >= 32 ? 0xFFFFFFFFu : ((1u << bits) - 1u);
  const int shift = (bits + 1) / 2;
  for (uint64_t r = 0; r < 4; ++r) {
    const uint64_t k = jx_draw(seed, 0x5045524Dull, r);
    x = (x * ((uint32_t)k | 1u)) & mask;
    x ^= x >> shift;
    x = (x + (uint32_t)(k >> 32)) & mask;
  }
  return x;
}

#endif /* JX_RNG_H */
