// Host random number generator for the default global pivot finder.
//
// The reference draws the random start points of DefaultGlobalPivotFinder
// from Julia's Random.default_rng() (globalpivotfinder.jl:156, called with
// rng=Random.default_rng() from tensorci2.jl:808).  That stream cannot be
// reproduced outside Julia, so this library and its CPU oracle share this
// generator instead: xoshiro256** (Blackman & Vigna, 2018) seeded through
// splitmix64, and rand(1:d) drawn with Lemire's multiply-and-reject method
// (unbiased).  Same seed => same start points on both sides.
#pragma once
#include <stdint.h>

typedef struct tci_rng { uint64_t s[4]; } tci_rng;

static inline uint64_t tci_splitmix64(uint64_t* x) {
  uint64_t z = (*x += 0x9e3779b97f4a7c15ULL);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

static inline void tci_rng_seed(tci_rng* r, uint64_t seed) {
  uint64_t x = seed;
  for (int i = 0; i < 4; ++i) r->s[i] = tci_splitmix64(&x);
}

static inline uint64_t tci_rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t tci_rng_next(tci_rng* r) {
  uint64_t* s = r->s;
  uint64_t result = tci_rotl64(s[1] * 5, 7) * 9;
  uint64_t t = s[1] << 17;
  s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
  s[2] ^= t;
  s[3] = tci_rotl64(s[3], 45);
  return result;
}

// Uniform integer in [1, d] (the reference's rand(rng, 1:d)).
static inline int64_t tci_rng_uniform1(tci_rng* r, uint64_t d) {
  uint64_t x = tci_rng_next(r);
  __uint128_t m = (__uint128_t)x * d;
  uint64_t l = (uint64_t)m;
  if (l < d) {
    uint64_t t = (0 - d) % d;
    while (l < t) {
      x = tci_rng_next(r);
      m = (__uint128_t)x * d;
      l = (uint64_t)m;
    }
  }
  return (int64_t)(m >> 64) + 1;
}

// Uniform double in [0, 1) with 53 random bits.
static inline double tci_rng_unit(tci_rng* r) {
  return (double)(tci_rng_next(r) >> 11) * (1.0 / 9007199254740992.0);
}
