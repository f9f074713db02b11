// lfsr88.cuh -- L'Ecuyer's combined Tausworthe generator (LFSR88) with the exact integer
// and float32 semantics of brainpy/_src/math/tifunc.py:47-180, for device code.
//
// The remainder by the (call-constant) connection length uses the exact "direct
// remainder" method of Lemire, Kaser and Kurz ("Faster remainder by direct computation",
// 2019): with M = floor((2^64 - 1) / d) + 1, x mod d = mulhi64((M * x) mod 2^64, d) for every
// 32-bit x and d.
#pragma once

#include <stdint.h>

namespace bp {

struct Lfsr88 {
  uint32_t s0, s1, s2;
};

struct FastMod {
  uint64_t M;
  uint32_t d;
};

inline FastMod make_fastmod(uint32_t d) {
  FastMod f;
  f.d = d;
  f.M = (d == 0) ? 0 : (0xFFFFFFFFFFFFFFFFull / d + 1ull);
  return f;
}

__device__ __forceinline__ uint32_t fastmod(uint32_t x, FastMod f) {
  const uint64_t low = f.M * (uint64_t)x;  // mod 2^64
  // high 64 bits of the 128-bit product low * d, with d < 2^32: two 32x32->64 products
  const uint64_t t = (uint64_t)(uint32_t)low * f.d;
  const uint64_t u = (uint64_t)(uint32_t)(low >> 32) * f.d + (t >> 32);
  return (uint32_t)(u >> 32);
}

// tifunc.py:47-67
__device__ __forceinline__ Lfsr88 lfsr88_key(uint32_t seed) {
  Lfsr88 k;
  k.s0 = seed + 1u;
  k.s1 = seed + 7u;
  k.s2 = seed + 15u;
  return k;
}

// tifunc.py:70-86; returns k0 ^ k1 ^ k2 of the advanced key
__device__ __forceinline__ uint32_t lfsr88_next(Lfsr88& k) {
  uint32_t b = ((k.s0 << 13) ^ k.s0) >> 19;
  k.s0 = ((k.s0 & 4294967294u) << 12) ^ b;
  b = ((k.s1 << 2) ^ k.s1) >> 25;
  k.s1 = ((k.s1 & 4294967288u) << 4) ^ b;
  b = ((k.s2 << 3) ^ k.s2) >> 11;
  k.s2 = ((k.s2 & 4294967280u) << 17) ^ b;
  return k.s0 ^ k.s1 ^ k.s2;
}

// tifunc.py:136-147 with low = 1, high = clen: x % clen + 1
__device__ __forceinline__ uint32_t lfsr88_inc(Lfsr88& k, FastMod fm) { return fastmod(lfsr88_next(k), fm) + 1u; }

// tifunc.py:136-147 with low = 0, high = clen - 1: x % clen
__device__ __forceinline__ uint32_t lfsr88_start(Lfsr88& k, FastMod fm) { return fastmod(lfsr88_next(k), fm); }

// tifunc.py:171-180: float32(x) * float32(2.3283064365386963e-10)
__device__ __forceinline__ float lfsr88_rand(Lfsr88& k) {
  return __fmul_rn(__uint2float_rn(lfsr88_next(k)), 2.3283064365386963e-10f);
}

// tifunc.py:156-168: r * (high - low) + low, each step rounded in float32
__device__ __forceinline__ float lfsr88_uniform(Lfsr88& k, float lo, float hi) {
  const float r = lfsr88_rand(k);
  return __fadd_rn(__fmul_rn(r, __fsub_rn(hi, lo)), lo);
}

// tifunc.py:89-133: Box-Muller (sin branch) with u1 clamped to 1e-10
__device__ __forceinline__ float lfsr88_normal(Lfsr88& k, float mu, float sigma) {
  float u1 = lfsr88_rand(k);
  const float u2 = lfsr88_rand(k);
  if (u1 < 1e-10f) u1 = 1e-10f;
  const float mag = sqrtf(__fmul_rn(-2.0f, logf(u1)));
  const float z = __fmul_rn(mag, sinf(__fmul_rn(6.28318530717958648f, u2)));
  return __fadd_rn(mu, __fmul_rn(sigma, z));
}

}  // namespace bp
