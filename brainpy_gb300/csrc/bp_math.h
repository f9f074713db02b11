/*
 * bp_math.h -- deterministic float32 helpers shared by host and device code.
 *
 * Every operation below is written as an explicit, individually rounded IEEE
 * float32 operation (no contraction into FMA unless spelled out), so that the
 * same source produces bit-identical results on the GPU and on the CPU.
 *
 * bp_expf: exp(x) by Cody-Waite argument reduction (x = n ln2 + r with ln2 split
 * into a 16-bit-exact high part and a low correction, |r| <= ln2/2) followed by
 * the degree-7 Taylor polynomial of e^r evaluated by Horner's rule with fused
 * multiply-adds, and an exact scaling by 2^n.  Truncation error of the
 * polynomial is below r^8/8! < 6e-9, i.e. below 0.15 ulp on [0.5, 2).
 *
 * bp_exprel: (exp(x) - 1) / x with the small-|x| series branch, as in
 * brainpy/_src/math/others.py:94-103 (threshold 1e-5 for float32, :120-124).
 */
#ifndef BP_MATH_H_
#define BP_MATH_H_

#include <stdint.h>

#if defined(__CUDACC__)
#define BP_HD __host__ __device__ __forceinline__
#else
#define BP_HD static inline
#include <math.h>
#include <string.h>
#endif

#if defined(__CUDA_ARCH__)
#define BP_FADD(a, b) __fadd_rn((a), (b))
#define BP_FSUB(a, b) __fsub_rn((a), (b))
#define BP_FMUL(a, b) __fmul_rn((a), (b))
#define BP_FDIV(a, b) __fdiv_rn((a), (b))
#define BP_FFMA(a, b, c) __fmaf_rn((a), (b), (c))
#define BP_RINT(a) rintf(a)
#else
/* host code is compiled with -ffp-contract=off so these stay separate roundings */
#define BP_FADD(a, b) ((float)((float)(a) + (float)(b)))
#define BP_FSUB(a, b) ((float)((float)(a) - (float)(b)))
#define BP_FMUL(a, b) ((float)((float)(a) * (float)(b)))
#define BP_FDIV(a, b) ((float)((float)(a) / (float)(b)))
#define BP_FFMA(a, b, c) fmaf((a), (b), (c))
#define BP_RINT(a) rintf(a)
#endif

BP_HD float bp_bits_to_float(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

/* 2^n for n in [-126, 127], exact. */
BP_HD float bp_pow2i(int n) { return bp_bits_to_float((uint32_t)(n + 127) << 23); }

BP_HD float bp_expf(float x) {
  if (!(x == x)) return x;                       /* NaN */
  if (x > 88.72f) return bp_bits_to_float(0x7f800000u);
  if (x < -103.98f) return 0.0f;
  const float log2e = 1.44269504088896341f;
  const float ln2_hi = 0.693145751953125f;       /* ln 2 rounded to 16 significant bits */
  const float ln2_lo = 1.42860682030941723e-6f;  /* ln 2 - ln2_hi */
  float n = BP_RINT(BP_FMUL(x, log2e));
  float r = BP_FFMA(-n, ln2_hi, x);
  r = BP_FFMA(-n, ln2_lo, r);
  /* Taylor coefficients 1/k!, k = 7..0 */
  float p = 1.98412698412698413e-4f;             /* 1/5040 */
  p = BP_FFMA(p, r, 1.38888888888888889e-3f);    /* 1/720 */
  p = BP_FFMA(p, r, 8.33333333333333333e-3f);    /* 1/120 */
  p = BP_FFMA(p, r, 4.16666666666666667e-2f);    /* 1/24 */
  p = BP_FFMA(p, r, 1.66666666666666667e-1f);    /* 1/6 */
  p = BP_FFMA(p, r, 0.5f);
  p = BP_FFMA(p, r, 1.0f);
  p = BP_FFMA(p, r, 1.0f);
  int ni = (int)n;
  if (ni > 127) return BP_FMUL(BP_FMUL(p, bp_pow2i(ni - 1)), 2.0f);
  if (ni >= -126) return BP_FMUL(p, bp_pow2i(ni));
  /* subnormal result: scale in two exact steps */
  return BP_FMUL(BP_FMUL(p, bp_pow2i(ni + 64)), bp_pow2i(-64));
}

/* brainpy/_src/math/others.py:94-103:
 *   where(|x| <= thr, 1 + x/2 + x*x/6, (exp(x) - 1) / x),  thr = 1e-5 for float32. */
BP_HD float bp_exprel(float x) {
  float ax = x < 0.0f ? -x : x;
  if (ax <= 1e-5f) {
    return BP_FADD(BP_FADD(1.0f, BP_FDIV(x, 2.0f)), BP_FDIV(BP_FMUL(x, x), 6.0f));
  }
  return BP_FDIV(BP_FSUB(bp_expf(x), 1.0f), x);
}

#endif /* BP_MATH_H_ */
