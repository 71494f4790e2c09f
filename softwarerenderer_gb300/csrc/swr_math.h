// Exact binary32 arithmetic shared by the CUDA kernels and the CPU oracle port.
//
// The reference computes every interpolant by incremental stepping
// (PixelData::stepX/stepY, PixelData.h:61-125; EdgeData::stepX/stepY,
// EdgeData.h:37-80), i.e. v <- fl(v + a) repeated k times.  A GPU thread that owns
// one pixel must reproduce the value the reference reaches after k steps without
// replaying the steps of every pixel to its left.  swr_fold() does that exactly:
// inside one binade the rounded increment of v + a is a constant integer number of
// ulps (after at most one parity step when a sits exactly on a half ulp), so a run
// of steps collapses into one integer multiply-add; binade changes, zeros,
// subnormals and non-finite values fall back to single IEEE steps.
//
// Every helper here is correctly rounded IEEE-754 binary32 (round to nearest even,
// subnormals preserved) on both sides: the device uses the _rn intrinsics (never
// contracted into FMA); the host relies on -ffp-contract=off and SSE/NEON scalar
// float arithmetic.
#pragma once
#include <math.h>
#include <stdint.h>
#ifndef __CUDACC__
#include <string.h>
#endif
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __CUDACC__
#define SWR_HD __host__ __device__ __forceinline__
#elif defined(__cplusplus)
#define SWR_HD inline
#else
#define SWR_HD static inline
#endif

SWR_HD uint32_t swr_f2u(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
#endif
}

SWR_HD float swr_u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  memcpy(&f, &u, 4);
  return f;
#endif
}

SWR_HD float swr_add(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}

SWR_HD float swr_sub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}

SWR_HD float swr_mul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}

SWR_HD float swr_div(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdiv_rn(a, b);
#else
  return a / b;
#endif
}

SWR_HD float swr_sqrt(float a) {
#ifdef __CUDA_ARCH__
  return __fsqrt_rn(a);
#else
  return __builtin_sqrtf(a);
#endif
}

// C/C++ (int) conversion of a float: truncation toward zero.  Values outside the
// int range are undefined behaviour in C++; callers only pass in-range values.
SWR_HD int swr_trunc_int(float f) {
#ifdef __CUDA_ARCH__
  return __float2int_rz(f);
#else
  return (int)f;
#endif
}

// std::min / std::max as used by the reference: min(a,b) = (b < a) ? b : a,
// max(a,b) = (a < b) ? b : a.  (Order matters for signed zeros and NaN.)
SWR_HD float swr_minf(float a, float b) { return (b < a) ? b : a; }
SWR_HD float swr_maxf(float a, float b) { return (a < b) ? b : a; }
SWR_HD int swr_mini(int a, int b) { return (b < a) ? b : a; }
SWR_HD int swr_maxi(int a, int b) { return (a < b) ? b : a; }

// Plane evaluation a*x + b*y + c in the reference's association order
// (EdgeEquation::evaluate, EdgeEquation.h:46-49; ParameterEquation::evaluate,
// ParameterEquation.h:51-54): (a*x + b*y) + c, three roundings, no FMA.
SWR_HD float swr_eval(float a, float b, float c, float x, float y) {
  return swr_add(swr_add(swr_mul(a, x), swr_mul(b, y)), c);
}

// Value of v after k repetitions of v = fl(v + a).  k <= 0 returns v unchanged.
SWR_HD float swr_fold(float v, float a, int k) {
  while (k > 0) {
    if (k <= 6) {
      for (; k > 0; --k) v = swr_add(v, a);
      return v;
    }
    const uint32_t vb = swr_f2u(v), ab = swr_f2u(a);
    const uint32_t ve = (vb >> 23) & 0xffu, ae = (ab >> 23) & 0xffu;
    // a == +-0, or a / v not finite: the first step reaches a fixed point
    // (x + 0 = x except -0 + +0 = +0; inf and NaN absorb every later step).
    if ((ab << 1) == 0u || ae == 0xffu || ve == 0xffu) return swr_add(v, a);
    // v zero or subnormal: take plain steps until v is normal.
    if (ve == 0u) {
      v = swr_add(v, a);
      --k;
      continue;
    }
    // v = s * N * u with u = 2^(ve-150), N in [2^23, 2^24);
    // |a| = ma * 2^(ea-150)  ->  |a|/u = ma / 2^shift.
    const int32_t N = (int32_t)((vb & 0x7fffffu) | 0x800000u);
    const uint32_t ma = ae ? ((ab & 0x7fffffu) | 0x800000u) : (ab & 0x7fffffu);
    const int ea = ae ? (int)ae : 1;
    const int shift = (int)ve - ea;
    const bool grow = ((vb ^ ab) >> 31) == 0u;  // a has the sign of v
    if (shift <= 0) {  // |a| is at least half of |v|: the binade changes fast
      v = swr_add(v, a);
      --k;
      continue;
    }
    int32_t qm, Dm, nz;
    if (shift >= 31) {
      // |a| < u / 2^7: each step rounds back to v while the exact sum stays in
      // this binade; only shrinking from exactly 2^E can reach the finer grid below.
      if (grow || N > 0x800000) return v;
      v = swr_add(v, a);
      --k;
      continue;
    }
    {
      const uint32_t rem = ma & ((1u << shift) - 1u);
      const uint32_t half = 1u << (shift - 1);
      qm = (int32_t)(ma >> shift);
      nz = rem != 0u;
      const bool tie = rem == half;
      Dm = qm + ((rem > half || (tie && ((N + qm) & 1))) ? 1 : 0);
      if (tie && (Dm & 1)) {  // the rounding direction alternates once
        v = swr_add(v, a);
        --k;
        continue;
      }
    }
    // Largest run of steps whose exact sums stay inside [2^23, 2^24] ulps.
    const int32_t slack = grow ? (0x1000000 - N - qm - nz) : (N - qm - nz - 0x800000);
    if (slack < 0) {
      v = swr_add(v, a);
      --k;
      continue;
    }
    if (Dm == 0) return v;
    // m = min(k, slack / Dm + 1); the whole run usually fits, which needs no division
    int32_t m = (int64_t)(k - 1) * Dm <= (int64_t)slack ? k : slack / Dm + 1;
    const int32_t N2 = grow ? N + m * Dm : N - m * Dm;
    // N2 == 2^24 carries into the exponent (and into +-inf from the top binade).
    v = swr_u2f((vb & 0x80000000u) + ((ve << 23) + (uint32_t)(N2 - 0x800000)));
    k -= m;
  }
  return v;
}

// ---------------------------------------------------------------------------
// Helpers of the texture sampler (exact on both sides: fmod, floor and ceil are exact
// operations; log2 is computed here from binary64 +, -, *, / only).

SWR_HD float swr_fmodf(float a, float b) { return fmodf(a, b); }
SWR_HD float swr_floorf(float a) { return floorf(a); }
SWR_HD float swr_ceilf(float a) { return ceilf(a); }
SWR_HD bool swr_isnan(float a) { return a != a; }

SWR_HD double swr_dadd(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
SWR_HD double swr_dsub(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
SWR_HD double swr_dmul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
SWR_HD double swr_ddiv(double a, double b) {
#ifdef __CUDA_ARCH__
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}

// log2(x) rounded to binary32, identical on every IEEE-754 machine.  x = m * 2^e with m in
// [sqrt(1/2), sqrt(2)); ln m = 2 atanh(s) = 2 (s + s^3/3 + s^5/5 + ...), s = (m - 1) / (m + 1),
// |s| < 0.1716 (the series ln((1 + s) / (1 - s)), Abramowitz & Stegun 4.1.28), summed in
// binary64 to s^23 (truncation below 1e-19 relative), scaled by 1/ln 2 and rounded once.
// Special values: log2(+0) = -inf, log2(+inf) = +inf, negative or NaN input -> NaN.
SWR_HD float swr_log2(float x) {
  if (!(x > 0.0f)) return x == 0.0f ? -INFINITY : NAN;
  uint32_t b = swr_f2u(x);
  if (b >= 0x7f800000u) return x;  // +inf
  int e = 0;
  if (b < 0x00800000u) {  // subnormal: scale by 2^32 into the normal range
    b = swr_f2u(swr_mul(x, 4294967296.0f));
    e = -32;
  }
  e += (int)(b >> 23) - 127;
  float m = swr_u2f((b & 0x007fffffu) | 0x3f800000u);  // [1, 2)
  if (m > 1.41421353816986083984375f) {  // sqrt(2) rounded down to binary32
    m = swr_mul(m, 0.5f);
    e += 1;
  }
  const double md = (double)m;
  const double s = swr_ddiv(swr_dsub(md, 1.0), swr_dadd(md, 1.0));
  const double s2 = swr_dmul(s, s);
  double poly = 1.0 / 23.0;
  poly = swr_dadd(swr_dmul(poly, s2), 1.0 / 21.0);
  poly = swr_dadd(swr_dmul(poly, s2), 1.0 / 19.0);
  poly = swr_dadd(swr_dmul(poly, s2), 1.0 / 17.0);
  poly = swr_dadd(swr_dmul(poly, s2), 1.0 / 15.0);
  poly = swr_dadd(swr_dmul(poly, s2), 1.0 / 13.0);
  poly = swr_dadd(swr_dmul(poly, s2), 1.0 / 11.0);
  poly = swr_dadd(swr_dmul(poly, s2), 1.0 / 9.0);
  poly = swr_dadd(swr_dmul(poly, s2), 1.0 / 7.0);
  poly = swr_dadd(swr_dmul(poly, s2), 1.0 / 5.0);
  poly = swr_dadd(swr_dmul(poly, s2), 1.0 / 3.0);
  poly = swr_dadd(swr_dmul(poly, s2), 1.0);
  const double ln_m = swr_dmul(2.0, swr_dmul(s, poly));
  const double inv_ln2 = 1.4426950408889634;  // 1 / ln 2 rounded to binary64
  return (float)swr_dadd((double)e, swr_dmul(ln_m, inv_ln2));
}
