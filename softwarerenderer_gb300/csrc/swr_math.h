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
    int32_t m = slack / Dm + 1;
    if (m > k) m = k;
    const int32_t N2 = grow ? N + m * Dm : N - m * Dm;
    // N2 == 2^24 carries into the exponent (and into +-inf from the top binade).
    v = swr_u2f((vb & 0x80000000u) + ((ve << 23) + (uint32_t)(N2 - 0x800000)));
    k -= m;
  }
  return v;
}
