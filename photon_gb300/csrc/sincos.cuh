// Single-precision sine and cosine that are correctly rounded except on a
// vanishing fraction of arguments, for the path tracer's sampling.
//
// Why: the reference runs on the host C library, whose sinf / cosf are
// within half an ulp plus a little of the exact value; CUDA's sinf / cosf
// differ from them on 16-21% of the sampling's arguments (at most one ulp),
// and in textured scenes with deep paths those ulps move enough paths by more
// than the per-sample tolerance.  These functions differ from the host's
// only where the host's are not correctly rounded (about 1.3% of the
// arguments), which brings the renders to the agreement of two correct
// libms.
//
// How (standard methods; every operation an IEEE float add, multiply or
// fused multiply-add, so host and device builds give identical bits):
//   * Cody-Waite reduction x = k pi/2 + r with pi/2 split into an 18-bit
//     head (k * head is exact for |k| <= 8) and two 24-bit tails, the
//     remainder r kept as an unevaluated sum of two floats (float-float,
//     Dekker's error-free sum and product; the product through fmaf);
//   * Taylor series of sin and cos on |r| <= pi/4 (the coefficients are
//     1 / n!), the leading coefficients and every product that carries them
//     in float-float, the small tail terms in plain float;
//   * one final float rounding of hi + lo, whose error before rounding is
//     below 2^-40 relative.
// Arguments with |x| > 8 (no call site passes one) and non-finite ones
// return CUDA's (or the host library's) sinf / cosf.
#pragma once

#include <cuda_runtime.h>
#ifndef __CUDA_ARCH__
#include <cmath>
#endif

#ifndef PHC_HD
#define PHC_HD __host__ __device__ __forceinline__
#endif

namespace phc {

struct FFloat {
  float hi, lo;
};

// a + b exactly as hi + lo (Knuth's two-sum)
PHC_HD FFloat ff_two_sum(float a, float b)
{
  const float s = a + b;
  const float bb = s - a;
  return FFloat{s, (a - (s - bb)) + (b - bb)};
}
// a + b exactly as hi + lo when |a| >= |b| (Dekker's fast two-sum)
PHC_HD FFloat ff_fast_sum(float a, float b)
{
  const float s = a + b;
  return FFloat{s, b - (s - a)};
}
PHC_HD FFloat ff_mul(FFloat a, FFloat b)
{
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return ff_fast_sum(p, e);
}
PHC_HD FFloat ff_add(FFloat a, FFloat b)
{
  const FFloat s = ff_two_sum(a.hi, b.hi);
  return ff_fast_sum(s.hi, (s.lo + a.lo) + b.lo);
}
PHC_HD FFloat ff(float hi, float lo = 0.f) { return FFloat{hi, lo}; }

// x = k pi/2 + (r.hi + r.lo), |r| <= pi/4 (a little more at the quadrant
// boundaries), for |x| <= 8; returns k.
PHC_HD int ff_reduce_pio2(float x, FFloat &r)
{
  const float C1 = 0x1.921f8p+0f;     // pi/2, first 18 bits
  const float C2 = 0x1.aa2216p-19f;   // next 24 bits
  const float C3 = 0x1.184698p-44f;   // next 24 bits
  const float k = rintf(x * 0x1.45f306p-1f); // x * 2/pi
  const float r1 = x - k * C1;              // exact: k * C1 has <= 22 bits, and x is near k * C1
  const float p2 = k * C2;
  const float e2 = fmaf(k, C2, -p2);        // k * C2 = p2 + e2 exactly
  const FFloat s = ff_two_sum(r1, -p2);
  r = ff_fast_sum(s.hi, (s.lo - e2) - k * C3);
  return int(k);
}

// sin(r) and cos(r) as float-float for |r| <= pi/4 + a little: Taylor
// series through r^13 / 13! and r^14 / 14! (truncation below 2^-41).
PHC_HD void ff_sincos_poly(FFloat r, FFloat &s, FFloat &c)
{
  const FFloat z = ff_mul(r, r);
  const float zh = z.hi;
  // sin r = r + r z (-1/3! + z (1/5! + z (-1/7! + z (1/9! + z (-1/11! + z / 13!)))))
  const float qs = -0x1.a01a02p-13f + zh * (0x1.71de3ap-19f + zh * (-0x1.ae6456p-26f + zh * 0x1.612462p-33f));
  const FFloat us = ff_add(ff(0x1.111112p-7f, -0x1.dddddep-32f), ff_mul(z, ff(qs)));
  const FFloat ps = ff_add(ff(-0x1.555556p-3f, 0x1.555556p-28f), ff_mul(z, us));
  s = ff_add(r, ff_mul(ff_mul(r, z), ps));
  // cos r = 1 + z (-1/2 + z (1/4! + z (-1/6! + z (1/8! + z (-1/10! + z (1/12! - z / 14!))))))
  const float qc = -0x1.6c16c2p-10f +
      zh * (0x1.a01a02p-16f + zh * (-0x1.27e4fcp-22f + zh * (0x1.1eed8ep-29f + zh * -0x1.93974ap-37f)));
  const FFloat uc = ff_add(ff(0x1.555556p-5f, -0x1.555556p-30f), ff_mul(z, ff(qc)));
  const FFloat rc = ff_add(ff(-0.5f), ff_mul(z, uc));
  c = ff_add(ff(1.f), ff_mul(z, rc));
}

PHC_HD float acc_sin(float x)
{
  if (!(fabsf(x) <= 8.f))
    return sinf(x);
  if (x == 0.f)
    return x; // sin(+-0) = +-0
  FFloat r, s, c;
  const int k = ff_reduce_pio2(x, r);
  ff_sincos_poly(r, s, c);
  switch (k & 3) {
  case 0: return s.hi + s.lo;
  case 1: return c.hi + c.lo;
  case 2: return -(s.hi + s.lo);
  default: return -(c.hi + c.lo);
  }
}

PHC_HD float acc_cos(float x)
{
  if (!(fabsf(x) <= 8.f))
    return cosf(x);
  FFloat r, s, c;
  const int k = ff_reduce_pio2(x, r);
  ff_sincos_poly(r, s, c);
  switch (k & 3) {
  case 0: return c.hi + c.lo;
  case 1: return -(s.hi + s.lo);
  case 2: return -(c.hi + c.lo);
  default: return s.hi + s.lo;
  }
}

} // namespace phc
