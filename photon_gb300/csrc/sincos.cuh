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
//     1 / n!), the terms above 2^-9 of the result in float-float, the small
//     tail terms in plain float;
//   * one final float rounding, whose error before rounding is below 2^-35
//     relative.
// Call sites that need both use acc_sincos (one reduction, both series).
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

// sin(r) and cos(r) for |r| <= pi/4 + a little (r = r.hi + r.lo), rounded
// once to float: Taylor series through r^13 / 13! and r^14 / 14!
// (truncation below 2^-41).  The terms above 2^-9 of the result (r, r^3/3!,
// r^5/5! for the sine; 1, z/2, z^2/4! for the cosine, z = r^2) are formed as
// float-float with exact products (fmaf); the rest in float, whose error is
// then below 2^-35 of the result.
PHC_HD void ff_sincos_poly(FFloat r, float &sn, float &cs)
{
  // z = r^2 = zh + zl
  const float zh = r.hi * r.hi;
  const float zl = fmaf(r.hi, r.hi, -zh) + 2.f * r.hi * r.lo;
  // sine: r^3 = p + pe, r^5 = q + qe, -r^3/3! = t + te, r^5/5! = u + ue
  const float p = r.hi * zh;
  const float pe = fmaf(r.hi, zh, -p) + fmaf(r.hi, zl, r.lo * zh);
  const float q = p * zh;
  const float qe = fmaf(p, zh, -q) + fmaf(p, zl, pe * zh);
  const float t = p * -0x1.555556p-3f;
  const float te = fmaf(p, -0x1.555556p-3f, -t) + fmaf(p, 0x1.555556p-28f, pe * -0x1.555556p-3f);
  const float u = q * 0x1.111112p-7f;
  const float ue = fmaf(q, 0x1.111112p-7f, -u) + fmaf(q, -0x1.dddddep-32f, qe * 0x1.111112p-7f);
  // r^7 (-1/7! + z (1/9! - z (1/11! - z / 13!)))
  const float st = q * zh * fmaf(zh, fmaf(zh, fmaf(zh, 0x1.612462p-33f, -0x1.ae6456p-26f), 0x1.71de3ap-19f),
      -0x1.a01a02p-13f);
  const FFloat sa = ff_two_sum(r.hi, t);
  const FFloat sb = ff_fast_sum(sa.hi, u);
  sn = sb.hi + (((sa.lo + sb.lo) + (r.lo + te)) + (ue + st));
  // cosine: -z/2 = -(zh + zl)/2 exactly, z^2 = w + we, z^2/4! = v + ve
  const float w = zh * zh;
  const float we = fmaf(zh, zh, -w) + 2.f * zh * zl;
  const float v = w * 0x1.555556p-5f;
  const float ve = fmaf(w, 0x1.555556p-5f, -v) + fmaf(w, -0x1.555556p-30f, we * 0x1.555556p-5f);
  // z^3 (-1/6! + z (1/8! - z (1/10! - z (1/12! - z / 14!))))
  const float ct = w * zh *
      fmaf(zh, fmaf(zh, fmaf(zh, fmaf(zh, -0x1.93974ap-37f, 0x1.1eed8ep-29f), -0x1.27e4fcp-22f), 0x1.a01a02p-16f),
          -0x1.6c16c2p-10f);
  const FFloat ca = ff_two_sum(1.f, -0.5f * zh);
  const FFloat cb = ff_fast_sum(ca.hi, v);
  cs = cb.hi + (((ca.lo + cb.lo) + (-0.5f * zl + ve)) + ct);
}

// sin(x) and cos(x) together (one reduction, both series).
PHC_HD void acc_sincos(float x, float &sn, float &cs)
{
  if (!(fabsf(x) <= 8.f)) {
    sn = sinf(x);
    cs = cosf(x);
    return;
  }
  FFloat r;
  const int k = ff_reduce_pio2(x, r);
  float s, c;
  ff_sincos_poly(r, s, c);
  switch (k & 3) {
  case 0: sn = s; cs = c; break;
  case 1: sn = c; cs = -s; break;
  case 2: sn = -s; cs = -c; break;
  default: sn = -c; cs = s; break;
  }
  if (x == 0.f)
    sn = x; // sin(+-0) = +-0
}

PHC_HD float acc_sin(float x)
{
  float s, c;
  acc_sincos(x, s, c);
  return s;
}

PHC_HD float acc_cos(float x)
{
  float s, c;
  acc_sincos(x, s, c);
  return c;
}

} // namespace phc
