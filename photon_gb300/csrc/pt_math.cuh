// Device math for the path-tracing kernels.
//
// The float expressions keep the association of Photon's math.h / sampling.h /
// rng.h (include/photon/pt/) so that, with the translation units compiled with
// --fmad=false (no contraction of a*b+c into one rounding), every IEEE add,
// multiply, divide and square root rounds exactly as the reference's host and
// Kokkos builds do.  Only the transcendental functions may differ from the
// host's C library (by an ulp, on the arguments where one of the two is not
// correctly rounded), which is what the per-sample parity tolerance covers.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#ifndef PHC_HD
#define PHC_HD __host__ __device__ __forceinline__
#endif

#ifndef __CUDA_ARCH__
#include <cmath>
#include <cstring>
#endif

#include "sincos.cuh"

namespace phc {

using u32 = uint32_t;
using i32 = int32_t;

// The transcendental functions of the path-tracing code, in one place.
// Sine and cosine are the float-float ones of sincos.cuh, correctly rounded
// but for a vanishing fraction of arguments, in host and device builds
// alike: the reference calls the host C library's sinf / cosf, which are
// correctly rounded on all but about 1% of the arguments, while CUDA's
// differ from them on 16-21%, enough to move deep paths of textured scenes
// past the per-sample tolerance.  The other functions are CUDA's on the
// device (the host library's in host builds): their ulp differences move no
// path measurably (tracking distances, environment directions).
PHC_HD float m_sin(float x) { return acc_sin(x); }
PHC_HD float m_cos(float x) { return acc_cos(x); }
PHC_HD void m_sincos(float x, float &s, float &c) { acc_sincos(x, s, c); }
PHC_HD float m_log(float x) { return logf(x); }
PHC_HD float m_acos(float x) { return acosf(x); }
PHC_HD float m_atan2(float y, float x) { return atan2f(y, x); }
PHC_HD float m_pow(float x, float y) { return powf(x, y); }
PHC_HD float m_tan(float x) { return tanf(x); }

// Bit casts and bit scans that compile for the device and, for host-side
// tests of the same traversal code, for the host.
PHC_HD uint32_t f2u(float f)
{
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
PHC_HD float u2f(uint32_t u)
{
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}
PHC_HD uint32_t ffs32(uint32_t x) // 1 + index of the lowest set bit, 0 for none
{
#ifdef __CUDA_ARCH__
  return uint32_t(__ffs(int(x)));
#else
  return uint32_t(__builtin_ffs(int(x)));
#endif
}
PHC_HD uint32_t popc32(uint32_t x)
{
#ifdef __CUDA_ARCH__
  return uint32_t(__popc(x));
#else
  return uint32_t(__builtin_popcount(x));
#endif
}

struct V3 {
  float x, y, z;
};

PHC_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
PHC_HD V3 v3(float4 a) { return V3{a.x, a.y, a.z}; }
PHC_HD V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
PHC_HD V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
PHC_HD V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
PHC_HD V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
PHC_HD V3 operator*(float s, V3 a) { return {a.x * s, a.y * s, a.z * s}; }
PHC_HD V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
PHC_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
PHC_HD V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
PHC_HD float length(V3 v) { return sqrtf(dot(v, v)); }
PHC_HD V3 normalize(V3 v)
{
  const float len = length(v);
  return len > 0.f ? v * (1.f / len) : V3{0.f, 0.f, 0.f};
}
PHC_HD V3 lerp(V3 a, V3 b, float t) { return a + (b - a) * t; }
PHC_HD V3 reflect(V3 i, V3 n) { return i - (2.f * dot(i, n)) * n; }
PHC_HD V3 refract(V3 i, V3 n, float eta)
{
  const float cosi = -dot(i, n);
  const float k = 1.f - eta * eta * (1.f - cosi * cosi);
  if (k < 0.f)
    return V3{0.f, 0.f, 0.f};
  return eta * i + (eta * cosi - sqrtf(k)) * n;
}
PHC_HD float4 f4(V3 v, float w) { return make_float4(v.x, v.y, v.z, w); }
PHC_HD float4 add4(float4 a, float4 b) { return make_float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
PHC_HD float4 mul4(float4 a, float s) { return make_float4(a.x * s, a.y * s, a.z * s, a.w * s); }
// Row-major 4x4 matrix times column vector.
PHC_HD float4 mat4_mul(const float *m, float4 v)
{
  return make_float4(m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * v.w,
      m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7] * v.w, m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11] * v.w,
      m[12] * v.x + m[13] * v.y + m[14] * v.z + m[15] * v.w);
}
PHC_HD float lum(V3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
PHC_HD float saturate(float x) { return fminf(1.f, fmaxf(0.f, x)); }
PHC_HD float clamp01(float x) { return x < 0.f ? 0.f : (x > 1.f ? 1.f : x); }
PHC_HD bool finite3(V3 c) { return c.x == c.x && c.y == c.y && c.z == c.z; }

constexpr float PI = 3.14159265358979323846f;
constexpr float INV_PI = 1.f / PI;
constexpr float TWO_PI = 2.f * PI;
constexpr float INV_TWO_PI = 1.f / TWO_PI;

// xorshift32 stream (rng.h:9-30) seeded per (pixel, sample, dimension)
// through the integer hash of pathtracer.cpp:20-34.
struct Rng {
  u32 s;
  PHC_HD explicit Rng(u32 seed) : s(seed ? seed : 1u) {}
  PHC_HD float next()
  {
    u32 x = s;
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    s = x;
    return (x >> 8) * (1.0f / 16777216.0f);
  }
};
PHC_HD u32 hash_u32(u32 x)
{
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}
PHC_HD Rng path_rng(u32 pixel, u32 sample, u32 dim)
{
  return Rng(hash_u32(pixel + hash_u32(sample + hash_u32(dim + 0x9e3779b9U))));
}

// sampling.h helpers
PHC_HD float power_heuristic(float f, float g)
{
  const float f2 = f * f, g2 = g * g;
  return (f2 + g2) > 0.f ? f2 / (f2 + g2) : 0.f;
}
PHC_HD void onb(V3 n, V3 &t, V3 &b)
{
  if (n.z < -0.9999999f) {
    t = V3{0.f, -1.f, 0.f};
    b = V3{-1.f, 0.f, 0.f};
    return;
  }
  const float a = 1.f / (1.f + n.z);
  const float c = -n.x * n.y * a;
  t = normalize(V3{1.f - n.x * n.x * a, c, -n.x});
  b = normalize(V3{c, 1.f - n.y * n.y * a, -n.y});
}
PHC_HD void concentric_disk(Rng &rng, float &dx, float &dy)
{
  const float u = 2.f * rng.next() - 1.f;
  const float v = 2.f * rng.next() - 1.f;
  if (u == 0.f && v == 0.f) {
    dx = dy = 0.f;
    return;
  }
  float r, th;
  if (fabsf(u) > fabsf(v)) {
    r = fabsf(u);
    th = (PI / 4.f) * (v / u);
  } else {
    r = fabsf(v);
    th = (PI / 2.f) - (PI / 4.f) * (u / v);
  }
  float sth, cth;
  m_sincos(th, sth, cth);
  dx = r * cth;
  dy = r * sth;
}
PHC_HD V3 cosine_hemisphere(V3 n, Rng &rng)
{
  V3 t, b;
  onb(n, t, b);
  float dx, dy;
  concentric_disk(rng, dx, dy);
  const float z = sqrtf(fmaxf(0.f, 1.f - dx * dx - dy * dy));
  return normalize(dx * t + dy * b + z * n);
}
PHC_HD V3 uniform_sphere(Rng &rng)
{
  const float z = 1.f - 2.f * rng.next();
  const float r = sqrtf(fmaxf(0.f, 1.f - z * z));
  const float phi = TWO_PI * rng.next();
  float sp, cp;
  m_sincos(phi, sp, cp);
  return V3{r * cp, r * sp, z};
}

} // namespace phc
