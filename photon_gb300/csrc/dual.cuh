// Forward-mode dual numbers for the adjoint: a value and its partial
// derivatives with respect to N parameters.  Arithmetic follows the usual
// rules; min / max / comparisons act on the value (the branch taken is the
// primal's, the derivative of the taken branch is propagated).
#pragma once

#include "pt_math.cuh"

namespace phc {

template <int N> struct Dual {
  float v;
  float d[N];
};

template <int N> __device__ __forceinline__ Dual<N> dconst(float v)
{
  Dual<N> r;
  r.v = v;
#pragma unroll
  for (int i = 0; i < N; ++i)
    r.d[i] = 0.f;
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> dvar(float v, int k)
{
  Dual<N> r = dconst<N>(v);
  r.d[k] = 1.f;
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator+(const Dual<N> &a, const Dual<N> &b)
{
  Dual<N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i)
    r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator-(const Dual<N> &a, const Dual<N> &b)
{
  Dual<N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i)
    r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator*(const Dual<N> &a, const Dual<N> &b)
{
  Dual<N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i)
    r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator/(const Dual<N> &a, const Dual<N> &b)
{
  Dual<N> r;
  r.v = a.v / b.v;
  const float inv = 1.f / b.v;
#pragma unroll
  for (int i = 0; i < N; ++i)
    r.d[i] = (a.d[i] - r.v * b.d[i]) * inv;
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator+(const Dual<N> &a, float b)
{
  Dual<N> r = a;
  r.v = a.v + b;
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator+(float b, const Dual<N> &a) { return a + b; }
template <int N> __device__ __forceinline__ Dual<N> operator-(const Dual<N> &a, float b)
{
  Dual<N> r = a;
  r.v = a.v - b;
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator-(float b, const Dual<N> &a)
{
  Dual<N> r;
  r.v = b - a.v;
#pragma unroll
  for (int i = 0; i < N; ++i)
    r.d[i] = -a.d[i];
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator*(const Dual<N> &a, float b)
{
  Dual<N> r;
  r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < N; ++i)
    r.d[i] = a.d[i] * b;
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator*(float b, const Dual<N> &a) { return a * b; }
template <int N> __device__ __forceinline__ Dual<N> operator/(const Dual<N> &a, float b)
{
  Dual<N> r;
  r.v = a.v / b;
#pragma unroll
  for (int i = 0; i < N; ++i)
    r.d[i] = a.d[i] / b;
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> operator/(float a, const Dual<N> &b)
{
  return dconst<N>(a) / b;
}
template <int N> __device__ __forceinline__ Dual<N> dsqrt(const Dual<N> &a)
{
  Dual<N> r;
  r.v = sqrtf(a.v);
  const float k = r.v > 0.f ? 0.5f / r.v : 0.f;
#pragma unroll
  for (int i = 0; i < N; ++i)
    r.d[i] = a.d[i] * k;
  return r;
}
template <int N> __device__ __forceinline__ Dual<N> dmax(const Dual<N> &a, float b)
{
  return a.v >= b || a.v != a.v ? a : dconst<N>(b);
}
template <int N> __device__ __forceinline__ Dual<N> dmin(const Dual<N> &a, float b)
{
  return a.v <= b || a.v != a.v ? a : dconst<N>(b);
}
template <int N> __device__ __forceinline__ Dual<N> dsat(const Dual<N> &a) { return dmin(dmax(a, 0.f), 1.f); }

// float overloads so one template body serves both types
__device__ __forceinline__ float dsqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ float dmax(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ float dmin(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ float dsat(float a) { return fminf(1.f, fmaxf(0.f, a)); }
__device__ __forceinline__ float val(float a) { return a; }
template <int N> __device__ __forceinline__ float val(const Dual<N> &a) { return a.v; }

} // namespace phc
