// The CDF searches of light and environment sampling, with optional guide
// tables (DevScene::emissive_guide / env_mguide / env_cguide).
//
// cdf_search_le: the largest i in [0, n - 1] with cdf[i] <= u, found by the
//   bisection of EnvironmentMap::sample_direction
//   (include/photon/pt/environment_map.h:62-104);
// cdf_search_gt: the first i in [0, n - 2] with cdf[i] > u, else n - 1, the
//   bisection of the emissive-triangle pick (src/photon/pt/pathtracer.cpp:
//   296-306).
// A guide of G = 2^bits + 1 entries holds the search's result for u = k / G
// at entry k (k / G is exact in float) and the largest result at entry G.
// Both results are non-decreasing in u over a non-decreasing CDF, so for
// k / G <= u < (k + 1) / G the result lies in [guide[k], guide[k + 1]] and
// bisecting only that range returns the same index as bisecting the whole
// table, in a few probes instead of log2(n) dependent loads.  The scene build
// writes guides only for non-decreasing CDFs.  __host__ __device__ so the
// CPU tests run the same code against the plain bisection.
#pragma once

#include "pt_math.cuh"

namespace phc {

PHC_HD float ldg_f(const float *p)
{
#ifdef __CUDA_ARCH__
  return __ldg(p);
#else
  return *p;
#endif
}
PHC_HD uint32_t ldg_u(const uint32_t *p)
{
#ifdef __CUDA_ARCH__
  return __ldg(p);
#else
  return *p;
#endif
}

PHC_HD uint32_t cdf_search_le(const float *cdf, uint32_t n, const uint32_t *guide, uint32_t bits, float u)
{
  uint32_t lo = 0, hi = n;
  if (guide) {
    const uint32_t k = uint32_t(u * float(1u << bits)); // u in [0, 1): k < G
    lo = ldg_u(guide + k);
    hi = ldg_u(guide + k + 1) + 1u;
  }
  while (lo + 1 < hi) {
    const uint32_t mid = (lo + hi) / 2;
    if (ldg_f(cdf + mid) <= u)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

PHC_HD uint32_t cdf_search_gt(const float *cdf, uint32_t n, const uint32_t *guide, uint32_t bits, float u)
{
  uint32_t lo = 0, hi = n - 1;
  if (guide) {
    const uint32_t k = uint32_t(u * float(1u << bits));
    lo = ldg_u(guide + k);
    hi = ldg_u(guide + k + 1);
  }
  while (lo < hi) {
    const uint32_t mid = (lo + hi) / 2;
    if (ldg_f(cdf + mid) <= u)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

} // namespace phc
