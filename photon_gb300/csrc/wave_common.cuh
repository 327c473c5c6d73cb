// Helpers shared by the wavefront kernels (wavefront.cu, shade_kernels.cu).
#pragma once

#include "shade.cuh"
#include "wavefront.h"

namespace phc {

constexpr uint32_t WARP_FULL = 0xffffffffu;
constexpr uint32_t EMISSION_ONLY = 0x80000000u;

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Next `k`-item batch of a warp; uniform across the warp.  Every lane of
// the warp calls it.  The __syncwarp makes the reconvergence explicit: a
// lane that ran long divergent work (a tracking loop, a shading call) must
// be back before the warp votes, or the lanes' views of the batch differ.
__device__ __forceinline__ uint32_t warp_fetch(uint32_t *ctr, uint32_t k = 32u)
{
  __syncwarp();
  uint32_t base = 0;
  if (lane_id() == 0)
    base = atomicAdd(ctr, k);
  return __shfl_sync(WARP_FULL, base, 0);
}

// Reserves one output slot per lane with pred set, keeping lane order; all
// lanes of the warp call it (ballot + popc prefix, one atomic per warp).
__device__ __forceinline__ uint32_t warp_append(uint32_t *ctr, bool pred)
{
  __syncwarp();
  const uint32_t mask = __ballot_sync(WARP_FULL, pred);
  if (mask == 0u)
    return 0u;
  const uint32_t leader = uint32_t(__ffs(int(mask)) - 1);
  uint32_t base = 0;
  if (lane_id() == leader)
    base = atomicAdd(ctr, uint32_t(__popc(mask)));
  base = __shfl_sync(WARP_FULL, base, int(leader));
  return base + uint32_t(__popc(mask & ((1u << lane_id()) - 1u)));
}

__device__ __forceinline__ V3 rc3(const float *p) { return V3{p[0], p[1], p[2]}; }

// clamp_contribution, pathtracer.cpp:36-47
__device__ __forceinline__ V3 clamp_contrib(V3 c, int light_bounce, float direct_sum, float indirect_sum)
{
  const float limit = light_bounce > 0 ? indirect_sum : direct_sum;
  if (!(limit > 0.f))
    return c;
  const float sum = fabsf(c.x) + fabsf(c.y) + fabsf(c.z);
  return sum > limit ? c * (limit / sum) : c;
}

// count_bounce, pathtracer.cpp:49-58
__device__ __forceinline__ bool count_bounce(uint32_t &kinds, uint32_t shift, int limit)
{
  uint32_t count = (kinds >> shift) & 0x7fu;
  if (count < 0x7fu)
    ++count;
  kinds = (kinds & ~(0x7fu << shift)) | (count << shift);
  return limit >= 0 && int(count) > limit;
}

// Camera::clip_range, camera.h:118-134
__device__ __forceinline__ void clip_range(const RenderConst &rc, V3 dir, float &tn, float &tf)
{
  tn = 0.f;
  tf = 1e30f;
  if (rc.clip_near <= 0.f && rc.clip_far >= 1e30f)
    return;
  const float ca = dot(dir, rc3(rc.cw) * -1.f);
  if (ca <= 1e-6f) {
    tn = 1.f;
    tf = 0.f;
    return;
  }
  if (rc.clip_near > 0.f)
    tn = rc.clip_near / ca;
  if (rc.clip_far < 1e30f)
    tf = rc.clip_far / ca;
}

// Jittered camera ray of one pixel sample (pathtracer.cpp:727-743 with
// Camera::ray and clip_range, camera.h:118-157).
__device__ __forceinline__ void camera_ray(const RenderConst &rc, uint32_t pixel, uint32_t sample_index, V3 &ro,
    V3 &rd, float &tmin, float &tmax)
{
  const uint32_t x = pixel % rc.w, y = pixel / rc.w;
  Rng rng = path_rng(pixel, sample_index, 0u);
  float u = (float(x) + rng.next()) / float(rc.w);
  float v = (float(y) + rng.next()) / float(rc.h); // rows from the bottom (bridge: bottom_up)
  u = rc.region[0] + (rc.region[2] - rc.region[0]) * u;
  v = rc.region[1] + (rc.region[3] - rc.region[1]) * v;
  const V3 ll = rc3(rc.lower_left), hz = rc3(rc.horizontal), vt = rc3(rc.vertical), org = rc3(rc.origin);
  if (rc.ortho) {
    ro = ll + hz * u + vt * v;
    rd = -rc3(rc.cw);
  } else if (rc.lens_radius <= 0.f) {
    ro = org;
    rd = normalize(ll + hz * u + vt * v - org);
  } else {
    float dx, dy;
    concentric_disk(rng, dx, dy);
    dx = dx * rc.lens_radius;
    dy = dy * rc.lens_radius;
    const V3 off = rc3(rc.cu) * dx + rc3(rc.cv) * dy;
    const V3 target = ll + hz * u + vt * v;
    ro = org + off;
    rd = normalize(target - org - off);
  }
  clip_range(rc, rd, tmin, tmax);
}

// sample_background_image, pathtracer.cpp:370-389
__device__ __forceinline__ float4 bg_image(const RenderConst &rc, float s, float t)
{
  const int h = int(rc.bg_h), w = int(rc.bg_w);
  const float fx = s * float(w) - 0.5f;
  const float fy = t * float(h) - 0.5f;
  const float flx = floorf(fx), fly = floorf(fy);
  const float tx = fx - flx, ty = fy - fly;
  auto ci = [](int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); };
  const int x0 = ci(int(flx), w), x1 = ci(int(flx) + 1, w), y0 = ci(int(fly), h), y1 = ci(int(fly) + 1, h);
  const float4 a = add4(mul4(__ldg(rc.bg_image + size_t(y0) * w + x0), 1.f - tx),
      mul4(__ldg(rc.bg_image + size_t(y0) * w + x1), tx));
  const float4 b = add4(mul4(__ldg(rc.bg_image + size_t(y1) * w + x0), 1.f - tx),
      mul4(__ldg(rc.bg_image + size_t(y1) * w + x1), tx));
  return add4(mul4(a, 1.f - ty), mul4(b, ty));
}

} // namespace phc
