// Scene tables built on the GPU at upload, with the same code as the host
// builders (these functions are __host__ __device__): the macro-cell
// majorant grid of a transfer-function volume (RenderBridge.cpp:668-780),
// the environment map's row and marginal CDFs (environment_map.cpp:8-65),
// the emissive triangles' selection CDF and area densities
// (pathtracer.cpp:439-487), and the guide tables of the CDF searches.
// Every operation is an IEEE add, multiply, divide, floor, ceil or compare
// (the translation units are compiled without contraction), so the device
// tables are bit-identical to the host's.
#pragma once

#include <cfloat>
#include <cstddef>
#include <cstdint>

#include "pt_math.cuh"
#include "scene_types.h"

namespace phc {

// One volume's majorant grid: per macro cell the largest extinction the
// transfer function reaches over the values the trilinear field can take in
// it, with a 1% margin.  sub[d] > 0 on an axis of <= 32 cells: macro cells
// subdivide voxel cells (refined, corner values of the interpolated field);
// otherwise a macro cell covers several voxels (their values, one voxel of
// margin on each side).
struct MajorantJob {
  uint32_t dims[3];
  uint32_t macro_dims[3];
  uint32_t sub[3];
  uint32_t refined;  // all three axes subdivided
  uint32_t complete; // the field holds dims[0]*dims[1]*dims[2] values
  uint32_t table;    // transfer-function entries (RGBA)
  float value_lo, range, density_scale, max_opacity;
};

// std::min / std::max as the host builder uses them: the second argument
// when it compares below / above the first, else the first.
PHC_HD float tbl_min(float a, float b) { return b < a ? b : a; }
PHC_HD float tbl_max(float a, float b) { return a < b ? b : a; }

PHC_HD float majorant_node(const MajorantJob &j, const float *vals, uint32_t x, uint32_t y, uint32_t z)
{
  x = x < j.dims[0] - 1u ? x : j.dims[0] - 1u;
  y = y < j.dims[1] - 1u ? y : j.dims[1] - 1u;
  z = z < j.dims[2] - 1u ? z : j.dims[2] - 1u;
  return vals[(size_t(z) * j.dims[1] + y) * j.dims[0] + x];
}

PHC_HD float majorant_interp(const MajorantJob &j, const float *vals, float gx, float gy, float gz)
{
  const uint32_t x = uint32_t(gx), y = uint32_t(gy), z = uint32_t(gz);
  const float fx = gx - float(x), fy = gy - float(y), fz = gz - float(z);
  const float c00 = majorant_node(j, vals, x, y, z) * (1.f - fx) + majorant_node(j, vals, x + 1, y, z) * fx;
  const float c10 = majorant_node(j, vals, x, y + 1, z) * (1.f - fx) + majorant_node(j, vals, x + 1, y + 1, z) * fx;
  const float c01 = majorant_node(j, vals, x, y, z + 1) * (1.f - fx) + majorant_node(j, vals, x + 1, y, z + 1) * fx;
  const float c11 =
      majorant_node(j, vals, x, y + 1, z + 1) * (1.f - fx) + majorant_node(j, vals, x + 1, y + 1, z + 1) * fx;
  return (c00 * (1.f - fy) + c10 * fy) * (1.f - fz) + (c01 * (1.f - fy) + c11 * fy) * fz;
}

// The majorant of macro cell (mx, my, mz); alpha(t) is the opacity of
// transfer-function entry t.
template <class Alpha>
PHC_HD float majorant_cell(const MajorantJob &j, const float *vals, Alpha alpha, uint32_t mx, uint32_t my, uint32_t mz)
{
  float bound = 0.f;
  if (j.complete && j.table > 0) {
    const uint32_t m[3] = {mx, my, mz};
    float vmin = FLT_MAX, vmax = -FLT_MAX;
    if (j.refined) {
      for (int corner = 0; corner < 8; ++corner) {
        float g[3];
        for (int d = 0; d < 3; ++d)
          g[d] = float(m[d] + ((corner >> d) & 1)) / float(j.sub[d]);
        const float value = majorant_interp(j, vals, g[0], g[1], g[2]);
        vmin = tbl_min(vmin, value);
        vmax = tbl_max(vmax, value);
      }
    } else {
      uint32_t first[3], last[3];
      for (int d = 0; d < 3; ++d) {
        const float cells = float(j.dims[d] > 1 ? j.dims[d] - 1 : 1);
        const float lo = float(m[d]) / float(j.macro_dims[d]) * cells;
        const float hi = float(m[d] + 1) / float(j.macro_dims[d]) * cells;
        first[d] = uint32_t(tbl_max(floorf(lo) - 1.f, 0.f));
        const uint32_t l = uint32_t(ceilf(hi)) + 1u;
        last[d] = l < j.dims[d] - 1u ? l : j.dims[d] - 1u;
      }
      for (uint32_t z = first[2]; z <= last[2]; ++z)
        for (uint32_t y = first[1]; y <= last[1]; ++y)
          for (uint32_t x = first[0]; x <= last[0]; ++x) {
            const float value = vals[(size_t(z) * j.dims[1] + y) * j.dims[0] + x];
            vmin = tbl_min(vmin, value);
            vmax = tbl_max(vmax, value);
          }
    }
    auto tpos = [&](float value) {
      float x = j.range != 0.f ? (value - j.value_lo) / j.range : 0.f;
      x = tbl_min(tbl_max(x, 0.f), 1.f);
      return x * float(j.table - 1);
    };
    const size_t i0 = size_t(floorf(tpos(vmin)));
    const size_t c1 = size_t(ceilf(tpos(vmax)));
    const size_t i1 = c1 < size_t(j.table - 1) ? c1 : size_t(j.table - 1);
    for (size_t t = i0; t <= i1; ++t)
      bound = tbl_max(bound, alpha(t));
    if (!(vmin <= vmax))
      bound = j.max_opacity;
  }
  return bound * j.density_scale * 1.01f;
}

// Luminance weights of the environment CDF and the emitters' power
// (environment_map.cpp:20, pathtracer.cpp:455).
PHC_HD float tbl_lum(float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; }

// A material that can emit (RenderBridge.cpp:780-813): positive strength and
// a textured or positive emission colour.
PHC_HD bool tbl_may_emit(const DevMaterial &m)
{
  if (m.emission_strength <= 0.f)
    return false;
  return m.src_kind[SRC_EMIT] != 0 || m.emission[0] > 0.f || m.emission[1] > 0.f || m.emission[2] > 0.f;
}

// Area of the triangle (p0, p1, p2): half the length of the cross product
// of its edges from p0.
PHC_HD float tbl_tri_area(const float *p0, const float *p1, const float *p2)
{
  const float ax = p1[0] - p0[0], ay = p1[1] - p0[1], az = p1[2] - p0[2];
  const float bx = p2[0] - p0[0], by = p2[1] - p0[1], bz = p2[2] - p0[2];
  const float cx = ay * bz - az * by, cy = az * bx - ax * bz, cz = ax * by - ay * bx;
  return 0.5f * sqrtf(cx * cx + cy * cy + cz * cz);
}

// Selection weight of an emissive triangle of the given area: area times
// the emitter's power (constant emission: the luminance of colour times
// strength; textured: the strength), the power floored at 1e-6.
PHC_HD double tbl_emit_weight(const DevMaterial &m, float area)
{
  const bool constant = m.src_kind[SRC_EMIT] == 0;
  const float power = constant ? tbl_lum(m.emission[0] * m.emission_strength, m.emission[1] * m.emission_strength,
                                     m.emission[2] * m.emission_strength)
                               : m.emission_strength;
  return area > 0.f ? double(area) * double(power > 1e-6f ? power : 1e-6f) : 0.0;
}

// Guide entries of non-decreasing CDFs, for the grid point u = k / G.
// guide_le: max{i in [0, n - 1] : cdf[i] <= u}, 0 when none (the row /
// column searches, environment_map.h:62-104); guide_gt: min({i in [0, n - 2]
// : cdf[i] > u} U {n - 1}) (the emissive search, pathtracer.cpp:296-306).
// The host builder walks the CDF in order; on a non-decreasing CDF these
// bisections return the same indices.
PHC_HD uint32_t guide_le(const float *cdf, uint32_t n, float u)
{
  uint32_t lo = 1, hi = n; // first i in [1, n) with cdf[i] > u, n when none
  while (lo < hi) {
    const uint32_t mid = lo + (hi - lo) / 2;
    if (cdf[mid] <= u)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo - 1;
}

PHC_HD uint32_t guide_gt(const float *cdf, uint32_t n, float u)
{
  uint32_t lo = 0, hi = n - 1; // first i in [0, n - 1) with cdf[i] > u, n - 1 when none
  while (lo < hi) {
    const uint32_t mid = lo + (hi - lo) / 2;
    if (cdf[mid] <= u)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

} // namespace phc
