// Volume sampling of the shading kernels: delta tracking (scattering) and
// ratio tracking (transmittance) through the transfer-function volumes over
// their macro-cell majorant grids (include/photon/pt/tf_volume.h:43-283), and
// the same tracking as a resumable state machine for persistent warps.
// __host__ __device__ so the CPU tests run the state machine against the
// plain tracking on the host.
#pragma once

#include "cdf_search.cuh"
#include "pt_math.cuh"
#include "scene_types.h"
#include "traverse.cuh"

#ifdef __CUDACC__
#define PHC_HD_NOINLINE __host__ __device__ __noinline__
#else
#define PHC_HD_NOINLINE __attribute__((noinline))
#endif

namespace phc {

// ------------------------------------------------------------- volumes
PHC_HD V3 vol_point(const DevVolume &v, V3 p)
{
  const float *m = v.w2l;
  return V3{m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
      m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]};
}
PHC_HD V3 vol_vector(const DevVolume &v, V3 d)
{
  const float *m = v.w2l;
  return V3{m[0] * d.x + m[1] * d.y + m[2] * d.z, m[4] * d.x + m[5] * d.y + m[6] * d.z,
      m[8] * d.x + m[9] * d.y + m[10] * d.z};
}
PHC_HD bool vol_clip(const DevVolume &v, V3 org, V3 dir, float &t0, float &t1)
{
  const float o[3] = {org.x, org.y, org.z}, d[3] = {dir.x, dir.y, dir.z};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float hi = v.origin[a] + v.spacing[a] * float(v.dims[a] > 1 ? v.dims[a] - 1 : 1);
    if (d[a] == 0.f) {
      if (o[a] < v.origin[a] || o[a] > hi)
        return false;
      continue;
    }
    const float inv = 1.f / d[a];
    const float ta = (v.origin[a] - o[a]) * inv;
    const float tb = (hi - o[a]) * inv;
    const float tn = ta < tb ? ta : tb;
    const float tf = ta < tb ? tb : ta;
    t0 = tn > t0 ? tn : t0;
    t1 = tf < t1 ? tf : t1;
    if (t1 <= t0)
      return false;
  }
  return true;
}
PHC_HD float vol_field(const DevScene &sc, const DevVolume &v, V3 p)
{
  const float g[3] = {(p.x - v.origin[0]) / v.spacing[0], (p.y - v.origin[1]) / v.spacing[1],
      (p.z - v.origin[2]) / v.spacing[2]};
  int i0[3], i1[3];
  float fr[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int n = int(v.dims[a]);
    float x = g[a];
    x = x < 0.f ? 0.f : (x > float(n - 1) ? float(n - 1) : x);
    if (v.linear) {
      int i = int(x);
      if (i > n - 2)
        i = n - 2;
      if (i < 0)
        i = 0;
      i0[a] = i;
      i1[a] = i + 1 < n ? i + 1 : i;
      fr[a] = x - float(i);
    } else {
      int i = int(x + 0.5f);
      i = i > n - 1 ? n - 1 : i;
      i0[a] = i1[a] = i;
      fr[a] = 0.f;
    }
  }
  const uint32_t sx = v.dims[0], sxy = v.dims[0] * v.dims[1];
  const float *base = sc.vol_values + v.data_offset;
  auto at = [&](int x, int y, int z) { return ldg_f(base + uint32_t(z) * sxy + uint32_t(y) * sx + uint32_t(x)); };
  if (!v.linear)
    return at(i0[0], i0[1], i0[2]);
  const float c00 = at(i0[0], i0[1], i0[2]) * (1.f - fr[0]) + at(i1[0], i0[1], i0[2]) * fr[0];
  const float c10 = at(i0[0], i1[1], i0[2]) * (1.f - fr[0]) + at(i1[0], i1[1], i0[2]) * fr[0];
  const float c01 = at(i0[0], i0[1], i1[2]) * (1.f - fr[0]) + at(i1[0], i0[1], i1[2]) * fr[0];
  const float c11 = at(i0[0], i1[1], i1[2]) * (1.f - fr[0]) + at(i1[0], i1[1], i1[2]) * fr[0];
  const float c0 = c00 * (1.f - fr[1]) + c10 * fr[1];
  const float c1 = c01 * (1.f - fr[1]) + c11 * fr[1];
  return c0 * (1.f - fr[2]) + c1 * fr[2];
}
PHC_HD float4 vol_classify(const DevScene &sc, const DevVolume &v, V3 p)
{
  const float value = vol_field(sc, v, p);
  const float range = v.value_hi - v.value_lo;
  float x = range != 0.f ? (value - v.value_lo) / range : 0.f;
  x = x < 0.f ? 0.f : (x > 1.f ? 1.f : x);
  const float f = x * float(v.tf_size - 1);
  uint32_t i = uint32_t(f);
  if (i > v.tf_size - 2)
    i = v.tf_size >= 2 ? v.tf_size - 2 : 0;
  const float fr = v.tf_size >= 2 ? f - float(i) : 0.f;
  const float4 a = ldg4(sc.vol_tf + v.tf_offset + i);
  const float4 b = ldg4(sc.vol_tf + v.tf_offset + (v.tf_size >= 2 ? i + 1 : i));
  float4 c = add4(mul4(a, 1.f - fr), mul4(b, fr));
  c.w = c.w * v.density_scale;
  return c;
}
// VolumeSet::track, tf_volume.h:150-232
static PHC_HD_NOINLINE float vol_track(const DevScene &sc, const DevVolume &v, V3 org, V3 dir, float t0, float t1,
    Rng &rng, bool scatter, V3 &albedo, float &tr)
{
  const float o[3] = {org.x, org.y, org.z}, d[3] = {dir.x, dir.y, dir.z};
  int cell[3], step[3];
  float t_next[3], t_delta[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const int m = int(v.macro_dims[a]);
    const float extent = v.spacing[a] * float(v.dims[a] > 1 ? v.dims[a] - 1 : 1);
    const float cpu = float(m) / extent;
    const float g = (o[a] + d[a] * t0 - v.origin[a]) * cpu;
    int c = int(g);
    c = c < 0 ? 0 : (c > m - 1 ? m - 1 : c);
    cell[a] = c;
    const float speed = d[a] * cpu;
    if (speed > 0.f) {
      step[a] = 1;
      t_delta[a] = 1.f / speed;
      t_next[a] = t0 + (float(c + 1) - g) * t_delta[a];
    } else if (speed < 0.f) {
      step[a] = -1;
      t_delta[a] = -1.f / speed;
      t_next[a] = t0 + (g - float(c)) * t_delta[a];
    } else {
      step[a] = 0;
      t_delta[a] = 1e30f;
      t_next[a] = 1e30f;
    }
  }
  float t = t0;
  int lookups = 0;
  for (int visited = 0; visited < 4096; ++visited) {
    const int axis = t_next[0] < t_next[1] ? (t_next[0] < t_next[2] ? 0 : 2) : (t_next[1] < t_next[2] ? 1 : 2);
    const float t_exit = t_next[axis] < t1 ? t_next[axis] : t1;
    const float bound = ldg_f(sc.vol_majorants + v.macro_offset +
        (uint32_t(cell[2]) * v.macro_dims[1] + uint32_t(cell[1])) * v.macro_dims[0] + uint32_t(cell[0]));
    if (bound > 0.f) {
      const float inv_bound = 1.f / bound;
      while (lookups < 8192) {
        t -= m_log(1.f - rng.next()) * inv_bound;
        if (t >= t_exit)
          break;
        ++lookups;
        const float4 c = vol_classify(sc, v, org + dir * t);
        if (scatter) {
          if (rng.next() * bound < c.w) {
            albedo = V3{c.x, c.y, c.z};
            return t;
          }
        } else {
          tr *= 1.f - c.w * inv_bound;
          if (tr < 0.05f) {
            if (!(tr > 0.f) || rng.next() * 0.05f >= tr) {
              tr = 0.f;
              return -1.f;
            }
            tr = 0.05f;
          }
        }
      }
    }
    t = t_exit;
    if (t_exit >= t1 || lookups >= 8192)
      break;
    cell[axis] += step[axis];
    if (cell[axis] < 0 || cell[axis] >= int(v.macro_dims[axis]))
      break;
    t_next[axis] += t_delta[axis];
  }
  return -1.f;
}
static PHC_HD_NOINLINE float vol_sample_scatter(const DevScene &sc, V3 ro, V3 rd, float tmin, float tmax, Rng &rng,
    V3 &albedo)
{
  float t_event = -1.f, t_limit = tmax, unused = 1.f;
  for (uint32_t vi = 0; vi < sc.volume_count; ++vi) {
    const DevVolume &v = sc.volumes[vi];
    if (v.majorant <= 0.f || v.tf_size == 0)
      continue;
    const V3 org = vol_point(v, ro), dir = vol_vector(v, rd);
    float t0 = tmin, t1 = t_limit;
    if (!vol_clip(v, org, dir, t0, t1))
      continue;
    V3 ea{0.f, 0.f, 0.f};
    const float t = vol_track(sc, v, org, dir, t0, t1, rng, true, ea, unused);
    if (t >= 0.f) {
      t_event = t;
      t_limit = t;
      albedo = ea;
    }
  }
  return t_event;
}
static PHC_HD_NOINLINE float vol_transmittance(const DevScene &sc, V3 ro, V3 rd, float tmin, float tmax, Rng &rng)
{
  float tr = 1.f;
  V3 unused{0.f, 0.f, 0.f};
  for (uint32_t vi = 0; vi < sc.volume_count; ++vi) {
    const DevVolume &v = sc.volumes[vi];
    if (v.majorant <= 0.f || v.tf_size == 0)
      continue;
    const V3 org = vol_point(v, ro), dir = vol_vector(v, rd);
    float t0 = tmin, t1 = tmax;
    if (!vol_clip(v, org, dir, t0, t1))
      continue;
    vol_track(sc, v, org, dir, t0, t1, rng, false, unused, tr);
    if (tr <= 0.f)
      return 0.f;
  }
  return tr;
}

// ------------------------------------------------- resumable volume tracking
// vol_sample_scatter (SCATTER) and vol_transmittance as a state machine that
// stops after each density lookup, so that persistent warps can hand a lane
// that finished its ray a new one and every step of a warp does one lookup
// per busy lane (the tracking loops differ in length by orders of magnitude
// from ray to ray).  vt_step runs the same arithmetic, in the same order, with
// the same random draws and loop limits as vol_track over the volumes in
// order, so a ray's result and its random-number state after the tracking
// are those of the plain functions.
struct VolTrack {
  V3 ro, rd;            // world ray
  float tmin, tmax;     // world segment
  uint32_t vi;          // current volume
  float t_limit;        // scatter: end of the search (the last event)
  float t_event;        // scatter: the event, -1 none
  V3 albedo;            // scatter: albedo at the event
  float tr;             // transmittance
  V3 org, dir;          // ray in the current volume's frame
  float t, t1, t_exit, bound, inv_bound;
  int cell[3], step[3];
  float t_next[3], t_delta[3];
  int visited, lookups, axis;
  bool in_vol, cell_ready, done;
};

PHC_HD void vt_init(VolTrack &s, V3 ro, V3 rd, float tmin, float tmax)
{
  s.ro = ro;
  s.rd = rd;
  s.tmin = tmin;
  s.tmax = tmax;
  s.vi = 0;
  s.t_limit = tmax;
  s.t_event = -1.f;
  s.albedo = V3{0.f, 0.f, 0.f};
  s.tr = 1.f;
  s.in_vol = false;
  s.cell_ready = false;
  s.done = false;
}

// The end of vol_track on the current volume (its return value `t_res`).
template <bool SCATTER>
PHC_HD void vt_end_volume(VolTrack &s, float t_res, V3 ea)
{
  if (SCATTER) {
    if (t_res >= 0.f) {
      s.t_event = t_res;
      s.t_limit = t_res;
      s.albedo = ea;
    }
  } else if (s.tr <= 0.f) { // vol_transmittance returns 0
    s.tr = 0.f;
    s.done = true;
  }
  s.in_vol = false;
  ++s.vi;
}

// After the cell's delta steps: `t = t_exit`, the loop's exit tests and the
// step to the next macro cell (vol_track's outer loop body end).
template <bool SCATTER>
PHC_HD void vt_next_cell(const DevScene &sc, VolTrack &s)
{
  const DevVolume &v = sc.volumes[s.vi];
  s.t = s.t_exit;
  s.cell_ready = false;
  if (s.t_exit >= s.t1 || s.lookups >= 8192) {
    vt_end_volume<SCATTER>(s, -1.f, V3{0.f, 0.f, 0.f});
    return;
  }
  // cell[axis] += step[axis], range test, t_next[axis] += t_delta[axis];
  // constant indices only, so that the state stays in registers
  bool out;
  if (s.axis == 0) {
    s.cell[0] += s.step[0];
    out = s.cell[0] < 0 || s.cell[0] >= int(v.macro_dims[0]);
    if (!out)
      s.t_next[0] += s.t_delta[0];
  } else if (s.axis == 1) {
    s.cell[1] += s.step[1];
    out = s.cell[1] < 0 || s.cell[1] >= int(v.macro_dims[1]);
    if (!out)
      s.t_next[1] += s.t_delta[1];
  } else {
    s.cell[2] += s.step[2];
    out = s.cell[2] < 0 || s.cell[2] >= int(v.macro_dims[2]);
    if (!out)
      s.t_next[2] += s.t_delta[2];
  }
  if (out) {
    vt_end_volume<SCATTER>(s, -1.f, V3{0.f, 0.f, 0.f});
    return;
  }
  ++s.visited;
}

// One unit of the tracking: entering a volume, leaving a macro cell or
// stepping over an empty one, or one delta-tracking step with its density
// lookup (after setting up its cell).  The persistent kernels make at most
// a few passes per lane and loop trip (vt_passes), so that a lane walking a
// long run of empty cells does not hold the warp's other lanes (each lane
// still makes its own operations and random draws in order).
enum : int { VT_CONTINUE = 0, VT_LOOKUP = 1, VT_DONE = 2 };
template <bool SCATTER>
PHC_HD int vt_pass(const DevScene &sc, VolTrack &s, Rng &rng)
{
  {
    if (s.done)
      return VT_DONE;
    if (!s.in_vol) { // enter the next volume the segment crosses
      if (s.vi >= sc.volume_count) {
        s.done = true;
        return VT_DONE;
      }
      const DevVolume &v = sc.volumes[s.vi];
      if (v.majorant <= 0.f || v.tf_size == 0) {
        ++s.vi;
        return VT_CONTINUE;
      }
      s.org = vol_point(v, s.ro);
      s.dir = vol_vector(v, s.rd);
      float t0 = s.tmin, t1 = SCATTER ? s.t_limit : s.tmax;
      if (!vol_clip(v, s.org, s.dir, t0, t1)) {
        ++s.vi;
        return VT_CONTINUE;
      }
      // the macro-cell walk of vol_track, from t0
      const float o[3] = {s.org.x, s.org.y, s.org.z}, d[3] = {s.dir.x, s.dir.y, s.dir.z};
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const int m = int(v.macro_dims[a]);
        const float extent = v.spacing[a] * float(v.dims[a] > 1 ? v.dims[a] - 1 : 1);
        const float cpu = float(m) / extent;
        const float g = (o[a] + d[a] * t0 - v.origin[a]) * cpu;
        int c = int(g);
        c = c < 0 ? 0 : (c > m - 1 ? m - 1 : c);
        s.cell[a] = c;
        const float speed = d[a] * cpu;
        if (speed > 0.f) {
          s.step[a] = 1;
          s.t_delta[a] = 1.f / speed;
          s.t_next[a] = t0 + (float(c + 1) - g) * s.t_delta[a];
        } else if (speed < 0.f) {
          s.step[a] = -1;
          s.t_delta[a] = -1.f / speed;
          s.t_next[a] = t0 + (g - float(c)) * s.t_delta[a];
        } else {
          s.step[a] = 0;
          s.t_delta[a] = 1e30f;
          s.t_next[a] = 1e30f;
        }
      }
      s.t = t0;
      s.t1 = t1;
      s.lookups = 0;
      s.visited = 0;
      s.in_vol = true;
      s.cell_ready = false;
    }
    const DevVolume &v = sc.volumes[s.vi];
    if (!s.cell_ready) { // the top of vol_track's outer loop
      if (s.visited >= 4096) {
        vt_end_volume<SCATTER>(s, -1.f, V3{0.f, 0.f, 0.f});
        return s.done ? VT_DONE : VT_CONTINUE;
      }
      s.axis = s.t_next[0] < s.t_next[1] ? (s.t_next[0] < s.t_next[2] ? 0 : 2) : (s.t_next[1] < s.t_next[2] ? 1 : 2);
      const float tn = s.axis == 0 ? s.t_next[0] : (s.axis == 1 ? s.t_next[1] : s.t_next[2]);
      s.t_exit = tn < s.t1 ? tn : s.t1;
      s.bound = ldg_f(sc.vol_majorants + v.macro_offset +
          (uint32_t(s.cell[2]) * v.macro_dims[1] + uint32_t(s.cell[1])) * v.macro_dims[0] + uint32_t(s.cell[0]));
      s.cell_ready = true;
      if (!(s.bound > 0.f)) {
        vt_next_cell<SCATTER>(sc, s);
        return s.done ? VT_DONE : VT_CONTINUE;
      }
      s.inv_bound = 1.f / s.bound;
    }
    // one delta-tracking step of the cell
    if (s.lookups >= 8192) {
      vt_next_cell<SCATTER>(sc, s);
      return s.done ? VT_DONE : VT_CONTINUE;
    }
    s.t -= m_log(1.f - rng.next()) * s.inv_bound;
    if (s.t >= s.t_exit) {
      vt_next_cell<SCATTER>(sc, s);
      return s.done ? VT_DONE : VT_CONTINUE;
    }
    ++s.lookups;
    const float4 c = vol_classify(sc, v, s.org + s.dir * s.t);
    if (SCATTER) {
      if (rng.next() * s.bound < c.w)
        vt_end_volume<SCATTER>(s, s.t, V3{c.x, c.y, c.z});
    } else {
      s.tr *= 1.f - c.w * s.inv_bound;
      if (s.tr < 0.05f) {
        if (!(s.tr > 0.f) || rng.next() * 0.05f >= s.tr) {
          s.tr = 0.f;
          vt_end_volume<SCATTER>(s, -1.f, V3{0.f, 0.f, 0.f});
        } else {
          s.tr = 0.05f;
        }
      }
    }
    return VT_LOOKUP;
  }
}

// Up to max_passes passes, stopping at a density lookup or the end of the
// tracking; returns the last pass's result.
template <bool SCATTER>
PHC_HD int vt_passes(const DevScene &sc, VolTrack &s, Rng &rng, uint32_t max_passes)
{
  int r = VT_CONTINUE;
  for (uint32_t k = 0; k < max_passes && r == VT_CONTINUE; ++k)
    r = vt_pass<SCATTER>(sc, s, rng);
  return r;
}

// Advances the ray to its next density lookup and makes it (passes until a
// lookup, at most 4096 + 64 per call: a longer run of empty cells resumes at
// the next call); sets s.done when the tracking is over.  Returns whether it
// made a lookup.
template <bool SCATTER>
PHC_HD bool vt_step(const DevScene &sc, VolTrack &s, Rng &rng)
{
  for (int pass = 0; pass < 4096 + 64; ++pass) {
    const int r = vt_pass<SCATTER>(sc, s, rng);
    if (r != VT_CONTINUE)
      return r == VT_LOOKUP;
  }
  return false;
}

} // namespace phc
