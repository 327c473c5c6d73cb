// Wavefront kernels of the GB300 path tracer.
//
//   k_raygen   pt_init_sample      pathtracer.cpp:691-760
//   k_trace    trace_closest       kokkos_backend.cpp:21-61 (BVH8, traverse.cuh)
//   k_shade    pt_shade            pathtracer.cpp:765-1090
//   k_shadow   trace_occluded + pt_nee_accum_pack  pathtracer.cpp:1092-1123
//   k_wave_end pt_update_variance  pathtracer.cpp:1129-1139 (+ wave bookkeeping)
//   k_resolve  pt_resolve + frame accumulation  pathtracer.cpp:1143-1155,
//              RenderBridge.cpp:386-410
//
// Unlike the reference, which sweeps all w*h slots in every kernel and keeps
// dead paths as empty rays (pathtracer.cpp:1113-1121), live paths are
// compacted into dense queues: each warp reserves its outputs with one atomic
// (ballot + popc prefix), and every kernel reads a dense, coalesced range.
// Kernels are persistent: a fixed grid of warps pulls 32-item batches from a
// device counter until the queue length (also in device memory) is reached.
#include "shade.cuh"
#include "wavefront.h"

namespace phc {
namespace {

constexpr uint32_t FULL = 0xffffffffu;
constexpr uint32_t EMISSION_ONLY = 0x80000000u;

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Next 32-item batch of a warp; uniform across the warp.
__device__ __forceinline__ uint32_t warp_fetch(uint32_t *ctr)
{
  uint32_t base = 0;
  if (lane_id() == 0)
    base = atomicAdd(ctr, 32u);
  return __shfl_sync(FULL, base, 0);
}

// Reserves one output slot per lane with pred set; all lanes call it.
__device__ __forceinline__ uint32_t warp_append(uint32_t *ctr, bool pred)
{
  const uint32_t mask = __ballot_sync(FULL, pred);
  if (mask == 0u)
    return 0u;
  const uint32_t leader = uint32_t(__ffs(int(mask)) - 1);
  uint32_t base = 0;
  if (lane_id() == leader)
    base = atomicAdd(ctr, uint32_t(__popc(mask)));
  base = __shfl_sync(FULL, base, int(leader));
  return base + uint32_t(__popc(mask & ((1u << lane_id()) - 1u)));
}

__device__ __forceinline__ V3 rc3(const float *p) { return V3{p[0], p[1], p[2]}; }

__device__ __forceinline__ V3 clamp_contrib(V3 c, int light_bounce, float direct_sum, float indirect_sum)
{
  const float limit = light_bounce > 0 ? indirect_sum : direct_sum;
  if (!(limit > 0.f))
    return c;
  const float sum = fabsf(c.x) + fabsf(c.y) + fabsf(c.z);
  return sum > limit ? c * (limit / sum) : c;
}

__device__ __forceinline__ bool count_bounce(uint32_t &kinds, uint32_t shift, int limit)
{
  uint32_t count = (kinds >> shift) & 0x7fu;
  if (count < 0x7fu)
    ++count;
  kinds = (kinds & ~(0x7fu << shift)) | (count << shift);
  return limit >= 0 && int(count) > limit;
}

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

__device__ __forceinline__ float4 bg_image(const RenderConst &rc, float s, float t)
{
  const int h = int(rc.bg_h), w = int(rc.bg_w);
  const float fx = s * float(w) - 0.5f;
  const float fy = t * float(h) - 0.5f;
  const float flx = floorf(fx), fly = floorf(fy);
  const float tx = fx - flx, ty = fy - fly;
  auto ci = [](int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); };
  const int x0 = ci(int(flx), w), x1 = ci(int(flx) + 1, w), y0 = ci(int(fly), h), y1 = ci(int(fly) + 1, h);
  const float4 a = add4(mul4(__ldg(rc.bg_image + size_t(y0) * w + x0), 1.f - tx), mul4(__ldg(rc.bg_image + size_t(y0) * w + x1), tx));
  const float4 b = add4(mul4(__ldg(rc.bg_image + size_t(y1) * w + x0), 1.f - tx), mul4(__ldg(rc.bg_image + size_t(y1) * w + x1), tx));
  return add4(mul4(a, 1.f - ty), mul4(b, ty));
}

// ----------------------------------------------------------------- raygen
__global__ void __launch_bounds__(256) k_raygen(const RenderConst *__restrict__ rcp, DevScene sc, PathSoA out,
    Accum acc, WaveCounters wc)
{
  const RenderConst &rc = *rcp;
  const uint32_t wave = *wc.wave;
  const uint32_t total = rc.npix * rc.lanes;
  for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < total;
       base += gridDim.x * blockDim.x) {
    const uint32_t i = base + lane_id();
    bool live = false;
    uint32_t pixel = 0, slot = 0, sample_index = 0;
    V3 ro{0.f, 0.f, 0.f}, rd{0.f, 0.f, 0.f};
    float tmin = 0.f, tmax = 0.f;
    if (i < total) {
      const uint32_t lane = i / rc.npix;
      pixel = i - lane * rc.npix;
      slot = i;
      const uint32_t s = wave * rc.lanes + lane; // sample number within the render call
      if (s < rc.spp) {
        live = true;
        if (rc.adaptive && s >= 16u) { // variance gate (pathtracer.cpp:710-725), lanes == 1
          const uint32_t ns = acc.nsamp[slot];
          if (ns >= 16u) {
            const float4 a = acc.acc[slot], q = acc.acc_sq[slot];
            const V3 mean = V3{a.x, a.y, a.z} * (1.f / float(ns));
            const V3 sq = V3{q.x, q.y, q.z} * (1.f / float(ns));
            const V3 var = sq - V3{mean.x * mean.x, mean.y * mean.y, mean.z * mean.z};
            const float max_var = fmaxf(var.x, fmaxf(var.y, var.z));
            const float l = fmaxf(0.2126f * mean.x + 0.7152f * mean.y + 0.0722f * mean.z, 1e-4f);
            if (max_var / (l * l) < 0.01f)
              live = false;
          }
        }
        if (live) {
          sample_index = s + rc.sample_offset;
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
          if (rc.adaptive)
            acc.start[slot] = acc.acc[slot];
          acc.nsamp[slot] += 1u;
        }
      }
    }
    const uint32_t o = warp_append(wc.count, live);
    if (live) {
      out.ray_o[o] = f4(ro, tmin);
      out.ray_d[o] = f4(rd, tmax);
      out.tp[o] = make_float4(1.f, 1.f, 1.f, -1.f);
      out.info[o] = make_uint4(slot, sample_index, 0u, 1u << 16);
      out.pdist[o] = 0.f;
    }
  }
}

// ------------------------------------------------------------ closest hit
template <bool COUNT>
__global__ void __launch_bounds__(128) k_trace(DevScene sc, PathSoA in, float4 *__restrict__ hits, WaveCounters wc,
    int it, uint64_t *stats)
{
  const uint32_t n = wc.count[it];
  uint32_t *fetch = wc.fetch + 3 * it;
  TravCounters ctr{0u, 0u};
  for (;;) {
    const uint32_t base = warp_fetch(fetch);
    if (base >= n)
      break;
    const uint32_t i = base + lane_id();
    if (i < n) {
      const float4 o = in.ray_o[i], d = in.ray_d[i];
      const RayHit h = trace_ray<false, COUNT>(sc, v3(o), v3(d), o.w, d.w, &ctr);
      hits[i] = make_float4(h.t, __uint_as_float(h.prim), h.u, h.v);
    }
  }
  if (COUNT) {
    atomicAdd((unsigned long long *)&stats[0], (unsigned long long)ctr.nodes);
    atomicAdd((unsigned long long *)&stats[1], (unsigned long long)ctr.tris);
  }
}

// ------------------------------------------------------------------ shade
struct NextPath {
  float4 o, d, tp;
  uint4 info;
  float pdist;
};
struct ShadowRec {
  float4 a, b, c;
};

// pt_shade for one path (pathtracer.cpp:765-1090).  Returns whether the path
// continues (next filled) and whether it casts a shadow ray (sh filled).
__device__ __noinline__ void shade_path(const RenderConst &rc, const DevScene &sc, const float4 ro4,
    const float4 rd4, const float4 tp4, const uint4 info, const float pdist, const float4 hit, Accum &acc, int it,
    bool &cont, NextPath &next, bool &has_shadow, ShadowRec &sh)
{
  cont = false;
  has_shadow = false;
  const uint32_t slot = info.x, sample_index = info.y;
  const uint32_t pixel = slot % rc.npix;
  uint32_t kinds = info.z;
  const uint32_t depth = info.w & 0xffffu;
  bool primary = (info.w >> 16) & 1u;
  const bool emission_only = (kinds & EMISSION_ONLY) != 0u;
  const V3 ray_org = v3(ro4), ray_dir = v3(rd4);
  V3 tp = v3(tp4);
  const float prev_pdf = tp4.w;
  const uint32_t max_depth = rc.max_depth;
  const float eps = sc.eps;
  const uint32_t prim = __float_as_uint(hit.y);
  const bool is_hit = prim != 0xffffffffu;
  Rng rng = path_rng(pixel, sample_index, 1u + uint32_t(it));
  float4 a = acc.acc[slot]; // radiance.xyz, alpha
  bool a_dirty = false;

  auto write_primary_aov = [&](float depth_v, V3 n, V3 albedo) {
    float4 an = acc.aov_a[slot];
    if (__float_as_uint(an.w) == 0u) {
      acc.aov_n[slot] = f4(n, depth_v);
      acc.aov_a[slot] = f4(albedo, __uint_as_float(sample_index + 1u));
    }
  };

  // Scattering inside a volume in front of the surface (pathtracer.cpp:789-858)
  if (sc.volume_count > 0) {
    V3 albedo{0.f, 0.f, 0.f};
    const float t_end = is_hit ? hit.x : rd4.w;
    const float t_sc = vol_sample_scatter(sc, ray_org, ray_dir, ro4.w, t_end, rng, albedo);
    if (t_sc >= 0.f) {
      const V3 p = ray_org + ray_dir * t_sc;
      if (primary) {
        primary = false;
        a.w = a.w + 1.f;
        a_dirty = true;
        write_primary_aov(pdist + t_sc, -ray_dir, albedo);
      }
      if (depth >= max_depth || emission_only) {
        if (a_dirty)
          acc.acc[slot] = a;
        return;
      }
      const V3 tpa = tp * albedo;
      const float phase = 0.25f * INV_PI;
      const DirectSample ds = sample_direct(sc, p, rng);
      if (ds.valid) {
        const float w_mis = ds.mis ? power_heuristic(ds.pdf, phase) : 1.f;
        const V3 c = clamp_contrib(tpa * ds.radiance * (phase * w_mis / ds.pdf), int(depth), rc.clamp_direct,
            rc.clamp_indirect);
        has_shadow = true;
        const float tmax = ds.dist < 1e29f ? ds.dist * (1.f - 1e-4f) : 1e30f;
        sh.a = f4(p, tmax);
        sh.b = f4(ds.wi, c.x);
        sh.c = make_float4(c.y, c.z, __uint_as_float(slot), __uint_as_float(sample_index));
      }
      V3 tp_next = tpa;
      if (depth >= 2) {
        const float max_tp = fmaxf(tpa.x, fmaxf(tpa.y, tpa.z));
        const float survive = fminf(fmaxf(max_tp, 0.05f), 0.95f);
        if (rng.next() >= survive) {
          if (a_dirty)
            acc.acc[slot] = a;
          return;
        }
        tp_next = tpa * (1.f / survive);
      }
      if (count_bounce(kinds, 24u, rc.max_volume))
        kinds |= EMISSION_ONLY;
      const V3 nd = uniform_sphere(rng);
      cont = true;
      next.o = f4(p, 0.f);
      next.d = f4(nd, 1e30f);
      next.tp = f4(tp_next, phase);
      next.info = make_uint4(slot, sample_index, kinds, (depth + 1u) | (primary ? 1u << 16 : 0u));
      next.pdist = pdist;
      if (a_dirty)
        acc.acc[slot] = a;
      return;
    }
  }

  if (!is_hit) { // miss (pathtracer.cpp:860-899)
    V3 L{0.f, 0.f, 0.f};
    if (primary) {
      if (sc.has_env && sc.env_visible) {
        L = env_eval(sc, ray_dir);
        a.w = a.w + 1.f;
      } else if (rc.bg_image) {
        const uint32_t x = pixel % rc.w, y = pixel / rc.w;
        const float bs = (float(x) + 0.5f) / float(rc.w);
        const float bt = (float(y) + 0.5f) / float(rc.h);
        const float4 bg = bg_image(rc, bs, bt);
        L = V3{bg.x, bg.y, bg.z} * bg.w;
        a.w = a.w + bg.w;
      } else {
        L = rc3(rc.bg) * rc.bg[3];
        a.w = a.w + rc.bg[3];
      }
    } else {
      L = rc3(rc.ambient);
      if (sc.has_env) {
        float w_mis = 1.f;
        if (prev_pdf > 0.f) {
          const float light_pdf = env_pdf(sc, ray_dir) / float(sc.strategy_count);
          w_mis = power_heuristic(prev_pdf, light_pdf);
        }
        L = L + env_eval(sc, ray_dir) * w_mis;
      }
    }
    V3 from_miss = tp * L;
    if (!primary || (sc.has_env && sc.env_visible))
      from_miss = clamp_contrib(from_miss, int(depth) - 1, rc.clamp_direct, rc.clamp_indirect);
    const V3 s = V3{a.x, a.y, a.z} + from_miss;
    acc.acc[slot] = make_float4(s.x, s.y, s.z, a.w);
    return;
  }

  // surface hit
  const RayHit rh{hit.x, prim, hit.z, hit.w};
  const HitAttr ha = hit_attributes(sc, ray_org, ray_dir, rh);
  const V3 p = ha.p;
  const V3 wo = -ray_dir;
  V3 hit_sn = ha.sn;
  if (!(dot(hit_sn, hit_sn) > 0.25f))
    hit_sn = ha.n;
  else if (dot(hit_sn, ha.n) < 0.f)
    hit_sn = hit_sn * -1.f;
  Query q;
  q.prim = prim;
  q.vidx = ha.vidx;
  q.b1 = rh.u;
  q.b2 = rh.v;
  q.p = p;
  q.sn = hit_sn;
  float alpha_val = 1.f;
  const DevMaterial &dm = sc.materials[ha.material_id];
  const Mat mat = resolve_material(sc, dm, q, alpha_val);
  const bool hidden = (mat.flags & MF_HIDDEN) != 0 && primary;
  if (hidden || (alpha_val < 1.f && rng.next() >= alpha_val)) { // stochastic transparency
    float tmin = eps, tmax = 1e30f;
    const float nd = pdist + rh.t;
    if (primary) {
      float tn, tf;
      clip_range(rc, ray_dir, tn, tf);
      if (tf < 1e30f) {
        tmax = tf - nd;
        if (tmax < eps) {
          tmin = 1.f;
          tmax = 0.f;
        }
      }
    }
    cont = true;
    next.o = f4(p, tmin);
    next.d = f4(ray_dir, tmax);
    next.tp = f4(tp, -1.f);
    next.info = make_uint4(slot, sample_index, kinds, depth | (primary ? 1u << 16 : 0u));
    next.pdist = nd;
    return;
  }
  V3 n = ha.n;
  V3 sn = hit_sn;
  const bool front = dot(n, wo) >= 0.f;
  if (!(mat.transmission > 0.f) && !front) {
    n = n * -1.f;
    sn = sn * -1.f;
  }
  if (dm.src_kind[SRC_NORMAL] != 0)
    sn = apply_normal_map(sc, dm.src_kind[SRC_NORMAL], dm.src_index[SRC_NORMAL], q, sn);
  if (primary) {
    primary = false;
    a.w = a.w + 1.f;
    a_dirty = true;
    write_primary_aov(pdist + rh.t, normalize(sn), mat.base_color);
  }
  if (may_emit(dm) && emits_on_side(mat.flags, front)) {
    float w_mis = 1.f;
    if (prev_pdf > 0.f && sc.emissive_count > 0) {
      const float pdf_area = __ldg(sc.prim_light_pdf + prim);
      const float cos_light = fabsf(dot(ha.n, wo));
      if (pdf_area > 0.f && cos_light > 0.f) {
        const float light_pdf = pdf_area * rh.t * rh.t / cos_light / float(sc.strategy_count);
        w_mis = power_heuristic(prev_pdf, light_pdf);
      }
    }
    const V3 s = V3{a.x, a.y, a.z} +
        clamp_contrib(tp * mat_emission(mat) * w_mis, int(depth) - 1, rc.clamp_direct, rc.clamp_indirect);
    a.x = s.x;
    a.y = s.y;
    a.z = s.z;
    a_dirty = true;
  }
  if (a_dirty)
    acc.acc[slot] = a;
  if ((mat.flags & MF_EMITTER_ONLY) != 0 || depth >= max_depth || emission_only)
    return;
  { // next event estimation
    const DirectSample ds = sample_direct(sc, p, rng);
    if (ds.valid) {
      const V3 f = bsdf_eval(mat, wo, ds.wi, n, sn);
      if (f.x > 0.f || f.y > 0.f || f.z > 0.f) {
        float w_mis = 1.f;
        if (ds.mis)
          w_mis = power_heuristic(ds.pdf, bsdf_pdf(mat, wo, ds.wi, n, sn));
        const V3 c = clamp_contrib(tp * f * ds.radiance * (w_mis / ds.pdf), int(depth), rc.clamp_direct,
            rc.clamp_indirect);
        const V3 so = p + n * eps;
        V3 sd;
        float stmax;
        if (ds.dist < 1e29f) {
          const V3 to_light = p + ds.wi * ds.dist - so;
          const float sdist = length(to_light);
          sd = sdist > 0.f ? to_light * (1.f / sdist) : ds.wi;
          stmax = sdist * (1.f - 1e-3f);
        } else {
          sd = ds.wi;
          stmax = 1e30f;
        }
        has_shadow = true;
        sh.a = f4(so, stmax);
        sh.b = f4(sd, c.x);
        sh.c = make_float4(c.y, c.z, __uint_as_float(slot), __uint_as_float(sample_index));
      }
    }
  }
  const BSample bs = bsdf_sample(mat, wo, n, sn, rng);
  if (bs.pdf <= 0.f || (bs.f.x <= 0.f && bs.f.y <= 0.f && bs.f.z <= 0.f))
    return;
  V3 tpn = tp * (bs.f * (1.f / bs.pdf));
  if (depth >= 2) {
    const float max_tp = fmaxf(tpn.x, fmaxf(tpn.y, tpn.z));
    const float survive = fminf(fmaxf(max_tp, 0.05f), 0.95f);
    if (rng.next() >= survive)
      return;
    tpn = tpn * (1.f / survive);
  }
  if (rc.tp_clamp > 0.f) {
    const float mx = fmaxf(tpn.x, fmaxf(tpn.y, tpn.z));
    if (mx > rc.tp_clamp)
      tpn = tpn * (rc.tp_clamp / mx);
  }
  if (!finite3(tpn))
    return;
  const V3 wi = normalize(bs.wi);
  const float side = dot(wi, ha.n) < 0.f ? -1.f : 1.f;
  const bool through = (dot(wi, ha.n) < 0.f) != (dot(wo, ha.n) < 0.f);
  const bool exceeded = through ? count_bounce(kinds, 16u, rc.max_transmission)
                                : (bs.diff ? count_bounce(kinds, 0u, rc.max_diffuse)
                                           : count_bounce(kinds, 8u, rc.max_glossy));
  if (exceeded)
    kinds |= EMISSION_ONLY;
  cont = true;
  next.o = f4(p + ha.n * (side * eps), 0.f);
  next.d = f4(wi, 1e30f);
  next.tp = f4(tpn, bs.spec ? -1.f : bs.pdf);
  next.info = make_uint4(slot, sample_index, kinds, depth + 1u);
  next.pdist = pdist;
}

__global__ void __launch_bounds__(128) k_shade(const RenderConst *__restrict__ rcp, DevScene sc, PathSoA in,
    PathSoA out, const float4 *__restrict__ hits, ShadowSoA sh, Accum acc, WaveCounters wc, int it)
{
  const RenderConst &rc = *rcp;
  const uint32_t n = wc.count[it];
  uint32_t *fetch = wc.fetch + 3 * it + 1;
  for (;;) {
    const uint32_t base = warp_fetch(fetch);
    if (base >= n)
      break;
    const uint32_t i = base + lane_id();
    bool cont = false, has_sh = false;
    NextPath np;
    ShadowRec sr;
    if (i < n)
      shade_path(rc, sc, in.ray_o[i], in.ray_d[i], in.tp[i], in.info[i], in.pdist[i], hits[i], acc, it, cont, np,
          has_sh, sr);
    const uint32_t o = warp_append(wc.count + it + 1, cont);
    if (cont) {
      out.ray_o[o] = np.o;
      out.ray_d[o] = np.d;
      out.tp[o] = np.tp;
      out.info[o] = np.info;
      out.pdist[o] = np.pdist;
    }
    const uint32_t so = warp_append(wc.scount + it, has_sh);
    if (has_sh) {
      sh.a[so] = sr.a;
      sh.b[so] = sr.b;
      sh.c[so] = sr.c;
    }
  }
}

// ----------------------------------------------------------------- shadow
// Any-hit traversal of the shadow queue, then the NEE contribution of the
// unoccluded rays times the ratio-tracking transmittance of the volumes
// (stream dimension 0x10000 + iteration), added to the path's pixel slot.
template <bool COUNT>
__global__ void __launch_bounds__(128) k_shadow(const RenderConst *__restrict__ rcp, DevScene sc, ShadowSoA sh,
    Accum acc, WaveCounters wc, int it, uint64_t *stats)
{
  const uint32_t npix = rcp->npix;
  const uint32_t n = wc.scount[it];
  uint32_t *fetch = wc.fetch + 3 * it + 2;
  TravCounters ctr{0u, 0u};
  for (;;) {
    const uint32_t base = warp_fetch(fetch);
    if (base >= n)
      break;
    const uint32_t i = base + lane_id();
    if (i < n) {
      const float4 a = sh.a[i], b = sh.b[i], c = sh.c[i];
      const V3 o = v3(a), d = v3(b);
      const RayHit h = trace_ray<true, COUNT>(sc, o, d, 0.f, a.w, &ctr);
      if (h.prim == 0xffffffffu) {
        V3 contrib{b.w, c.x, c.y};
        const uint32_t slot = __float_as_uint(c.z), sample_index = __float_as_uint(c.w);
        if (sc.volume_count > 0) {
          Rng rs = path_rng(slot % npix, sample_index, 0x10000u + uint32_t(it));
          contrib = contrib * vol_transmittance(sc, o, d, 0.f, a.w, rs);
        }
        if (finite3(contrib)) {
          float4 v = acc.acc[slot];
          v.x = v.x + contrib.x;
          v.y = v.y + contrib.y;
          v.z = v.z + contrib.z;
          acc.acc[slot] = v;
        }
      }
    }
  }
  if (COUNT) {
    atomicAdd((unsigned long long *)&stats[0], (unsigned long long)ctr.nodes);
    atomicAdd((unsigned long long *)&stats[1], (unsigned long long)ctr.tris);
  }
}

// End of a wave: adaptive variance update (pathtracer.cpp:1129-1139), ray
// totals, and the wave index for the next replay.  Runs as one grid over the
// pixel slots; block 0 thread 0 does the bookkeeping after reading counters.
__global__ void __launch_bounds__(256) k_wave_end(const RenderConst *__restrict__ rcp, Accum acc, WaveCounters wc,
    uint32_t npix, int adaptive, int max_iter, unsigned long long *ray_totals)
{
  if (adaptive) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x) {
      const float4 a = acc.acc[i], s = acc.start[i];
      const V3 sv = V3{a.x, a.y, a.z} - V3{s.x, s.y, s.z};
      float4 q = acc.acc_sq[i];
      q.x = q.x + sv.x * sv.x;
      q.y = q.y + sv.y * sv.y;
      q.z = q.z + sv.z * sv.z;
      acc.acc_sq[i] = q;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    unsigned long long cr = 0, sr = 0;
    for (int k = 0; k < max_iter; ++k) {
      cr += wc.count[k];
      sr += wc.scount[k];
    }
    ray_totals[0] += wc.count[0];
    ray_totals[1] += cr;
    ray_totals[2] += sr;
    *wc.wave += 1u;
  }
}

// pt_resolve + accumulate_frame: per pixel the lanes' sums in lane order,
// divided by the samples started, weighted into the frame.  The depth,
// normal and albedo of the earliest sample that reached a primary event.
__global__ void __launch_bounds__(256) k_resolve(Accum acc, Frame fr, uint32_t npix, uint32_t lanes, float weight,
    int first)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
    float4 sum = acc.acc[p];
    uint32_t ns = acc.nsamp[p];
    float4 an = acc.aov_n[p], aa = acc.aov_a[p];
    for (uint32_t l = 1; l < lanes; ++l) {
      const size_t s = size_t(l) * npix + p;
      const float4 v = acc.acc[s];
      sum.x = sum.x + v.x;
      sum.y = sum.y + v.y;
      sum.z = sum.z + v.z;
      sum.w = sum.w + v.w;
      ns += acc.nsamp[s];
      const float4 a2 = acc.aov_a[s];
      const uint32_t w2 = __float_as_uint(a2.w), w1 = __float_as_uint(aa.w);
      if (w2 != 0u && (w1 == 0u || w2 < w1)) {
        aa = a2;
        an = acc.aov_n[s];
      }
    }
    const float inv = ns > 0 ? (1.f / float(ns)) : 0.f;
    const float4 color = make_float4(sum.x * inv, sum.y * inv, sum.z * inv, sum.w * inv);
    const bool written = __float_as_uint(aa.w) != 0u;
    const float depth = written ? an.w : 1e30f;
    if (first) {
      fr.color[p] = make_float4(color.x * weight, color.y * weight, color.z * weight, color.w * weight);
      fr.normal[p] = written ? make_float4(an.x, an.y, an.z, depth) : make_float4(0.f, 0.f, 0.f, depth);
      fr.albedo[p] = written ? make_float4(aa.x, aa.y, aa.z, 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
      float4 c = fr.color[p];
      c.x = c.x + color.x * weight;
      c.y = c.y + color.y * weight;
      c.z = c.z + color.z * weight;
      c.w = c.w + color.w * weight;
      fr.color[p] = c;
    }
  }
}

// Channels in the bridge's read-back layout (RenderBridge.cpp:1082-1172).
__global__ void __launch_bounds__(256) k_read(Frame fr, uint32_t npix, float inv, int channel, float *out)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
    if (channel == 0) {
      const float4 c = fr.color[p];
      const float a = c.w * inv;
      reinterpret_cast<float4 *>(out)[p] =
          make_float4(c.x * inv, c.y * inv, c.z * inv, a < 0.f ? 0.f : (a > 1.f ? 1.f : a));
    } else if (channel == 1) {
      const float d = fr.normal[p].w;
      out[p] = d < 1e29f ? d : __int_as_float(0x7f800000);
    } else {
      const float4 v = channel == 2 ? fr.normal[p] : fr.albedo[p];
      out[3 * p] = v.x;
      out[3 * p + 1] = v.y;
      out[3 * p + 2] = v.z;
    }
  }
}

} // namespace

// ------------------------------------------------------------- launchers

void launch_raygen(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, PathSoA out, Accum acc,
    WaveCounters wc)
{
  k_raygen<<<c.blocks_raygen, 256, 0, s>>>(rc, sc, out, acc, wc);
}

void launch_trace(const LaunchCfg &c, cudaStream_t s, DevScene sc, PathSoA in, float4 *hits, WaveCounters wc, int it,
    uint64_t *stats)
{
  if (stats)
    k_trace<true><<<c.blocks_trace, 128, 0, s>>>(sc, in, hits, wc, it, stats);
  else
    k_trace<false><<<c.blocks_trace, 128, 0, s>>>(sc, in, hits, wc, it, nullptr);
}

void launch_shade(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, PathSoA in, PathSoA out,
    const float4 *hits, ShadowSoA sh, Accum acc, WaveCounters wc, int it)
{
  k_shade<<<c.blocks_shade, 128, 0, s>>>(rc, sc, in, out, hits, sh, acc, wc, it);
}

void launch_shadow(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, ShadowSoA sh, Accum acc,
    WaveCounters wc, int it, uint64_t *stats)
{
  if (stats)
    k_shadow<true><<<c.blocks_trace, 128, 0, s>>>(rc, sc, sh, acc, wc, it, stats);
  else
    k_shadow<false><<<c.blocks_trace, 128, 0, s>>>(rc, sc, sh, acc, wc, it, nullptr);
}

void launch_wave_end(cudaStream_t s, const RenderConst *rc, Accum acc, WaveCounters wc, uint32_t npix, int adaptive,
    int max_iter, uint64_t *ray_totals)
{
  const uint32_t blocks = adaptive ? (npix + 255) / 256 : 1u;
  k_wave_end<<<blocks, 256, 0, s>>>(rc, acc, wc, npix, adaptive, max_iter, (unsigned long long *)ray_totals);
}

void launch_resolve(cudaStream_t s, Accum acc, Frame fr, uint32_t npix, uint32_t lanes, float weight, int first)
{
  k_resolve<<<(npix + 255) / 256, 256, 0, s>>>(acc, fr, npix, lanes, weight, first);
}

void launch_read(cudaStream_t s, Frame fr, uint32_t npix, float inv_samples, int channel, float *out)
{
  k_read<<<(npix + 255) / 256, 256, 0, s>>>(fr, npix, inv_samples, channel, out);
}

int max_active_blocks(int which, int threads)
{
  int n = 0;
  switch (which) {
  case 0: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_trace<false>, threads, 0); break;
  case 1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_shade, threads, 0); break;
  case 2: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_shadow<false>, threads, 0); break;
  default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_raygen, threads, 0); break;
  }
  return n;
}

} // namespace phc
