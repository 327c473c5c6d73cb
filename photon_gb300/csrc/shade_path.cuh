// The shading of one path (pt_shade, src/photon/pt/pathtracer.cpp:765-1090)
// and the persistent hit / miss / all-path shading kernel, shared by the
// translation units that instantiate its variants (shade_kernels.cu: the
// general kernels; shade_classes_*.cu: the lean hit kernels of the shading
// classes).
//
// The reference shades every pixel slot in one megakernel.  Profiling that
// design on GB300 showed the warps stalled on instruction fetch (a large,
// divergent kernel), so the shading is split:
//   FULL = false  compiled without volumes, attribute/sampler sources,
//                 normal maps and analytic lights, for scenes that use none;
//   PART 1 / 2    hits and misses of the closest-hit query in separate
//                 kernels over the index queues the trace kernel wrote
//                 (scenes without volumes, where a miss cannot scatter);
//   PART 0        every path of the iteration (volume scenes);
//   PART 3        volume scenes with split queues: the paths that scatter in
//                 a volume, while those that reach their surface hit or
//                 escape go to PART 1 / 2 (the tracking pre-pass routes them);
//   CLS           lean hit kernels specialised to the lobes of a shading
//                 class (scene_types.h), each over its class's run of the
//                 class-sorted hit queue: smaller kernels with fewer live
//                 registers, and the same results (a class leaves out only
//                 lobes that are exactly +0 for its materials).
// The arithmetic of every branch is the reference's, in its order.
#pragma once

#include "wave_common.cuh"

namespace phc {
namespace {

struct NextPath {
  float4 o, d, tp;
  uint4 info;
  float pdist;
};
struct ShadowRec {
  float4 a, b, c;
};
// Result of k_vol_scatter for one path: the scattering distance (or -1) and
// albedo, and the random-number state after the tracking.
struct VolPre {
  float4 s;
  uint32_t rng;
};

template <bool FULL, int PART, uint32_t LOBES = LB_ALL>
__device__ __forceinline__ void shade_path(const RenderConst &rc, const DevScene &sc, const float4 ro4,
    const float4 rd4, const float4 tp4, const uint4 info, const float pdist, const float4 hit, const Accum &acc,
    int it, bool &cont, NextPath &next, bool &has_shadow, ShadowRec &sh, uint32_t inst = INST_NONE,
    const VolPre *pre = nullptr)
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
  const bool is_hit = PART == 1 ? true : (PART == 2 ? false : prim != 0xffffffffu);
  Rng rng = path_rng(pixel, sample_index, 1u + uint32_t(it));
  if (FULL && (PART == 1 || PART == 2) && pre) // split volume queues: the path did not scatter
    rng = Rng(pre->rng);
  // The slot's radiance and alpha, read only on the branches that update them
  // (a secondary hit on a surface that does not emit toward the ray leaves
  // them alone): one scattered 16-byte load and four live registers fewer
  // for most paths.
  float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
  bool a_dirty = false;

  auto write_primary_aov = [&](float depth_v, V3 n, V3 albedo) {
    const float4 an = acc.aov_a[slot];
    if (__float_as_uint(an.w) == 0u) {
      acc.aov_n[slot] = f4(n, depth_v);
      acc.aov_a[slot] = f4(albedo, __uint_as_float(sample_index + 1u));
    }
  };

  // Scattering inside a volume in front of the surface (pathtracer.cpp:789-858)
  if (FULL && (PART == 0 || PART == 3) && sc.volume_count > 0) {
    V3 albedo{0.f, 0.f, 0.f};
    float t_sc;
    if (pre) { // tracked by k_vol_scatter: continue its random-number stream
      t_sc = pre->s.x;
      albedo = V3{pre->s.y, pre->s.z, pre->s.w};
      rng = Rng(pre->rng);
    } else {
      const float t_end = is_hit ? hit.x : rd4.w;
      t_sc = vol_sample_scatter(sc, ray_org, ray_dir, ro4.w, t_end, rng, albedo);
    }
    if (t_sc >= 0.f) {
      const V3 p = ray_org + ray_dir * t_sc;
      if (primary) {
        a = acc.acc[slot];
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
      const DirectSample ds = sample_direct<FULL>(sc, p, rng);
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
  if (PART == 3) // the scattering queue holds only paths that scatter
    return;

  if (PART != 1 && !is_hit) { // miss (pathtracer.cpp:860-899)
    a = acc.acc[slot];
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
        float w_mis = 1.f, env_p = 0.f;
        const V3 le = env_eval_pdf(sc, ray_dir, prev_pdf > 0.f, env_p);
        if (prev_pdf > 0.f) {
          const float light_pdf = env_p / float(sc.strategy_count);
          w_mis = power_heuristic(prev_pdf, light_pdf);
        }
        L = L + le * w_mis;
      }
    }
    V3 from_miss = tp * L;
    if (!primary || (sc.has_env && sc.env_visible))
      from_miss = clamp_contrib(from_miss, int(depth) - 1, rc.clamp_direct, rc.clamp_indirect);
    const V3 s = V3{a.x, a.y, a.z} + from_miss;
    acc.acc[slot] = make_float4(s.x, s.y, s.z, a.w);
    return;
  }
  if (PART == 2)
    return;

  // surface hit
  const RayHit rh{hit.x, prim, hit.z, hit.w};
  const HitAttr ha = hit_attributes(sc, ray_org, ray_dir, rh, inst);
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
  q.inst = inst;
  float alpha_val = 1.f;
  const DevMaterial &dm = sc.materials[ha.material_id];
  const Mat mat = resolve_material<FULL>(sc, dm, q, alpha_val);
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
  if (FULL && dm.src_kind[SRC_NORMAL] != 0)
    sn = apply_normal_map(sc, dm.src_kind[SRC_NORMAL], dm.src_index[SRC_NORMAL], q, sn);
  const bool emits = may_emit(dm) && emits_on_side(mat.flags, front);
  if (primary || emits)
    a = acc.acc[slot];
  if (primary) {
    primary = false;
    a.w = a.w + 1.f;
    a_dirty = true;
    write_primary_aov(pdist + rh.t, normalize(sn), mat.base_color);
  }
  if (emits) {
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
    const DirectSample ds = sample_direct<FULL>(sc, p, rng);
    if (ds.valid) {
      const V3 f = bsdf_eval<LOBES>(mat, wo, ds.wi, n, sn);
      if (f.x > 0.f || f.y > 0.f || f.z > 0.f) {
        float w_mis = 1.f;
        if (ds.mis)
          w_mis = power_heuristic(ds.pdf, bsdf_pdf<LOBES>(mat, wo, ds.wi, n, sn));
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
  const BSample bs = bsdf_sample<LOBES>(mat, wo, n, sn, rng);
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

// BATCH: the path's job (PathSoA::info.w bits 17..) selects scene, constants
// and accumulators, and travels with the continued path and its shadow ray.
// Minimum resident 128-thread blocks per SM that the register allocation
// must allow, per variant.  Shading is latency-bound (scattered path-state,
// material and texture loads); a capped register count with some spilling
// keeps more warps resident and hides more of that latency.
#ifndef PHC_SHADE_MIN_BLOCKS_LEAN
#define PHC_SHADE_MIN_BLOCKS_LEAN 12
#endif
#ifndef PHC_SHADE_MIN_BLOCKS_FULL
#define PHC_SHADE_MIN_BLOCKS_FULL 16
#endif
// CLS: the shading class (lean hit kernels only; 0 = every lobe).  With a
// class-sorted hit queue (hq.cls_end) a class kernel shades its class's run
// of it, with its own work counter; otherwise only class 0 runs, over the
// whole queue.
template <bool FULL, int PART, bool BATCH, uint32_t CLS = 0>
__global__ void __launch_bounds__(128, FULL ? PHC_SHADE_MIN_BLOCKS_FULL : PHC_SHADE_MIN_BLOCKS_LEAN) k_shade(const RenderConst *__restrict__ rcp, DevScene sc, BatchTable bt,
    PathSoA in, PathSoA out, const float4 *__restrict__ hits, ShadowSoA sh, Accum acc, WaveCounters wc, int it,
    HitQueues hq)
{
  static_assert(CLS == 0 || (PART == 1 && !FULL), "class kernels are lean hit kernels");
  if (wave_failed(wc))
    return;
  const uint32_t n_all =
      PART == 0 ? wc.count[it] : (PART == 1 ? wc.hcount[it] : (PART == 2 ? wc.mcount[it] : wc.vcount[it]));
  const bool sorted = PART == 1 && hq.sort_threshold != 0u && n_all >= hq.sort_threshold;
  uint32_t lo = 0, n = n_all;
  if (PART == 1 && hq.cls_end && sorted) {
    lo = CLS == 0 ? 0u : hq.cls_end[CLS * MAT_CLASS_BINS - 1];
    n = hq.cls_end[(CLS + 1) * MAT_CLASS_BINS - 1] - lo;
  } else if (CLS != 0) {
    return;
  }
  uint32_t *fetch = CLS != 0 ? wc.cfetch + it * SHADE_CLASSES + CLS
                             : (PART == 3 ? wc.vqfetch + it : wc.fetch + 4 * it + (PART == 2 ? 2 : 1));
  for (;;) {
    const uint32_t base = warp_fetch(fetch);
    if (base >= n)
      break;
    const uint32_t j = base + lane_id();
    bool cont = false, has_sh = false;
    NextPath np;
    ShadowRec sr;
    uint32_t job_bits = 0;
    if (j < n) {
      const uint32_t i = PART == 0 ? j
          : PART == 1          ? (sorted ? hq.sorted[lo + j] : hq.hitq[j])
          : PART == 2          ? hq.missq[j]
                               : hq.vscatq[j];
      const uint4 info = in.info[i];
      if (BATCH) {
        job_bits = info.w & ~((1u << BATCH_JOB_SHIFT) - 1u);
        const BatchJob &J = bt.jobs[info.w >> BATCH_JOB_SHIFT];
        shade_path<FULL, PART, SHADE_CLASS_LOBES[CLS]>(J.rc, J.sc, in.ray_o[i], in.ray_d[i], in.tp[i], info,
            in.pdist[i], hits[i], J.acc, it, cont, np, has_sh, sr);
      } else {
        const uint32_t inst = (PART != 2 && sc.inst_count) ? hq.inst[i] : INST_NONE;
        VolPre pre;
        const bool has_pre = FULL && hq.vscatter != nullptr; // volume scenes (PART 1 / 2: split queues)
        if (has_pre) {
          pre.s = hq.vscatter[i];
          pre.rng = hq.vrng[i];
        }
        shade_path<FULL, PART, SHADE_CLASS_LOBES[CLS]>(*rcp, sc, in.ray_o[i], in.ray_d[i], in.tp[i], info,
            in.pdist[i], hits[i], acc, it, cont, np, has_sh, sr, inst, has_pre ? &pre : nullptr);
      }
    }
    if (PART != 2) { // misses never continue nor cast shadow rays
      const uint32_t o = warp_append(wc.count + it + 1, cont);
      if (cont) {
        out.ray_o[o] = np.o;
        out.ray_d[o] = np.d;
        out.tp[o] = np.tp;
        out.info[o] = make_uint4(np.info.x, np.info.y, np.info.z, np.info.w | job_bits);
        out.pdist[o] = np.pdist;
      }
      const uint32_t so = warp_append(wc.scount + it, has_sh);
      if (has_sh) {
        sh.a[so] = sr.a;
        sh.b[so] = sr.b;
        sh.c[so] = sr.c;
        if (BATCH)
          sh.job[so] = job_bits >> BATCH_JOB_SHIFT;
      }
    }
  }
}

} // namespace
} // namespace phc
