// Host build of the device BVH8 traversal (photon_gb300/csrc/traverse.cuh)
// over the host BVH8 builder, for CPU tests of the traversal logic against the
// oracle before any GPU run.  Test infrastructure only.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "bvh8.h"
#include "cdf_search.cuh"
#include "traverse.cuh"
#include "volume_track.cuh"

using namespace phc;

extern "C" int ht_trace(const float *pos, uint64_t nv, const uint32_t *idx, uint64_t nt, const float *orgs,
    const float *dirs, const float *tmin, const float *tmax, uint32_t n, int any_hit, int max_leaf, float *out4,
    uint64_t *stats)
{
  Bvh8Host b;
  build_bvh8(pos, nv, idx, nt, b, max_leaf);
  DevScene sc{};
  sc.nodes = reinterpret_cast<const uint4 *>(b.nodes.data());
  sc.tris = reinterpret_cast<const float4 *>(b.tris.data());
  uint64_t nodes = 0, tris = 0;
#pragma omp parallel for reduction(+ : nodes, tris) schedule(dynamic, 256)
  for (int64_t i = 0; i < int64_t(n); ++i) {
    const V3 o{orgs[3 * i], orgs[3 * i + 1], orgs[3 * i + 2]};
    const V3 d{dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]};
    TravCounters c{0, 0};
    const RayHit h = any_hit ? trace_ray<true, true>(sc, o, d, tmin[i], tmax[i], &c)
                             : trace_ray<false, true>(sc, o, d, tmin[i], tmax[i], &c);
    out4[4 * i] = h.t;
    std::memcpy(&out4[4 * i + 1], &h.prim, 4);
    out4[4 * i + 2] = h.u;
    out4[4 * i + 3] = h.v;
    nodes += c.nodes;
    tris += c.tris;
  }
  stats[0] = nodes;
  stats[1] = tris;
  stats[2] = b.node_count;
  stats[3] = b.max_depth;
  stats[4] = b.tri_count;
  return 0;
}

// Two-level traversal (trav_step2) of a scene with instances, built by the
// renderer's own host scene build (build_host_scene): per ray (t, prim, u, v)
// of the closest hit and the object id of its instance (0xffffffff: the
// scene's own triangles or a miss), world hit position and world normals
// as the shading kernels compute them (hit_attributes).
#include "scene_build.h"
#include "bvh_gpu.h"
#include "tuning.h"

#include <stdexcept>

namespace phc {
// The harness never uploads a scene, so the GPU builder (bvh_gpu.cu, compiled
// by nvcc) is not linked in; scene_build.cpp's upload refers to it.
GpuBvh8 build_bvh8_gpu(const float4 *, const uint4 *, uint32_t, cudaStream_t, int, int, float)
{
  throw std::runtime_error("the host harness builds no BVH on the GPU");
}
// Likewise the GPU majorant grid (scene_tables.cu): the harness has every
// table built on the host (host_scene).
std::string launch_majorants(const MajorantJob &, const float *, const float4 *, float *, cudaStream_t)
{
  return "the host harness builds no tables on the GPU";
}
std::string launch_pack_texels_u8(const float4 *, size_t, const float *, uchar4 *, uint32_t *, cudaStream_t)
{
  return "the host harness packs no texels on the GPU";
}
std::string launch_env_tables(const EnvTablesJob &, cudaStream_t) { return "the host harness builds no tables on the GPU"; }
size_t scan_u32_scratch(uint32_t n) { return n; }
void scan_u32(const uint32_t *, uint32_t *, uint32_t, uint32_t *, uint32_t *, cudaStream_t) {}
std::string launch_emissive_ids(const EmissiveJob &, cudaStream_t) { return "the host harness builds no tables on the GPU"; }
std::string launch_emissive_weights(const EmissiveJob &, cudaStream_t)
{
  return "the host harness builds no tables on the GPU";
}
std::string launch_emissive_tables(const EmissiveJob &, double, cudaStream_t)
{
  return "the host harness builds no tables on the GPU";
}
void host_scene(const phc_scene_desc &desc, HostScene &h)
{
  tuning().gpu_tables = 0;
  build_host_scene(desc, h);
}
} // namespace phc

extern "C" int ht_trace_instanced(const phc_scene_desc *desc, const float *orgs, const float *dirs,
    const float *tmin, const float *tmax, uint32_t n, int any_hit, float *out4, uint32_t *obj, float *geo9,
    uint64_t *stats)
{
  HostScene h;
  host_scene(*desc, h);
  DevScene sc{};
  sc.nodes = reinterpret_cast<const uint4 *>(h.bvh.nodes.data());
  sc.tris = reinterpret_cast<const float4 *>(h.bvh.tris.data());
  sc.prim_geo = reinterpret_cast<const float4 *>(h.prim_geo.data());
  sc.prim_vidx = reinterpret_cast<const uint4 *>(h.prim_vidx.data());
  sc.normals = h.normals4.empty() ? nullptr : reinterpret_cast<const float4 *>(h.normals4.data());
  sc.inst_w2o = reinterpret_cast<const float4 *>(h.inst_w2o.data());
  sc.inst_info = reinterpret_cast<const uint4 *>(h.inst_info.data());
  sc.inst_count = h.inst_count;
  sc.scene_normals = h.scene_normals ? 1 : 0;
  if (h.inst_count == 0)
    return -1;
  uint64_t nodes = 0, tris = 0;
#pragma omp parallel for reduction(+ : nodes, tris) schedule(dynamic, 256)
  for (int64_t i = 0; i < int64_t(n); ++i) {
    const V3 o{orgs[3 * i], orgs[3 * i + 1], orgs[3 * i + 2]};
    const V3 d{dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]};
    TravCounters c{0, 0};
    TravState2 s;
    trav_init2(s, o, d, tmin[i], tmax[i]);
    uint2 stack[PHC_STACK_SIZE];
    if (s.g_hits != 0u) {
      if (any_hit)
        while (trav_step2<true, true>(sc.nodes, sc.tris, sc.inst_w2o, sc.inst_info, s, stack, &c)) {
        }
      else
        while (trav_step2<false, true>(sc.nodes, sc.tris, sc.inst_w2o, sc.inst_info, s, stack, &c)) {
        }
    }
    out4[4 * i] = s.best.t;
    std::memcpy(&out4[4 * i + 1], &s.best.prim, 4);
    out4[4 * i + 2] = s.best.u;
    out4[4 * i + 3] = s.best.v;
    obj[i] = 0xffffffffu;
    for (int k = 0; k < 9; ++k)
      geo9[9 * i + k] = 0.f;
    if (s.best.prim != 0xffffffffu) {
      const uint32_t inst = s.best_inst; // INST_NONE: the scene's own triangles
      obj[i] = inst == INST_NONE ? 0xffffffffu : h.inst_info[4 * size_t(inst) + 1];
      const HitAttr a = hit_attributes(sc, o, d, s.best, inst);
      const float g[9] = {a.p.x, a.p.y, a.p.z, a.n.x, a.n.y, a.n.z, a.sn.x, a.sn.y, a.sn.z};
      std::memcpy(&geo9[9 * i], g, sizeof(g));
    }
    nodes += c.nodes;
    tris += c.tris;
  }
  stats[0] = nodes;
  stats[1] = tris;
  stats[2] = h.bvh.node_count;
  stats[3] = h.bvh.max_depth;
  stats[4] = h.inst_count;
  return 0;
}

// The guided CDF searches of the shading kernels (cdf_search.cuh) against
// the plain bisection, over the scene's emissive CDF and environment CDFs:
// every u of `us` and, per CDF, every u at and next to one of its entries
// (RNG values: multiples of 2^-24 in [0, 1)).  counts: [0] guides present
// (bit 0 emissive, 1 marginal, 2 rows), [1] emissive, [2] marginal, [3] row
// searches compared, [4] mismatches.
extern "C" int ht_guide_check(const phc_scene_desc *desc, const float *us, uint32_t n, uint64_t *counts)
{
  HostScene h;
  host_scene(*desc, h);
  for (int k = 0; k < 5; ++k)
    counts[k] = 0;
  counts[0] = (h.emissive_guide.empty() ? 0u : 1u) | (h.env_mguide.empty() ? 0u : 2u) |
      (h.env_cguide.empty() ? 0u : 4u);
  const float q = 1.f / 16777216.f;
  // the RNG values at and next to each entry of a CDF
  auto near_entries = [&](const float *c, uint32_t m, std::vector<float> &out) {
    out.clear();
    for (uint32_t i = 0; i < m; ++i) {
      if (!(c[i] >= 0.f && c[i] < 1.f))
        continue;
      const float b = std::floor(c[i] / q) * q;
      for (float v : {b - q, b, b + q})
        if (v >= 0.f && v < 1.f)
          out.push_back(v);
    }
  };
  std::vector<float> extra;
  const uint32_t ne = uint32_t(h.emissive_cdf.size());
  if (ne > 0) {
    const uint32_t *g = h.emissive_guide.empty() ? nullptr : h.emissive_guide.data();
    near_entries(h.emissive_cdf.data(), ne, extra);
    for (int pass = 0; pass < 2; ++pass) {
      const float *vals = pass ? extra.data() : us;
      const size_t m = pass ? extra.size() : n;
      for (size_t i = 0; i < m; ++i) {
        const uint32_t a = cdf_search_gt(h.emissive_cdf.data(), ne, nullptr, EMISSIVE_GUIDE_BITS, vals[i]);
        const uint32_t b = cdf_search_gt(h.emissive_cdf.data(), ne, g, EMISSIVE_GUIDE_BITS, vals[i]);
        counts[1]++;
        counts[4] += a != b;
      }
    }
  }
  if (h.has_env) {
    const uint32_t w = h.env_w, hh = h.env_h;
    const uint32_t *gm = h.env_mguide.empty() ? nullptr : h.env_mguide.data();
    near_entries(h.env_marginal.data(), hh + 1, extra);
    for (int pass = 0; pass < 2; ++pass) {
      const float *vals = pass ? extra.data() : us;
      const size_t m = pass ? extra.size() : n;
      for (size_t i = 0; i < m; ++i) {
        const uint32_t a = cdf_search_le(h.env_marginal.data(), hh, nullptr, ENV_MGUIDE_BITS, vals[i]);
        const uint32_t b = cdf_search_le(h.env_marginal.data(), hh, gm, ENV_MGUIDE_BITS, vals[i]);
        counts[2]++;
        counts[4] += a != b;
      }
    }
    for (uint32_t row = 0; row < hh; ++row) {
      const float *c = &h.env_conditional[size_t(row) * (w + 1)];
      const uint32_t *g = h.env_cguide.empty() ? nullptr
                                               : &h.env_cguide[size_t(row) * ((1u << ENV_CGUIDE_BITS) + 1)];
      near_entries(c, w + 1, extra);
      for (int pass = 0; pass < 2; ++pass) {
        const float *vals = pass ? extra.data() : us;
        const size_t m = pass ? extra.size() : std::min<size_t>(n, 4096);
        for (size_t i = 0; i < m; ++i) {
          const uint32_t x = cdf_search_le(c, w, nullptr, ENV_CGUIDE_BITS, vals[i]);
          const uint32_t y = cdf_search_le(c, w, g, ENV_CGUIDE_BITS, vals[i]);
          counts[3]++;
          counts[4] += x != y;
        }
      }
    }
  }
  return 0;
}

// The resumable volume tracking of the shading kernels (VolTrack / vt_step,
// volume_track.cuh) against the plain tracking (vol_sample_scatter,
// vol_transmittance), both run on the host over the scene's volumes: for
// every ray the scattering distance and albedo, the transmittance and the
// random-number state after the tracking must be identical bit for bit.
// seeds: the initial random-number state per ray.  counts: [0] rays that
// met a volume event or attenuation, [1] mismatches, [2] vt_step calls.
extern "C" int ht_volume_check(const phc_scene_desc *desc, const float *orgs, const float *dirs, const float *tmin,
    const float *tmax, const uint32_t *seeds, uint32_t n, uint64_t *counts)
{
  HostScene h;
  host_scene(*desc, h);
  std::vector<float> values(h.vol_values);
  for (const HostScene::Span &sp : h.vol_value_spans)
    values.insert(values.end(), sp.p, sp.p + sp.floats);
  DevScene sc{};
  sc.volumes = h.volumes.data();
  sc.volume_count = uint32_t(h.volumes.size());
  sc.vol_values = values.data();
  sc.vol_tf = reinterpret_cast<const float4 *>(h.vol_tf.data());
  sc.vol_majorants = h.vol_majorants.data();
  uint64_t events = 0, bad = 0, steps = 0;
  for (uint32_t i = 0; i < n; ++i) {
    const V3 o{orgs[3 * i], orgs[3 * i + 1], orgs[3 * i + 2]};
    const V3 d{dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]};
    for (int mode = 0; mode < 2; ++mode) {
      Rng a(seeds[i]), b(seeds[i]);
      VolTrack s;
      vt_init(s, o, d, tmin[i], tmax[i]);
      bool same = true;
      if (mode == 0) {
        V3 albedo{0.f, 0.f, 0.f};
        const float t = vol_sample_scatter(sc, o, d, tmin[i], tmax[i], a, albedo);
        while (!s.done) {
          vt_step<true>(sc, s, b);
          ++steps;
        }
        same = f2u(t) == f2u(s.t_event) && f2u(albedo.x) == f2u(s.albedo.x) &&
            f2u(albedo.y) == f2u(s.albedo.y) && f2u(albedo.z) == f2u(s.albedo.z);
        events += t >= 0.f;
      } else {
        const float tr = vol_transmittance(sc, o, d, tmin[i], tmax[i], a);
        while (!s.done) {
          vt_step<false>(sc, s, b);
          ++steps;
        }
        same = f2u(tr) == f2u(s.tr);
        events += tr < 1.f;
      }
      same = same && a.s == b.s;
      bad += same ? 0u : 1u;
    }
  }
  counts[0] = events;
  counts[1] = bad;
  counts[2] = steps;
  return 0;
}

// The float-float sine and cosine of the shading code (sincos.cuh), and the
// host C library's sinf / cosf on the same arguments.
extern "C" void ht_sincos(const float *x, uint32_t n, float *s, float *c, float *libm_s, float *libm_c)
{
  for (uint32_t i = 0; i < n; ++i) {
    s[i] = phc::acc_sin(x[i]);
    c[i] = phc::acc_cos(x[i]);
    libm_s[i] = std::sin(x[i]);
    libm_c[i] = std::cos(x[i]);
  }
}
