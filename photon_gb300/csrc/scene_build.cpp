// Scene build of the GB300 renderer: the tables the reference's render bridge
// and path tracer derive from a scene (src/photon/anari/RenderBridge.cpp:
// 441-826, src/photon/pt/pathtracer.cpp:411-503, src/photon/pt/
// environment_map.cpp:8-65), computed on the host with the same float
// arithmetic (this file is compiled with -ffp-contract=off) so the device sees
// identical CDFs, majorants and light densities, then uploaded to HBM.
#include "scene_build.h"
#include "bvh_gpu.h"
#include "scene_tables.cuh"
#include "tuning.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <stdexcept>

namespace phc {
namespace {

struct F3 {
  float x, y, z;
};
inline F3 f3(const float *p) { return {p[0], p[1], p[2]}; }
inline F3 sub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline F3 crs(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float len(F3 v) { return std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
inline float lum(float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; }

// The bridge's material conversion (RenderBridge.cpp:324-370).
DevMaterial convert_material(const phc_material &in)
{
  DevMaterial m{};
  std::memcpy(m.base_color, in.base_color, sizeof(m.base_color));
  m.metallic = in.metallic;
  m.roughness = in.roughness * in.roughness;
  m.ior = in.ior;
  m.transmission = in.transmission;
  m.specular = 0.5f * in.specular;
  m.clearcoat = in.clearcoat;
  m.clearcoat_roughness = in.clearcoat_roughness;
  m.sheen = in.sheen;
  std::memcpy(m.emission, in.emission, sizeof(m.emission));
  m.emission_strength = 1.f;
  m.alpha = in.opacity;
  const phc_param_source *src[7] = {&in.base_color_src, &in.opacity_src, &in.metallic_src, &in.roughness_src,
      &in.emission_src, &in.transmission_src, &in.normal_src};
  for (int k = 0; k < 7; ++k) {
    m.src_kind[k] = src[k]->kind == 1 ? 1 : (src[k]->kind == 2 ? 2 : 0);
    m.src_index[k] = src[k]->index;
  }
  m.base_color_alpha = in.base_color_alpha ? 1 : 0;
  m.base_tex = -1;
  m.alpha_tex = -1;
  if (m.src_kind[SRC_ALPHA] != 0)
    m.alpha = 1.f;
  m.alpha_mode = in.alpha_mode == 0 ? 0 : (in.alpha_mode == 2 ? 2 : 1);
  m.alpha_cutoff = in.alpha_cutoff;
  m.thin = in.thin_walled ? 1 : 0;
  m.flags = MF_REFRACTIVE;
  if (in.emitter_only)
    m.flags |= MF_EMITTER_ONLY;
  if (in.hidden_to_camera)
    m.flags |= MF_HIDDEN;
  if (in.emission_side == 2)
    m.flags |= MF_EMIT_BOTH;
  else if (in.emission_side == 1)
    m.flags |= MF_EMIT_BACK;
  return m;
}

// The lobes a material's BSDF can have (LB_*), from the constants the lean
// and full shading kernels read (resolve_material clamps metallic and
// specTrans to [0, 1]).  A bit is cleared only where the shading code gives
// that lobe exactly +0 for every direction:
//   diffuse (and the sheen share of its weight): weight and value carry the
//     factor (1 - metallic)(1 - specTrans), 0 here, times finite terms;
//   specular reflection: with metallic 0 and the dielectric F0 / F90 scaled
//     by the opacity both 0, F0 = F90 = +0, so its weight and value are +0;
//   transmission: its branch needs specTrans > 0;
//   clear coat, sheen: their code returns +0 for clearcoat <= 0, for
//     sheen <= 0 or metallic >= 1.
// Materials whose base colour, metallic or specTrans come from attributes or
// textures, or with non-finite constants, keep every lobe.
uint32_t material_lobes(const DevMaterial &m)
{
  if (m.src_kind[SRC_BASE] != 0 || m.src_kind[SRC_METAL] != 0 || m.src_kind[SRC_TRANS] != 0 || m.base_tex >= 0)
    return LB_ALL;
  const float vals[9] = {m.base_color[0], m.base_color[1], m.base_color[2], m.metallic, m.transmission,
      m.specular, m.ior, m.clearcoat, m.sheen};
  for (float v : vals)
    if (!std::isfinite(v))
      return LB_ALL;
  auto clamp01 = [](float x) { return x < 0.f ? 0.f : (x > 1.f ? 1.f : x); };
  const float metallic = clamp01(m.metallic), trans = clamp01(m.transmission);
  const float dielectric = 1.f - metallic, opaque = 1.f - trans;
  uint32_t lb = 0;
  if (dielectric * opaque > 0.f)
    lb |= LB_DIFF;
  const float scale = std::fmax(2.f * m.specular, 0.f);
  const float a = (1.f - m.ior) / (1.f + m.ior);
  const float f0d = std::fmin(a * a * scale, 1.f) * opaque;
  const float f90d = std::fmin(scale, 1.f) * opaque;
  if (!(metallic == 0.f && f0d == 0.f && f90d == 0.f))
    lb |= LB_SPEC;
  if (trans > 0.f)
    lb |= LB_TRANS;
  if (m.clearcoat > 0.f)
    lb |= LB_COAT;
  if (m.sheen > 0.f && metallic < 1.f)
    lb |= LB_SHEEN;
  return lb;
}

// The shading class of a material: the first class from 1 whose lobes
// include the material's, else class 0 (every lobe).
uint32_t shade_class_of(uint32_t lobes)
{
  for (uint32_t c = 1; c < SHADE_CLASSES; ++c)
    if ((lobes & ~SHADE_CLASS_LOBES[c]) == 0u)
      return c;
  return 0u;
}

// photon::pt::Material{} defaults (material.h:35-82), used when the scene has
// no material at all (RenderBridge.cpp:518-519).
DevMaterial default_material()
{
  DevMaterial m{};
  m.base_color[0] = m.base_color[1] = m.base_color[2] = 0.8f;
  m.metallic = 0.f;
  m.roughness = 0.5f;
  m.ior = 1.5f;
  m.transmission = 0.f;
  m.specular = 0.5f;
  m.clearcoat = 0.f;
  m.clearcoat_roughness = 0.03f;
  m.sheen = 0.f;
  m.alpha = 1.f;
  m.emission_strength = 0.f;
  m.alpha_mode = 0;
  m.alpha_cutoff = 0.5f;
  m.flags = 0;
  m.base_tex = -1;
  m.alpha_tex = -1;
  return m;
}

// A material of a scene built at the path tracer's level (the pbrt reader,
// pbrt_to_photon.cpp:98-170): pt::Material as given, with its defaults for
// the fields such scenes leave alone (material.h:35-82).
DevMaterial pt_material(const phc_pt_material &in, uint32_t texture_count)
{
  DevMaterial m = default_material();
  std::memcpy(m.base_color, in.base_color, sizeof(m.base_color));
  m.metallic = in.metallic;
  m.roughness = in.roughness;
  m.ior = in.ior;
  m.transmission = in.transmission;
  m.specular = in.specular;
  m.clearcoat = in.clearcoat;
  m.clearcoat_roughness = in.clearcoat_roughness;
  m.sheen = in.sheen;
  m.alpha = in.alpha;
  std::memcpy(m.emission, in.emission, sizeof(m.emission));
  m.emission_strength = in.emission_strength;
  m.flags = in.flags & (MF_EMITTER_ONLY | MF_HIDDEN | MF_EMIT_BOTH | MF_REFRACTIVE | MF_EMIT_BACK);
  // TextureAtlas::sample returns white for an id past the list; with no
  // textures at all the ids are not looked at (pathtracer.cpp:190-199)
  m.base_tex = texture_count ? (in.base_color_tex < 0 ? -1 : in.base_color_tex) : -1;
  m.alpha_tex = texture_count ? (in.alpha_tex < 0 ? -1 : in.alpha_tex) : -1;
  return m;
}

bool may_emit(const DevMaterial &m)
{
  if (m.emission_strength <= 0.f)
    return false;
  return m.src_kind[SRC_EMIT] != 0 || m.emission[0] > 0.f || m.emission[1] > 0.f || m.emission[2] > 0.f;
}

// RGBA8 images reach the seam as floats k / 255 (the reference's
// SamplerTable holds fp32 RGBA, sampler.h:56-138; the bridge copies the
// caller's floats).  When every value of a sampler's texels is one of the
// 256 floats float(k) / 255 bit for bit (s.u8_decode), its texels are kept
// as k in 8 bits and the device decodes them through the same table, so
// lookups return the identical floats from a quarter of the bytes.  Appends
// to s.texels_u8 and returns true, or leaves it unchanged and returns false.
bool pack_texels_u8(const float *src, size_t floats, HostScene &s)
{
  const size_t at = s.texels_u8.size();
  s.texels_u8.resize(at + floats);
  uint8_t *dst = s.texels_u8.data() + at;
  const float *dec = s.u8_decode.data();
  int ok = 1;
#pragma omp parallel for reduction(&& : ok) schedule(static)
  for (int64_t i = 0; i < int64_t(floats); ++i) {
    const float x = src[i];
    const float y = x * 255.f;
    if (!(y >= 0.f && y <= 255.f)) { // NaN, negative or above 1
      ok = 0;
      continue;
    }
    const uint32_t k = uint32_t(y + 0.5f);
    uint32_t a, b;
    std::memcpy(&a, &x, 4);
    std::memcpy(&b, dec + k, 4);
    if (a != b) { // not exactly k / 255 (-0.0 included)
      ok = 0;
      continue;
    }
    dst[i] = uint8_t(k);
  }
  if (!ok)
    s.texels_u8.resize(at);
  return ok != 0;
}

// sin(theta) of row y of an environment map of h rows, with the host C
// library's sinf as the reference evaluates it (environment_map.cpp:31).
static float env_row_sin(uint32_t y, uint32_t h)
{
  const float PI = 3.14159265358979323846f;
  return std::sin(((float)y + 0.5f) * (PI / (float)h));
}

// EnvironmentMap::build_cdf (environment_map.cpp:8-65): row CDFs of texel
// luminance and a marginal CDF of row sums weighted by sin(theta).
void build_env_cdf(HostScene &s)
{
  const uint32_t w = s.env_w, h = s.env_h;
  s.env_marginal.assign(h + 1, 0.f);
  s.env_conditional.assign(size_t(h) * (w + 1), 0.f);
  std::vector<float> row_w(h, 0.f);
  for (uint32_t y = 0; y < h; ++y) {
    float *c = &s.env_conditional[size_t(y) * (w + 1)];
    c[0] = 0.f;
    const float st = env_row_sin(y, h);
    float sum = 0.f;
    for (uint32_t x = 0; x < w; ++x) {
      const float *p = &s.env_pixels4[(size_t(y) * w + x) * 4];
      sum += tbl_lum(p[0], p[1], p[2]);
      c[x + 1] = sum;
    }
    if (sum > 0.f) {
      const float inv = 1.f / sum;
      for (uint32_t x = 0; x <= w; ++x)
        c[x] *= inv;
      c[w] = 1.f;
    } else {
      for (uint32_t x = 0; x <= w; ++x)
        c[x] = (float)x / (float)w;
    }
    row_w[y] = sum * st;
  }
  float total = 0.f;
  for (uint32_t y = 0; y < h; ++y) {
    total += row_w[y];
    s.env_marginal[y + 1] = total;
  }
  if (total > 0.f) {
    const float inv = 1.f / total;
    for (uint32_t y = 0; y <= h; ++y)
      s.env_marginal[y] *= inv;
    s.env_marginal[h] = 1.f;
  } else {
    for (uint32_t y = 0; y <= h; ++y)
      s.env_marginal[y] = (float)y / (float)h;
  }
}

// Guide tables for the CDF searches of the shading kernels.  The searches
// themselves are the reference's: the largest row / column i with
// cdf[i] <= u (environment_map.h:62-104) and the first emissive triangle with
// cdf[i] > u (pathtracer.cpp:296-306).  Both results are non-decreasing in u
// when the CDF is, so the result for u lies between the results for the two
// grid points k / G <= u < (k + 1) / G, which the guide stores; the device
// bisects only that range.  A CDF that is not non-decreasing (NaN texels)
// keeps the plain bisection, whose probe order then decides the result.
static bool non_decreasing(const float *c, uint32_t n)
{
  for (uint32_t i = 1; i < n; ++i)
    if (!(c[i - 1] <= c[i]))
      return false;
  return true;
}

// guide[k] = max{i in [0, n - 1] : cdf[i] <= k / G} (0 when none), guide[G] = n - 1
static void le_guide(const float *cdf, uint32_t n, uint32_t bits, uint32_t *out)
{
  const uint32_t G = 1u << bits;
  uint32_t i = 0;
  for (uint32_t k = 0; k < G; ++k) {
    const float u = float(k) / float(G);
    while (i + 1 < n && cdf[i + 1] <= u)
      ++i;
    out[k] = i;
  }
  out[G] = n - 1;
}

void build_search_guides(HostScene &s)
{
  s.emissive_guide.clear();
  s.env_mguide.clear();
  s.env_cguide.clear();
  const uint32_t ne = uint32_t(s.emissive_cdf.size());
  if (ne > 1 && non_decreasing(s.emissive_cdf.data(), ne)) {
    // guide[k] = min({i in [0, n - 2] : cdf[i] > k / G} U {n - 1}), guide[G] = n - 1
    const uint32_t G = 1u << EMISSIVE_GUIDE_BITS;
    s.emissive_guide.resize(G + 1);
    uint32_t i = 0;
    for (uint32_t k = 0; k < G; ++k) {
      const float u = float(k) / float(G);
      while (i < ne - 1 && s.emissive_cdf[i] <= u)
        ++i;
      s.emissive_guide[k] = i;
    }
    s.emissive_guide[G] = ne - 1;
  }
  if (s.has_env && s.env_w > 0 && s.env_h > 0 && !s.env_rgb) {
    const uint32_t w = s.env_w, h = s.env_h;
    bool ok = non_decreasing(s.env_marginal.data(), h + 1);
    for (uint32_t y = 0; ok && y < h; ++y)
      ok = non_decreasing(&s.env_conditional[size_t(y) * (w + 1)], w + 1);
    if (ok) {
      const uint32_t gm = (1u << ENV_MGUIDE_BITS) + 1, gc = (1u << ENV_CGUIDE_BITS) + 1;
      s.env_mguide.resize(gm);
      le_guide(s.env_marginal.data(), h, ENV_MGUIDE_BITS, s.env_mguide.data());
      s.env_cguide.resize(size_t(h) * gc);
      for (uint32_t y = 0; y < h; ++y)
        le_guide(&s.env_conditional[size_t(y) * (w + 1)], w, ENV_CGUIDE_BITS, &s.env_cguide[size_t(y) * gc]);
    }
  }
}

// Volume tables and the macro-cell majorant grid (RenderBridge.cpp:622-778):
// per macro cell the largest extinction the transfer function reaches over
// the values the trilinear field can take inside it, with a 1% margin.
void build_volumes(const phc_scene_desc &in, HostScene &s)
{
  size_t value_offset = 0, tf_offset = 0;
  for (uint32_t i = 0; i < in.volume_count; ++i) {
    const phc_volume &vd = in.volumes[i];
    DevVolume v{};
    std::memcpy(v.w2l, vd.world_to_local, sizeof(v.w2l));
    std::memcpy(v.origin, vd.origin, sizeof(v.origin));
    std::memcpy(v.spacing, vd.spacing, sizeof(v.spacing));
    for (int d = 0; d < 3; ++d)
      v.dims[d] = std::max<uint32_t>(vd.dims[d], 1);
    v.data_offset = uint32_t(value_offset);
    v.tf_offset = uint32_t(tf_offset);
    const size_t table = vd.transfer ? vd.transfer_count : 0;
    v.tf_size = uint32_t(table);
    v.value_lo = vd.value_range[0];
    v.value_hi = vd.value_range[1];
    v.density_scale = vd.density_scale;
    v.linear = vd.linear ? 1u : 0u;
    float max_opacity = 0.f;
    for (size_t t = 0; t < table; ++t) {
      for (int k = 0; k < 4; ++k)
        s.vol_tf.push_back(vd.transfer[4 * t + k]);
      max_opacity = std::max(max_opacity, vd.transfer[4 * t + 3]);
    }
    v.majorant = max_opacity * vd.density_scale;
    const size_t nvals = vd.values ? size_t(vd.value_count) : 0;
    const bool complete = nvals >= size_t(v.dims[0]) * v.dims[1] * v.dims[2];
    if (!complete)
      v.majorant = 0.f;
    v.macro_offset = uint32_t(s.vol_majorants.size());
    uint32_t sub[3] = {0, 0, 0};
    for (int d = 0; d < 3; ++d) {
      const uint32_t cells = v.dims[d] > 1 ? v.dims[d] - 1 : 1;
      if (cells <= 32) {
        sub[d] = std::min<uint32_t>(std::max<uint32_t>((32 + cells - 1) / cells, 1), 16);
        v.macro_dims[d] = cells * sub[d];
      } else {
        v.macro_dims[d] = std::min<uint32_t>(std::max<uint32_t>((v.dims[d] + 2) / 4, 1), 128);
      }
    }
    const float range = vd.value_range[1] - vd.value_range[0];
    const bool refined = sub[0] > 0 && sub[1] > 0 && sub[2] > 0;
    if (!refined)
      for (int d = 0; d < 3; ++d)
        if (sub[d] > 0)
          v.macro_dims[d] = std::min<uint32_t>(std::max<uint32_t>((v.dims[d] + 2) / 4, 1), 128);
    MajorantJob job{};
    for (int d = 0; d < 3; ++d) {
      job.dims[d] = v.dims[d];
      job.macro_dims[d] = v.macro_dims[d];
      job.sub[d] = sub[d];
    }
    job.refined = refined ? 1u : 0u;
    job.complete = complete ? 1u : 0u;
    job.table = uint32_t(table);
    job.value_lo = vd.value_range[0];
    job.range = range;
    job.density_scale = vd.density_scale;
    job.max_opacity = max_opacity;
    const size_t cells_total = size_t(v.macro_dims[0]) * v.macro_dims[1] * v.macro_dims[2];
    const size_t base = s.vol_majorants.size();
    s.vol_majorants.resize(base + cells_total);
    if (tuning().gpu_tables && nvals) { // computed on the device from the uploaded field (upload)
      s.majorant_tasks.push_back({job, uint32_t(base), uint32_t(value_offset), uint32_t(tf_offset)});
    } else {
      const float *vals = vd.values;
      const float *tf = vd.transfer;
      auto alpha = [&](size_t t) { return tf[4 * t + 3]; };
#pragma omp parallel for schedule(dynamic, 1)
      for (int64_t mz = 0; mz < int64_t(v.macro_dims[2]); ++mz)
        for (uint32_t my = 0; my < v.macro_dims[1]; ++my)
          for (uint32_t mx = 0; mx < v.macro_dims[0]; ++mx) {
            const size_t cell = (size_t(mz) * v.macro_dims[1] + my) * v.macro_dims[0] + mx;
            s.vol_majorants[base + cell] = majorant_cell(job, vals, alpha, mx, my, uint32_t(mz));
          }
    }
    if (nvals)
      s.vol_value_spans.push_back({vd.values, nvals}); // copied to the device from the caller's array
    value_offset += nvals;
    tf_offset += table;
    s.volumes.push_back(v);
  }
}

} // namespace

// Appends bottom level `b` (node and triangle indices rebased, triangle
// records' primitive ids offset by prim_base) to the combined arrays.
uint32_t append_blas(Bvh8Host &all, const Bvh8Host &b, uint32_t prim_base)
{
  const uint32_t node_off = all.node_count, tri_off = all.tri_count;
  const size_t n0 = all.nodes.size();
  all.nodes.insert(all.nodes.end(), b.nodes.begin(), b.nodes.end());
  for (size_t k = n0; k < all.nodes.size(); k += 20) {
    all.nodes[k + 4] += node_off; // child base (read only where imask has bits)
    all.nodes[k + 5] += tri_off;  // triangle base
  }
  const size_t t0 = all.tris.size();
  all.tris.insert(all.tris.end(), b.tris.begin(), b.tris.end());
  for (size_t k = t0; k < all.tris.size(); k += 12) {
    uint32_t id;
    std::memcpy(&id, &all.tris[k + 3], 4);
    id += prim_base;
    std::memcpy(&all.tris[k + 3], &id, 4);
  }
  all.node_count += b.node_count;
  all.tri_count += b.tri_count;
  all.max_depth = std::max(all.max_depth, b.max_depth);
  return node_off;
}

// Two-level BVH of a pt scene with instanced geometry (scene.h:18-39): the
// objects' triangles are appended to the vertex and primitive arrays in
// object space, each object gets its own bottom level, and the top level
// holds one leaf per instance plus one for the scene's own triangles (an
// identity placement), the layout of the reference's instanced back-end
// (optix_backend.cpp:502-590) on this renderer's BVH8.
void build_instancing(const phc_pt_scene &pt, bool has_scene_tris, const float lo[3], const float hi[3],
    HostScene &s, int max_leaf)
{
  const uint32_t n_obj = pt.object_count;
  if (!pt.objects)
    throw std::invalid_argument("scene: objects pointer is null");
  if (!pt.instances)
    throw std::invalid_argument("scene: instances pointer is null");
  const uint32_t material_count = uint32_t(s.materials.size());
  const size_t vc0 = s.positions4.size() / 4;
  bool any_normals = s.scene_normals;
  for (uint32_t o = 0; o < n_obj; ++o)
    any_normals = any_normals || (pt.objects[o].normals && pt.objects[o].triangle_count);
  if (any_normals && s.normals4.empty())
    s.normals4.assign(vc0 * 4, 0.f);

  // bottom levels: the scene's triangles, then every object with triangles
  Bvh8Host all;
  all.node_count = 0;
  Bvh8Host scene_blas = std::move(s.bvh);
  std::vector<uint32_t> obj_root(n_obj, 0u), obj_flags(n_obj, 0u);
  std::vector<char> obj_ok(n_obj, 0);
  std::vector<uint64_t> obj_tris(n_obj, 0u);
  std::vector<Bvh8Host> blas(n_obj);
  std::vector<uint32_t> obj_prim_base(n_obj, 0u);
  for (uint32_t o = 0; o < n_obj; ++o) {
    const phc_object &ob = pt.objects[o];
    if (ob.triangle_count == 0 || ob.vertex_count == 0)
      continue;
    if (!ob.positions || !ob.indices)
      throw std::invalid_argument("scene: object positions/indices pointer is null");
    if (ob.triangle_count > 0x3fffffffull || ob.vertex_count > 0xffffffffull)
      throw std::length_error("scene: object too large");
    for (size_t i = 0; i < ob.triangle_count * 3; ++i)
      if (ob.indices[i] >= ob.vertex_count)
        throw std::out_of_range("scene: object vertex index out of range");
    const uint32_t prim_base = uint32_t(s.prim_vidx.size() / 4);
    const uint32_t vbase = uint32_t(s.positions4.size() / 4);
    if (uint64_t(prim_base) + ob.triangle_count > 0x3fffffffull)
      throw std::length_error("scene: too many primitives");
    for (size_t v = 0; v < ob.vertex_count; ++v) {
      for (int a = 0; a < 3; ++a)
        s.positions4.push_back(ob.positions[3 * v + a]);
      s.positions4.push_back(0.f);
      if (any_normals) {
        for (int a = 0; a < 3; ++a)
          s.normals4.push_back(ob.normals ? ob.normals[3 * v + a] : 0.f);
        s.normals4.push_back(0.f);
      }
    }
    const uint32_t mat = ob.material_id < material_count ? ob.material_id : 0u;
    for (size_t t = 0; t < ob.triangle_count; ++t) {
      s.prim_vidx.push_back(vbase + ob.indices[3 * t]);
      s.prim_vidx.push_back(vbase + ob.indices[3 * t + 1]);
      s.prim_vidx.push_back(vbase + ob.indices[3 * t + 2]);
      s.prim_vidx.push_back(mat);
    }
    std::vector<float> geo(size_t(ob.triangle_count) * 12);
    build_prim_records(ob.positions, ob.indices, ob.triangle_count, geo.data());
    for (size_t t = 0; t < ob.triangle_count; ++t) { // record ids are global primitive ids
      const uint32_t id = prim_base + uint32_t(t);
      std::memcpy(&geo[12 * t + 3], &id, 4);
    }
    s.prim_geo.insert(s.prim_geo.end(), geo.begin(), geo.end());
    build_bvh8(ob.positions, ob.vertex_count, ob.indices, ob.triangle_count, blas[o], max_leaf);
    obj_flags[o] = ob.normals ? INST_NORMALS : 0u;
    obj_ok[o] = 1;
    obj_tris[o] = ob.triangle_count;
    obj_prim_base[o] = prim_base;
  }

  // top-level entries: the scene's triangles (identity), then the instances
  struct Entry {
    uint32_t object; // n_obj: the scene's triangles
    double w2o[12];
    float box[6];
  };
  std::vector<Entry> ent;
  if (has_scene_tris) {
    Entry e{};
    e.object = n_obj;
    e.w2o[0] = e.w2o[5] = e.w2o[10] = 1.0;
    for (int a = 0; a < 3; ++a) {
      e.box[a] = lo[a];
      e.box[3 + a] = hi[a];
    }
    ent.push_back(e);
  }
  for (uint32_t i = 0; i < pt.instance_count; ++i) {
    const phc_instance &in = pt.instances[i];
    if (in.object_id >= n_obj || !obj_ok[in.object_id])
      continue; // as the reference's back-end skips them (optix_backend.cpp:511-513)
    // object-to-world rows from the column-major transform
    double m[3][4];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 4; ++c)
        m[r][c] = double(in.transform[c * 4 + r]);
    const double det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
        m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) + m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    if (!(std::fabs(det) > 1e-30) || !std::isfinite(det))
      continue; // a singular placement has no world-to-object map
    Entry e{};
    e.object = in.object_id;
    const double id = 1.0 / det;
    double inv[3][3];
    inv[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) * id;
    inv[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
    inv[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
    inv[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) * id;
    inv[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
    inv[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
    inv[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) * id;
    inv[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
    inv[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
    for (int r = 0; r < 3; ++r) {
      for (int c = 0; c < 3; ++c)
        e.w2o[r * 4 + c] = inv[r][c];
      e.w2o[r * 4 + 3] = -(inv[r][0] * m[0][3] + inv[r][1] * m[1][3] + inv[r][2] * m[2][3]);
    }
    // world box of the placed vertices (tight, unlike the transformed object
    // box), padded so float rounding of the transform never shrinks it below
    // the placed geometry
    const phc_object &obd = pt.objects[in.object_id];
    double wl[3] = {1e300, 1e300, 1e300}, wh[3] = {-1e300, -1e300, -1e300};
    for (size_t v = 0; v < obd.vertex_count; ++v) {
      const float *p = &obd.positions[3 * v];
      for (int r = 0; r < 3; ++r) {
        const double w = m[r][0] * p[0] + m[r][1] * p[1] + m[r][2] * p[2] + m[r][3];
        wl[r] = std::min(wl[r], w);
        wh[r] = std::max(wh[r], w);
      }
    }
    double ext = 0.0;
    for (int r = 0; r < 3; ++r)
      ext = std::max(ext, std::max(std::fabs(wl[r]), std::fabs(wh[r])));
    const double pad = 1e-5 * ext + 1e-30;
    for (int r = 0; r < 3; ++r) {
      e.box[r] = float(wl[r] - pad);
      e.box[3 + r] = float(wh[r] + pad);
    }
    ent.push_back(e);
    s.instanced_triangles += obj_tris[in.object_id];
  }
  if (ent.empty())
    return; // nothing placed: the scene stays single-level
  std::vector<float> boxes(ent.size() * 6);
  for (size_t i = 0; i < ent.size(); ++i)
    std::memcpy(&boxes[6 * i], ent[i].box, sizeof(ent[i].box));
  Bvh8Host tlas;
  build_bvh8_boxes(boxes.data(), boxes.size() / 6, tlas, 1);

  // combined arrays: top level at node 0, then the bottom levels
  all = Bvh8Host{};
  all.nodes = tlas.nodes;
  all.node_count = tlas.node_count;
  all.max_depth = 0;
  uint32_t scene_root = 0;
  if (has_scene_tris)
    scene_root = append_blas(all, scene_blas, 0u);
  for (uint32_t o = 0; o < n_obj; ++o)
    if (obj_ok[o])
      obj_root[o] = append_blas(all, blas[o], obj_prim_base[o]);
  const uint32_t blas_depth = all.max_depth;
  all.max_depth = tlas.max_depth + blas_depth + 1;
  all.sah_cost = tlas.sah_cost;

  // instance records in top-level leaf order
  s.inst_count = uint32_t(tlas.leaf_prims.size());
  s.inst_w2o.assign(size_t(s.inst_count) * 12, 0.f);
  s.inst_info.assign(size_t(s.inst_count) * 4, 0u);
  for (uint32_t j = 0; j < s.inst_count; ++j) {
    const Entry &e = ent[tlas.leaf_prims[j]];
    for (int k = 0; k < 12; ++k)
      s.inst_w2o[12 * size_t(j) + k] = float(e.w2o[k]);
    uint32_t *info = &s.inst_info[4 * size_t(j)];
    if (e.object == n_obj) {
      info[0] = scene_root;
      info[1] = n_obj;
      info[2] = INST_IDENTITY | (s.scene_normals ? INST_NORMALS : 0u);
      info[3] = 0u;
    } else {
      info[0] = obj_root[e.object];
      info[1] = e.object;
      info[2] = obj_flags[e.object];
      info[3] = obj_prim_base[e.object]; // local primitive id = global - base
    }
  }
  s.bvh = std::move(all);
  s.obj_prim_base = obj_prim_base;
  s.obj_prim_count.assign(n_obj, 0u);
  for (uint32_t o = 0; o < n_obj; ++o)
    s.obj_prim_count[o] = uint32_t(obj_tris[o]);
  // primitives of objects have no light pdf (instances do not emit light)
  if (!s.prim_light_pdf.empty())
    s.prim_light_pdf.resize(s.prim_vidx.size() / 4, 0.f);
}

void build_host_scene(const phc_scene_desc &in, HostScene &s)
{
  s = HostScene{};
  size_t vc = in.vertex_count, tc = in.triangle_count;
  if ((vc && !in.positions) || (tc && !in.indices))
    throw std::invalid_argument("scene: positions/indices pointer is null");
  const bool empty = tc == 0 || vc == 0;
  if (empty) { // one degenerate triangle, never hit (RenderBridge.cpp:445-453)
    vc = 3;
    tc = 1;
  }
  if (tc > 0x3fffffffull || vc > 0xffffffffull)
    throw std::length_error("scene: too many triangles or vertices");
  // the per-vertex and per-triangle arrays, each filled by one parallel loop
  // (element by element the same values as a sequential copy)
  HostVec<float> pos3(vc * 3);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < int64_t(vc * 3); ++i)
    pos3[size_t(i)] = empty ? 0.f : in.positions[i];
  // the scene's extent, in vertex order (RenderBridge.cpp:815-820)
  float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
  for (size_t i = 0; i < vc; ++i)
    for (int a = 0; a < 3; ++a) {
      const float p = pos3[3 * i + a];
      lo[a] = lo[a] < p ? lo[a] : p;
      hi[a] = hi[a] > p ? hi[a] : p;
    }
  s.indices.resize(tc * 3);
  int bad_index = 0;
#pragma omp parallel for schedule(static) reduction(| : bad_index)
  for (int64_t i = 0; i < int64_t(tc * 3); ++i) {
    const uint32_t v = empty ? uint32_t(i) : in.indices[i];
    bad_index |= v >= vc ? 1 : 0;
    s.indices[size_t(i)] = v;
  }
  if (bad_index)
    throw std::out_of_range("scene: vertex index out of range");
  const uint32_t material_count = uint32_t(std::max<size_t>(in.material_count, 1));
  s.material_ids.resize(tc);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < int64_t(tc); ++i) {
    const uint32_t id =
        (!empty && in.material_ids && uint64_t(i) < in.material_id_count) ? in.material_ids[i] : 0u;
    s.material_ids[size_t(i)] = id < material_count ? id : 0u;
  }
  s.positions4.resize(vc * 4);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < int64_t(vc); ++i) {
    s.positions4[4 * size_t(i)] = pos3[3 * size_t(i)];
    s.positions4[4 * size_t(i) + 1] = pos3[3 * size_t(i) + 1];
    s.positions4[4 * size_t(i) + 2] = pos3[3 * size_t(i) + 2];
    s.positions4[4 * size_t(i) + 3] = 0.f;
  }
  if (!empty && in.normals) {
    s.normals4.resize(vc * 4);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < int64_t(vc); ++i) {
      s.normals4[4 * size_t(i)] = in.normals[3 * i];
      s.normals4[4 * size_t(i) + 1] = in.normals[3 * i + 1];
      s.normals4[4 * size_t(i) + 2] = in.normals[3 * i + 2];
      s.normals4[4 * size_t(i) + 3] = 0.f;
    }
  }
  s.prim_vidx.resize(tc * 4);
#pragma omp parallel for schedule(static)
  for (int64_t t = 0; t < int64_t(tc); ++t) {
    s.prim_vidx[4 * size_t(t)] = s.indices[3 * size_t(t)];
    s.prim_vidx[4 * size_t(t) + 1] = s.indices[3 * size_t(t) + 1];
    s.prim_vidx[4 * size_t(t) + 2] = s.indices[3 * size_t(t) + 2];
    s.prim_vidx[4 * size_t(t) + 3] = s.material_ids[size_t(t)];
  }
  s.prim_geo.resize(tc * 12);
  build_prim_records(pos3.data(), s.indices.data(), tc, s.prim_geo.data());
  const phc_pt_scene *pt = in.pt;
  if (pt) {
    if (in.material_count && !pt->materials)
      throw std::invalid_argument("scene: pt materials pointer is null");
    if (pt->texture_count && !pt->textures)
      throw std::invalid_argument("scene: pt textures pointer is null");
    // texture coordinates (mesh.texcoords) ride in attribute slot 0 as (u, v,
    // 0, 1): its barycentric interpolation is the hit's uv
    // (mesh_intersector.h:146-163)
    if (!empty && pt->texcoords) {
      s.attr_offset[0] = 0;
      s.attr_values.resize(vc * 4);
      for (size_t i = 0; i < vc; ++i) {
        s.attr_values[4 * i] = pt->texcoords[2 * i];
        s.attr_values[4 * i + 1] = pt->texcoords[2 * i + 1];
        s.attr_values[4 * i + 2] = 0.f;
        s.attr_values[4 * i + 3] = 1.f;
      }
    }
    for (uint32_t i = 0; i < in.material_count; ++i)
      s.materials.push_back(pt_material(pt->materials[i], pt->texture_count));
  } else {
    // attributes (RenderBridge.cpp:489-511)
    size_t total = 0;
    for (int slot = 0; slot < 5; ++slot)
      if (!empty && in.attributes[slot]) {
        s.attr_offset[slot] = int32_t(total);
        total += vc;
      }
    s.attr_values.resize(total * 4);
    for (int slot = 0; slot < 5; ++slot)
      if (s.attr_offset[slot] >= 0)
        std::memcpy(&s.attr_values[size_t(s.attr_offset[slot]) * 4], in.attributes[slot], vc * 16);
    for (uint32_t i = 0; i < in.material_count; ++i)
      s.materials.push_back(convert_material(in.materials[i]));
  }
  if (s.materials.empty())
    s.materials.push_back(default_material());
  for (DevMaterial &m : s.materials)
    m.shade_class = shade_class_of(material_lobes(m));
  // samplers (RenderBridge.cpp:527-571); a pt scene has atlas textures
  // (texture.h:11-65) in their place, RGB widened to float4
  size_t offset = 0;
  for (uint32_t i = 0; pt && i < pt->texture_count; ++i) {
    const phc_texture &td = pt->textures[i];
    DevSampler si{};
    si.type = 4;
    si.size[0] = td.width;
    si.size[1] = td.height;
    si.size[2] = 1;
    si.offset = uint32_t(offset);
    si.grad_offset = uint32_t(offset);
    const size_t n = size_t(td.width) * td.height;
    if (n && !td.rgb)
      throw std::invalid_argument("scene: texture pixels pointer is null");
    const size_t at = s.texels.size();
    s.texels.resize(at + 4 * n);
    for (size_t k = 0; k < n; ++k) {
      s.texels[at + 4 * k] = td.rgb[3 * k];
      s.texels[at + 4 * k + 1] = td.rgb[3 * k + 1];
      s.texels[at + 4 * k + 2] = td.rgb[3 * k + 2];
      s.texels[at + 4 * k + 3] = 1.f;
    }
    offset += n;
    s.samplers.push_back(si);
  }
  // storage offsets: float4 texels (atlas, then fp32 samplers) and uchar4
  // texels (8-bit samplers); `offset` runs over every sampler in order
  size_t f_offset = offset;
  if (!pt && in.sampler_count) {
    s.u8_decode.resize(256);
    for (int k = 0; k < 256; ++k)
      s.u8_decode[size_t(k)] = float(k) / 255.f;
    // room for every sampler's texels, so that packing never moves the array
    size_t cap = 0;
    for (uint32_t i = 0; i < in.sampler_count; ++i)
      cap += in.samplers[i].texels ? 4 * size_t(in.samplers[i].texel_count) : 0;
    if (tuning().texels_u8 && !tuning().gpu_tables)
      s.texels_u8.reserve(cap);
  }
  for (uint32_t i = 0; !pt && i < in.sampler_count; ++i) {
    const phc_sampler &sd = in.samplers[i];
    DevSampler si{};
    si.type = sd.type == 0 ? 0 : (sd.type == 2 ? 2 : (sd.type == 3 ? 3 : 1));
    si.in_attribute = sd.in_attribute;
    si.linear = sd.linear ? 1u : 0u;
    for (int d = 0; d < 3; ++d) {
      si.wrap[d] = sd.wrap[d] == 1 ? 1 : (sd.wrap[d] == 2 ? 2 : 0);
      si.size[d] = std::max<uint32_t>(sd.size[d], 1);
    }
    si.grad_offset = uint32_t(offset);
    std::memcpy(si.in_t, sd.in_transform, sizeof(si.in_t));
    std::memcpy(si.in_o, sd.in_offset, sizeof(si.in_o));
    std::memcpy(si.out_t, sd.out_transform, sizeof(si.out_t));
    std::memcpy(si.out_o, sd.out_offset, sizeof(si.out_o));
    const size_t n = sd.texels ? size_t(sd.texel_count) : 0;
    if (si.type != 3 && n < size_t(si.size[0]) * si.size[1] * si.size[2])
      si.type = 3; // incomplete image: a transform keeps lookups in bounds
    const bool try_u8 = n && si.type != 3 && tuning().texels_u8;
    if (try_u8 && tuning().gpu_tables) { // packed and checked by the upload
      si.u8 = 1;
      si.offset = uint32_t(s.texels_u8_device);
      s.texel_pack_tasks.push_back({sd.texels, n, uint32_t(s.samplers.size()), s.texels_u8_device});
      s.texels_u8_device += n;
    } else if (try_u8 && pack_texels_u8(sd.texels, 4 * n, s)) {
      si.u8 = 1;
      si.offset = uint32_t(s.texels_u8.size() / 4 - n);
    } else {
      si.offset = uint32_t(f_offset);
      if (n)
        s.texel_spans.push_back({sd.texels, 4 * n});
      f_offset += n;
    }
    offset += n;
    s.samplers.push_back(si);
  }
  if (offset > 0xffffffffull)
    throw std::length_error("scene: too many sampler texels");
  s.texel_logical_count = offset;
  for (uint32_t i = 0; i < in.light_count; ++i) {
    const phc_light &ld = in.lights[i];
    DevLight l{};
    l.type = ld.type == 1 ? 1 : (ld.type == 2 ? 2 : 0);
    std::memcpy(l.position, ld.position, sizeof(l.position));
    std::memcpy(l.direction, ld.direction, sizeof(l.direction));
    std::memcpy(l.color, ld.color, sizeof(l.color));
    l.intensity = ld.intensity;
    l.radius = ld.radius;
    l.spot_angle = ld.spot_angle;
    l.spot_falloff = ld.spot_falloff;
    s.lights.push_back(l);
  }
  const phc_environment &env = in.environment;
  if (env.present && env.width > 0 && env.height > 0 && env.pixels) {
    s.env_w = env.width;
    s.env_h = env.height;
    const size_t n = size_t(env.width) * env.height;
    if (tuning().gpu_tables) { // texels and CDFs built by the upload
      s.env_rgb = env.pixels;
      s.env_row_sin.resize(env.height);
      for (uint32_t y = 0; y < env.height; ++y)
        s.env_row_sin[y] = env_row_sin(y, env.height);
    } else {
      s.env_pixels4.resize(n * 4);
      for (size_t k = 0; k < n; ++k) {
        for (int c = 0; c < 3; ++c) {
          const float v = env.pixels[3 * k + c];
          s.env_pixels4[4 * k + c] = std::isfinite(v) && v > 0.f ? v : 0.f;
        }
        s.env_pixels4[4 * k + 3] = 0.f;
      }
    }
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        s.env_w2t[r * 3 + c] = env.world_to_map[r * 3 + c];
        s.env_t2w[c * 3 + r] = env.world_to_map[r * 3 + c];
      }
    if (pt && pt->env_map_to_world_given) // pbrt_to_photon.cpp:455-466
      std::memcpy(s.env_t2w, pt->env_map_to_world, sizeof(s.env_t2w));
    if (!s.env_rgb)
      build_env_cdf(s);
    s.has_env = true;
    s.env_visible = env.visible != 0;
  }
  build_volumes(in, s);
  // emissive triangles (RenderBridge.cpp:780-813) and their selection CDF
  // and area densities (pathtracer.cpp:439-487)
  std::vector<uint32_t> ids;
  std::vector<float> areas;
  const bool instanced = pt && pt->instance_count && pt->object_count;
  s.emissive_on_gpu = !empty && !instanced && tuning().gpu_tables; // built by the upload
  if (!empty && !s.emissive_on_gpu) {
    for (size_t t = 0; t < tc; ++t) {
      const uint32_t mid = s.material_ids[t];
      if (!tbl_may_emit(s.materials[mid]))
        continue;
      const float area = tbl_tri_area(&pos3[3 * size_t(s.indices[3 * t])], &pos3[3 * size_t(s.indices[3 * t + 1])],
          &pos3[3 * size_t(s.indices[3 * t + 2])]);
      if (!(area > 0.f))
        continue;
      ids.push_back(uint32_t(t));
      areas.push_back(area);
    }
  }
  if (!ids.empty()) {
    const uint32_t n = uint32_t(ids.size());
    std::vector<double> weights(n, 0.0);
    double total_w = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
      weights[i] = tbl_emit_weight(s.materials[s.material_ids[ids[i]]], areas[i]);
      total_w += weights[i];
    }
    if (total_w > 0.0) {
      s.emissive_ids = ids;
      s.emissive_cdf.assign(n, 0.f);
      s.prim_light_pdf.assign(tc, 0.f);
      double running = 0.0;
      for (uint32_t i = 0; i < n; ++i) {
        running += weights[i];
        s.emissive_cdf[i] = float(running / total_w);
        if (weights[i] > 0.0 && ids[i] < tc)
          s.prim_light_pdf[ids[i]] = float(weights[i] / total_w / double(areas[i]));
      }
      s.emissive_cdf[n - 1] = 1.f;
    }
  }
  // ray offset relative to the scene size (RenderBridge.cpp:815-820)
  s.eps = 1e-3f;
  if (!empty && hi[0] >= lo[0]) {
    const F3 d{hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    const float e = 1e-4f * len(d);
    s.eps = std::min(std::max(e, 1e-6f), 1e-2f);
  }
  s.strategy_count = uint32_t(s.lights.size()) + (s.emissive_cdf.empty() ? 0u : 1u) + (s.has_env ? 1u : 0u);
  build_search_guides(s);
  s.scene_normals = !empty && in.normals;
  if (tuning().gpu_bvh && !instanced && !empty) {
    s.bvh_on_gpu = true; // single-level scenes: the upload builds the BVH8 on the GPU
    return;
  }
  build_bvh8(pos3.data(), vc, s.indices.data(), tc, s.bvh, tuning().max_leaf);
  if (instanced)
    build_instancing(*pt, !empty, lo, hi, s, tuning().max_leaf);
}

// ------------------------------------------------------------------ upload

DeviceScene::~DeviceScene() { release(); }

void DeviceScene::release()
{
  for (void *p : allocations)
    cudaFree(p);
  allocations.clear();
  dev = DevScene{};
  bytes = 0;
}

template <class T, class A> T *DeviceScene::put(const std::vector<T, A> &v, cudaStream_t s, std::string &err)
{
  if (v.empty() || !err.empty())
    return nullptr;
  void *p = nullptr;
  const size_t n = v.size() * sizeof(T);
  cudaError_t e = cudaMalloc(&p, n);
  if (e != cudaSuccess) {
    err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return nullptr;
  }
  allocations.push_back(p);
  bytes += n;
  e = cudaMemcpyAsync(p, v.data(), n, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess)
    err = std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e);
  return static_cast<T *>(p);
}

// An owned host array followed by spans of the caller's arrays, in one
// device array (texels: the atlas, then every sampler's texels; volume
// values: every volume's field), in the offsets build_host_scene assigned.
float *DeviceScene::put_spans(const std::vector<float> &owned, const std::vector<HostScene::Span> &spans,
    cudaStream_t s, std::string &err)
{
  size_t total = owned.size();
  for (const HostScene::Span &sp : spans)
    total += sp.floats;
  if (total == 0 || !err.empty())
    return nullptr;
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, total * sizeof(float));
  if (e != cudaSuccess) {
    err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return nullptr;
  }
  allocations.push_back(p);
  bytes += total * sizeof(float);
  float *dst = static_cast<float *>(p);
  if (!owned.empty())
    e = cudaMemcpyAsync(dst, owned.data(), owned.size() * sizeof(float), cudaMemcpyHostToDevice, s);
  size_t at = owned.size();
  for (const HostScene::Span &sp : spans) {
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(dst + at, sp.p, sp.floats * sizeof(float), cudaMemcpyHostToDevice, s);
    at += sp.floats;
  }
  if (e != cudaSuccess)
    err = std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e);
  return dst;
}

template <class T> T *DeviceScene::alloc(size_t n, std::string &err, bool keep)
{
  if (!err.empty() || n == 0)
    return nullptr;
  void *p = nullptr;
  const cudaError_t e = cudaMalloc(&p, n * sizeof(T));
  if (e != cudaSuccess) {
    err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
    return nullptr;
  }
  if (keep) {
    allocations.push_back(p);
    bytes += n * sizeof(T);
  }
  return static_cast<T *>(p);
}

// The environment and emitter tables of h built on the device
// (scene_tables.cu; h.env_rgb, h.emissive_on_gpu) into d, with the host
// builders' arithmetic and order, so that they equal the host tables bit for
// bit.  Reads the emitter count, the emitters' weights and the
// monotonicity flags back (waits for the stream); sets the guides only for
// non-decreasing CDFs, and the emitter tables only when their weights sum
// above 0, as the host does.
std::string DeviceScene::device_tables(const HostScene &h, DevScene &d, cudaStream_t s)
{
  std::string err;
  std::vector<void *> scratch;
  auto tmp = [&](size_t bytes_) -> void * {
    void *p = alloc<uint8_t>(bytes_, err, false);
    if (p)
      scratch.push_back(p);
    return p;
  };
  auto ck = [&](cudaError_t e, const char *what) {
    if (e != cudaSuccess && err.empty())
      err = std::string(what) + ": " + cudaGetErrorString(e);
  };
  uint32_t *flags = static_cast<uint32_t *>(tmp(16)); // bad, count
  double tw = 0.0;                                       // the emitters' total weight
  if (flags)
    ck(cudaMemsetAsync(flags, 0, 16, s), "table flags");
  const uint32_t w = h.env_w, eh = h.env_h;
  uint32_t *mguide = nullptr, *cguide = nullptr;
  if (h.env_rgb && err.empty()) {
    EnvTablesJob j{};
    const size_t n = size_t(w) * eh;
    float *rgb = static_cast<float *>(tmp(n * 3 * sizeof(float)));
    float *row_sin = static_cast<float *>(tmp(eh * sizeof(float)));
    j.row_weight = static_cast<float *>(tmp(eh * sizeof(float)));
    if (err.empty()) {
      ck(cudaMemcpyAsync(rgb, h.env_rgb, n * 3 * sizeof(float), cudaMemcpyHostToDevice, s), "environment texels");
      ck(cudaMemcpyAsync(row_sin, h.env_row_sin.data(), eh * sizeof(float), cudaMemcpyHostToDevice, s),
          "environment rows");
    }
    j.rgb = rgb;
    j.row_sin = row_sin;
    j.w = w;
    j.h = eh;
    j.pixels = alloc<float4>(n, err);
    j.conditional = alloc<float>(size_t(eh) * (w + 1), err);
    j.marginal = alloc<float>(size_t(eh) + 1, err);
    j.mguide = mguide = alloc<uint32_t>((1u << ENV_MGUIDE_BITS) + 1, err);
    j.cguide = cguide = alloc<uint32_t>(size_t(eh) * ((1u << ENV_CGUIDE_BITS) + 1), err);
    j.bad = flags;
    if (err.empty())
      err = launch_env_tables(j, s);
    d.env_pixels = j.pixels;
    d.env_conditional = j.conditional;
    d.env_marginal = j.marginal;
    table_floats[PHC_TABLE_ENV_MARGINAL] = size_t(eh) + 1;
    table_floats[PHC_TABLE_ENV_CONDITIONAL] = size_t(eh) * (w + 1);
  }
  EmissiveJob ej{};
  uint32_t counts[4] = {0, 0, 0, 0};
  const uint32_t tc = uint32_t(h.prim_vidx.size() / 4);
  if (h.emissive_on_gpu && err.empty() && tc) {
    ej.pos = d.positions;
    ej.vidx = d.prim_vidx;
    ej.mats = d.materials;
    ej.tc = tc;
    ej.flag = static_cast<uint32_t *>(tmp(size_t(tc) * sizeof(uint32_t)));
    ej.rank = static_cast<uint32_t *>(tmp(size_t(tc) * sizeof(uint32_t)));
    ej.scan_scratch = static_cast<uint32_t *>(tmp(scan_u32_scratch(tc) * sizeof(uint32_t)));
    ej.count = flags + 1;
    ej.bad = flags;
    if (err.empty())
      err = launch_emissive_ids(ej, s);
    if (err.empty()) {
      ck(cudaMemcpyAsync(counts, flags, 8, cudaMemcpyDeviceToHost, s), "emitter count");
      ck(cudaStreamSynchronize(s), "emitter count");
    }
    ej.n = counts[1];
    if (ej.n && err.empty()) {
      ej.ids = alloc<uint32_t>(ej.n, err);
      ej.weight = static_cast<double *>(tmp(size_t(ej.n) * sizeof(double)));
      ej.prefix = static_cast<double *>(tmp(size_t(ej.n) * sizeof(double)));
      ej.cdf = alloc<float>(ej.n, err);
      ej.pdf = alloc<float>(tc, err);
      ej.guide = alloc<uint32_t>((1u << EMISSIVE_GUIDE_BITS) + 1, err);
      if (err.empty())
        ck(cudaMemsetAsync(ej.pdf, 0, size_t(tc) * sizeof(float), s), "emitter densities");
      if (err.empty())
        err = launch_emissive_weights(ej, s);
      // the running sum of the weights is sequential in the reference's
      // double order: one host core runs it (about 1 ns per emitter, against
      // tens of ns for one GPU thread's dependent FP64 adds), between a read
      // of the weights and an upload of the sums
      std::vector<double> w(err.empty() ? ej.n : 0);
      if (err.empty()) {
        ck(cudaMemcpyAsync(w.data(), ej.weight, w.size() * sizeof(double), cudaMemcpyDeviceToHost, s),
            "emitter weights");
        ck(cudaStreamSynchronize(s), "emitter weights");
      }
      if (err.empty()) {
        for (double &x : w) {
          tw += x;
          x = tw;
        }
        ck(cudaMemcpyAsync(ej.prefix, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, s),
            "emitter sums");
      }
      if (err.empty())
        err = launch_emissive_tables(ej, tw, s);
    }
  }
  if (err.empty()) {
    ck(cudaMemcpyAsync(counts, flags, 8, cudaMemcpyDeviceToHost, s), "table flags");
    ck(cudaStreamSynchronize(s), "device tables");
  }
  for (void *p : scratch)
    cudaFree(p);
  if (!err.empty())
    return err;
  if (h.env_rgb) {
    const bool ok = (counts[0] & 3u) == 0;
    d.env_mguide = ok ? mguide : nullptr;
    d.env_cguide = ok ? cguide : nullptr;
  }
  if (h.emissive_on_gpu) {
    const bool any = ej.n > 0 && tw > 0.0;
    d.emissive_ids = any ? ej.ids : nullptr;
    d.emissive_cdf = any ? ej.cdf : nullptr;
    d.prim_light_pdf = any ? ej.pdf : nullptr;
    d.emissive_count = any ? ej.n : 0u;
    d.emissive_guide = any && ej.n > 1 && (counts[0] & 4u) == 0 ? ej.guide : nullptr;
    d.strategy_count = h.strategy_count + (any ? 1u : 0u);
    table_floats[PHC_TABLE_EMISSIVE_CDF] = any ? ej.n : 0;
    table_floats[PHC_TABLE_PRIM_LIGHT_PDF] = any ? tc : 0;
  }
  return std::string();
}

// The samplers of h.texel_pack_tasks: the packing kernel reads their fp32
// texels through a staging buffer and writes the uchar4 array and a flag
// per sampler; a sampler whose flag is set is switched to fp32 storage
// (samplers[i].u8 = 0, its texels appended to the float4 array's spans).
// Waits for the stream.
const uchar4 *DeviceScene::pack_texels(const HostScene &h, std::vector<DevSampler> &samplers,
    std::vector<HostScene::Span> &spans, const float *dec, cudaStream_t s, std::string &err)
{
  constexpr size_t kStage = size_t(1) << 23; // texels per staging copy (128 MiB)
  const size_t n_tasks = h.texel_pack_tasks.size();
  size_t most = 0;
  for (const HostScene::TexelPackTask &t : h.texel_pack_tasks)
    most = std::max(most, t.texels);
  void *out = nullptr, *stage = nullptr, *bad = nullptr;
  cudaError_t e = cudaMalloc(&out, h.texels_u8_device * sizeof(uchar4));
  if (e == cudaSuccess) {
    allocations.push_back(out);
    bytes += h.texels_u8_device * sizeof(uchar4);
    e = cudaMalloc(&bad, n_tasks * sizeof(uint32_t));
  }
  if (e == cudaSuccess)
    e = cudaMemsetAsync(bad, 0, n_tasks * sizeof(uint32_t), s);
  uchar4 *dst = static_cast<uchar4 *>(out);
  // the caller's texels are staged (a kernel reading them in place through
  // the host's page tables measured slower on a first upload: 4 GB/s)
  for (size_t i = 0; i < n_tasks && e == cudaSuccess && err.empty(); ++i) {
    const HostScene::TexelPackTask &t = h.texel_pack_tasks[i];
    if (!stage)
      e = cudaMalloc(&stage, std::min(most, kStage) * sizeof(float4));
    for (size_t at = 0; at < t.texels && e == cudaSuccess && err.empty(); at += kStage) {
      const size_t m = std::min(kStage, t.texels - at);
      e = cudaMemcpyAsync(stage, t.src + 4 * at, m * sizeof(float4), cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess)
        err = launch_pack_texels_u8(static_cast<const float4 *>(stage), m, dec, dst + t.u8_offset + at,
            static_cast<uint32_t *>(bad) + i, s);
    }
  }
  std::vector<uint32_t> flags(n_tasks, 0);
  if (e == cudaSuccess && err.empty())
    e = cudaMemcpyAsync(flags.data(), bad, n_tasks * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && err.empty())
    e = cudaStreamSynchronize(s);
  if (stage)
    cudaFree(stage);
  if (bad)
    cudaFree(bad);
  if (e != cudaSuccess && err.empty())
    err = std::string("texel packing: ") + cudaGetErrorString(e);
  if (!err.empty())
    return nullptr;
  size_t f_end = h.texels.size() / 4;
  for (const HostScene::Span &sp : spans)
    f_end += sp.floats / 4;
  for (size_t i = 0; i < n_tasks; ++i) {
    if (!flags[i])
      continue;
    const HostScene::TexelPackTask &t = h.texel_pack_tasks[i];
    samplers[t.sampler].u8 = 0;
    samplers[t.sampler].offset = uint32_t(f_end);
    spans.push_back({t.src, 4 * t.texels});
    f_end += t.texels;
  }
  return dst;
}

std::string DeviceScene::upload(const HostScene &h, cudaStream_t s)
{
  release();
  std::string err;
  DevScene d{};
  d.nodes = reinterpret_cast<const uint4 *>(put(h.bvh.nodes, s, err));
  d.tris = reinterpret_cast<const float4 *>(put(h.bvh.tris, s, err));
  d.prim_geo = reinterpret_cast<const float4 *>(put(h.prim_geo, s, err));
  d.prim_vidx = reinterpret_cast<const uint4 *>(put(h.prim_vidx, s, err));
  d.normals = reinterpret_cast<const float4 *>(put(h.normals4, s, err));
  d.positions = reinterpret_cast<const float4 *>(put(h.positions4, s, err));
  d.node_count = h.bvh.node_count;
  d.prim_count = uint32_t(h.material_ids.size());
  d.materials = put(h.materials, s, err);
  d.material_count = uint32_t(h.materials.size());
  d.attr_values = reinterpret_cast<const float4 *>(put(h.attr_values, s, err));
  std::memcpy(d.attr_offset, h.attr_offset, sizeof(d.attr_offset));
  d.u8_decode = put(h.u8_decode, s, err);
  std::vector<DevSampler> samplers = h.samplers;
  std::vector<HostScene::Span> texel_spans = h.texel_spans;
  if (h.texel_pack_tasks.empty())
    d.texels_u8 = reinterpret_cast<const uchar4 *>(put(h.texels_u8, s, err));
  else if (err.empty())
    d.texels_u8 = pack_texels(h, samplers, texel_spans, d.u8_decode, s, err);
  d.samplers = put(samplers, s, err);
  d.sampler_count = uint32_t(samplers.size());
  d.texels = reinterpret_cast<const float4 *>(put_spans(h.texels, texel_spans, s, err));
  d.lights = put(h.lights, s, err);
  d.light_count = uint32_t(h.lights.size());
  d.emissive_ids = put(h.emissive_ids, s, err);
  d.emissive_cdf = put(h.emissive_cdf, s, err);
  d.prim_light_pdf = put(h.prim_light_pdf, s, err);
  d.emissive_count = uint32_t(h.emissive_cdf.size());
  d.env_pixels = reinterpret_cast<const float4 *>(put(h.env_pixels4, s, err));
  d.env_marginal = put(h.env_marginal, s, err);
  d.env_conditional = put(h.env_conditional, s, err);
  d.emissive_guide = h.emissive_guide.empty() ? nullptr : put(h.emissive_guide, s, err);
  d.env_mguide = h.env_mguide.empty() ? nullptr : put(h.env_mguide, s, err);
  d.env_cguide = h.env_cguide.empty() ? nullptr : put(h.env_cguide, s, err);
  d.env_w = h.env_w;
  d.env_h = h.env_h;
  std::memcpy(d.env_w2t, h.env_w2t, sizeof(d.env_w2t));
  std::memcpy(d.env_t2w, h.env_t2w, sizeof(d.env_t2w));
  d.has_env = h.has_env ? 1 : 0;
  d.env_visible = h.env_visible ? 1 : 0;
  d.volumes = put(h.volumes, s, err);
  d.volume_count = uint32_t(h.volumes.size());
  d.vol_values = put_spans(h.vol_values, h.vol_value_spans, s, err);
  d.vol_tf = reinterpret_cast<const float4 *>(put(h.vol_tf, s, err));
  float *majorants = put(h.vol_majorants, s, err);
  d.vol_majorants = majorants;
  for (const HostScene::MajorantTask &t : h.majorant_tasks)
    if (err.empty())
      err = launch_majorants(t.job, d.vol_values + t.data_offset, d.vol_tf + t.tf_offset,
          majorants + t.macro_offset, s);
  d.strategy_count = h.strategy_count;
  d.eps = h.eps;
  d.inst_w2o = reinterpret_cast<const float4 *>(put(h.inst_w2o, s, err));
  d.inst_info = reinterpret_cast<const uint4 *>(put(h.inst_info, s, err));
  d.inst_count = h.inst_count;
  d.scene_object_id = uint32_t(h.obj_prim_base.size());
  d.scene_normals = h.scene_normals ? 1 : 0;
  d.features = h.inst_count ? SCENE_INSTANCES : 0u;
  if (!h.volumes.empty())
    d.features |= SCENE_VOLUMES;
  if (!h.lights.empty())
    d.features |= SCENE_LIGHTS;
  for (const DevMaterial &m : h.materials) {
    for (int k = 0; k < 7; ++k)
      if (m.src_kind[k] != 0)
        d.features |= SCENE_SOURCES;
    if (m.base_tex >= 0 || m.alpha_tex >= 0)
      d.features |= SCENE_SOURCES;
  }
  node_bytes = uint64_t(h.bvh.nodes.size()) * 4;
  tri_bytes = uint64_t(h.bvh.tris.size()) * 4;
  bvh_depth = h.bvh.max_depth;
  texel_count = h.texel_logical_count;
  uint32_t class_mask = 0u;
  for (const DevMaterial &m : h.materials)
    class_mask |= 1u << (m.shade_class % SHADE_CLASSES);
  shade_class_count = uint32_t(__builtin_popcount(class_mask));
  table_floats[PHC_TABLE_MAJORANTS] = h.vol_majorants.size();
  table_floats[PHC_TABLE_ENV_MARGINAL] = h.env_marginal.size();
  table_floats[PHC_TABLE_ENV_CONDITIONAL] = h.env_conditional.size();
  table_floats[PHC_TABLE_EMISSIVE_CDF] = h.emissive_cdf.size();
  table_floats[PHC_TABLE_PRIM_LIGHT_PDF] = h.prim_light_pdf.size();
  if (err.empty() && (h.env_rgb || h.emissive_on_gpu))
    err = device_tables(h, d, s);
  if (!err.empty()) {
    release();
    return err;
  }
  if (h.bvh_on_gpu) {
    try {
      const GpuBvh8 g = build_bvh8_gpu(d.positions, d.prim_vidx, uint32_t(h.prim_vidx.size() / 4), s,
          tuning().gpu_max_leaf, tuning().ploc_radius, 0.01f * float(tuning().collapse_tri_cost));
      allocations.push_back(g.nodes);
      allocations.push_back(g.tris);
      bytes += size_t(g.node_cap) * 80 + size_t(g.tri_count) * 48;
      d.nodes = static_cast<const uint4 *>(g.nodes);
      d.tris = static_cast<const float4 *>(g.tris);
      d.node_count = g.node_count;
      node_bytes = uint64_t(g.node_count) * 80;
      tri_bytes = uint64_t(g.tri_count) * 48;
      bvh_depth = g.max_depth;
    } catch (const std::exception &ex) {
      release();
      return ex.what();
    }
  }
  const cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    release();
    return std::string("scene upload: ") + cudaGetErrorString(e);
  }
  dev = d;
  return std::string();
}

} // namespace phc
