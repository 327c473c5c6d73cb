// C entry points over the reference's own pbrt path: parse_pbrt_file
// (src/photon/pbrt/pbrt_parser.cpp), convert_pbrt_scene
// (src/photon/pbrt/pbrt_to_photon.cpp) and PathTracer::render, compiled
// unmodified against the project's Kokkos and stb_image stand-ins
// (oracle/kokkos_shim, oracle/stb_shim) into oracle/_ref/libphoton_ref.so.
// TEST INFRASTRUCTURE ONLY: the pbrt tests and the fixture generator read the
// converted scene and the reference's render through it, to pin the
// product's pbrt reader (photon_gb300/csrc/pbrt_reader.cpp).
//
// ref_pbrt_render runs the scene the way app/photon_pbrt_render.cpp:141-161
// does (KokkosBackend::build_accel_instanced, PathTracer with the file's
// size, spp and depth and RenderParams' defaults), with two switches for
// per-sample comparisons: adaptive sampling, and bottom_up (the bridge
// renders bottom-up, RenderBridge.cpp:913; the application top-down).
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>

#include "photon/pbrt/pbrt_parser.h"
#include "photon/pbrt/pbrt_to_photon.h"
#include "photon/pt/backend/ray_backend.h"
#include "photon/pt/pathtracer.h"
#include "photon_cuda.h"

namespace {

struct RefPbrt {
  photon::pbrt::PbrtScene parsed;
  photon::pbrt::ConvertedScene conv;
};

void put3(float *d, const photon::pt::Vec3 &v)
{
  d[0] = v.x;
  d[1] = v.y;
  d[2] = v.z;
}

} // namespace

extern "C" {

void *ref_pbrt_load(const char *path, int use_instancing, int width, int height, int spp, int max_depth)
{
  auto h = std::make_unique<RefPbrt>();
  h->parsed = photon::pbrt::parse_pbrt_file(path, use_instancing != 0);
  if (width > 0)
    h->parsed.width = width;
  if (height > 0)
    h->parsed.height = height;
  if (spp > 0)
    h->parsed.spp = spp;
  if (max_depth > 0)
    h->parsed.max_depth = max_depth;
  std::string base;
  const std::string p(path);
  const size_t s = p.find_last_of("/\\");
  if (s != std::string::npos)
    base = p.substr(0, s + 1);
  h->conv = photon::pbrt::convert_pbrt_scene(h->parsed, base);
  return h.release();
}

void ref_pbrt_free(void *h) { delete static_cast<RefPbrt *>(h); }

// counts: triangles, materials, emissive, textures, lights, width, height,
// spp, max_depth, meshes, named materials, object defs, object instances,
// has env map
int ref_pbrt_counts(void *hv, uint64_t *out)
{
  const auto *h = static_cast<RefPbrt *>(hv);
  const auto &sc = h->conv.scene;
  out[0] = sc.mesh.triangle_count();
  out[1] = sc.material_count;
  out[2] = sc.emissive_count;
  out[3] = sc.textures.count;
  out[4] = sc.light_count;
  out[5] = uint64_t(h->parsed.width);
  out[6] = uint64_t(h->parsed.height);
  out[7] = uint64_t(h->parsed.spp);
  out[8] = uint64_t(h->parsed.max_depth);
  out[9] = h->parsed.meshes.size();
  out[10] = h->parsed.named_materials.size();
  out[11] = h->parsed.object_defs.size();
  out[12] = h->parsed.object_instances.size();
  out[13] = sc.env_map.has_value() ? 1u : 0u;
  return 0;
}

// The flattened mesh: 3 * triangles vertices (positions, normals xyz, uv).
int ref_pbrt_mesh(void *hv, float *positions, float *normals, float *uv, uint32_t *material_ids, uint32_t *indices)
{
  const auto &m = static_cast<RefPbrt *>(hv)->conv.scene.mesh;
  const size_t nv = m.positions.extent(0);
  for (size_t i = 0; i < nv; ++i) {
    put3(positions + 3 * i, m.positions(i));
    put3(normals + 3 * i, m.normals(i));
    uv[2 * i] = m.texcoords(i).x;
    uv[2 * i + 1] = m.texcoords(i).y;
  }
  for (size_t i = 0; i < m.indices.extent(0); ++i)
    indices[i] = m.indices(i);
  for (size_t t = 0; t < m.material_ids.extent(0); ++t)
    material_ids[t] = m.material_ids(t);
  return 0;
}

int ref_pbrt_materials(void *hv, phc_pt_material *out)
{
  const auto &sc = static_cast<RefPbrt *>(hv)->conv.scene;
  for (uint32_t i = 0; i < sc.material_count; ++i) {
    const photon::pt::Material &m = sc.materials(i);
    phc_pt_material &d = out[i];
    std::memset(&d, 0, sizeof(d));
    put3(d.base_color, m.base_color);
    d.metallic = m.metallic;
    d.roughness = m.roughness;
    d.ior = m.ior;
    d.transmission = m.transmission;
    d.specular = m.specular;
    d.clearcoat = m.clearcoat;
    d.clearcoat_roughness = m.clearcoat_roughness;
    d.sheen = m.sheen;
    d.alpha = m.alpha;
    put3(d.emission, m.emission);
    d.emission_strength = m.emission_strength;
    d.flags = m.flags;
    d.base_color_tex = m.base_color_tex;
    d.alpha_tex = m.alpha_tex;
  }
  return 0;
}

int ref_pbrt_emissive(void *hv, uint32_t *ids, float *areas)
{
  const auto &sc = static_cast<RefPbrt *>(hv)->conv.scene;
  for (uint32_t i = 0; i < sc.emissive_count; ++i) {
    ids[i] = sc.emissive_prim_ids(i);
    areas[i] = sc.emissive_prim_areas(i);
  }
  return 0;
}

// origin, lower_left, horizontal, vertical, u, v, w (21 floats), lens
// radius, focus distance
int ref_pbrt_camera(void *hv, float *out)
{
  const auto &c = static_cast<RefPbrt *>(hv)->conv.camera;
  put3(out, c.origin);
  put3(out + 3, c.lower_left);
  put3(out + 6, c.horizontal);
  put3(out + 9, c.vertical);
  put3(out + 12, c.u);
  put3(out + 15, c.v);
  put3(out + 18, c.w);
  out[21] = c.lens_radius;
  out[22] = c.focus_dist;
  return 0;
}

// width, height; pixels (row 0 first, may be null); world_to_tex, tex_to_world
int ref_pbrt_env(void *hv, uint32_t *wh, float *pixels, float *w2t, float *t2w)
{
  const auto &sc = static_cast<RefPbrt *>(hv)->conv.scene;
  if (!sc.env_map.has_value()) {
    wh[0] = wh[1] = 0;
    return 0;
  }
  const auto &e = *sc.env_map;
  wh[0] = e.width;
  wh[1] = e.height;
  if (pixels)
    for (uint32_t y = 0; y < e.height; ++y)
      for (uint32_t x = 0; x < e.width; ++x)
        put3(pixels + 3 * (size_t(y) * e.width + x), e.pixels(y, x));
  std::memcpy(w2t, e.world_to_tex, sizeof(e.world_to_tex));
  std::memcpy(t2w, e.tex_to_world, sizeof(e.tex_to_world));
  return 0;
}

// texture i of the atlas: width, height, then RGB when rgb is not null
int ref_pbrt_texture(void *hv, uint32_t i, uint32_t *wh, float *rgb)
{
  const auto &t = static_cast<RefPbrt *>(hv)->conv.scene.textures;
  if (i >= t.count)
    return -1;
  const photon::pt::TextureInfo ti = t.infos(i);
  wh[0] = ti.width;
  wh[1] = ti.height;
  if (rgb)
    for (uint32_t k = 0; k < ti.width * ti.height; ++k)
      put3(rgb + 3 * size_t(k), t.pixels(ti.offset + k));
  return 0;
}

// Instanced geometry of the conversion (ConvertedScene::instanced_geometry):
// counts of objects and instances.
int ref_pbrt_ig_counts(void *hv, uint64_t *out)
{
  const auto &ig = static_cast<RefPbrt *>(hv)->conv.instanced_geometry;
  out[0] = ig.objects.size();
  out[1] = ig.instances.size();
  return 0;
}

// Object i: sizes (position floats, indices, normal floats, material id),
// then the arrays when the pointers are not null.
int ref_pbrt_ig_object(void *hv, uint32_t i, uint64_t *sizes, float *pos, int32_t *idx, float *nrm)
{
  const auto &ig = static_cast<RefPbrt *>(hv)->conv.instanced_geometry;
  if (i >= ig.objects.size())
    return -1;
  const auto &o = ig.objects[i];
  sizes[0] = o.positions.size();
  sizes[1] = o.indices.size();
  sizes[2] = o.normals.size();
  sizes[3] = o.material_id;
  if (pos)
    std::memcpy(pos, o.positions.data(), o.positions.size() * sizeof(float));
  if (idx)
    std::memcpy(idx, o.indices.data(), o.indices.size() * sizeof(int32_t));
  if (nrm)
    std::memcpy(nrm, o.normals.data(), o.normals.size() * sizeof(float));
  return 0;
}

int ref_pbrt_ig_instance(void *hv, uint32_t i, uint32_t *object_id, float *xf16)
{
  const auto &ig = static_cast<RefPbrt *>(hv)->conv.instanced_geometry;
  if (i >= ig.instances.size())
    return -1;
  *object_id = ig.instances[i].object_id;
  std::memcpy(xf16, ig.instances[i].transform, 16 * sizeof(float));
  return 0;
}

// Renders the converted scene; rgb gets width*height*3 floats, row 0 first.
int ref_pbrt_render(void *hv, int adaptive, int bottom_up, float *rgb)
{
  auto *h = static_cast<RefPbrt *>(hv);
  auto backend = photon::pt::create_best_backend();
  backend->build_accel_instanced(h->conv.scene, h->conv.instanced_geometry);
  photon::pt::PathTracer pt;
  pt.params.width = uint32_t(h->parsed.width);
  pt.params.height = uint32_t(h->parsed.height);
  pt.params.samples_per_pixel = uint32_t(h->parsed.spp);
  pt.params.max_depth = uint32_t(h->parsed.max_depth);
  pt.params.adaptive_sampling = adaptive != 0;
  pt.params.bottom_up = bottom_up != 0;
  pt.camera = h->conv.camera;
  pt.set_scene(h->conv.scene);
  pt.set_backend(std::move(backend));
  const auto result = pt.render();
  for (uint32_t y = 0; y < pt.params.height; ++y)
    for (uint32_t x = 0; x < pt.params.width; ++x)
      put3(rgb + 3 * (size_t(y) * pt.params.width + x), result.color(y, x));
  return 0;
}

} // extern "C"
