// C entry points over Photon's own path-tracing sources, compiled unmodified
// against the project's Kokkos stand-in (oracle/kokkos_shim) into
// oracle/_ref/libphoton_ref.so.  TEST INFRASTRUCTURE ONLY: the tests and the
// fixture generator call it to pin the CPU restatement (photon_oracle.cpp) and
// the CUDA path against the reference's own code.  Nothing in the product
// links or loads it.
//
// The scene, camera and settings arrive as the C-ABI structs of
// include/photon_cuda.h and are converted field by field into
// photon::bridge::SceneData / CameraData / RenderSettings
// (src/photon/anari/RenderBridge.h:21-170), then handed to the reference's
// bridge::Renderer (RenderBridge.cpp:1012-1172), which runs PathTracer::render
// (src/photon/pt/pathtracer.cpp:564-1159) over KokkosBackend
// (src/photon/pt/backend/kokkos_backend.cpp).
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "photon/anari/RenderBridge.h"
#include "photon/pt/backend/kokkos_backend.h"
#include "photon/pt/disney_bsdf.h"
#include "photon/pt/geom/mesh_intersector.h"
#include "photon/pt/scene.h"
#include "photon_cuda.h"

namespace {

using namespace photon;

thread_local std::string g_error;

bridge::ParamSourceData conv(const phc_param_source &s)
{
  bridge::ParamSourceData d;
  d.kind = s.kind;
  d.index = s.index;
  return d;
}

void convert_scene(const phc_scene_desc &in, bridge::SceneData &out)
{
  out.positions.assign(in.positions, in.positions + 3 * in.vertex_count);
  if (in.normals)
    out.normals.assign(in.normals, in.normals + 3 * in.vertex_count);
  for (int s = 0; s < 5; ++s)
    if (in.attributes[s])
      out.attributes[s].assign(in.attributes[s], in.attributes[s] + 4 * in.vertex_count);
  out.indices.assign(in.indices, in.indices + 3 * in.triangle_count);
  if (in.material_ids)
    out.material_ids.assign(in.material_ids, in.material_ids + in.material_id_count);
  for (uint32_t i = 0; i < in.material_count; ++i) {
    const phc_material &m = in.materials[i];
    bridge::MaterialData d;
    std::memcpy(d.base_color, m.base_color, sizeof(d.base_color));
    d.opacity = m.opacity;
    d.metallic = m.metallic;
    d.roughness = m.roughness;
    d.ior = m.ior;
    d.transmission = m.transmission;
    d.specular = m.specular;
    std::memcpy(d.emission, m.emission, sizeof(d.emission));
    d.clearcoat = m.clearcoat;
    d.clearcoat_roughness = m.clearcoat_roughness;
    d.sheen = m.sheen;
    d.base_color_src = conv(m.base_color_src);
    d.opacity_src = conv(m.opacity_src);
    d.metallic_src = conv(m.metallic_src);
    d.roughness_src = conv(m.roughness_src);
    d.emission_src = conv(m.emission_src);
    d.transmission_src = conv(m.transmission_src);
    d.normal_src = conv(m.normal_src);
    d.alpha_mode = m.alpha_mode;
    d.alpha_cutoff = m.alpha_cutoff;
    d.base_color_alpha = m.base_color_alpha != 0;
    d.thin_walled = m.thin_walled != 0;
    d.emitter_only = m.emitter_only != 0;
    d.hidden_to_camera = m.hidden_to_camera != 0;
    d.emission_side = m.emission_side;
    out.materials.push_back(d);
  }
  for (uint32_t i = 0; i < in.sampler_count; ++i) {
    const phc_sampler &s = in.samplers[i];
    bridge::SamplerData d;
    d.type = s.type;
    d.in_attribute = s.in_attribute;
    d.linear = s.linear != 0;
    for (int k = 0; k < 3; ++k) {
      d.wrap[k] = s.wrap[k];
      d.size[k] = s.size[k];
    }
    std::memcpy(d.in_transform, s.in_transform, sizeof(d.in_transform));
    std::memcpy(d.in_offset, s.in_offset, sizeof(d.in_offset));
    std::memcpy(d.out_transform, s.out_transform, sizeof(d.out_transform));
    std::memcpy(d.out_offset, s.out_offset, sizeof(d.out_offset));
    if (s.texels)
      d.texels.assign(s.texels, s.texels + 4 * s.texel_count);
    out.samplers.push_back(std::move(d));
  }
  for (uint32_t i = 0; i < in.light_count; ++i) {
    const phc_light &l = in.lights[i];
    bridge::LightData d;
    d.type = l.type;
    std::memcpy(d.position, l.position, sizeof(d.position));
    std::memcpy(d.direction, l.direction, sizeof(d.direction));
    std::memcpy(d.color, l.color, sizeof(d.color));
    d.intensity = l.intensity;
    d.radius = l.radius;
    d.spot_angle = l.spot_angle;
    d.spot_falloff = l.spot_falloff;
    out.lights.push_back(d);
  }
  const phc_environment &e = in.environment;
  out.environment.present = e.present != 0;
  out.environment.visible = e.visible != 0;
  out.environment.width = e.width;
  out.environment.height = e.height;
  if (e.pixels)
    out.environment.pixels.assign(e.pixels, e.pixels + size_t(e.width) * e.height * 3);
  std::memcpy(out.environment.world_to_map, e.world_to_map, sizeof(e.world_to_map));
  for (uint32_t i = 0; i < in.volume_count; ++i) {
    const phc_volume &v = in.volumes[i];
    bridge::VolumeData d;
    std::memcpy(d.world_to_local, v.world_to_local, sizeof(d.world_to_local));
    std::memcpy(d.origin, v.origin, sizeof(d.origin));
    std::memcpy(d.spacing, v.spacing, sizeof(d.spacing));
    for (int k = 0; k < 3; ++k)
      d.dims[k] = v.dims[k];
    if (v.values)
      d.values.assign(v.values, v.values + v.value_count);
    if (v.transfer)
      d.transfer.assign(v.transfer, v.transfer + 4 * size_t(v.transfer_count));
    d.value_range[0] = v.value_range[0];
    d.value_range[1] = v.value_range[1];
    d.density_scale = v.density_scale;
    d.linear = v.linear != 0;
    out.volumes.push_back(std::move(d));
  }
}

void convert_camera(const phc_camera &c, bridge::CameraData &d)
{
  std::memcpy(d.position, c.position, sizeof(d.position));
  std::memcpy(d.direction, c.direction, sizeof(d.direction));
  std::memcpy(d.up, c.up, sizeof(d.up));
  d.orthographic = c.orthographic != 0;
  d.fovy = c.fovy;
  d.height = c.height;
  d.aspect = c.aspect;
  d.aperture_radius = c.aperture_radius;
  d.focus_distance = c.focus_distance;
  std::memcpy(d.image_region, c.image_region, sizeof(d.image_region));
  d.clip_near = c.clip_near;
  d.clip_far = c.clip_far;
}

void convert_settings(const phc_settings &s, bridge::RenderSettings &d)
{
  d.width = s.width;
  d.height = s.height;
  d.pixel_samples = s.pixel_samples;
  d.max_depth = s.max_depth;
  std::memcpy(d.background, s.background, sizeof(d.background));
  d.background_image = s.background_image;
  d.background_width = s.background_width;
  d.background_height = s.background_height;
  std::memcpy(d.ambient_color, s.ambient_color, sizeof(d.ambient_color));
  d.ambient_radiance = s.ambient_radiance;
  d.adaptive_sampling = s.adaptive_sampling != 0;
  d.throughput_clamp = s.throughput_clamp;
  d.max_diffuse_bounces = s.max_diffuse_bounces;
  d.max_glossy_bounces = s.max_glossy_bounces;
  d.max_transmission_bounces = s.max_transmission_bounces;
  d.max_volume_bounces = s.max_volume_bounces;
  d.clamp_direct = s.clamp_direct;
  d.clamp_indirect = s.clamp_indirect;
}

struct RefRenderer
{
  bridge::Renderer renderer;
  std::string error;
};

int fail(RefRenderer *r, const std::string &msg)
{
  if (r)
    r->error = msg;
  g_error = msg;
  return -1;
}

} // namespace

extern "C" {

const char *ref_global_error() { return g_error.c_str(); }

void *ref_renderer_create()
{
  auto *r = new RefRenderer();
  std::string err;
  if (!r->renderer.initialize(err)) {
    g_error = err;
    delete r;
    return nullptr;
  }
  return r;
}

void ref_renderer_destroy(void *h) { delete static_cast<RefRenderer *>(h); }

const char *ref_last_error(void *h) { return static_cast<RefRenderer *>(h)->error.c_str(); }

const char *ref_backend_name(void *h)
{
  static thread_local std::string name;
  name = static_cast<RefRenderer *>(h)->renderer.backend_name();
  return name.c_str();
}

int ref_set_scene(void *h, const phc_scene_desc *desc)
{
  auto *r = static_cast<RefRenderer *>(h);
  bridge::SceneData scene;
  convert_scene(*desc, scene);
  std::string err;
  if (!r->renderer.set_scene(scene, err))
    return fail(r, err);
  return 0;
}

int ref_render(void *h, const phc_camera *cam, const phc_settings *settings, int reset)
{
  auto *r = static_cast<RefRenderer *>(h);
  bridge::CameraData c;
  bridge::RenderSettings s;
  convert_camera(*cam, c);
  convert_settings(*settings, s);
  std::string err;
  if (!r->renderer.render(c, s, reset != 0, err))
    return fail(r, err);
  return 0;
}

uint32_t ref_accumulated_samples(void *h) { return static_cast<RefRenderer *>(h)->renderer.accumulated_samples(); }

int ref_read_color(void *h, float *out)
{
  auto *r = static_cast<RefRenderer *>(h);
  std::string err;
  return r->renderer.read_color(out, err) ? 0 : fail(r, err);
}

int ref_read_depth(void *h, float *out)
{
  auto *r = static_cast<RefRenderer *>(h);
  std::string err;
  return r->renderer.read_depth(out, err) ? 0 : fail(r, err);
}

int ref_read_normal(void *h, float *out)
{
  auto *r = static_cast<RefRenderer *>(h);
  std::string err;
  return r->renderer.read_normal(out, err) ? 0 : fail(r, err);
}

int ref_read_albedo(void *h, float *out)
{
  auto *r = static_cast<RefRenderer *>(h);
  std::string err;
  return r->renderer.read_albedo(out, err) ? 0 : fail(r, err);
}

// Level A through the reference's KokkosBackend: builds Bvh::build_cpu over
// the mesh and traces n rays (host arrays).  any_hit selects trace_occluded.
int ref_trace(const float *positions, uint64_t vertex_count, const uint32_t *indices, uint64_t triangle_count,
    const float *normals, const uint32_t *material_ids, const float *orgs, const float *dirs, const float *tmin,
    const float *tmax, uint32_t n, int any_hit, phc_hit_result *hits, uint32_t *occluded)
{
  using namespace photon::pt;
  Scene scene;
  scene.mesh.positions = Kokkos::View<Vec3 *>("pos", vertex_count);
  scene.mesh.indices = Kokkos::View<u32 *>("idx", triangle_count * 3);
  for (uint64_t i = 0; i < vertex_count; ++i)
    scene.mesh.positions(i) = Vec3{positions[3 * i], positions[3 * i + 1], positions[3 * i + 2]};
  for (uint64_t i = 0; i < triangle_count * 3; ++i)
    scene.mesh.indices(i) = indices[i];
  if (normals) {
    scene.mesh.normals = Kokkos::View<Vec3 *>("nrm", vertex_count);
    for (uint64_t i = 0; i < vertex_count; ++i)
      scene.mesh.normals(i) = Vec3{normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]};
  }
  if (material_ids) {
    scene.mesh.material_ids = Kokkos::View<u32 *>("mat", triangle_count);
    for (uint64_t i = 0; i < triangle_count; ++i)
      scene.mesh.material_ids(i) = material_ids[i];
  }
  KokkosBackend backend;
  backend.build_accel(scene);
  RayBatch rays;
  rays.origins = Kokkos::View<Vec3 *>("o", n);
  rays.directions = Kokkos::View<Vec3 *>("d", n);
  rays.tmin = Kokkos::View<f32 *>("tmin", n);
  rays.tmax = Kokkos::View<f32 *>("tmax", n);
  rays.count = n;
  for (uint32_t i = 0; i < n; ++i) {
    rays.origins(i) = Vec3{orgs[3 * i], orgs[3 * i + 1], orgs[3 * i + 2]};
    rays.directions(i) = Vec3{dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]};
    rays.tmin(i) = tmin[i];
    rays.tmax(i) = tmax[i];
  }
  if (any_hit) {
    Kokkos::View<u32 *> occ("occ", n);
    backend.trace_occluded(rays, occ);
    for (uint32_t i = 0; i < n; ++i)
      occluded[i] = occ(i);
    return 0;
  }
  HitBatch hb;
  hb.hits = Kokkos::View<HitResult *>("hits", n);
  hb.count = n;
  backend.trace_closest(rays, hb);
  static_assert(sizeof(HitResult) == sizeof(phc_hit_result), "hit record layout");
  for (uint32_t i = 0; i < n; ++i) {
    const HitResult &h = hb.hits(i);
    phc_hit_result &o = hits[i];
    std::memset(&o, 0, sizeof(o));
    o.hit = h.hit ? 1 : 0;
    if (!h.hit)
      continue;
    o.t = h.t;
    o.position[0] = h.position.x; o.position[1] = h.position.y; o.position[2] = h.position.z;
    o.normal[0] = h.normal.x; o.normal[1] = h.normal.y; o.normal[2] = h.normal.z;
    o.shading_normal[0] = h.shading_normal.x; o.shading_normal[1] = h.shading_normal.y;
    o.shading_normal[2] = h.shading_normal.z;
    o.uv[0] = h.uv.x; o.uv[1] = h.uv.y;
    o.bary[0] = h.bary.x; o.bary[1] = h.bary.y;
    o.interpolated_color[0] = h.interpolated_color.x; o.interpolated_color[1] = h.interpolated_color.y;
    o.interpolated_color[2] = h.interpolated_color.z;
    o.prim_id = h.prim_id;
    o.geom_id = h.geom_id;
    o.inst_id = h.inst_id;
    o.material_id = h.material_id;
    o.has_interpolated_color = h.has_interpolated_color ? 1 : 0;
  }
  return 0;
}

// Disney BSDF probes (include/photon/pt/disney_bsdf.h:288-521) on a material
// given as the bridge does it (convert_material, RenderBridge.cpp:324-370),
// for unit-level parity of the BSDF: for each of n (wo, wi, seed) cases,
// out[8*i .. 8*i+7] = eval.xyz, pdf, sample.wi.xyz, sample.pdf and
// out2[4*i .. 4*i+3] = sample.f.xyz, flags (1 specular | 2 diffuse).
int ref_bsdf_probe(const phc_material *m, const float *n_geo, const float *n_shade, const float *wo, const float *wi,
    const uint32_t *seeds, uint32_t n, float *out, float *out2)
{
  using namespace photon::pt;
  bridge::SceneData scene;
  phc_scene_desc d{};
  (void)d;
  // Same conversion the bridge applies (RenderBridge.cpp:324-370).
  Material mat;
  mat.base_color = Vec3{m->base_color[0], m->base_color[1], m->base_color[2]};
  mat.metallic = m->metallic;
  mat.roughness = m->roughness * m->roughness;
  mat.ior = m->ior;
  mat.transmission = m->transmission;
  mat.specular = 0.5f * m->specular;
  mat.clearcoat = m->clearcoat;
  mat.clearcoat_roughness = m->clearcoat_roughness;
  mat.sheen = m->sheen;
  mat.thin = m->thin_walled ? 1 : 0;
  mat.flags = MATERIAL_FLAG_REFRACTIVE;
  for (uint32_t i = 0; i < n; ++i) {
    const Vec3 ng{n_geo[3 * i], n_geo[3 * i + 1], n_geo[3 * i + 2]};
    const Vec3 ns{n_shade[3 * i], n_shade[3 * i + 1], n_shade[3 * i + 2]};
    const Vec3 o{wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]};
    const Vec3 w{wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]};
    const Vec3 f = disney_bsdf_eval(mat, o, w, ng, ns);
    const f32 pdf = disney_bsdf_pdf(mat, o, w, ng, ns);
    Rng rng(seeds[i]);
    const BsdfSample s = disney_bsdf_sample(mat, o, ng, ns, rng);
    float *r = out + 8 * i;
    r[0] = f.x; r[1] = f.y; r[2] = f.z; r[3] = pdf;
    r[4] = s.wi.x; r[5] = s.wi.y; r[6] = s.wi.z; r[7] = s.pdf;
    float *r2 = out2 + 4 * i;
    r2[0] = s.f.x; r2[1] = s.f.y; r2[2] = s.f.z;
    r2[3] = float((s.is_specular ? 1 : 0) | (s.is_diffuse ? 2 : 0));
  }
  return 0;
}

} // extern "C"
