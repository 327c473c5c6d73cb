// Level B of the drop-in: photon::bridge::Renderer (the reference's
// src/photon/anari/RenderBridge.h:175-214) implemented over
// libphoton_cuda.so, in place of src/photon/anari/RenderBridge.cpp.  Its
// consumer, the ANARI Frame (Frame.cpp:139-241), sees the same class: the
// scene, camera and settings go across as the C-ABI's field-for-field
// mirrors, errors come back as false plus a message (RenderBridge.cpp:83-110),
// every call blocks, and the frame is read in the bridge's layout (rows from
// the bottom).  The library copies the scene during phc_set_scene, so the
// SceneData may change or go away afterwards.
#include <cstring>
#include <string>
#include <vector>

#include "photon/anari/RenderBridge.h"
#include "photon_cuda.h"

namespace photon::bridge {

// Field-for-field mirrors: the arrays must keep their extents.
static_assert(kMeshAttributeCount == 5, "phc_scene_desc::attributes holds five slots");
static_assert(sizeof(CameraData::image_region) == sizeof(phc_camera::image_region), "image_region");
static_assert(sizeof(SamplerData::in_transform) == sizeof(phc_sampler::in_transform), "in_transform");
static_assert(sizeof(SamplerData::out_transform) == sizeof(phc_sampler::out_transform), "out_transform");
static_assert(sizeof(EnvironmentData::world_to_map) == sizeof(phc_environment::world_to_map), "world_to_map");
static_assert(sizeof(VolumeData::world_to_local) == sizeof(phc_volume::world_to_local), "world_to_local");
static_assert(sizeof(RenderSettings::background) == sizeof(phc_settings::background), "background");

namespace {

phc_param_source source(const ParamSourceData &s) { return phc_param_source{s.kind, s.index}; }

phc_material material(const MaterialData &m)
{
  phc_material o;
  phc_material_default(&o);
  std::memcpy(o.base_color, m.base_color, sizeof(o.base_color));
  o.opacity = m.opacity;
  o.metallic = m.metallic;
  o.roughness = m.roughness;
  o.ior = m.ior;
  o.transmission = m.transmission;
  o.specular = m.specular;
  std::memcpy(o.emission, m.emission, sizeof(o.emission));
  o.clearcoat = m.clearcoat;
  o.clearcoat_roughness = m.clearcoat_roughness;
  o.sheen = m.sheen;
  o.base_color_src = source(m.base_color_src);
  o.opacity_src = source(m.opacity_src);
  o.metallic_src = source(m.metallic_src);
  o.roughness_src = source(m.roughness_src);
  o.emission_src = source(m.emission_src);
  o.transmission_src = source(m.transmission_src);
  o.normal_src = source(m.normal_src);
  o.alpha_mode = m.alpha_mode;
  o.alpha_cutoff = m.alpha_cutoff;
  o.base_color_alpha = m.base_color_alpha;
  o.thin_walled = m.thin_walled;
  o.emitter_only = m.emitter_only;
  o.hidden_to_camera = m.hidden_to_camera;
  o.emission_side = m.emission_side;
  return o;
}

phc_sampler sampler(const SamplerData &s)
{
  phc_sampler o;
  phc_sampler_default(&o);
  o.type = s.type;
  o.in_attribute = s.in_attribute;
  o.linear = s.linear;
  for (int k = 0; k < 3; ++k) {
    o.wrap[k] = s.wrap[k];
    o.size[k] = s.size[k];
  }
  std::memcpy(o.in_transform, s.in_transform, sizeof(o.in_transform));
  std::memcpy(o.in_offset, s.in_offset, sizeof(o.in_offset));
  std::memcpy(o.out_transform, s.out_transform, sizeof(o.out_transform));
  std::memcpy(o.out_offset, s.out_offset, sizeof(o.out_offset));
  o.texels = s.texels.empty() ? nullptr : s.texels.data();
  o.texel_count = s.texels.size() / 4;
  return o;
}

phc_light light(const LightData &l)
{
  phc_light o;
  phc_light_default(&o);
  o.type = l.type;
  std::memcpy(o.position, l.position, sizeof(o.position));
  std::memcpy(o.direction, l.direction, sizeof(o.direction));
  std::memcpy(o.color, l.color, sizeof(o.color));
  o.intensity = l.intensity;
  o.radius = l.radius;
  o.spot_angle = l.spot_angle;
  o.spot_falloff = l.spot_falloff;
  return o;
}

phc_volume volume(const VolumeData &v)
{
  phc_volume o;
  phc_volume_default(&o);
  std::memcpy(o.world_to_local, v.world_to_local, sizeof(o.world_to_local));
  std::memcpy(o.origin, v.origin, sizeof(o.origin));
  std::memcpy(o.spacing, v.spacing, sizeof(o.spacing));
  std::memcpy(o.dims, v.dims, sizeof(o.dims));
  o.values = v.values.empty() ? nullptr : v.values.data();
  o.value_count = v.values.size();
  o.transfer = v.transfer.empty() ? nullptr : v.transfer.data();
  o.transfer_count = uint32_t(v.transfer.size() / 4);
  std::memcpy(o.value_range, v.value_range, sizeof(o.value_range));
  o.density_scale = v.density_scale;
  o.linear = v.linear;
  return o;
}

phc_camera camera(const CameraData &c)
{
  phc_camera o;
  phc_camera_default(&o);
  std::memcpy(o.position, c.position, sizeof(o.position));
  std::memcpy(o.direction, c.direction, sizeof(o.direction));
  std::memcpy(o.up, c.up, sizeof(o.up));
  o.orthographic = c.orthographic;
  o.fovy = c.fovy;
  o.height = c.height;
  o.aspect = c.aspect;
  o.aperture_radius = c.aperture_radius;
  o.focus_distance = c.focus_distance;
  std::memcpy(o.image_region, c.image_region, sizeof(o.image_region));
  o.clip_near = c.clip_near;
  o.clip_far = c.clip_far;
  return o;
}

phc_settings settings(const RenderSettings &s)
{
  phc_settings o;
  phc_settings_default(&o);
  o.width = s.width;
  o.height = s.height;
  o.pixel_samples = s.pixel_samples;
  o.max_depth = s.max_depth;
  std::memcpy(o.background, s.background, sizeof(o.background));
  o.background_image = s.background_image;
  o.background_width = s.background_width;
  o.background_height = s.background_height;
  std::memcpy(o.ambient_color, s.ambient_color, sizeof(o.ambient_color));
  o.ambient_radiance = s.ambient_radiance;
  o.adaptive_sampling = s.adaptive_sampling;
  o.throughput_clamp = s.throughput_clamp;
  o.max_diffuse_bounces = s.max_diffuse_bounces;
  o.max_glossy_bounces = s.max_glossy_bounces;
  o.max_transmission_bounces = s.max_transmission_bounces;
  o.max_volume_bounces = s.max_volume_bounces;
  o.clamp_direct = s.clamp_direct;
  o.clamp_indirect = s.clamp_indirect;
  return o;
}

} // namespace

struct Renderer::Impl {
  phc_renderer *r = nullptr;
};

Renderer::Renderer() = default;

Renderer::~Renderer()
{
  if (m_impl) {
    phc_destroy(m_impl->r);
    delete m_impl;
  }
}

bool Renderer::initialize(std::string &error)
{
  if (m_impl)
    return true;
  phc_renderer *r = nullptr;
  if (phc_create(&r) != PHC_OK) {
    error = phc_global_error();
    return false;
  }
  m_impl = new Impl{r};
  return true;
}

std::string Renderer::backend_name() const { return m_impl ? phc_backend_name(m_impl->r) : ""; }

std::string Renderer::execution_space() const { return m_impl ? "Cuda" : ""; }

bool Renderer::set_scene(const SceneData &scene, std::string &error)
{
  if (!initialize(error))
    return false;
  phc_scene_desc d;
  phc_scene_desc_default(&d);
  d.positions = scene.positions.empty() ? nullptr : scene.positions.data();
  d.vertex_count = scene.positions.size() / 3;
  d.normals = !scene.normals.empty() && scene.normals.size() >= scene.positions.size() ? scene.normals.data() : nullptr;
  for (int k = 0; k < kMeshAttributeCount; ++k)
    d.attributes[k] =
        !scene.attributes[k].empty() && scene.attributes[k].size() >= 4 * d.vertex_count ? scene.attributes[k].data()
                                                                                         : nullptr;
  d.indices = scene.indices.empty() ? nullptr : scene.indices.data();
  d.triangle_count = scene.indices.size() / 3;
  d.material_ids = scene.material_ids.empty() ? nullptr : scene.material_ids.data();
  d.material_id_count = scene.material_ids.size();
  std::vector<phc_material> materials;
  for (const MaterialData &m : scene.materials)
    materials.push_back(material(m));
  std::vector<phc_sampler> samplers;
  for (const SamplerData &s : scene.samplers)
    samplers.push_back(sampler(s));
  std::vector<phc_light> lights;
  for (const LightData &l : scene.lights)
    lights.push_back(light(l));
  std::vector<phc_volume> volumes;
  for (const VolumeData &v : scene.volumes)
    volumes.push_back(volume(v));
  d.materials = materials.data();
  d.material_count = uint32_t(materials.size());
  d.samplers = samplers.data();
  d.sampler_count = uint32_t(samplers.size());
  d.lights = lights.data();
  d.light_count = uint32_t(lights.size());
  d.volumes = volumes.data();
  d.volume_count = uint32_t(volumes.size());
  const EnvironmentData &env = scene.environment;
  d.environment.present = env.present;
  d.environment.visible = env.visible;
  d.environment.width = env.width;
  d.environment.height = env.height;
  d.environment.pixels = env.pixels.empty() ? nullptr : env.pixels.data();
  std::memcpy(d.environment.world_to_map, env.world_to_map, sizeof(d.environment.world_to_map));
  if (phc_set_scene(m_impl->r, &d) != PHC_OK) {
    error = phc_last_error(m_impl->r);
    return false;
  }
  m_samples = 0;
  return true;
}

bool Renderer::render(const CameraData &camera_data, const RenderSettings &render_settings, bool reset,
    std::string &error)
{
  if (!m_impl) {
    error = "renderer not initialized";
    return false;
  }
  const phc_camera c = camera(camera_data);
  const phc_settings s = settings(render_settings);
  if (phc_render(m_impl->r, &c, &s, reset ? 1 : 0) != PHC_OK) {
    error = phc_last_error(m_impl->r);
    return false;
  }
  m_samples = phc_accumulated_samples(m_impl->r);
  return true;
}

uint32_t Renderer::accumulated_samples() const { return m_samples; }

namespace {
template <class Read>
bool read_channel(phc_renderer *r, Read read, float *out, std::string &error)
{
  if (!r) {
    error = "renderer not initialized";
    return false;
  }
  if (read(r, out) != PHC_OK) {
    error = phc_last_error(r);
    return false;
  }
  return true;
}
} // namespace

bool Renderer::read_color(float *rgba, std::string &error)
{
  return read_channel(m_impl ? m_impl->r : nullptr, phc_read_color, rgba, error);
}
bool Renderer::read_depth(float *depth, std::string &error)
{
  return read_channel(m_impl ? m_impl->r : nullptr, phc_read_depth, depth, error);
}
bool Renderer::read_normal(float *xyz, std::string &error)
{
  return read_channel(m_impl ? m_impl->r : nullptr, phc_read_normal, xyz, error);
}
bool Renderer::read_albedo(float *rgb, std::string &error)
{
  return read_channel(m_impl ? m_impl->r : nullptr, phc_read_albedo, rgb, error);
}

// The CUDA library keeps no process-wide state to finalize (each renderer
// owns its device memory and stream; phc_destroy releases them).
void Renderer::shutdown() {}

} // namespace photon::bridge
