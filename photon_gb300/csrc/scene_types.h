// Device-side scene layout of the GB300 path tracer (host and device view).
//
// Everything lives in HBM as flat arrays; a DevScene of raw pointers is passed
// to every kernel by value (kernel parameters sit in the constant bank).
//
//   nodes      uint4[5 * node_count]   80-byte quantised BVH8 nodes (bvh8.h)
//   tris       float4[3 * tri_count]   leaf-ordered triangle records:
//                                      (v0.xyz, prim id bits), (e1.xyz, -), (e2.xyz, -)
//                                      with e1 = v1 - v0, e2 = v2 - v0 rounded as the
//                                      reference's intersect_triangle computes them
//   prim_geo   float4[3 * prims]       the same record by primitive id (shading)
//   prim_vidx  uint4[prims]            (i0, i1, i2, material id) by primitive id
//   normals    float4[verts]           optional vertex normals (w unused)
//   ...        materials, attributes, samplers, lights, env map, volumes,
//              emissive-triangle CDF: the tables of the reference's scene build
//              (src/photon/anari/RenderBridge.cpp:441-826) and light tables
//              (src/photon/pt/pathtracer.cpp:411-503).
#pragma once

#include <cstdint>

namespace phc {

// Material after the bridge's conversion (RenderBridge.cpp:324-370); the
// fields of photon::pt::Material (include/photon/pt/material.h:35-82) that the
// seam can set, laid out for 16-byte loads.
struct DevMaterial {
  float base_color[3];
  float metallic;
  float roughness; // GGX alpha (perceptual squared)
  float ior;
  float transmission;
  float specular; // Disney specular (0.5 x bridge value)
  float clearcoat;
  float clearcoat_roughness;
  float sheen;
  float alpha;
  float emission[3];
  float emission_strength;
  int32_t src_kind[7];  // base_color, alpha, metallic, roughness, emission, transmission, normal
  int32_t src_index[7];
  int32_t alpha_mode; // 0 blend, 1 opaque, 2 mask
  float alpha_cutoff;
  int32_t flags;
  int32_t thin;
  int32_t base_color_alpha;
  int32_t base_tex;  // atlas texture of the base colour (pt::Material::base_color_tex), -1: none
  int32_t alpha_tex; // atlas texture of alpha (pt::Material::alpha_tex), -1: none
  uint32_t shade_class; // shading kernel class (SHADE_CLASS_LOBES), set by the scene build
};

// Lobes a material's BSDF can have.  A bit is clear only where the scene
// build proved that lobe's weight and value exactly +0 for every direction
// (material_lobes), so a shading kernel compiled without it returns the
// same results for that material.
enum : uint32_t { LB_DIFF = 1u, LB_SPEC = 2u, LB_TRANS = 4u, LB_COAT = 8u, LB_SHEEN = 16u, LB_ALL = 31u };
// Material classes with a hit-shading kernel of their own: class c is
// shaded with the lobes SHADE_CLASS_LOBES[c]; a material goes to the first
// class (from 1) whose lobes include its own, else to class 0 (all lobes).
constexpr uint32_t SHADE_CLASSES = 8;
constexpr uint32_t SHADE_CLASS_LOBES[SHADE_CLASSES] = {LB_ALL, LB_SPEC | LB_COAT, LB_DIFF | LB_SPEC | LB_COAT,
    LB_TRANS | LB_COAT, LB_SPEC | LB_TRANS | LB_COAT, LB_SPEC, LB_DIFF | LB_SPEC, LB_DIFF};

enum : int32_t { SRC_BASE = 0, SRC_ALPHA = 1, SRC_METAL = 2, SRC_ROUGH = 3, SRC_EMIT = 4, SRC_TRANS = 5, SRC_NORMAL = 6 };
enum : int32_t {
  MF_EMITTER_ONLY = 1,
  MF_HIDDEN = 2,
  MF_EMIT_BOTH = 4,
  MF_REFRACTIVE = 8,
  MF_EMIT_BACK = 16
};

struct DevSampler { // include/photon/pt/sampler.h:49-63
  int32_t type; // 0 1D, 1 2D, 2 3D, 3 transform, 4 atlas texture (pt::TextureAtlas entry)
  int32_t in_attribute;
  uint32_t linear;
  int32_t wrap[3];
  uint32_t offset;
  uint32_t size[3];
  float in_t[16];
  float in_o[4];
  float out_t[16];
  float out_o[4];
  // Storage of the texels: u8 = 0: float4 at DevScene::texels + offset;
  // u8 = 1: uchar4 at DevScene::texels_u8 + offset (images whose every value
  // is k / 255, decoded through DevScene::u8_decode).  grad_offset is the
  // sampler's first texel in the scene's texel order (all samplers' texels
  // in sequence), the index of the adjoint's texel gradients.
  uint32_t u8;
  uint32_t grad_offset;
};

struct DevLight { // include/photon/pt/light.h:19-35 (point, directional, spot)
  int32_t type;
  float position[3];
  float direction[3];
  float color[3];
  float intensity;
  float spot_angle;
  float spot_falloff;
  float radius;
};

struct DevVolume { // include/photon/pt/tf_volume.h:14-33
  float w2l[12];
  float origin[3];
  float spacing[3];
  uint32_t dims[3];
  uint32_t data_offset;
  uint32_t tf_offset;
  uint32_t tf_size;
  float value_lo, value_hi, density_scale, majorant;
  uint32_t linear;
  uint32_t macro_offset;
  uint32_t macro_dims[3];
};

constexpr uint32_t EMISSIVE_GUIDE_BITS = 10;
constexpr uint32_t ENV_MGUIDE_BITS = 10;
constexpr uint32_t ENV_CGUIDE_BITS = 8;

struct DevScene {
  // geometry
  const uint4 *nodes;
  const float4 *tris;
  const float4 *prim_geo;
  const uint4 *prim_vidx;
  const float4 *normals; // nullptr: none
  const float4 *positions; // vertex positions (w unused)
  uint32_t node_count;
  uint32_t prim_count;
  // shading tables
  const DevMaterial *materials;
  uint32_t material_count;
  const float4 *attr_values;
  int32_t attr_offset[5];
  const DevSampler *samplers;
  uint32_t sampler_count;
  const float4 *texels;
  const uchar4 *texels_u8;  // 8-bit RGBA samplers (DevSampler::u8)
  const float *u8_decode;   // 256 entries: float(k) / 255 (IEEE division)
  const DevLight *lights;
  uint32_t light_count;
  const uint32_t *emissive_ids;
  const float *emissive_cdf;
  const float *prim_light_pdf;
  uint32_t emissive_count;
  // Guide tables of the three CDF searches (nullptr: plain binary search).
  // Entry k of a guide is the search's result for u = k / G (G = 2^bits,
  // exact in float), entry G its largest result; a search for u then only
  // bisects [guide[k], guide[k + 1]] with k = u * G, which returns the same
  // index as the bisection of the whole table for every u of the reference's
  // RNG (multiples of 2^-24 in [0, 1)) when the CDF is non-decreasing.
  const uint32_t *emissive_guide; // EMISSIVE_GUIDE_BITS: G + 1 entries
  const uint32_t *env_mguide;     // ENV_MGUIDE_BITS: G + 1 entries (marginal)
  const uint32_t *env_cguide;     // ENV_CGUIDE_BITS: h x (G + 1) entries (rows)
  // environment (environment_map.h)
  const float4 *env_pixels; // (h, w)
  const float *env_marginal; // h + 1
  const float *env_conditional; // h x (w + 1)
  uint32_t env_w, env_h;
  float env_w2t[9], env_t2w[9];
  int32_t has_env, env_visible;
  // volumes (tf_volume.h)
  const DevVolume *volumes;
  uint32_t volume_count;
  const float *vol_values;
  const float4 *vol_tf;
  const float *vol_majorants;
  uint32_t strategy_count;
  float eps;
  uint32_t features; // SCENE_* bits: which shading features the scene uses
  // two-level BVH (SCENE_INSTANCES): `nodes` holds the top level (root at
  // node 0, leaves address instance slots) followed by every bottom level;
  // per top-level leaf slot the world-to-object rows and
  // (bottom-level root, object id, INST_* flags, 0)
  const float4 *inst_w2o; // 3 per instance
  const uint4 *inst_info;
  uint32_t inst_count;
  uint32_t scene_object_id; // instance id a ray back-end reports for the scene's own triangles
  int32_t scene_normals; // the scene's own triangles carry vertex normals
};

enum : uint32_t {
  INST_IDENTITY = 1u, // the scene's own triangles: world space, no transform
  INST_NORMALS = 2u,  // the object has vertex normals
  INST_NONE = 0xffffffffu
};

enum : uint32_t {
  SCENE_VOLUMES = 1u,  // transfer-function volumes (delta / ratio tracking)
  SCENE_SOURCES = 2u,  // material parameters from attributes or samplers, normal maps
  SCENE_LIGHTS = 4u,   // analytic point / directional / spot lights
  SCENE_INSTANCES = 8u // instanced geometry: two-level traversal
};

} // namespace phc
