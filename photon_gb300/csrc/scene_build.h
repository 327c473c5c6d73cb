// Host-side scene build: phc_scene_desc -> device tables.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/photon_cuda.h"
#include "bvh8.h"
#include "scene_types.h"
#include "scene_tables.cuh"

namespace phc {

// Sets the message phc_global_error returns on this thread.
void set_global_error(const std::string &msg);

// Scene tables in host memory, exactly the content the reference's bridge
// builds (RenderBridge.cpp:441-826) plus the light tables of
// PathTracer::build_light_tables (pathtracer.cpp:411-503).
struct HostScene {
  std::vector<float> positions4;      // vertices as float4
  std::vector<uint32_t> indices;      // 3 per triangle
  std::vector<uint32_t> material_ids; // clamped like the bridge
  std::vector<float> normals4;        // empty: none
  std::vector<uint32_t> prim_vidx;    // (i0, i1, i2, material) per triangle
  std::vector<float> prim_geo;        // 12 floats per triangle
  std::vector<DevMaterial> materials;
  std::vector<float> attr_values;     // float4
  int32_t attr_offset[5]{-1, -1, -1, -1, -1};
  std::vector<DevSampler> samplers;
  std::vector<float> texels;          // float4 (atlas textures, converted from RGB)
  // sampler texels, read from the caller's arrays (valid for the set-scene
  // call that builds and uploads this scene) and copied straight to the
  // device after `texels`
  struct Span {
    const float *p;
    size_t floats;
  };
  std::vector<Span> texel_spans;
  // 8-bit RGBA texels (4 bytes per texel) of the samplers whose every value
  // is one of u8_decode's, and that table
  std::vector<uint8_t> texels_u8;
  std::vector<float> u8_decode;
  uint64_t texel_logical_count{0}; // texels in the scene's texel order (atlas or every sampler)
  std::vector<Span> vol_value_spans; // volume fields, likewise
  std::vector<DevLight> lights;
  std::vector<uint32_t> emissive_ids;
  std::vector<float> emissive_cdf, prim_light_pdf;
  bool has_env{false}, env_visible{true};
  uint32_t env_w{0}, env_h{0};
  std::vector<float> env_pixels4, env_marginal, env_conditional;
  // guide tables of the CDF searches (empty: plain bisection on the device)
  std::vector<uint32_t> emissive_guide, env_mguide, env_cguide;
  float env_w2t[9]{1, 0, 0, 0, 1, 0, 0, 0, 1}, env_t2w[9]{1, 0, 0, 0, 1, 0, 0, 0, 1};
  std::vector<DevVolume> volumes;
  // majorant grids the upload computes on the device (tuning key gpu_tables):
  // the grid's parameters and its offsets in vol_majorants / vol_values /
  // vol_tf (transfer-function entries)
  struct MajorantTask {
    MajorantJob job;
    uint32_t macro_offset, data_offset, tf_offset;
  };
  std::vector<MajorantTask> majorant_tasks;
  std::vector<float> vol_values, vol_tf, vol_majorants;
  uint32_t strategy_count{0};
  float eps{1e-3f};
  Bvh8Host bvh;
  // instancing: one record per top-level leaf slot (3 float4 world-to-object
  // rows; uint4 bottom-level root, object id, INST_* flags, 0)
  std::vector<float> inst_w2o;
  std::vector<uint32_t> inst_info;
  uint32_t inst_count{0};
  bool scene_normals{false};
  uint64_t instanced_triangles{0}; // triangles the instances place (not stored)
  std::vector<uint32_t> obj_prim_base, obj_prim_count; // per object: its primitives
  bool bvh_on_gpu{false}; // `bvh` left empty: DeviceScene::upload builds it on the GPU
};

void build_host_scene(const phc_scene_desc &in, HostScene &out);

// Owns the device copies of a HostScene.
struct DeviceScene {
  std::vector<void *> allocations;
  DevScene dev{};
  size_t bytes{0};
  uint64_t node_bytes{0}, tri_bytes{0};
  uint64_t texel_count{0};
  uint32_t bvh_depth{0};
  uint64_t table_floats[5]{}; // lengths of the tables phc_scene_table reads (PHC_TABLE_*)
  ~DeviceScene();
  void release();
  // Returns an empty string on success, else the failure message.
  std::string upload(const HostScene &h, cudaStream_t stream);

private:
  template <class T> T *put(const std::vector<T> &v, cudaStream_t s, std::string &err);
  float *put_spans(const std::vector<float> &owned, const std::vector<HostScene::Span> &spans, cudaStream_t s,
      std::string &err);
};

// Launches the majorant grid of one volume on the device (scene_tables.cu);
// returns an empty string on success, else the failure message.
std::string launch_majorants(const MajorantJob &job, const float *vals, const float4 *tf, float *out,
    cudaStream_t stream);

} // namespace phc
