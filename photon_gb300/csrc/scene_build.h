// Host-side scene build: phc_scene_desc -> device tables.
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/photon_cuda.h"
#include "bvh8.h"
#include "scene_types.h"
#include "scene_tables.cuh"

namespace phc {

// Allocator whose resize leaves new elements uninitialised (for arrays that
// a parallel loop fills right after: no serial zeroing pass, and the pages
// are first touched by the threads that write them).
template <class T> struct UninitAlloc : std::allocator<T> {
  template <class U> struct rebind {
    using other = UninitAlloc<U>;
  };
  UninitAlloc() = default;
  template <class U> UninitAlloc(const UninitAlloc<U> &) noexcept {}
  template <class U> void construct(U *p) noexcept { ::new (static_cast<void *>(p)) U; }
  template <class U, class... A> void construct(U *p, A &&...a)
  {
    ::new (static_cast<void *>(p)) U(std::forward<A>(a)...);
  }
};

// Host arrays of a scene's geometry: filled by parallel loops right after
// they are sized.
template <class T> using HostVec = std::vector<T, UninitAlloc<T>>;

// Sets the message phc_global_error returns on this thread.
void set_global_error(const std::string &msg);

// Scene tables in host memory, exactly the content the reference's bridge
// builds (RenderBridge.cpp:441-826) plus the light tables of
// PathTracer::build_light_tables (pathtracer.cpp:411-503).
struct HostScene {
  HostVec<float> positions4;      // vertices as float4
  HostVec<uint32_t> indices;      // 3 per triangle
  HostVec<uint32_t> material_ids; // clamped like the bridge
  HostVec<float> normals4;        // empty: none
  HostVec<uint32_t> prim_vidx;    // (i0, i1, i2, material) per triangle
  HostVec<float> prim_geo;        // 12 floats per triangle
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
  std::vector<uint8_t, UninitAlloc<uint8_t>> texels_u8;
  std::vector<float> u8_decode;
  // samplers the upload packs to 8 bits on the device (tuning key
  // gpu_tables): their fp32 texels in the caller's array, the sampler, and
  // its place in the device's uchar4 array; a sampler whose values are not
  // all k / 255 falls back to fp32 at the end of the float4 array
  struct TexelPackTask {
    const float *src;
    size_t texels;
    uint32_t sampler;
    size_t u8_offset;
  };
  std::vector<TexelPackTask> texel_pack_tasks;
  size_t texels_u8_device{0}; // uchar4 texels the device array holds for them
  uint64_t texel_logical_count{0}; // texels in the scene's texel order (atlas or every sampler)
  std::vector<Span> vol_value_spans; // volume fields, likewise
  std::vector<DevLight> lights;
  std::vector<uint32_t> emissive_ids;
  std::vector<float> emissive_cdf, prim_light_pdf;
  bool has_env{false}, env_visible{true};
  uint32_t env_w{0}, env_h{0};
  // environment and emitter tables the upload builds on the device (tuning
  // key gpu_tables): the caller's RGB environment texels (valid for the
  // set-scene call) and each row's sin(theta); the emitters of a
  // single-level scene
  const float *env_rgb{nullptr};
  std::vector<float> env_row_sin;
  bool emissive_on_gpu{false};
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
  uint32_t shade_class_count{0}; // distinct shading classes among the materials
  uint32_t bvh_depth{0};
  uint64_t table_floats[5]{}; // lengths of the tables phc_scene_table reads (PHC_TABLE_*)
  ~DeviceScene();
  void release();
  // Returns an empty string on success, else the failure message.
  std::string upload(const HostScene &h, cudaStream_t stream);

private:
  template <class T, class A> T *put(const std::vector<T, A> &v, cudaStream_t s, std::string &err);
  float *put_spans(const std::vector<float> &owned, const std::vector<HostScene::Span> &spans, cudaStream_t s,
      std::string &err);
  std::string device_tables(const HostScene &h, DevScene &d, cudaStream_t s);
  template <class T> T *alloc(size_t n, std::string &err, bool keep = true);
  const uchar4 *pack_texels(const HostScene &h, std::vector<DevSampler> &samplers,
      std::vector<HostScene::Span> &spans, const float *dec, cudaStream_t s, std::string &err);
};

// Launches the majorant grid of one volume on the device (scene_tables.cu);
// returns an empty string on success, else the failure message.
std::string launch_majorants(const MajorantJob &job, const float *vals, const float4 *tf, float *out,
    cudaStream_t stream);

// The environment map's tables on the device (scene_tables.cu): texels
// from the caller's RGB (staged on the device), row CDFs, row weights, the
// marginal CDF and both guides; bad |= 1 when a row CDF, 2 when the
// marginal is not non-decreasing (the guides are then not used).
struct EnvTablesJob {
  const float *rgb;      // w x h RGB on the device
  const float *row_sin;  // h: sin(theta) of each row, host libm as the reference
  uint32_t w, h;
  float4 *pixels;        // w x h
  float *conditional;    // h x (w + 1)
  float *marginal;       // h + 1
  float *row_weight;     // h (scratch)
  uint32_t *mguide;      // 2^ENV_MGUIDE_BITS + 1
  uint32_t *cguide;      // h x (2^ENV_CGUIDE_BITS + 1)
  uint32_t *bad;
};
std::string launch_env_tables(const EnvTablesJob &job, cudaStream_t stream);

// The emissive triangles' tables on the device (scene_tables.cu), in three
// launches: flags of the triangles whose material may emit and whose area
// is positive, their exclusive scan and their number (count[0] = n); their
// ids in triangle order and their weights; then, from the running sum of the weights (computed by
// the caller, in the reference's double order, into prefix) and its total,
// the CDF, the per-triangle area densities and the guide (bad |= 4 when the
// CDF is not non-decreasing).
struct EmissiveJob {
  const float4 *pos;
  const uint4 *vidx; // (i0, i1, i2, material) per triangle
  const DevMaterial *mats;
  uint32_t tc;       // triangles
  uint32_t *flag;    // tc (scratch)
  uint32_t *rank;    // tc (scratch): exclusive scan of flag
  uint32_t *scan_scratch; // scan_u32_scratch(tc) words
  uint32_t *ids;     // n
  uint32_t *count;
  uint32_t n;        // emitters
  double *weight, *prefix; // n, n
  float *cdf;        // n
  float *pdf;        // tc, zero-filled by the caller
  uint32_t *guide;   // 2^EMISSIVE_GUIDE_BITS + 1
  uint32_t *bad;
};
std::string launch_emissive_ids(const EmissiveJob &job, cudaStream_t stream);
std::string launch_emissive_weights(const EmissiveJob &job, cudaStream_t stream);
std::string launch_emissive_tables(const EmissiveJob &job, double total, cudaStream_t stream);

// Packs n fp32 RGBA texels to 8 bits on the device (scene_tables.cu): dst[i]
// channel c = k where src[i].c is bit for bit dec[k] (dec: the 256 floats
// float(k) / 255); sets *bad to nonzero if any value is not one of them.
std::string launch_pack_texels_u8(const float4 *src, size_t n, const float *dec, uchar4 *dst, uint32_t *bad,
    cudaStream_t stream);

} // namespace phc
