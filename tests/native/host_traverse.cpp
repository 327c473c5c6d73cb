// Host build of the device BVH8 traversal (photon_gb300/csrc/traverse.cuh)
// over the host BVH8 builder, for CPU tests of the traversal logic against the
// oracle before any GPU run.  Test infrastructure only.
#include <cstdint>
#include <cstring>
#include <vector>

#include "bvh8.h"
#include "traverse.cuh"

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

#include <stdexcept>

namespace phc {
// The harness never uploads a scene, so the GPU builder (bvh_gpu.cu, compiled
// by nvcc) is not linked in; scene_build.cpp's upload refers to it.
GpuBvh8 build_bvh8_gpu(const float4 *, const uint4 *, uint32_t, cudaStream_t)
{
  throw std::runtime_error("the host harness builds no BVH on the GPU");
}
} // namespace phc

extern "C" int ht_trace_instanced(const phc_scene_desc *desc, const float *orgs, const float *dirs,
    const float *tmin, const float *tmax, uint32_t n, int any_hit, float *out4, uint32_t *obj, float *geo9,
    uint64_t *stats)
{
  HostScene h;
  build_host_scene(*desc, h);
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
