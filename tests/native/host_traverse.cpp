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
