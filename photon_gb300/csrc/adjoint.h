// Path-replay adjoint on the wavefront (adjoint.cu): launchers and queues.
#pragma once

#include <cuda_runtime.h>

#include "wavefront.h"

namespace phc {

// Gradient layout per material (ADJ_MATERIAL_PARAMS floats): base colour
// r, g, b, roughness (the bridge's perceptual roughness r, GGX alpha = r^2),
// metallic, specTrans, sheen, clearcoat.  Per volume (ADJ_VOLUME_PARAMS):
// density scale, albedo r, g, b (the transfer function's colour, taken as
// constant over the volume).  Per texel: float4 (r, g, b, unused).
constexpr int ADJ_MATERIAL_PARAMS = 8;
constexpr int ADJ_VOLUME_PARAMS = 4;
constexpr int ADJ_MAX_VOLUMES = 4;
constexpr uint32_t ADJ_VTX_VALID = 0x80000000u; // VtxSoA::q.w: a surface vertex is stored
constexpr uint32_t ADJ_PREV_VALID = 1u << 30;   // PathSoA::info.w: the path carries a previous sample
constexpr uint32_t ADJ_NO_NEXT = 0xffffffffu;

// A surface vertex, enough to find its material and base-colour texels again:
// q = (prim, b1 bits, b2 bits, material | ADJ_VTX_VALID), p = position,
// sn = the hit's shading normal (before flips and normal maps).
struct VtxSoA {
  uint4 *q;
  float4 *p, *sn;
};

// The replayed paths of one bounce: the forward state plus what the
// derivative needs.
struct AdjPathSoA {
  PathSoA p;
  float4 *rem;     // radiance still to be collected (xyz)
  float4 *g0, *g1; // previous surface sample (ADJ_PREV_VALID): d log pu / d theta, 8 values
  VtxSoA v;        // previous surface vertex
};

// Shadow rays of one bounce with their deferred gradient: when the ray is
// unoccluded with transmittance T, the vertex's parameters get T * (g0, g1)
// and the continued path (next) loses T * contribution from its remainder.
struct AdjShadowSoA {
  ShadowSoA s;    // a: origin, tmax (< 0 once k_shadow found it occluded); b: direction, contribution.x;
                  // c: contribution.yz, slot, sample index
  uint32_t *next; // the continued path's index in the next queue, or ADJ_NO_NEXT
  float4 *g0, *g1;
  VtxSoA v;       // the shading vertex (q.w without ADJ_VTX_VALID: a volume scattering event)
};

struct AdjointArgs {
  const float4 *primal;  // radiance of each pixel sample (slot = sample-in-chunk * npix + pixel)
  const float4 *d_image; // dLoss/dI per pixel (rgb), pixel order of the frame
  float4 *collected;     // per slot: radiance the replay collected (checked against primal)
  float *radiance;       // optional: per pixel, sum of the pass's sample radiances (3 floats)
  float *mat_grads;      // material_count * ADJ_MATERIAL_PARAMS
  float *vol_grads;      // min(volume_count, ADJ_MAX_VOLUMES) * ADJ_VOLUME_PARAMS
  float4 *texel_grads;   // one per texel of the scene's sampler table, or nullptr
  unsigned long long *mismatches; // pixel samples whose replay radiance differs from the primal
  uint32_t npix;
  float inv_spp; // the image is the mean of 1 / inv_spp samples
};

void launch_adj_shade(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, AdjPathSoA in,
    AdjPathSoA out, const float4 *hits, AdjShadowSoA sh, WaveCounters wc, int it, AdjointArgs a,
    HitQueues hq);
void launch_adj_resolve(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, AdjShadowSoA sh,
    AdjPathSoA next, WaveCounters wc, int it, AdjointArgs a);
void launch_adj_finish(cudaStream_t s, int blocks, uint32_t slots, AdjointArgs a);
int adj_shade_max_active_blocks(int threads);

} // namespace phc
