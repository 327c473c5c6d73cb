// Launcher of the path-replay adjoint kernel (adjoint.cu).
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

struct AdjointArgs {
  const float4 *primal;  // radiance of each pixel sample, slot s * npix + pixel (the wavefront's accumulators)
  const float4 *d_image; // dLoss/dI per pixel (rgb; w unused), pixel order of the frame
  float *radiance;       // optional: sum over the pass's samples of the path radiance (3 per pixel)
  float *mat_grads;      // material_count * ADJ_MATERIAL_PARAMS
  float *vol_grads;      // min(volume_count, ADJ_MAX_VOLUMES) * ADJ_VOLUME_PARAMS
  float4 *texel_grads;   // one per texel of the scene's sampler table, or nullptr
  // Self-check: status[0] != 0 when a path exceeded its budget (then every
  // thread stops and the host reports an error): 1 + the bounce index, or
  // 0x10000 for a ray whose traversal exceeded ADJ_MAX_TRAVERSAL_STEPS.
  // status[1] = the largest clock count of one pixel sample; status[2] =
  // pixel samples whose replayed radiance differs from the primal one.
  unsigned long long *status;
  unsigned long long cycle_budget; // per pixel sample
  uint32_t npix, spp, sample_offset; // this launch: samples sample_offset .. + spp - 1
  float inv_spp;         // the image is the mean of inv_spp^-1 samples
};
constexpr uint32_t ADJ_MAX_TRAVERSAL_STEPS = 1u << 20;

void launch_adjoint(cudaStream_t s, int blocks, const RenderConst *rc, DevScene sc, AdjointArgs a);
int adjoint_max_active_blocks(int threads);

} // namespace phc
