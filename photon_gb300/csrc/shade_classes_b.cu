// Lean hit-shading kernels of shading classes 5-7 (see shade_classes_a.cu).
#include "shade_path.cuh"

namespace phc {

namespace {
template <uint32_t C>
void launch_cls(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, PathSoA in, PathSoA out,
    const float4 *hits, ShadowSoA sh, Accum acc, WaveCounters wc, int it, HitQueues hq)
{
  k_shade<false, 1, false, C><<<c.blocks_shade_lean, 128, 0, s>>>(rc, sc, BatchTable{}, in, out, hits, sh, acc, wc, it,
      hq);
}
} // namespace

void launch_shade_class_b(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, PathSoA in,
    PathSoA out, const float4 *hits, ShadowSoA sh, Accum acc, WaveCounters wc, int it, uint32_t cls, HitQueues hq)
{
  static_assert(SHADE_CLASSES == 8, "classes 1-4 in shade_classes_a.cu, 5-7 here");
  switch (cls) {
  case 5: launch_cls<5>(c, s, rc, sc, in, out, hits, sh, acc, wc, it, hq); break;
  case 6: launch_cls<6>(c, s, rc, sc, in, out, hits, sh, acc, wc, it, hq); break;
  case 7: launch_cls<7>(c, s, rc, sc, in, out, hits, sh, acc, wc, it, hq); break;
  default: break;
  }
}

} // namespace phc
