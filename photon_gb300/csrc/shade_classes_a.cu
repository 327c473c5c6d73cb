// Lean hit-shading kernels of shading classes 1-4 (shade_path.cuh,
// scene_types.h SHADE_CLASS_LOBES); classes 5-7 are in shade_classes_b.cu so
// that the two compile in parallel.
#include "shade_path.cuh"

namespace phc {

void launch_shade_class_b(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, PathSoA in,
    PathSoA out, const float4 *hits, ShadowSoA sh, Accum acc, WaveCounters wc, int it, uint32_t cls, HitQueues hq);

namespace {
template <uint32_t C>
void launch_cls(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, PathSoA in, PathSoA out,
    const float4 *hits, ShadowSoA sh, Accum acc, WaveCounters wc, int it, HitQueues hq)
{
  k_shade<false, 1, false, C><<<c.blocks_shade_lean, 128, 0, s>>>(rc, sc, BatchTable{}, in, out, hits, sh, acc, wc, it,
      hq);
}
} // namespace

void launch_shade_class(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, PathSoA in,
    PathSoA out, const float4 *hits, ShadowSoA sh, Accum acc, WaveCounters wc, int it, uint32_t cls, HitQueues hq)
{
  switch (cls) {
  case 1: launch_cls<1>(c, s, rc, sc, in, out, hits, sh, acc, wc, it, hq); break;
  case 2: launch_cls<2>(c, s, rc, sc, in, out, hits, sh, acc, wc, it, hq); break;
  case 3: launch_cls<3>(c, s, rc, sc, in, out, hits, sh, acc, wc, it, hq); break;
  case 4: launch_cls<4>(c, s, rc, sc, in, out, hits, sh, acc, wc, it, hq); break;
  default: launch_shade_class_b(c, s, rc, sc, in, out, hits, sh, acc, wc, it, cls, hq); break;
  }
}

} // namespace phc
