// Lean hit-shading kernels of shading classes 1-7 for the batched wavefront
// (paths of many jobs, each shaded with its job's scene; shade_path.cuh),
// in a translation unit of their own so that they compile in parallel with
// the single-scene class kernels.
#include "shade_path.cuh"

namespace phc {

namespace {
template <uint32_t C>
void launch_cls_batch(const LaunchCfg &c, cudaStream_t s, BatchTable bt, PathSoA in, PathSoA out,
    const float4 *hits, ShadowSoA sh, WaveCounters wc, int it, HitQueues hq)
{
  k_shade<false, 1, true, C><<<c.blocks_shade_lean, 128, 0, s>>>(nullptr, DevScene{}, bt, in, out, hits, sh, Accum{},
      wc, it, hq);
}
} // namespace

void launch_shade_class_batch(const LaunchCfg &c, cudaStream_t s, BatchTable bt, PathSoA in, PathSoA out,
    const float4 *hits, ShadowSoA sh, WaveCounters wc, int it, uint32_t cls, HitQueues hq)
{
  static_assert(SHADE_CLASSES == 8, "classes 1-7");
  switch (cls) {
  case 1: launch_cls_batch<1>(c, s, bt, in, out, hits, sh, wc, it, hq); break;
  case 2: launch_cls_batch<2>(c, s, bt, in, out, hits, sh, wc, it, hq); break;
  case 3: launch_cls_batch<3>(c, s, bt, in, out, hits, sh, wc, it, hq); break;
  case 4: launch_cls_batch<4>(c, s, bt, in, out, hits, sh, wc, it, hq); break;
  case 5: launch_cls_batch<5>(c, s, bt, in, out, hits, sh, wc, it, hq); break;
  case 6: launch_cls_batch<6>(c, s, bt, in, out, hits, sh, wc, it, hq); break;
  case 7: launch_cls_batch<7>(c, s, bt, in, out, hits, sh, wc, it, hq); break;
  default: break;
  }
}

} // namespace phc
