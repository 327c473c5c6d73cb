// Shading kernels: pt_shade (src/photon/pt/pathtracer.cpp:765-1090) for the
// paths of one bounce iteration, in the general variants (shade_path.cuh),
// and the volume-scattering pre-pass of volume scenes.
#include "shade_path.cuh"

namespace phc {
namespace {

// The volume step of pt_shade (pathtracer.cpp:789-858) for every path of the
// iteration, ahead of the shading kernel: delta tracking along the path's
// segment (up to its hit, or its tmax for a miss) with the stream the shading
// would use (dimension 1 + iteration), whose state after the tracking goes
// with the result.  Tracking loops differ in length from path to path; in a
// kernel of their own they no longer hold the lanes of the shading code.
// lookups (or nullptr): density lookups made, added up over the grid.
__global__ void __launch_bounds__(128) k_vol_scatter(const RenderConst *__restrict__ rcp, DevScene sc, PathSoA in,
    const float4 *__restrict__ hits, WaveCounters wc, int it, HitQueues hq, unsigned long long *lookups)
{
  if (wave_failed(wc))
    return;
  // persistent warps with refill: a lane whose ray is done takes a new one
  // once wc.vol_refill lanes of its warp are idle; every trip is at most
  // wc.vol_passes passes of every busy lane's tracking (vt_pass: a macro-cell
  // step or a density lookup), ending at its next lookup
  const uint32_t n = wc.count[it];
  uint32_t *fetch = wc.vfetch + 2 * it;
  const uint32_t lane = lane_id();
  const uint32_t lt_mask = (1u << lane) - 1u;
  VolTrack s;
  Rng rng(1u);
  bool busy = false, exhausted = false;
  uint32_t idx = 0, idle = WARP_FULL, nlook = 0;
  for (uint32_t trips = 0;; ++trips) {
    if (trips >= wc.trip_cap) { // warp-uniform
      if (lane == 0)
        atomicCAS(wc.error, 0u, (WAVE_ERR_VOLUME << 16) | uint32_t(it));
      break;
    }
    if (!exhausted && (idle == WARP_FULL || uint32_t(__popc(idle)) >= wc.vol_refill)) {
      __syncwarp();
      const uint32_t k = uint32_t(__popc(idle));
      const uint32_t base = warp_fetch(fetch, k);
      if (base + k >= n)
        exhausted = true;
      if (!busy) {
        const uint32_t my = base + uint32_t(__popc(idle & lt_mask));
        if (my < n) {
          idx = my;
          const uint4 info = in.info[idx];
          const float4 ro4 = in.ray_o[idx], rd4 = in.ray_d[idx], hit = hits[idx];
          rng = path_rng(info.x % rcp->npix, info.y, 1u + uint32_t(it));
          const bool is_hit = __float_as_uint(hit.y) != 0xffffffffu;
          vt_init(s, v3(ro4), v3(rd4), ro4.w, is_hit ? hit.x : rd4.w);
          busy = true;
        }
      }
      idle = __ballot_sync(WARP_FULL, !busy);
    }
    if (idle == WARP_FULL) {
      if (exhausted)
        break;
      continue;
    }
    if (busy) {
      nlook += vt_passes<true>(sc, s, rng, wc.vol_passes) == VT_LOOKUP ? 1u : 0u;
      if (s.done) {
        hq.vscatter[idx] = make_float4(s.t_event, s.albedo.x, s.albedo.y, s.albedo.z);
        hq.vrng[idx] = rng.s;
        busy = false;
      }
    }
    __syncwarp(); // every lane back from the step's divergent work before the vote
    idle = __ballot_sync(WARP_FULL, !busy);
  }
  if (lookups) { // the loop ends for the whole warp at once
    const uint32_t w = __reduce_add_sync(WARP_FULL, nlook);
    if (lane == 0)
      atomicAdd(lookups, (unsigned long long)w);
  }
}

// Split queues, routed after the pre-pass: every path of the iteration joins
// the queue of its outcome (it scatters, reaches its hit, or escapes), in
// the order of the paths within each warp.  Routing inside k_vol_scatter,
// as paths finish their tracking, measured slower (235.9 against 238.3
// Msamples/s on the 2M scene).
__global__ void __launch_bounds__(256) k_vol_route(const float4 *__restrict__ hits, WaveCounters wc, int it,
    HitQueues hq)
{
  if (wave_failed(wc))
    return;
  const uint32_t n = wc.count[it];
  const uint32_t warps = gridDim.x * (blockDim.x / 32u);
  for (uint32_t base = (blockIdx.x * (blockDim.x / 32u) + (threadIdx.x >> 5)) * 32u; base < n; base += warps * 32u) {
    const uint32_t i = base + lane_id();
    uint32_t route = 0u;
    if (i < n)
      route = hq.vscatter[i].x >= 0.f ? 1u : (__float_as_uint(hits[i].y) != 0xffffffffu ? 2u : 3u);
    const uint32_t a = warp_append(wc.vcount + it, route == 1u);
    if (route == 1u)
      hq.vscatq[a] = i;
    const uint32_t b = warp_append(wc.hcount + it, route == 2u);
    if (route == 2u)
      hq.hitq[b] = i;
    const uint32_t m = warp_append(wc.mcount + it, route == 3u);
    if (route == 3u)
      hq.missq[m] = i;
  }
}

} // namespace

void launch_vol_route(const LaunchCfg &c, cudaStream_t s, const float4 *hits, WaveCounters wc, int it, HitQueues hq)
{
  k_vol_route<<<c.blocks_raygen, 256, 0, s>>>(hits, wc, it, hq);
}

void launch_vol_scatter(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, PathSoA in,
    const float4 *hits, WaveCounters wc, int it, HitQueues hq, uint64_t *lookups)
{
  k_vol_scatter<<<c.blocks_trace, 128, 0, s>>>(rc, sc, in, hits, wc, it, hq,
      reinterpret_cast<unsigned long long *>(lookups));
}

void launch_shade(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, PathSoA in, PathSoA out,
    const float4 *hits, ShadowSoA sh, Accum acc, WaveCounters wc, int it, ShadeVariant v, HitQueues hq)
{
  const int b = v.full ? c.blocks_shade : c.blocks_shade_lean;
  const BatchTable none{};
  if (v.full) {
    if (v.part == 0)
      k_shade<true, 0, false><<<b, 128, 0, s>>>(rc, sc, none, in, out, hits, sh, acc, wc, it, hq);
    else if (v.part == 1)
      k_shade<true, 1, false><<<b, 128, 0, s>>>(rc, sc, none, in, out, hits, sh, acc, wc, it, hq);
    else if (v.part == 2)
      k_shade<true, 2, false><<<b, 128, 0, s>>>(rc, sc, none, in, out, hits, sh, acc, wc, it, hq);
    else
      k_shade<true, 3, false><<<b, 128, 0, s>>>(rc, sc, none, in, out, hits, sh, acc, wc, it, hq);
  } else {
    if (v.part == 0)
      k_shade<false, 0, false><<<b, 128, 0, s>>>(rc, sc, none, in, out, hits, sh, acc, wc, it, hq);
    else if (v.part == 1)
      k_shade<false, 1, false><<<b, 128, 0, s>>>(rc, sc, none, in, out, hits, sh, acc, wc, it, hq);
    else
      k_shade<false, 2, false><<<b, 128, 0, s>>>(rc, sc, none, in, out, hits, sh, acc, wc, it, hq);
  }
}

void launch_shade_batch(const LaunchCfg &c, cudaStream_t s, BatchTable bt, PathSoA in, PathSoA out,
    const float4 *hits, ShadowSoA sh, WaveCounters wc, int it, ShadeVariant v, HitQueues hq)
{
  const int b = v.full ? c.blocks_shade : c.blocks_shade_lean;
  const DevScene sc{};
  const Accum acc{};
  if (v.full) {
    if (v.part == 0)
      k_shade<true, 0, true><<<b, 128, 0, s>>>(nullptr, sc, bt, in, out, hits, sh, acc, wc, it, hq);
    else if (v.part == 1)
      k_shade<true, 1, true><<<b, 128, 0, s>>>(nullptr, sc, bt, in, out, hits, sh, acc, wc, it, hq);
    else
      k_shade<true, 2, true><<<b, 128, 0, s>>>(nullptr, sc, bt, in, out, hits, sh, acc, wc, it, hq);
  } else {
    if (v.part == 0)
      k_shade<false, 0, true><<<b, 128, 0, s>>>(nullptr, sc, bt, in, out, hits, sh, acc, wc, it, hq);
    else if (v.part == 1)
      k_shade<false, 1, true><<<b, 128, 0, s>>>(nullptr, sc, bt, in, out, hits, sh, acc, wc, it, hq);
    else
      k_shade<false, 2, true><<<b, 128, 0, s>>>(nullptr, sc, bt, in, out, hits, sh, acc, wc, it, hq);
  }
}

int shade_max_active_blocks(int threads, bool full)
{
  int n = 0;
  if (full)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_shade<true, 0, false>, threads, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_shade<false, 1, false>, threads, 0);
  return n;
}

} // namespace phc
