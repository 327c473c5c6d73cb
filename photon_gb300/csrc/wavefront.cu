// Wavefront kernels of the GB300 path tracer (shading lives in shade_kernels.cu).
//
//   k_raygen   pt_init_sample      pathtracer.cpp:691-760
//   k_trace    trace_closest       kokkos_backend.cpp:21-61 (BVH8, traverse.cuh)
//   k_shadow   trace_occluded + pt_nee_accum_pack  pathtracer.cpp:1092-1123
//   k_shadow_volume  the transmittance of the unoccluded shadow rays of
//              volume scenes (the tracking loop, out of the voting loop)
//   k_wave_end pt_update_variance  pathtracer.cpp:1129-1139 (+ wave bookkeeping)
//   k_resolve  pt_resolve + frame accumulation  pathtracer.cpp:1143-1155,
//              RenderBridge.cpp:386-410
//
// Unlike the reference, which sweeps all w*h slots in every kernel and keeps
// dead paths as empty rays (pathtracer.cpp:1113-1121), live paths are
// compacted into dense queues: each warp reserves its outputs with one atomic
// (ballot + popc prefix), and every kernel reads a dense, coalesced range.
// Kernels are persistent: a fixed grid of warps pulls batches from a device
// counter until the queue length (also in device memory) is reached.
#include "wave_common.cuh"

#include <type_traits>

namespace phc {
namespace {

// ----------------------------------------------------------------- raygen
// Batched raygen: the items of this wave are the entries of its table (job,
// sample range, every pixel); each path lands in its job's lane of the
// sample (lane = sample % job lanes), exactly as the job's own render would.
__global__ void __launch_bounds__(256) k_raygen_batch(BatchTable bt, PathSoA out, WaveCounters wc)
{
  const uint32_t wave = *wc.wave;
  const uint32_t e0 = bt.wave_entry[wave], e1 = bt.wave_entry[wave + 1];
  const uint32_t total = bt.wave_items[wave];
  for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < total;
       base += gridDim.x * blockDim.x) {
    const uint32_t i = base + lane_id();
    const bool live = i < total;
    uint32_t slot = 0, sample_index = 0, job = 0;
    V3 ro{0.f, 0.f, 0.f}, rd{0.f, 0.f, 0.f};
    float tmin = 0.f, tmax = 0.f;
    if (live) {
      uint32_t lo = e0, hi = e1 - 1; // last entry with item_begin <= i
      while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) / 2;
        if (bt.entries[mid].item_begin <= i)
          lo = mid;
        else
          hi = mid - 1;
      }
      const BatchEntry e = bt.entries[lo];
      job = e.job;
      const RenderConst &rc = bt.jobs[job].rc;
      const uint32_t local = i - e.item_begin;
      const uint32_t s_local = local / rc.npix;
      const uint32_t pixel = local - s_local * rc.npix;
      const uint32_t s = e.sample_begin + s_local;
      slot = (s % rc.lanes) * rc.npix + pixel;
      sample_index = s + rc.sample_offset;
      camera_ray(rc, pixel, sample_index, ro, rd, tmin, tmax);
      bt.jobs[job].acc.nsamp[slot] += 1u;
    }
    const uint32_t o = warp_append(wc.count, live);
    if (live) {
      out.ray_o[o] = f4(ro, tmin);
      out.ray_d[o] = f4(rd, tmax);
      out.tp[o] = make_float4(1.f, 1.f, 1.f, -1.f);
      out.info[o] = make_uint4(slot, sample_index, 0u, (1u << 16) | (job << BATCH_JOB_SHIFT));
      out.pdist[o] = 0.f;
    }
  }
}

__global__ void __launch_bounds__(256) k_raygen(const RenderConst *__restrict__ rcp, DevScene sc, PathSoA out,
    Accum acc, WaveCounters wc)
{
  const RenderConst &rc = *rcp;
  const uint32_t wave = *wc.wave;
  const uint32_t total = rc.npix * rc.lanes;
  // Without adaptive sampling the live slots are a prefix of the slot order
  // (lane-major: the lanes below spp - wave * lanes), so the queue is the slot
  // order itself: position = slot, no atomic per warp.
  const bool dense = !rc.adaptive;
  if (dense) {
    const uint32_t first = wave * rc.lanes;
    const uint32_t live_lanes = first < rc.spp ? min(rc.lanes, rc.spp - first) : 0u;
    if (blockIdx.x == 0 && threadIdx.x == 0)
      wc.count[0] = live_lanes * rc.npix;
  }
  for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < total;
       base += gridDim.x * blockDim.x) {
    const uint32_t i = base + lane_id();
    bool live = false;
    uint32_t pixel = 0, slot = 0, sample_index = 0;
    V3 ro{0.f, 0.f, 0.f}, rd{0.f, 0.f, 0.f};
    float tmin = 0.f, tmax = 0.f;
    if (i < total) {
      const uint32_t lane = i / rc.npix;
      pixel = i - lane * rc.npix;
      slot = i;
      const uint32_t s = wave * rc.lanes + lane; // sample number within the render call
      if (s < rc.spp) {
        live = true;
        if (rc.adaptive && s >= 16u) { // variance gate (pathtracer.cpp:710-725), lanes == 1
          const uint32_t ns = acc.nsamp[slot];
          if (ns >= 16u) {
            const float4 a = acc.acc[slot], q = acc.acc_sq[slot];
            const V3 mean = V3{a.x, a.y, a.z} * (1.f / float(ns));
            const V3 sq = V3{q.x, q.y, q.z} * (1.f / float(ns));
            const V3 var = sq - V3{mean.x * mean.x, mean.y * mean.y, mean.z * mean.z};
            const float max_var = fmaxf(var.x, fmaxf(var.y, var.z));
            const float l = fmaxf(0.2126f * mean.x + 0.7152f * mean.y + 0.0722f * mean.z, 1e-4f);
            if (max_var / (l * l) < 0.01f)
              live = false;
          }
        }
        if (live) {
          sample_index = s + rc.sample_offset;
          camera_ray(rc, pixel, sample_index, ro, rd, tmin, tmax);
          if (rc.adaptive)
            acc.start[slot] = acc.acc[slot];
          acc.nsamp[slot] += 1u;
        }
      }
    }
    const uint32_t o = dense ? i : warp_append(wc.count, live);
    if (live) {
      out.ray_o[o] = f4(ro, tmin);
      out.ray_d[o] = f4(rd, tmax);
      out.tp[o] = make_float4(1.f, 1.f, 1.f, -1.f);
      out.info[o] = make_uint4(slot, sample_index, 0u, 1u << 16);
      out.pdist[o] = 0.f;
    }
  }
}

// Loop-trip cap reached (WAVE_TRIP_CAP): the first warp to report writes the
// error word and its record (the state of its first busy lane).  Called by
// every lane of the warp.
__device__ __forceinline__ void record_cap(const WaveCounters &wc, uint32_t code, uint32_t n, uint32_t fetched,
    bool busy, bool exhausted, uint32_t idx, float4 o, float4 d, const TravState &s, uint32_t steps, uint32_t rays,
    uint32_t fetch_trips, uint32_t step_trips, uint32_t max_steps, uint32_t max_idx, uint32_t trips)
{
  const uint32_t active = __activemask();
  const uint32_t bm = __ballot_sync(WARP_FULL, busy);
  // the busy lane with the most steps on its current ray
  uint32_t best = busy ? steps : 0u;
  for (int off = 16; off > 0; off >>= 1)
    best = max(best, __shfl_xor_sync(WARP_FULL, best, off));
  const uint32_t cand = __ballot_sync(WARP_FULL, busy && steps == best);
  uint32_t won = 0;
  if (lane_id() == 0)
    won = atomicCAS(wc.error, 0u, code) == 0u ? 1u : 0u;
  won = __shfl_sync(WARP_FULL, won, 0);
  if (!won)
    return;
  uint32_t *r = wc.dbg;
  if (lane_id() == 0) {
    r[0] = n;
    r[1] = fetched;
    r[2] = bm;
    r[3] = exhausted ? 1u : 0u;
  }
  if (cand != 0u && lane_id() == uint32_t(__ffs(int(cand)) - 1)) {
    r[4] = idx;
    r[5] = __float_as_uint(o.x);
    r[6] = __float_as_uint(o.y);
    r[7] = __float_as_uint(o.z);
    r[8] = __float_as_uint(o.w);
    r[9] = __float_as_uint(d.x);
    r[10] = __float_as_uint(d.y);
    r[11] = __float_as_uint(d.z);
    r[12] = uint32_t(s.sp);
    r[13] = s.g_base;
    r[14] = s.g_hits;
    r[15] = s.g_imask;
    r[16] = steps;
    r[17] = rays;
  }
  uint32_t ms = max_steps;
  for (int off = 16; off > 0; off >>= 1)
    ms = max(ms, __shfl_xor_sync(WARP_FULL, ms, off));
  const uint32_t mc = __ballot_sync(WARP_FULL, max_steps == ms);
  if (lane_id() == 0) {
    r[18] = fetch_trips;
    r[19] = step_trips;
    r[20] = ms;
    r[22] = trips;
    r[23] = active;
  }
  if (lane_id() == uint32_t(__ffs(int(mc)) - 1))
    r[21] = max_idx;
}

// ------------------------------------------------------------ closest hit
// Persistent warps with dynamic refill: a lane whose ray is finished idles
// until `refill` lanes of its warp are idle, then the warp fetches that many
// new rays with one atomic (ballot + popc), so long rays no longer hold a
// whole warp of finished lanes.  Each loop trip is one traversal step (one
// node and the triangles of its hit leaves) of every busy lane.  With SPLIT
// the finished queue positions also go to the hit or the miss index queue.
#ifndef PHC_TRACE_MIN_BLOCKS
#define PHC_TRACE_MIN_BLOCKS 8 // 64 registers: 8 resident 128-thread blocks per SM
#endif
#ifndef PHC_TRACE_MIN_BLOCKS_INST
#define PHC_TRACE_MIN_BLOCKS_INST 8 // the two-level variant (more state: the world ray)
#endif
// INST: the scene has instances (two-level traversal, trav_step2); the hit's
// instance slot goes to hq.inst.
template <bool COUNT, bool SPLIT, bool BATCH, bool INST = false>
__global__ void __launch_bounds__(128, INST ? PHC_TRACE_MIN_BLOCKS_INST : PHC_TRACE_MIN_BLOCKS) k_trace(DevScene sc, BatchTable bt, PathSoA in, float4 *__restrict__ hits,
    WaveCounters wc, int it, uint64_t *stats, uint32_t refill, HitQueues hq)
{
  if (wave_failed(wc))
    return;
  const uint32_t n = wc.count[it];
  uint32_t *fetch = wc.fetch + 4 * it;
  const uint32_t lane = lane_id();
  const uint32_t lt_mask = (1u << lane) - 1u;
  TravCounters ctr{0u, 0u};
  std::conditional_t<INST, TravState2, TravState> s;
  uint2 stack[PHC_STACK_SIZE];
  bool busy = false, exhausted = false;
  uint32_t idx = 0, steps = 0, rays = 0, fetch_trips = 0, step_trips = 0, max_steps = 0, max_idx = 0;
  const uint4 *nodes = sc.nodes;
  const float4 *tris = sc.tris;
  // The idle mask changes only when lanes finish or fetch, so the warp votes
  // (refill, queue appends) run only on trips where some lane finished.
  uint32_t idle = WARP_FULL;
  for (uint32_t trips = 0;; ++trips) {
    if (trips >= wc.trip_cap) { // warp-uniform: every lane counts the same trips
      record_cap(wc, (WAVE_ERR_TRACE << 16) | uint32_t(it), n, *fetch, busy, exhausted, idx, in.ray_o[idx],
          in.ray_d[idx], s, steps, rays, fetch_trips, step_trips, max_steps, max_idx, trips);
      break;
    }
    if (!exhausted && (idle == WARP_FULL || uint32_t(__popc(idle)) >= refill)) {
      __syncwarp();
      const uint32_t k = uint32_t(__popc(idle));
      const uint32_t base = warp_fetch(fetch, k);
      ++fetch_trips;
      if (base + k >= n)
        exhausted = true;
      if (!busy) {
        const uint32_t my = base + uint32_t(__popc(idle & lt_mask));
        if (my < n) {
          idx = my;
          const float4 o = in.ray_o[idx], d = in.ray_d[idx];
          if (BATCH) { // the BVH of the path's job
            const BatchJob &job = bt.jobs[in.info[idx].w >> BATCH_JOB_SHIFT];
            nodes = job.sc.nodes;
            tris = job.sc.tris;
          }
          if constexpr (INST)
            trav_init2(s, v3(o), v3(d), o.w, d.w);
          else
            trav_init(s, v3(o), v3(d), o.w, d.w);
          steps = 0;
          ++rays;
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
    bool done = false;
    ++step_trips;
    if (busy) {
      if constexpr (INST)
        done = !trav_step2<false, COUNT>(nodes, tris, sc.inst_w2o, sc.inst_info, s, stack, &ctr);
      else
        done = !trav_step<false, COUNT>(nodes, tris, s, stack, &ctr);
      ++steps;
      if (steps > max_steps) {
        max_steps = steps;
        max_idx = idx;
      }
    }
    __syncwarp(); // every lane back from the step's divergent work before the vote
    const uint32_t dm = __ballot_sync(WARP_FULL, done);
    if (dm == 0u)
      continue;
    if (SPLIT) {
      const bool is_hit = done && s.best.prim != 0xffffffffu;
      const uint32_t hm = __ballot_sync(WARP_FULL, is_hit);
      const uint32_t mm = dm & ~hm;
      uint32_t hb = 0, mb = 0;
      if (lane == 0) {
        if (hm)
          hb = atomicAdd(wc.hcount + it, uint32_t(__popc(hm)));
        if (mm)
          mb = atomicAdd(wc.mcount + it, uint32_t(__popc(mm)));
      }
      hb = __shfl_sync(WARP_FULL, hb, 0);
      mb = __shfl_sync(WARP_FULL, mb, 0);
      if (done) {
        if (is_hit)
          hq.hitq[hb + uint32_t(__popc(hm & lt_mask))] = idx;
        else
          hq.missq[mb + uint32_t(__popc(mm & lt_mask))] = idx;
      }
    }
    if (done) {
      hits[idx] = make_float4(s.best.t, __uint_as_float(s.best.prim), s.best.u, s.best.v);
      if constexpr (INST)
        hq.inst[idx] = s.best_inst;
      busy = false;
    }
    idle |= dm;
  }
  if (COUNT) {
    atomicAdd((unsigned long long *)&stats[0], (unsigned long long)ctr.nodes);
    atomicAdd((unsigned long long *)&stats[1], (unsigned long long)ctr.tris);
  }
}

// ------------------------------------------------------- material sort
// Counting sort of the hit queue by material, so that the hit-shading kernel
// sees runs of one material (coherent parameter branches, shared texture
// rows).  Histogram in shared memory, one-block exclusive scan, scatter with
// warp-aggregated atomics (lanes with the same bin take consecutive slots
// from one atomic).  Order within a bin is not preserved; every path's result
// is independent of the order it is shaded in.
// Bin of a queued hit: its material (batched renders: job and material).
// Sorting by shading class (hq.classes): the class's bins, then the material.
template <bool BATCH>
__device__ __forceinline__ uint32_t hit_bin(const DevScene &sc, const BatchTable &bt, const uint4 *info,
    const float4 *hits, const HitQueues &hq, uint32_t qi)
{
  const uint32_t prim = __float_as_uint(hits[qi].y);
  if (BATCH) {
    const uint32_t job = info[qi].w >> BATCH_JOB_SHIFT;
    const uint32_t mat = __ldg(&bt.jobs[job].sc.prim_vidx[prim].w);
    if (hq.classes)
      return __ldg(&bt.jobs[job].sc.materials[mat].shade_class) * MAT_CLASS_BINS + (job * 1031u + mat) % MAT_CLASS_BINS;
    return (job * 1031u + mat) % MAT_SORT_BINS;
  }
  const uint32_t mat = __ldg(&sc.prim_vidx[prim].w);
  if (hq.classes)
    return __ldg(&sc.materials[mat].shade_class) * MAT_CLASS_BINS + mat % MAT_CLASS_BINS;
  return mat % MAT_SORT_BINS;
}

template <bool BATCH>
__global__ void __launch_bounds__(256) k_mat_hist(DevScene sc, BatchTable bt, const uint4 *__restrict__ info,
    const float4 *__restrict__ hits, HitQueues hq, WaveCounters wc, int it, uint32_t *bins)
{
  if (wave_failed(wc))
    return;
  __shared__ uint32_t h[MAT_SORT_BINS];
  const uint32_t n = wc.hcount[it];
  if (n < hq.sort_threshold)
    return;
  for (uint32_t b = threadIdx.x; b < MAT_SORT_BINS; b += blockDim.x)
    h[b] = 0u;
  __syncthreads();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    atomicAdd(&h[hit_bin<BATCH>(sc, bt, info, hits, hq, hq.hitq[i])], 1u);
  __syncthreads();
  for (uint32_t b = threadIdx.x; b < MAT_SORT_BINS; b += blockDim.x)
    if (h[b])
      atomicAdd(&bins[b], h[b]);
}

// One block of MAT_SORT_BINS threads: bins[0..) counts -> bins[MAT_SORT_BINS..) starts.
__global__ void __launch_bounds__(MAT_SORT_BINS) k_mat_scan(HitQueues hq, WaveCounters wc, int it, uint32_t *bins)
{
  if (wave_failed(wc))
    return;
  __shared__ uint32_t t[MAT_SORT_BINS];
  if (wc.hcount[it] < hq.sort_threshold)
    return;
  const uint32_t b = threadIdx.x;
  t[b] = bins[b];
  __syncthreads();
  for (uint32_t off = 1; off < MAT_SORT_BINS; off <<= 1) { // Hillis-Steele inclusive scan
    const uint32_t v = b >= off ? t[b - off] : 0u;
    __syncthreads();
    t[b] += v;
    __syncthreads();
  }
  bins[MAT_SORT_BINS + b] = t[b] - bins[b];
}

// Scatter in chunks of 256 x MAT_SCATTER_PER_THREAD queue entries per block:
// ranks within the chunk from shared-memory counters (warp-aggregated), then
// one global atomic per (chunk, bin) reserves the chunk's run in that bin.
constexpr uint32_t MAT_SCATTER_PER_THREAD = 8;
template <bool BATCH>
__global__ void __launch_bounds__(256) k_mat_scatter(DevScene sc, BatchTable bt, const uint4 *__restrict__ info,
    const float4 *__restrict__ hits, HitQueues hq, WaveCounters wc, int it, uint32_t *bins)
{
  if (wave_failed(wc))
    return;
  __shared__ uint32_t cnt[MAT_SORT_BINS];
  const uint32_t n = wc.hcount[it];
  if (n < hq.sort_threshold)
    return;
  uint32_t *start = bins + MAT_SORT_BINS;
  const uint32_t chunk = blockDim.x * MAT_SCATTER_PER_THREAD;
  for (uint32_t c0 = blockIdx.x * chunk; c0 < n; c0 += gridDim.x * chunk) {
    for (uint32_t b = threadIdx.x; b < MAT_SORT_BINS; b += blockDim.x)
      cnt[b] = 0u;
    __syncthreads();
    uint32_t q[MAT_SCATTER_PER_THREAD], bin[MAT_SCATTER_PER_THREAD], rank[MAT_SCATTER_PER_THREAD];
#pragma unroll
    for (uint32_t k = 0; k < MAT_SCATTER_PER_THREAD; ++k) {
      const uint32_t i = c0 + k * blockDim.x + threadIdx.x;
      const bool live = i < n;
      q[k] = live ? hq.hitq[i] : 0u;
      bin[k] = live ? hit_bin<BATCH>(sc, bt, info, hits, hq, q[k]) : 0xffffffffu;
      const uint32_t grp = __match_any_sync(WARP_FULL, bin[k]);
      const uint32_t leader = uint32_t(__ffs(int(grp)) - 1);
      uint32_t r = 0;
      if (live && lane_id() == leader)
        r = atomicAdd(&cnt[bin[k]], uint32_t(__popc(grp)));
      r = __shfl_sync(WARP_FULL, r, int(leader));
      rank[k] = r + uint32_t(__popc(grp & ((1u << lane_id()) - 1u)));
    }
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < MAT_SORT_BINS; b += blockDim.x)
      if (cnt[b])
        cnt[b] = atomicAdd(&start[b], cnt[b]); // the chunk's run in bin b
    __syncthreads();
#pragma unroll
    for (uint32_t k = 0; k < MAT_SCATTER_PER_THREAD; ++k)
      if (bin[k] != 0xffffffffu)
        hq.sorted[cnt[bin[k]] + rank[k]] = q[k];
    __syncthreads();
  }
}

// ----------------------------------------------------------------- shadow
// Any-hit traversal of the shadow queue, then the NEE contribution of the
// unoccluded rays times the ratio-tracking transmittance of the volumes
// (stream dimension 0x10000 + iteration), added to the path's pixel slot.
template <bool COUNT, bool BATCH, bool DEFER = false, bool INST = false>
__global__ void __launch_bounds__(128) k_shadow(const RenderConst *__restrict__ rcp, DevScene sc, BatchTable bt,
    ShadowSoA sh, Accum acc_param, WaveCounters wc, int it, uint64_t *stats, uint32_t refill)
{
  if (wave_failed(wc))
    return;
  const uint32_t n = wc.scount[it];
  uint32_t *fetch = wc.fetch + 4 * it + 3;
  const uint32_t lane = lane_id();
  const uint32_t lt_mask = (1u << lane) - 1u;
  TravCounters ctr{0u, 0u};
  std::conditional_t<INST, TravState2, TravState> s;
  uint2 stack[PHC_STACK_SIZE];
  bool busy = false, exhausted = false;
  uint32_t idx = 0, job = 0, steps = 0, rays = 0, fetch_trips = 0, step_trips = 0, max_steps = 0, max_idx = 0;
  const uint4 *nodes = sc.nodes;
  const float4 *tris = sc.tris;
  // persistent warps with dynamic refill, as in k_trace: the idle mask
  // changes only where lanes finish or fetch
  uint32_t idle = WARP_FULL;
  for (uint32_t trips = 0;; ++trips) {
    if (trips >= wc.trip_cap) {
      record_cap(wc, (WAVE_ERR_SHADOW << 16) | uint32_t(it), n, *fetch, busy, exhausted, idx, sh.a[idx], sh.b[idx],
          s, steps, rays, fetch_trips, step_trips, max_steps, max_idx, trips);
      break;
    }
    if (!exhausted && (idle == WARP_FULL || uint32_t(__popc(idle)) >= refill)) {
      __syncwarp();
      const uint32_t k = uint32_t(__popc(idle));
      const uint32_t base = warp_fetch(fetch, k);
      ++fetch_trips;
      if (base + k >= n)
        exhausted = true;
      if (!busy) {
        const uint32_t my = base + uint32_t(__popc(idle & lt_mask));
        if (my < n) {
          idx = my;
          const float4 a = sh.a[idx], b = sh.b[idx];
          if (BATCH) {
            job = sh.job[idx];
            nodes = bt.jobs[job].sc.nodes;
            tris = bt.jobs[job].sc.tris;
          }
          if constexpr (INST)
            trav_init2(s, v3(a), v3(b), 0.f, a.w);
          else
            trav_init(s, v3(a), v3(b), 0.f, a.w);
          steps = 0;
          ++rays;
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
    ++step_trips;
    bool more = true;
    if (busy) {
      ++steps;
      if (steps > max_steps) {
        max_steps = steps;
        max_idx = idx;
      }
      if constexpr (INST)
        more = trav_step2<true, COUNT>(nodes, tris, sc.inst_w2o, sc.inst_info, s, stack, &ctr);
      else
        more = trav_step<true, COUNT>(nodes, tris, s, stack, &ctr);
    }
    if (busy && !more) {
      busy = false;
      // Unoccluded: add the contribution here when the ray's scene has no
      // volume; otherwise leave the ray (tmax >= 0) to k_shadow_volume, so
      // that no lane runs a tracking loop inside this warp-voting loop.
      // Occluded or done: tmax < 0.
      // DEFER: every unoccluded ray is left to a later kernel (the adjoint's).
      const bool vol = DEFER || (BATCH ? bt.jobs[job].sc.volume_count : sc.volume_count) > 0;
      const bool open = s.best.prim == 0xffffffffu;
      if (open && !vol) {
        const Accum &acc = BATCH ? bt.jobs[job].acc : acc_param;
        const float4 b = sh.b[idx], c = sh.c[idx];
        const V3 contrib{b.w, c.x, c.y};
        const uint32_t slot = __float_as_uint(c.z);
        if (finite3(contrib)) {
          float4 v = acc.acc[slot];
          v.x = v.x + contrib.x;
          v.y = v.y + contrib.y;
          v.z = v.z + contrib.z;
          acc.acc[slot] = v;
        }
      }
      if (!(open && vol))
        sh.a[idx].w = -1.f;
    }
    __syncwarp(); // every lane back from the step's divergent work before the vote
    idle = __ballot_sync(WARP_FULL, !busy);
  }
  if (COUNT) {
    atomicAdd((unsigned long long *)&stats[0], (unsigned long long)ctr.nodes);
    atomicAdd((unsigned long long *)&stats[1], (unsigned long long)ctr.tris);
  }
}

// The unoccluded shadow rays of volume scenes (tmax >= 0 after k_shadow):
// contribution times the ratio-tracking transmittance of the volumes along
// [0, tmax] (stream dimension 0x10000 + iteration), added to the path's slot.
// lookups (or nullptr): density lookups made, added up over the grid.
template <bool BATCH>
__global__ void __launch_bounds__(128) k_shadow_volume(const RenderConst *__restrict__ rcp, DevScene sc,
    BatchTable bt, ShadowSoA sh, Accum acc_param, WaveCounters wc, int it, unsigned long long *lookups)
{
  if (wave_failed(wc))
    return;
  // the unoccluded shadow rays (tmax >= 0) of the iteration: ratio-tracking
  // transmittance (stream dimension 0x10000 + iteration) times the NEE
  // contribution into the path's pixel slot; persistent warps with refill,
  // one tracking pass per busy lane and trip, as in k_vol_scatter
  const uint32_t n = wc.scount[it];
  uint32_t *fetch = wc.vfetch + 2 * it + 1;
  const uint32_t lane = lane_id();
  const uint32_t lt_mask = (1u << lane) - 1u;
  VolTrack s;
  Rng rng(1u);
  bool busy = false, exhausted = false;
  uint32_t idx = 0, job = 0, idle = WARP_FULL, nlook = 0;
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
          const float4 a = sh.a[my];
          if (a.w >= 0.f) { // occluded or already accumulated rays: tmax < 0
            idx = my;
            job = BATCH ? sh.job[idx] : 0u;
            const uint32_t npix = BATCH ? bt.jobs[job].rc.npix : rcp->npix;
            const float4 b = sh.b[idx], c = sh.c[idx];
            rng = path_rng(__float_as_uint(c.z) % npix, __float_as_uint(c.w), 0x10000u + uint32_t(it));
            vt_init(s, v3(a), v3(b), 0.f, a.w);
            busy = true;
          }
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
      const DevScene &S = BATCH ? bt.jobs[job].sc : sc;
      nlook += vt_passes<false>(S, s, rng, wc.vol_passes) == VT_LOOKUP ? 1u : 0u;
      if (s.done) {
        busy = false;
        const Accum &acc = BATCH ? bt.jobs[job].acc : acc_param;
        const float4 b = sh.b[idx], c = sh.c[idx];
        const uint32_t slot = __float_as_uint(c.z);
        const V3 contrib = V3{b.w, c.x, c.y} * s.tr;
        if (finite3(contrib)) {
          float4 v = acc.acc[slot];
          v.x = v.x + contrib.x;
          v.y = v.y + contrib.y;
          v.z = v.z + contrib.z;
          acc.acc[slot] = v;
        }
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

// End of a wave: adaptive variance update (pathtracer.cpp:1129-1139), ray
// totals, and the wave index for the next replay.
__global__ void __launch_bounds__(256) k_wave_end(const RenderConst *__restrict__ rcp, Accum acc, WaveCounters wc,
    uint32_t npix, int adaptive, int max_iter, unsigned long long *ray_totals)
{
  if (adaptive) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x) {
      const float4 a = acc.acc[i], s = acc.start[i];
      const V3 sv = V3{a.x, a.y, a.z} - V3{s.x, s.y, s.z};
      float4 q = acc.acc_sq[i];
      q.x = q.x + sv.x * sv.x;
      q.y = q.y + sv.y * sv.y;
      q.z = q.z + sv.z * sv.z;
      acc.acc_sq[i] = q;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    unsigned long long cr = 0, sr = 0;
    for (int k = 0; k < max_iter; ++k) {
      cr += wc.count[k];
      sr += wc.scount[k];
    }
    ray_totals[0] += wc.count[0];
    ray_totals[1] += cr;
    ray_totals[2] += sr;
    *wc.wave += 1u;
  }
}

// pt_resolve + accumulate_frame: per pixel the lanes' sums in lane order,
// divided by the samples started, weighted into the frame.  The depth,
// normal and albedo of the earliest sample that reached a primary event.
__global__ void __launch_bounds__(256) k_resolve(Accum acc, Frame fr, uint32_t npix, uint32_t lanes, float weight,
    int first)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
    float4 sum = acc.acc[p];
    uint32_t ns = acc.nsamp[p];
    float4 an = acc.aov_n[p], aa = acc.aov_a[p];
    for (uint32_t l = 1; l < lanes; ++l) {
      const size_t s = size_t(l) * npix + p;
      const float4 v = acc.acc[s];
      sum.x = sum.x + v.x;
      sum.y = sum.y + v.y;
      sum.z = sum.z + v.z;
      sum.w = sum.w + v.w;
      ns += acc.nsamp[s];
      const float4 a2 = acc.aov_a[s];
      const uint32_t w2 = __float_as_uint(a2.w), w1 = __float_as_uint(aa.w);
      if (w2 != 0u && (w1 == 0u || w2 < w1)) {
        aa = a2;
        an = acc.aov_n[s];
      }
    }
    const float inv = ns > 0 ? (1.f / float(ns)) : 0.f;
    const float4 color = make_float4(sum.x * inv, sum.y * inv, sum.z * inv, sum.w * inv);
    const bool written = __float_as_uint(aa.w) != 0u;
    const float depth = written ? an.w : 1e30f;
    if (first) {
      fr.color[p] = make_float4(color.x * weight, color.y * weight, color.z * weight, color.w * weight);
      fr.normal[p] = written ? make_float4(an.x, an.y, an.z, depth) : make_float4(0.f, 0.f, 0.f, depth);
      fr.albedo[p] = written ? make_float4(aa.x, aa.y, aa.z, 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
    } else {
      float4 c = fr.color[p];
      c.x = c.x + color.x * weight;
      c.y = c.y + color.y * weight;
      c.z = c.z + color.z * weight;
      c.w = c.w + color.w * weight;
      fr.color[p] = c;
    }
  }
}

// Channels in the bridge's read-back layout (RenderBridge.cpp:1082-1172).
__global__ void __launch_bounds__(256) k_read(Frame fr, uint32_t npix, float inv, int channel, float *out)
{
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
    if (channel == 0) {
      const float4 c = fr.color[p];
      const float a = c.w * inv;
      reinterpret_cast<float4 *>(out)[p] =
          make_float4(c.x * inv, c.y * inv, c.z * inv, a < 0.f ? 0.f : (a > 1.f ? 1.f : a));
    } else if (channel == 1) {
      const float d = fr.normal[p].w;
      out[p] = d < 1e29f ? d : __int_as_float(0x7f800000);
    } else {
      const float4 v = channel == 2 ? fr.normal[p] : fr.albedo[p];
      out[3 * p] = v.x;
      out[3 * p + 1] = v.y;
      out[3 * p + 2] = v.z;
    }
  }
}

} // namespace

// ------------------------------------------------------------- launchers

void launch_raygen(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, PathSoA out, Accum acc,
    WaveCounters wc)
{
  k_raygen<<<c.blocks_raygen, 256, 0, s>>>(rc, sc, out, acc, wc);
}

void launch_trace(const LaunchCfg &c, cudaStream_t s, DevScene sc, PathSoA in, float4 *hits, WaveCounters wc, int it,
    uint64_t *stats, int refill, HitQueues hq)
{
  const uint32_t r = uint32_t(refill < 1 ? 1 : (refill > 32 ? 32 : refill));
  const bool split = hq.hitq != nullptr;
  const BatchTable none{};
  if (sc.inst_count > 0) { // two-level traversal
    if (stats) {
      if (split)
        k_trace<true, true, false, true><<<c.blocks_trace, 128, 0, s>>>(sc, none, in, hits, wc, it, stats, r, hq);
      else
        k_trace<true, false, false, true><<<c.blocks_trace, 128, 0, s>>>(sc, none, in, hits, wc, it, stats, r, hq);
    } else {
      if (split)
        k_trace<false, true, false, true><<<c.blocks_trace, 128, 0, s>>>(sc, none, in, hits, wc, it, nullptr, r, hq);
      else
        k_trace<false, false, false, true><<<c.blocks_trace, 128, 0, s>>>(sc, none, in, hits, wc, it, nullptr, r, hq);
    }
    return;
  }
  if (stats) {
    if (split)
      k_trace<true, true, false><<<c.blocks_trace, 128, 0, s>>>(sc, none, in, hits, wc, it, stats, r, hq);
    else
      k_trace<true, false, false><<<c.blocks_trace, 128, 0, s>>>(sc, none, in, hits, wc, it, stats, r, hq);
  } else {
    if (split)
      k_trace<false, true, false><<<c.blocks_trace, 128, 0, s>>>(sc, none, in, hits, wc, it, nullptr, r, hq);
    else
      k_trace<false, false, false><<<c.blocks_trace, 128, 0, s>>>(sc, none, in, hits, wc, it, nullptr, r, hq);
  }
}

void launch_shadow(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, ShadowSoA sh, Accum acc,
    WaveCounters wc, int it, uint64_t *stats, int refill)
{
  const uint32_t r = uint32_t(refill < 1 ? 1 : (refill > 32 ? 32 : refill));
  const BatchTable none{};
  if (sc.inst_count > 0) {
    if (stats)
      k_shadow<true, false, false, true><<<c.blocks_trace, 128, 0, s>>>(rc, sc, none, sh, acc, wc, it, stats, r);
    else
      k_shadow<false, false, false, true><<<c.blocks_trace, 128, 0, s>>>(rc, sc, none, sh, acc, wc, it, nullptr, r);
  } else if (stats)
    k_shadow<true, false><<<c.blocks_trace, 128, 0, s>>>(rc, sc, none, sh, acc, wc, it, stats, r);
  else
    k_shadow<false, false><<<c.blocks_trace, 128, 0, s>>>(rc, sc, none, sh, acc, wc, it, nullptr, r);
}

void launch_shadow_volume(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, ShadowSoA sh,
    Accum acc, WaveCounters wc, int it, uint64_t *lookups)
{
  k_shadow_volume<false><<<c.blocks_trace, 128, 0, s>>>(rc, sc, BatchTable{}, sh, acc, wc, it,
      reinterpret_cast<unsigned long long *>(lookups));
}

void launch_raygen_batch(const LaunchCfg &c, cudaStream_t s, BatchTable bt, PathSoA out, WaveCounters wc)
{
  k_raygen_batch<<<c.blocks_raygen, 256, 0, s>>>(bt, out, wc);
}

void launch_trace_batch(const LaunchCfg &c, cudaStream_t s, BatchTable bt, PathSoA in, float4 *hits,
    WaveCounters wc, int it, int refill, HitQueues hq)
{
  const uint32_t r = uint32_t(refill < 1 ? 1 : (refill > 32 ? 32 : refill));
  const DevScene none{};
  if (hq.hitq)
    k_trace<false, true, true><<<c.blocks_trace, 128, 0, s>>>(none, bt, in, hits, wc, it, nullptr, r, hq);
  else
    k_trace<false, false, true><<<c.blocks_trace, 128, 0, s>>>(none, bt, in, hits, wc, it, nullptr, r, hq);
}

void launch_material_sort(const LaunchCfg &c, cudaStream_t s, DevScene sc, const float4 *hits, HitQueues hq,
    WaveCounters wc, int it, uint32_t *bins)
{
  const int blocks = c.blocks_raygen > 0 ? c.blocks_raygen : 1;
  const BatchTable none{};
  k_mat_hist<false><<<blocks, 256, 0, s>>>(sc, none, nullptr, hits, hq, wc, it, bins);
  k_mat_scan<<<1, MAT_SORT_BINS, 0, s>>>(hq, wc, it, bins);
  k_mat_scatter<false><<<blocks, 256, 0, s>>>(sc, none, nullptr, hits, hq, wc, it, bins);
}

void launch_material_sort_batch(const LaunchCfg &c, cudaStream_t s, BatchTable bt, const uint4 *info,
    const float4 *hits, HitQueues hq, WaveCounters wc, int it, uint32_t *bins)
{
  const int blocks = c.blocks_raygen > 0 ? c.blocks_raygen : 1;
  k_mat_hist<true><<<blocks, 256, 0, s>>>(DevScene{}, bt, info, hits, hq, wc, it, bins);
  k_mat_scan<<<1, MAT_SORT_BINS, 0, s>>>(hq, wc, it, bins);
  k_mat_scatter<true><<<blocks, 256, 0, s>>>(DevScene{}, bt, info, hits, hq, wc, it, bins);
}

void launch_shadow_deferred(const LaunchCfg &c, cudaStream_t s, DevScene sc, ShadowSoA sh, WaveCounters wc, int it,
    int refill)
{
  const uint32_t r = uint32_t(refill < 1 ? 1 : (refill > 32 ? 32 : refill));
  k_shadow<false, false, true><<<c.blocks_trace, 128, 0, s>>>(nullptr, sc, BatchTable{}, sh, Accum{}, wc, it, nullptr, r);
}

void launch_shadow_batch(const LaunchCfg &c, cudaStream_t s, BatchTable bt, ShadowSoA sh, WaveCounters wc, int it,
    int refill, bool volumes)
{
  const uint32_t r = uint32_t(refill < 1 ? 1 : (refill > 32 ? 32 : refill));
  k_shadow<false, true><<<c.blocks_trace, 128, 0, s>>>(nullptr, DevScene{}, bt, sh, Accum{}, wc, it, nullptr, r);
  if (volumes)
    k_shadow_volume<true><<<c.blocks_trace, 128, 0, s>>>(nullptr, DevScene{}, bt, sh, Accum{}, wc, it, nullptr);
}

void launch_wave_end(cudaStream_t s, const RenderConst *rc, Accum acc, WaveCounters wc, uint32_t npix, int adaptive,
    int max_iter, uint64_t *ray_totals)
{
  const uint32_t blocks = adaptive ? (npix + 255) / 256 : 1u;
  k_wave_end<<<blocks, 256, 0, s>>>(rc, acc, wc, npix, adaptive, max_iter, (unsigned long long *)ray_totals);
}

void launch_resolve(cudaStream_t s, Accum acc, Frame fr, uint32_t npix, uint32_t lanes, float weight, int first)
{
  k_resolve<<<(npix + 255) / 256, 256, 0, s>>>(acc, fr, npix, lanes, weight, first);
}

void launch_read(cudaStream_t s, Frame fr, uint32_t npix, float inv_samples, int channel, float *out)
{
  k_read<<<(npix + 255) / 256, 256, 0, s>>>(fr, npix, inv_samples, channel, out);
}

int shade_max_active_blocks(int threads, bool full);

int max_active_blocks(int which, int threads)
{
  int n = 0;
  switch (which) {
  case 0: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_trace<false, true, false>, threads, 0); break;
  case 1: n = shade_max_active_blocks(threads, true); break;
  case 4: n = shade_max_active_blocks(threads, false); break;
  case 2: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_shadow<false, false>, threads, 0); break;
  default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_raygen, threads, 0); break;
  }
  return n;
}

} // namespace phc
