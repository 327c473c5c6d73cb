// Wavefront state and kernel launchers of the renderer (host/device view).
//
// One render call runs the samples of every pixel as waves of `lanes`
// samples; one wave is a fixed sequence of launches (raygen, then per bounce
// iteration: closest-hit trace, shade, shadow trace) over SoA queues in HBM
// whose lengths live in device counters, so the host never waits between
// bounces (the reference reduces the active count to the host every bounce,
// pathtracer.cpp:1094-1126).  The sequence is captured once as a CUDA graph
// and replayed per wave.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "scene_types.h"

namespace phc {

// Per-render-call constants (camera, settings), in device memory.
struct RenderConst {
  float origin[3], lower_left[3], horizontal[3], vertical[3], cu[3], cv[3], cw[3];
  float lens_radius;
  int32_t ortho;
  float clip_near, clip_far;
  float region[4];
  uint32_t w, h, npix, spp;
  uint32_t sample_offset; // bridge sample counter when the render call began
  uint32_t max_depth, max_iter;
  float bg[4];
  const float4 *bg_image;
  uint32_t bg_w, bg_h;
  float ambient[3];
  int32_t adaptive;
  float tp_clamp;
  int32_t max_diffuse, max_glossy, max_transmission, max_volume;
  float clamp_direct, clamp_indirect;
  uint32_t lanes; // samples of one pixel in flight per wave
};

// Path state, structure of arrays over `cap` slots (two copies, ping-pong).
struct PathSoA {
  float4 *ray_o; // org.xyz, tmin
  float4 *ray_d; // dir.xyz, tmax
  float4 *tp;    // throughput.xyz, prev_pdf (< 0: delta / none)
  uint4 *info;   // pixel, sample index, bounce kinds, depth | primary << 16
  float *pdist;  // distance travelled by the camera ray
};

// Shadow ray queue: (o.xyz, tmax), (d.xyz, contrib.x), (contrib.yz, slot,
// sample); job: the batch job of each ray (batched renders only).
struct ShadowSoA {
  float4 *a, *b, *c;
  uint32_t *job;
};

// Per pixel-slot accumulators (slot = lane * npix + pixel).
struct Accum {
  float4 *acc;      // radiance.xyz, alpha
  float4 *acc_sq;   // adaptive: squared sample values
  float4 *start;    // adaptive: acc when the last sample began
  uint32_t *nsamp;  // samples started
  float4 *aov_n;    // normal.xyz, depth
  float4 *aov_a;    // albedo.xyz, (sample index + 1) of the write as float bits, 0 unwritten
};

// Device counters of one wave.
struct WaveCounters {
  uint32_t *count;   // [max_iter + 1] paths entering iteration it
  uint32_t *scount;  // [max_iter] shadow rays of iteration it
  uint32_t *hcount;  // [max_iter] closest-hit results that hit (split queues)
  uint32_t *mcount;  // [max_iter] closest-hit results that missed (split queues)
  uint32_t *fetch;   // [4 * max_iter] work counters: trace, shade (all/hits), shade misses, shadow
  uint32_t *vfetch;  // [2 * max_iter] work counters: volume scattering, shadow transmittance
  uint32_t *cfetch;  // [SHADE_CLASSES * max_iter] work counters of the class hit-shading kernels
  uint32_t *vcount;  // [max_iter] paths that scatter in a volume (volume scenes, split queues)
  uint32_t *vqfetch; // [max_iter] work counters of the shading of those paths
  uint32_t *wave;    // current wave index within the render call
  uint32_t *error;   // sticky error word
  uint32_t *dbg;     // [WAVE_DBG_WORDS] record of the first self-check failure
  uint32_t trip_cap; // loop trips after which a persistent warp stops (tuning key wave_trip_cap)
  uint32_t vol_refill; // a volume-tracking warp takes new rays once this many lanes are idle (tuning key vol_refill)
  uint32_t vol_passes; // tracking passes per lane and loop trip at most (tuning key vol_passes)
};
inline size_t wave_counter_words(int max_iter) { return size_t((12 + SHADE_CLASSES) * max_iter + 1); }

// Self-check of the persistent traversal loops: a warp that makes more than
// WaveCounters::trip_cap loop trips (each trip is one traversal step of every
// busy lane; legitimate work needs a few thousand; default WAVE_TRIP_CAP)
// stops and records (kernel << 16) | iteration in the error word, first
// writer wins.  Every later kernel of the wave then returns at entry
// (wave_failed), so nothing reads the results the stopped warps never wrote.
constexpr uint32_t WAVE_TRIP_CAP = 1u << 24;
__device__ __forceinline__ bool wave_failed(const WaveCounters &wc) { return *(volatile uint32_t *)wc.error != 0u; }
enum : uint32_t { WAVE_ERR_TRACE = 1u, WAVE_ERR_SHADOW = 2u, WAVE_ERR_VOLUME = 3u };
// dbg words: queue length, fetch counter, busy ballot, exhausted, then for
// the warp's first busy lane: ray index, origin xyz, tmax, direction xyz,
// stack depth, group base, group hits, group internal mask, steps of the ray.
constexpr uint32_t WAVE_DBG_WORDS = 24;
// Counter words after the per-wave block: wave, error, 2 spare, dbg.
inline size_t wave_counter_alloc_bytes(int max_iter) { return (wave_counter_words(max_iter) + 4 + WAVE_DBG_WORDS) * 4; }

// Indices (into the iteration's path queue) of the paths whose closest-hit
// query hit / missed, when the shading of misses and hits is split.
// sorted / sort_threshold: when the iteration has at least sort_threshold
// hits (0: never), the hit queue is also sorted by material into `sorted`
// (launch_material_sort) and the hit-shading kernel reads that order.
struct HitQueues {
  uint32_t *hitq;
  uint32_t *missq;
  uint32_t *sorted = nullptr;
  uint32_t sort_threshold = 0;
  uint32_t *inst = nullptr; // per path: instance slot of its hit (scenes with instances)
  // Scenes with volumes: the scattering event sampled along each path's
  // segment by k_vol_scatter before shading (t or -1, albedo.xyz) and the
  // path's random-number state after it, from which shading continues.
  float4 *vscatter = nullptr;
  uint32_t *vrng = nullptr;
  // Volume scenes with split queues: after k_vol_scatter, k_vol_route puts
  // every path in vscatq (it scatters in a volume; wc.vcount), hitq or missq
  // (it reaches its surface hit / escapes; wc.hcount / wc.mcount), and the
  // closest-hit kernel writes no queue.
  uint32_t *vscatq = nullptr;
  // Sorting by shading class (lean scenes): bins are grouped per class
  // (MAT_CLASS_BINS each, class-major), and after the sort cls_end[b] is
  // the end of bin b's run in `sorted`, so class c's hits are the run
  // [cls_end[c * MAT_CLASS_BINS - 1] (0 for c = 0), cls_end[(c + 1) *
  // MAT_CLASS_BINS - 1]), shaded by that class's kernel.
  uint32_t classes = 0;
  const uint32_t *cls_end = nullptr;
};
constexpr uint32_t MAT_SORT_BINS = 1024; // materials map to bin = id % MAT_SORT_BINS
constexpr uint32_t MAT_CLASS_BINS = MAT_SORT_BINS / SHADE_CLASSES; // sorting by class: bin = class * this + id % this

// Shading kernel variants: FULL compiles volumes, material sources and
// analytic lights; PART 0 shades every path, 1 the hit queue, 2 the misses,
// 3 the paths that scatter in a volume (FULL only).
struct ShadeVariant {
  bool full;
  int part;
};

// Frame accumulated across render calls (RenderBridge.cpp:386-410).
struct Frame {
  float4 *color;  // rgb * weight sum, alpha
  float4 *normal; // xyz, depth
  float4 *albedo;
};

struct LaunchCfg {
  int blocks_trace, blocks_shade, blocks_raygen;
  int blocks_shade_lean; // grid of the lean shading variant (its own occupancy)
  int threads;
};

// ---------------------------------------------------------------- batches
// One job of a batched render: its scene, constants and accumulators.  Paths
// of all jobs share the queues; bits 17..31 of PathSoA::info.w hold the job.
struct BatchJob {
  DevScene sc;
  RenderConst rc;
  Accum acc;
};
// One entry of a batch wave: `nsamples` consecutive samples (from
// sample_begin) of every pixel of `job`, as items [item_begin, item_begin +
// nsamples * npix) of the wave.
struct BatchEntry {
  uint32_t job;
  uint32_t sample_begin;
  uint32_t nsamples;
  uint32_t item_begin;
};
struct BatchTable {
  const BatchJob *jobs;
  const BatchEntry *entries;  // all waves' entries
  const uint32_t *wave_entry; // [waves + 1] first entry of each wave
  const uint32_t *wave_items; // [waves] paths of each wave
};
constexpr uint32_t BATCH_JOB_SHIFT = 17;
constexpr uint32_t MAX_BATCH_JOBS = 1u << (32 - BATCH_JOB_SHIFT);

void launch_raygen_batch(const LaunchCfg &c, cudaStream_t s, BatchTable bt, PathSoA out, WaveCounters wc);
void launch_trace_batch(const LaunchCfg &c, cudaStream_t s, BatchTable bt, PathSoA in, float4 *hits,
    WaveCounters wc, int it, int refill, HitQueues hq);
void launch_shade_batch(const LaunchCfg &c, cudaStream_t s, BatchTable bt, PathSoA in, PathSoA out,
    const float4 *hits, ShadowSoA sh, WaveCounters wc, int it, ShadeVariant v, HitQueues hq);
// volumes: some job of the batch has volumes (k_shadow_volume runs too).
void launch_shadow_batch(const LaunchCfg &c, cudaStream_t s, BatchTable bt, ShadowSoA sh, WaveCounters wc, int it,
    int refill, bool volumes);

void launch_raygen(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, PathSoA out, Accum acc,
    WaveCounters wc);
// refill: a warp takes new rays once at least this many of its lanes are
// idle (32: only when all are).  hq.hitq != nullptr: also write the hit and
// miss index queues.
void launch_trace(const LaunchCfg &c, cudaStream_t s, DevScene sc, PathSoA in, float4 *hits, WaveCounters wc, int it,
    uint64_t *stats, int refill, HitQueues hq);
void launch_shade(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, PathSoA in, PathSoA out,
    const float4 *hits, ShadowSoA sh, Accum acc, WaveCounters wc, int it, ShadeVariant v, HitQueues hq);
// The lean hit-shading kernel of shading class cls (1 .. SHADE_CLASSES - 1)
// over its run of the class-sorted hit queue (hq.cls_end); class 0 is
// launch_shade's lean hit kernel.
void launch_shade_class(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, PathSoA in,
    PathSoA out, const float4 *hits, ShadowSoA sh, Accum acc, WaveCounters wc, int it, uint32_t cls, HitQueues hq);
// The batched wavefront's class kernels (shade_classes_batch.cu).
void launch_shade_class_batch(const LaunchCfg &c, cudaStream_t s, BatchTable bt, PathSoA in, PathSoA out,
    const float4 *hits, ShadowSoA sh, WaveCounters wc, int it, uint32_t cls, HitQueues hq);
// Delta tracking of every path of iteration `it` through the scene's volumes
// (the first step of pt_shade for volume scenes), into hq.vscatter / hq.vrng.
// lookups (or nullptr): the density lookups are added to it.
void launch_vol_scatter(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, PathSoA in,
    const float4 *hits, WaveCounters wc, int it, HitQueues hq, uint64_t *lookups);
void launch_vol_route(const LaunchCfg &c, cudaStream_t s, const float4 *hits, WaveCounters wc, int it, HitQueues hq);
void launch_shadow(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, ShadowSoA sh, Accum acc,
    WaveCounters wc, int it, uint64_t *stats, int refill);
// Volume scenes, after launch_shadow: ratio-tracking transmittance of the
// unoccluded shadow rays times their contribution, into the pixel slots.
void launch_shadow_volume(const LaunchCfg &c, cudaStream_t s, const RenderConst *rc, DevScene sc, ShadowSoA sh,
    Accum acc, WaveCounters wc, int it, uint64_t *lookups);
// Counting sort of iteration it's hit queue by material (when hcount[it] >=
// hq.sort_threshold): bins = 2 * MAT_SORT_BINS words of scratch.
void launch_material_sort(const LaunchCfg &c, cudaStream_t s, DevScene sc, const float4 *hits, HitQueues hq,
    WaveCounters wc, int it, uint32_t *bins);
// Batched renders: bins by (job, material); info = the iteration's path info.
void launch_material_sort_batch(const LaunchCfg &c, cudaStream_t s, BatchTable bt, const uint4 *info,
    const float4 *hits, HitQueues hq, WaveCounters wc, int it, uint32_t *bins);
// Occlusion only: unoccluded rays keep tmax >= 0, occluded ones get tmax < 0.
void launch_shadow_deferred(const LaunchCfg &c, cudaStream_t s, DevScene sc, ShadowSoA sh, WaveCounters wc, int it,
    int refill);
void launch_wave_end(cudaStream_t s, const RenderConst *rc, Accum acc, WaveCounters wc, uint32_t npix, int adaptive,
    int max_iter, uint64_t *ray_totals);
void launch_resolve(cudaStream_t s, Accum acc, Frame fr, uint32_t npix, uint32_t lanes, float weight, int first);
void launch_read(cudaStream_t s, Frame fr, uint32_t npix, float inv_samples, int channel, float *out);
// Resident blocks per SM of a kernel (0 trace, 1 shade, 2 shadow, 3 raygen).
int max_active_blocks(int which, int threads);

} // namespace phc
