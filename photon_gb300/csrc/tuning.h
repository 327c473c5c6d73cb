// Launch and scheduling parameters of the renderer, set by the autotuner
// (photon_gb300/autotune.py) through phc_tuning_set or the PHC_TUNE_<KEY>
// environment variables, read once per render call.  The defaults are the
// autotuner's choice on the 500K-triangle workload (1024^2, 128 spp) on GB300;
// the GPU-built BVH8 traverses in 12.8 node visits per ray there against the
// host SAH build's 14.3 and uploads in 0.018 s against 0.21 s.
#pragma once

#include <cstdint>

namespace phc {

struct Tuning {
  int64_t wave_paths{1 << 27};       // paths in flight per wave (lanes = wave_paths / pixels); 2^27 holds a
                                     // 1024^2 x 128-spp frame in one wave (~36 GB of path state)
  int trace_blocks_per_sm{32};       // persistent grid of the traversal kernels (128 threads; capped by occupancy)
  int shade_blocks_per_sm{16};       // persistent grid of the shading kernel (128 threads; capped by occupancy)
  int use_graph{1};                  // replay each wave as a CUDA graph
  int count_traversal{0};            // node-visit / triangle-test counters (roofline runs)
  int max_leaf{1};                   // triangles per leaf child of the host-built BVH8 (1..3), read at scene build
  int time_kernels{0};               // CUDA events around every launch (no graph), per-kind times
  int trace_refill{8};               // closest-hit warps refill once this many lanes idle (32: never)
  int vol_refill{8};                 // volume-tracking warps refill once this many lanes idle
  int vol_passes{1};                 // volume tracking: passes per lane and loop trip at most
  int split_shade{1};                // misses and hits shaded by separate kernels (no-volume scenes)
  int split_volume{1};               // volume scenes: scattering, hit and miss paths shaded by separate kernels
  int adjoint_sort{1};               // the adjoint replay shades its hits sorted by material
  int64_t class_threshold{1 << 26};  // waves of at least this many paths shade hits with the class kernels
  int shade_lean{1};                 // lean shading kernels for scenes without volumes/sources/lights
  int shade_classes{1};              // lean scenes: hit queue sorted by shading class, one kernel per class
  int64_t batch_wave_paths{1 << 25}; // paths per wave of a batched render
  int64_t sort_threshold{1 << 18};   // sort the hit queue by material when it holds this many hits (0: never)
  int gpu_bvh{1};                    // build the BVH8 on the GPU (bvh_gpu.cu), read at scene build
  int gpu_max_leaf{2};               // triangles per leaf child of the GPU-built BVH8 (1..3), read at scene build
  int ploc_radius{8};                // clusters searched on each side by the GPU build's clustering (2..32)
  int collapse_tri_cost{30};         // GPU build: triangle test / node visit cost in percent for the collapse's
                                     // surface-area program; 0: greedy collapse (read at scene build)
  int gpu_tables{1};                 // build majorant grids, env / emissive CDFs and 8-bit texels on the GPU (scene_tables.cu), read at scene build
  int texels_u8{1};                  // keep samplers whose texels are all k / 255 as 8-bit RGBA, read at scene build
  int64_t wave_trip_cap{1 << 24};    // loop trips after which a persistent wave kernel's warp stops with
                                     // PHC_ERR_DEVICE (a self-check; lowered only to test that path)
};

Tuning &tuning();

} // namespace phc
