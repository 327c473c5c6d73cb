// GPU construction of the BVH8 (bvh_gpu.cu): Morton sort, parallel
// locally-ordered clustering, collapse into the quantised 8-wide nodes of
// bvh8.h with leaf children of up to max_leaf triangles.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace phc {

struct GpuBvh8 {
  void *nodes{nullptr}; // node_cap x 80 bytes (cudaMalloc; the caller frees)
  void *tris{nullptr};  // tri_count x 48 bytes (cudaMalloc; the caller frees)
  uint32_t node_count{0}, node_cap{0}, tri_count{0}, max_depth{0};
};

// positions: float4 per vertex; prim_vidx: (i0, i1, i2, material) per
// triangle, both on the device; max_leaf: triangles per leaf child (1..3);
// radius: clusters searched on each side by the clustering (2..32);
// tri_cost: a triangle test's cost relative to a node visit for the
// collapse's surface-area program, 0 for the greedy collapse (largest
// subtrees opened first).  Blocks on `s` until the build is done.
GpuBvh8 build_bvh8_gpu(const float4 *positions, const uint4 *prim_vidx, uint32_t triangle_count, cudaStream_t s,
    int max_leaf = 1, int radius = 16, float tri_cost = 0.f);

// Exclusive scan of n words (in == out allowed) on the device, in three
// launches on `s`; *total (if not null) receives the sum.  scratch holds
// scan_u32_scratch(n) words.
size_t scan_u32_scratch(uint32_t n);
void scan_u32(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *total, uint32_t *scratch, cudaStream_t s);

} // namespace phc
