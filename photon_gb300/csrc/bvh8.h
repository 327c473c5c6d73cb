// SAH-built 8-wide BVH with quantised child boxes (host builder).
//
// Replaces the reference's binary median-split BVH (src/photon/pt/bvh/bvh.cpp:
// 20-125, 44-byte AoS nodes, leaves of <= 4) with a layout made for 128-bit
// coalesced loads on GB300 SMs, after the compressed wide BVH of Ylitie,
// Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs Through
// Compressed Wide BVHs" (HPG 2017).  One node is 80 bytes = 5 x uint4:
//
//   word 0   float p[3]           origin of the child-box grid
//            u8 e[3], u8 imask    per-axis scale exponent (2^(e-127)); bit s of
//                                 imask = child slot s is an internal node
//   word 1   u32 child_base       first child node (internal children are
//                                 stored contiguously in slot order)
//            u32 tri_base         first triangle record of the leaf children
//            u8 meta[8]           per slot: 0 empty; 0x80 internal;
//                                 (count << 5) | offset for a leaf of 1..3
//                                 triangles at tri_base + offset
//   words 2-4 u8 qlo_x[8] qlo_y[8] qlo_z[8] qhi_x[8] qhi_y[8] qhi_z[8]
//                                 child boxes: p + q * 2^(e-127), rounded outward
//
// Child slots are assigned so that a ray whose direction has sign octant o
// visits slot (k ^ o) k-th, close to front-to-back order (the octant ordering
// of the paper); the builder solves that assignment greedily.
#pragma once

#include <cstdint>
#include <vector>

namespace phc {

struct Bvh8Host {
  std::vector<uint32_t> nodes; // 20 u32 per node
  std::vector<float> tris;     // 12 floats per triangle record, leaf order
  std::vector<uint32_t> leaf_prims; // box builds: primitive id per leaf entry, leaf order
  uint32_t node_count{0};
  uint32_t tri_count{0};
  uint32_t max_depth{0};
  double sah_cost{0.0};
};

// Builds the BVH8 over triangles (positions xyz per vertex, 3 indices per
// triangle).  Degenerate triangles are kept (they are never hit, as in the
// reference).  max_leaf is the largest triangle count of one leaf child (1..3).
void build_bvh8(const float *positions, uint64_t vertex_count, const uint32_t *indices, uint64_t triangle_count,
    Bvh8Host &out, int max_leaf = 3);

// Builds the BVH8 over axis-aligned boxes (lo xyz, hi xyz per primitive):
// the top level over instances.  Leaf children address `leaf_prims` (the
// box ids in leaf order) where a triangle build addresses its records.
void build_bvh8_boxes(const float *boxes, uint64_t count, Bvh8Host &out, int max_leaf = 1);

// Per-primitive triangle records (v0, e1, e2 as in the leaf records) in
// primitive order, for shading: 12 floats per triangle into prim_geo.
void build_prim_records(const float *positions, const uint32_t *indices, uint64_t triangle_count, float *prim_geo);

} // namespace phc
