// The surface-area program of the GPU BVH build's collapse (bvh_gpu.cu),
// __host__ __device__ so that host tests run the very code the kernels run.
//
// The binary tree: n leaves (0..n-1, one primitive each) and n-1 inner nodes
// (n..2n-2), children before parents; nchild[v] = (left, right), or (-1,
// primitive) for a leaf; nbox[6 v ..] = (lo xyz, hi xyz).
//
// cost(u, j), for j = 1..8: the least expected cost of covering binary
// subtree u with at most j child slots of its wide parent, each slot holding
// a descendant w of u as a leaf child (area(w) x primitives x tri_cost, when
// it has at most max_leaf primitives) or as a wide inner node (area(w) x 1 +
// the cheapest cover of w's two subtrees by 8 slots); for j >= 2 u may also
// be opened, its two subtrees sharing the j slots.  A binary leaf is always a
// one-primitive leaf child.  (The dynamic program of Ylitie, Karras and
// Laine, "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide
// BVHs", HPG 2017, restated for this layout's leaf children.)
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#ifndef PHC_HD
#define PHC_HD __host__ __device__ __forceinline__
#endif

namespace phc {

struct CollapseDp {
  float *cost;     // 8 per inner node (index v - n): cost(v, j + 1)
  uint8_t *split;  // 8 per inner node, entry j for j + 1 slots: 0 = v fills one slot, k = v opened, k slots
                   // for its left subtree
  uchar4 *info;    // per inner node: x = the split of v as a wide inner node, y = 1 when v fills one slot as a
                   // leaf child, z = its primitives (at most 255)
};

// surface area of binary node v's box
PHC_HD float dp_area(const float *nbox, uint32_t v)
{
  const float *b = nbox + 6 * size_t(v);
  const float dx = b[3] - b[0], dy = b[4] - b[1], dz = b[5] - b[2];
  return 2.f * (dx * dy + dy * dz + dz * dx);
}

PHC_HD float dp_cost(const CollapseDp &d, const float *nbox, uint32_t n, int u, int j, float ct)
{
  return uint32_t(u) < n ? dp_area(nbox, uint32_t(u)) * ct : d.cost[8 * size_t(uint32_t(u) - n) + j];
}

// The program's entries of inner node v; its children's must be final.
PHC_HD void collapse_dp_node(const CollapseDp &d, const float *nbox, const int2 *nchild, uint32_t n, uint32_t v,
    float ct, int max_leaf)
{
  const int2 c = nchild[v];
  float cl[8], cr[8];
  for (int j = 0; j < 8; ++j) {
    cl[j] = dp_cost(d, nbox, n, c.x, j, ct);
    cr[j] = dp_cost(d, nbox, n, c.y, j, ct);
  }
  const uint32_t pl = uint32_t(c.x) < n ? 1u : d.info[uint32_t(c.x) - n].z;
  const uint32_t pr = uint32_t(c.y) < n ? 1u : d.info[uint32_t(c.y) - n].z;
  const uint32_t p = pl + pr < 255u ? pl + pr : 255u;
  // open v: the cheapest share of j slots between its subtrees (j = 2..8)
  float sc[8];
  uint8_t sk[8];
  sc[0] = 3.4e38f;
  sk[0] = 0;
  for (int j = 2; j <= 8; ++j) {
    float best = 3.4e38f;
    int bk = 1;
    for (int k = 1; k < j; ++k) {
      const float x = cl[k - 1] + cr[j - k - 1];
      if (x < best) {
        best = x;
        bk = k;
      }
    }
    sc[j - 1] = best;
    sk[j - 1] = uint8_t(bk);
  }
  const float a = dp_area(nbox, v);
  const float c_inner = a + sc[7];
  const bool leaf = p <= uint32_t(max_leaf) && a * float(p) * ct <= c_inner;
  const float self = leaf ? a * float(p) * ct : c_inner;
  float *co = d.cost + 8 * size_t(v - n);
  uint8_t *sp = d.split + 8 * size_t(v - n);
  co[0] = self;
  sp[0] = 0;
  for (int j = 1; j < 8; ++j) {
    const bool open = sc[j] < self;
    co[j] = open ? sc[j] : self;
    sp[j] = open ? sk[j] : 0;
  }
  d.info[v - n] = make_uchar4(sk[7], leaf ? 1 : 0, uint8_t(p), 0);
}

// The children of the wide node over binary inner node `root` as the program
// chose them: the root's two subtrees share the 8 slots; each (subtree,
// slots) entry either fills one slot or, when the program opened it for that
// many slots, becomes two entries whose slots add up to its own, so at most
// 8 entries are ever pending.  ch[i]: binary node, lc[i]: its primitives as
// a leaf child (0: a wide inner node).  Returns the count, -1 if the choices
// are inconsistent (more than 8 children).
PHC_HD int sah_children(const int2 *nchild, const uint8_t *split, const uchar4 *info, uint32_t n, int root, int *ch,
    int *lc)
{
  int stk[8], slots[8], sp = 0, k = 0;
  int s0 = int(info[uint32_t(root) - n].x);
  s0 = s0 < 1 ? 1 : (s0 > 7 ? 7 : s0);
  stk[sp] = nchild[root].y;
  slots[sp++] = 8 - s0;
  stk[sp] = nchild[root].x;
  slots[sp++] = s0;
  while (sp > 0) {
    --sp;
    const int u = stk[sp], j = slots[sp];
    const bool bin_leaf = uint32_t(u) < n;
    const int open = bin_leaf || j < 2 ? 0 : int(split[8 * size_t(uint32_t(u) - n) + size_t(j - 1)]);
    if (open >= 1 && open < j && sp + 2 <= 8) {
      stk[sp] = nchild[u].y;
      slots[sp++] = j - open;
      stk[sp] = nchild[u].x;
      slots[sp++] = open;
      continue;
    }
    if (k == 8) // cannot happen: the entries' slots add up to 8
      return -1;
    ch[k] = u;
    if (bin_leaf) {
      lc[k] = 1;
    } else {
      const uchar4 in = info[uint32_t(u) - n];
      lc[k] = in.y ? int(in.z) : 0;
    }
    ++k;
  }
  return k;
}

} // namespace phc
