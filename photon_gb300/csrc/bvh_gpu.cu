// GPU construction of the BVH8 of bvh8.h (same node and triangle-record
// layout, so the traversal kernels read either build).
//
// The reference builds its BVH on the host (src/photon/pt/bvh/bvh.cpp:77-125,
// median split); so does this renderer's default builder (binned SAH,
// bvh8.cpp).  For scene upload latency (many scenes per second in the batched
// mode) this file builds on the GPU instead:
//
//   1. primitive boxes and centroids, scene bounds;
//   2. 30-bit Morton codes of the centroids, sorted with a stable LSD radix
//      sort (4 passes of 8 bits: block histograms, one scan, ranked scatter);
//   3. a binary tree by parallel locally-ordered clustering (Meister and
//      Bittner, "Parallel Locally-Ordered Clustering for Bounding Volume
//      Hierarchy Construction", IEEE TVCG 2018): every cluster finds, among
//      the `radius` clusters on each side in Morton order (2, 4, 8, 16 or 32;
//      tuning key ploc_radius), the one whose merged
//      box has the least surface area; mutual pairs merge; the survivors are
//      compacted in order; repeat until one cluster is left.  Ties in the
//      area are broken by the pair's indices, so the globally smallest pair
//      is always mutual and every iteration merges;
//   4. the binary tree collapsed into the 8-wide quantised nodes level by
//      level, each node taking the up to eight descendants of largest area
//      (subtrees of more than max_leaf primitives opened first), the octant
//      slot order and the outward-rounded 8-bit child grid of the host
//      builder; a descendant with at most max_leaf primitives (1..3) is one
//      leaf child.  With a triangle cost (tuning key collapse_tri_cost) the
//      descendants are chosen instead by the surface-area cost of the whole
//      wide tree (the dynamic program of Ylitie, Karras and Laine,
//      "Efficient Incoherent Ray Traversal on GPUs Through Compressed Wide
//      BVHs", HPG 2017): bottom-up, the cheapest way to cover every
//      binary subtree with 1..8 slots, then the collapse follows those
//      choices from the root down.
//
// The result is deterministic except for where nodes and leaf records land
// in memory (atomic allocation order), which changes no traversal result.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "bvh_collapse.cuh"
#include "bvh_gpu.h"

namespace phc {
namespace {

constexpr int SORT_BLOCK = 256;
constexpr int TILE = 256;    // clusters per block of the neighbour search

__device__ __forceinline__ float area(const float *lo, const float *hi)
{
  const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
  return 2.f * (dx * dy + dy * dz + dz * dx);
}

// ---------------------------------------------------------------- stage 1
// Primitive boxes (6 floats) and the scene's centroid bounds through ordered
// integer atomics on the float bits.
__device__ __forceinline__ uint32_t ord(float f)
{
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unord(uint32_t u)
{
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__global__ void k_prim_boxes(const float4 *__restrict__ pos, const uint4 *__restrict__ vidx, uint32_t n,
    float *__restrict__ boxes, uint32_t *cbounds)
{
  float clo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, chi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint4 v = vidx[i];
    const float4 a = pos[v.x], b = pos[v.y], c = pos[v.z];
    float *bx = boxes + 6 * size_t(i);
    bx[0] = fminf(fminf(a.x, b.x), c.x);
    bx[1] = fminf(fminf(a.y, b.y), c.y);
    bx[2] = fminf(fminf(a.z, b.z), c.z);
    bx[3] = fmaxf(fmaxf(a.x, b.x), c.x);
    bx[4] = fmaxf(fmaxf(a.y, b.y), c.y);
    bx[5] = fmaxf(fmaxf(a.z, b.z), c.z);
    for (int k = 0; k < 3; ++k) {
      const float cc = 0.5f * (bx[k] + bx[3 + k]);
      clo[k] = fminf(clo[k], cc);
      chi[k] = fmaxf(chi[k], cc);
    }
  }
  for (int k = 0; k < 3; ++k) {
    for (int o = 16; o > 0; o >>= 1) {
      clo[k] = fminf(clo[k], __shfl_xor_sync(0xffffffffu, clo[k], o));
      chi[k] = fmaxf(chi[k], __shfl_xor_sync(0xffffffffu, chi[k], o));
    }
  }
  if ((threadIdx.x & 31u) == 0)
    for (int k = 0; k < 3; ++k) {
      atomicMin(&cbounds[k], ord(clo[k]));
      atomicMax(&cbounds[3 + k], ord(chi[k]));
    }
}

__device__ __forceinline__ uint32_t spread10(uint32_t x)
{
  x &= 0x3ffu;
  x = (x | (x << 16)) & 0x030000ffu;
  x = (x | (x << 8)) & 0x0300f00fu;
  x = (x | (x << 4)) & 0x030c30c3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

__global__ void k_morton(const float *__restrict__ boxes, uint32_t n, const uint32_t *cbounds,
    uint32_t *__restrict__ keys, uint32_t *__restrict__ vals)
{
  float lo[3], sc[3];
  for (int k = 0; k < 3; ++k) {
    lo[k] = unord(cbounds[k]);
    const float ext = unord(cbounds[3 + k]) - lo[k];
    sc[k] = ext > 0.f ? 1023.99f / ext : 0.f;
  }
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float *bx = boxes + 6 * size_t(i);
    uint32_t q[3];
    for (int k = 0; k < 3; ++k) {
      const float c = 0.5f * (bx[k] + bx[3 + k]);
      const float f = (c - lo[k]) * sc[k];
      q[k] = uint32_t(fminf(fmaxf(f, 0.f), 1023.f));
    }
    keys[i] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
    vals[i] = i;
  }
}

// ---------------------------------------------------------------- stage 2
// Stable LSD radix sort, one element per thread: per-block digit counts,
// one exclusive scan over (digit, block), then each element's rank among the
// equal digits before it in its block (lanes through match_any, warps
// through shared counts).
__global__ void __launch_bounds__(SORT_BLOCK) k_digit_hist(const uint32_t *__restrict__ keys, uint32_t n, int shift,
    uint32_t *__restrict__ hist, uint32_t nblocks)
{
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0u;
  __syncthreads();
  const uint32_t i = blockIdx.x * SORT_BLOCK + threadIdx.x;
  if (i < n)
    atomicAdd(&h[(keys[i] >> shift) & 0xffu], 1u);
  __syncthreads();
  hist[size_t(threadIdx.x) * nblocks + blockIdx.x] = h[threadIdx.x]; // digit-major
}

// Exclusive scan of `count` words in place by one block (sequential chunks,
// in order, so the result is independent of the block size): the scan of
// the tile sums below.
__global__ void __launch_bounds__(1024) k_scan_inplace(uint32_t *__restrict__ v, uint32_t count, uint32_t *total)
{
  __shared__ uint32_t part[1024];
  const uint32_t per = (count + 1023u) / 1024u;
  const uint32_t b = threadIdx.x * per, e = min(count, b + per);
  uint32_t s = 0;
  for (uint32_t i = b; i < e; ++i)
    s += v[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (uint32_t off = 1; off < 1024u; off <<= 1) {
    const uint32_t x = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
    __syncthreads();
    part[threadIdx.x] += x;
    __syncthreads();
  }
  uint32_t run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
  for (uint32_t i = b; i < e; ++i) {
    const uint32_t x = v[i];
    v[i] = run;
    run += x;
  }
  if (threadIdx.x == 1023 && total)
    *total = part[1023];
}

// Multi-block exclusive scan: tiles of SCAN_TILE words, one block each;
// the tile sums, their scan by one block, then each tile's scan from its
// offset.  Integer sums, so the result is exact whatever the tiling.
constexpr int SCAN_T = 256, SCAN_ITEMS = 8, SCAN_TILE = SCAN_T * SCAN_ITEMS;

__device__ __forceinline__ uint32_t block_exclusive(uint32_t x, uint32_t &block_total)
{
  __shared__ uint32_t warp_sum[SCAN_T / 32];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t inc = x;
  for (uint32_t off = 1; off < 32u; off <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, off);
    if (lane >= off)
      inc += y;
  }
  if (lane == 31u)
    warp_sum[warp] = inc;
  __syncthreads();
  uint32_t before = 0, all = 0;
  for (uint32_t w = 0; w < SCAN_T / 32; ++w) {
    const uint32_t v = warp_sum[w];
    before += w < warp ? v : 0u;
    all += v;
  }
  __syncthreads(); // warp_sum is reused by the next call
  block_total = all;
  return before + inc - x;
}

__global__ void __launch_bounds__(SCAN_T) k_tile_sums(const uint32_t *__restrict__ in, uint32_t n,
    uint32_t *__restrict__ sums)
{
  const size_t base = size_t(blockIdx.x) * SCAN_TILE;
  uint32_t s = 0;
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    const size_t i = base + size_t(k) * SCAN_T + threadIdx.x;
    if (i < n)
      s += in[i];
  }
  uint32_t total;
  block_exclusive(s, total);
  if (threadIdx.x == 0)
    sums[blockIdx.x] = total;
}

// Padded shared index: thread t's SCAN_ITEMS consecutive words fall in
// different banks.
__device__ __forceinline__ uint32_t scan_pad(uint32_t i) { return i + (i >> 5); }

__global__ void __launch_bounds__(SCAN_T) k_tile_scan(const uint32_t *in, uint32_t n,
    const uint32_t *__restrict__ offsets, uint32_t *out)
{
  __shared__ uint32_t tile[SCAN_TILE + SCAN_TILE / 32];
  const size_t base = size_t(blockIdx.x) * SCAN_TILE;
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    const uint32_t j = uint32_t(k) * SCAN_T + threadIdx.x;
    tile[scan_pad(j)] = base + j < n ? in[base + j] : 0u;
  }
  __syncthreads();
  uint32_t v[SCAN_ITEMS], local = 0;
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    v[k] = tile[scan_pad(threadIdx.x * SCAN_ITEMS + k)];
    local += v[k];
  }
  uint32_t total;
  uint32_t run = offsets[blockIdx.x] + block_exclusive(local, total);
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    tile[scan_pad(threadIdx.x * SCAN_ITEMS + k)] = run;
    run += v[k];
  }
  __syncthreads();
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    const uint32_t j = uint32_t(k) * SCAN_T + threadIdx.x;
    if (base + j < n)
      out[base + j] = tile[scan_pad(j)];
  }
}

__global__ void __launch_bounds__(SORT_BLOCK) k_digit_scatter(const uint32_t *__restrict__ kin,
    const uint32_t *__restrict__ vin, uint32_t n, int shift, const uint32_t *__restrict__ hist, uint32_t nblocks,
    uint32_t *__restrict__ kout, uint32_t *__restrict__ vout)
{
  __shared__ uint32_t wcount[SORT_BLOCK / 32][256];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (uint32_t k = threadIdx.x; k < (SORT_BLOCK / 32) * 256; k += SORT_BLOCK)
    (&wcount[0][0])[k] = 0u;
  __syncthreads();
  const uint32_t i = blockIdx.x * SORT_BLOCK + threadIdx.x;
  const bool live = i < n;
  const uint32_t key = live ? kin[i] : 0u;
  const uint32_t dg = live ? (key >> shift) & 0xffu : 256u + lane; // dead lanes get private digits
  const uint32_t peers = __match_any_sync(0xffffffffu, dg);
  const uint32_t before = __popc(peers & ((1u << lane) - 1u));
  if (live && before == 0)
    wcount[warp][dg] = __popc(peers);
  __syncthreads();
  if (live) {
    uint32_t rank = before;
    for (uint32_t w = 0; w < warp; ++w)
      rank += wcount[w][dg];
    const uint32_t dst = hist[size_t(dg) * nblocks + blockIdx.x] + rank;
    kout[dst] = key;
    vout[dst] = vin[i];
  }
}

// ---------------------------------------------------------------- stage 3
// BVH2 nodes: n leaves (0..n-1, leaf j = the j-th primitive in Morton order)
// then n-1 internal nodes.  child.x = left (-1 for a leaf), child.y = right
// (the primitive id for a leaf).
__global__ void k_leaves(const float *__restrict__ boxes, const uint32_t *__restrict__ sorted_prim, uint32_t n,
    float *__restrict__ nbox, int2 *__restrict__ nchild, uint32_t *__restrict__ cid, float *__restrict__ cbox)
{
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const uint32_t p = sorted_prim[j];
    for (int k = 0; k < 6; ++k) {
      const float b = boxes[6 * size_t(p) + k];
      nbox[6 * size_t(j) + k] = b;
      cbox[6 * size_t(j) + k] = b;
    }
    nchild[j] = make_int2(-1, int(p));
    cid[j] = j;
  }
}

// Nearest neighbour of every cluster within RADIUS on each side; the pair
// order is (merged area, smaller index, larger index).
template <int RADIUS>
__global__ void __launch_bounds__(TILE) k_ploc_nn(const float *__restrict__ cbox, uint32_t n, uint32_t *__restrict__ nn)
{
  __shared__ float sb[TILE + 2 * RADIUS][6];
  const int base = int(blockIdx.x) * TILE;
  for (int t = threadIdx.x; t < TILE + 2 * RADIUS; t += TILE) {
    const int g = base - RADIUS + t;
    for (int k = 0; k < 6; ++k)
      sb[t][k] = (g >= 0 && g < int(n)) ? cbox[6 * size_t(g) + k] : 0.f;
  }
  __syncthreads();
  const int i = base + int(threadIdx.x);
  if (i >= int(n))
    return;
  const float *me = sb[threadIdx.x + RADIUS];
  float best = 3.4e38f;
  int bj = -1;
  const int j0 = max(0, i - RADIUS), j1 = min(int(n) - 1, i + RADIUS);
  for (int j = j0; j <= j1; ++j) {
    if (j == i)
      continue;
    const float *o = sb[j - base + RADIUS];
    float lo[3], hi[3];
    for (int k = 0; k < 3; ++k) {
      lo[k] = fminf(me[k], o[k]);
      hi[k] = fmaxf(me[3 + k], o[3 + k]);
    }
    const float a = area(lo, hi);
    // scanning j upward, a strict < keeps the smaller partner index on ties;
    // the pair order's other keys are i's own, equal for every candidate
    if (a < best) {
      best = a;
      bj = j;
    }
  }
  nn[i] = uint32_t(bj < 0 ? i : bj);
}

// flags.x: cluster i merges with its partner (mutual, i the smaller index);
// flags.y: cluster i survives the iteration (it merges or stays alone).
__global__ void k_ploc_flags(const uint32_t *__restrict__ nn, uint32_t n, uint32_t *__restrict__ merge,
    uint32_t *__restrict__ keep)
{
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t j = nn[i];
    const bool mutual = j != i && nn[j] == i;
    merge[i] = (mutual && i < j) ? 1u : 0u;
    keep[i] = (mutual && i > j) ? 0u : 1u;
  }
}

__global__ void k_ploc_write(const uint32_t *__restrict__ nn, uint32_t n, const uint32_t *__restrict__ merge_flag,
    const uint32_t *__restrict__ merge_rank, const uint32_t *__restrict__ keep_flag,
    const uint32_t *__restrict__ keep_rank, uint32_t node_base, const uint32_t *__restrict__ cid,
    const float *__restrict__ cbox, uint32_t *__restrict__ cid_out, float *__restrict__ cbox_out,
    float *__restrict__ nbox, int2 *__restrict__ nchild)
{
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (!keep_flag[i])
      continue;
    const uint32_t dst = keep_rank[i];
    if (merge_flag[i]) {
      const uint32_t j = nn[i];
      const uint32_t node = node_base + merge_rank[i];
      float b[6];
      for (int k = 0; k < 3; ++k) {
        b[k] = fminf(cbox[6 * size_t(i) + k], cbox[6 * size_t(j) + k]);
        b[3 + k] = fmaxf(cbox[6 * size_t(i) + 3 + k], cbox[6 * size_t(j) + 3 + k]);
      }
      for (int k = 0; k < 6; ++k) {
        nbox[6 * size_t(node) + k] = b[k];
        cbox_out[6 * size_t(dst) + k] = b[k];
      }
      nchild[node] = make_int2(int(cid[i]), int(cid[j]));
      cid_out[dst] = node;
    } else {
      for (int k = 0; k < 6; ++k)
        cbox_out[6 * size_t(dst) + k] = cbox[6 * size_t(i) + k];
      cid_out[dst] = cid[i];
    }
  }
}

// ---------------------------------------------------------------- stage 4
struct Collapse {
  const float *nbox;   // BVH2 boxes
  const int2 *nchild;  // BVH2 children
  const float4 *pos;
  const uint4 *vidx;
  uint32_t *nodes;     // 20 words per BVH8 node
  float4 *tris;        // 3 per triangle record
  uint32_t *counters;  // [0] nodes, [1] triangle records, [2] next queue length, [3] overflow
  uint32_t node_cap;
  int max_leaf;        // triangles per leaf child (1..3)
};

// The primitives of BVH2 subtree v when it has at most `limit` leaves (at
// most 3): their count, with the primitives in `prims` in left-to-right
// order; limit + 1 when it has more.
__device__ int subtree_prims(const int2 *__restrict__ nchild, int v, int limit, int *prims)
{
  int stack[4], sp = 0, n = 0;
  stack[sp++] = v;
  while (sp > 0) {
    const int u = stack[--sp];
    const int2 c = nchild[u];
    if (c.x < 0) {
      if (n == limit)
        return limit + 1;
      prims[n++] = c.y;
    } else {
      if (sp + 2 > 4)
        return limit + 1;
      stack[sp++] = c.y;
      stack[sp++] = c.x;
    }
  }
  return n;
}

__device__ __forceinline__ float node_area(const float *nbox, int v)
{
  const float *b = nbox + 6 * size_t(v);
  return area(b, b + 3);
}

// One BVH8 node per thread: queue entries (BVH8 node index, BVH2 root).
__global__ void __launch_bounds__(128) k_collapse(Collapse c, const uint2 *__restrict__ qin, uint32_t nq,
    uint2 *__restrict__ qout)
{
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq)
    return;
  const uint32_t ni = qin[t].x;
  const int root = int(qin[t].y);
  // candidates: child v, whether it is internal, its area, and whether it
  // has at most max_leaf primitives (it becomes one leaf child unless a free
  // slot opens it), each found once when the candidate is added
  int ch[8];
  bool inner[8], sm[8];
  float ar[8];
  int prims[3];
  int k = 0;
  auto add = [&](int slot, int v) {
    ch[slot] = v;
    inner[slot] = c.nchild[v].x >= 0;
    ar[slot] = inner[slot] ? node_area(c.nbox, v) : 0.f;
    sm[slot] = inner[slot] && c.max_leaf > 1 && subtree_prims(c.nchild, v, c.max_leaf, prims) <= c.max_leaf;
  };
  if (c.nchild[root].x < 0) {
    add(k++, root); // a leaf root: one leaf child
  } else {
    add(k++, c.nchild[root].x);
    add(k++, c.nchild[root].y);
  }
  while (k < 8) { // open the internal child of largest area, larger subtrees first
    int best = -1;
    for (int i = 0; i < k; ++i)
      if (inner[i] && (best < 0 || (sm[best] && !sm[i]) || (sm[i] == sm[best] && ar[i] > ar[best])))
        best = i;
    if (best < 0)
      break;
    const int2 cc = c.nchild[ch[best]];
    add(best, cc.x);
    add(k++, cc.y);
  }
  float nlo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, nhi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  for (int i = 0; i < k; ++i)
    for (int a = 0; a < 3; ++a) {
      nlo[a] = fminf(nlo[a], c.nbox[6 * size_t(ch[i]) + a]);
      nhi[a] = fmaxf(nhi[a], c.nbox[6 * size_t(ch[i]) + 3 + a]);
    }
  // octant slots, greedily by the smallest cost (the host builder's rule)
  float pc[3];
  for (int a = 0; a < 3; ++a)
    pc[a] = 0.5f * (nlo[a] + nhi[a]);
  float cost[8][8];
  for (int i = 0; i < k; ++i) {
    float cc[3];
    for (int a = 0; a < 3; ++a)
      cc[a] = 0.5f * (c.nbox[6 * size_t(ch[i]) + a] + c.nbox[6 * size_t(ch[i]) + 3 + a]) - pc[a];
    for (int s = 0; s < 8; ++s) {
      const float dx = (s & 4) ? -1.f : 1.f, dy = (s & 2) ? -1.f : 1.f, dz = (s & 1) ? -1.f : 1.f;
      cost[i][s] = cc[0] * dx + cc[1] * dy + cc[2] * dz;
    }
  }
  int child_at[8];
  for (int s = 0; s < 8; ++s)
    child_at[s] = -1;
  uint32_t used_c = 0u, used_s = 0u;
  for (int it = 0; it < k; ++it) {
    float best = 3.4e38f;
    int bc = -1, bs = -1;
    for (int i = 0; i < k; ++i) {
      if (used_c & (1u << i))
        continue;
      for (int s = 0; s < 8; ++s) {
        if (used_s & (1u << s))
          continue;
        if (cost[i][s] < best || bc < 0) {
          best = cost[i][s];
          bc = i;
          bs = s;
        }
      }
    }
    used_c |= 1u << bc;
    used_s |= 1u << bs;
    child_at[bs] = ch[bc];
  }
  // quantisation grid (double, exact powers of two: outward rounding)
  uint8_t e[3];
  double scale[3];
  for (int a = 0; a < 3; ++a) {
    const double ext = double(nhi[a]) - double(nlo[a]);
    int ex = -127;
    if (ext > 0.0) {
      ex = int(ceil(log2(ext / 255.0)));
      while (ldexp(255.0, ex) < ext)
        ++ex;
      while (ex > -127 && ldexp(255.0, ex - 1) >= ext)
        --ex;
    }
    ex = min(max(ex, -127), 127);
    e[a] = uint8_t(ex + 127);
    scale[a] = ex == -127 ? 0.0 : ldexp(1.0, ex);
  }
  // leaf children: single primitives, and internal children of at most
  // max_leaf primitives (lcount[s] primitives each)
  uint32_t internal = 0, leaves = 0;
  uint8_t imask = 0;
  int lcount[8];
  for (int s = 0; s < 8; ++s) {
    lcount[s] = 0;
    if (child_at[s] < 0)
      continue;
    const int v = child_at[s];
    if (c.nchild[v].x < 0)
      lcount[s] = 1;
    else if (c.max_leaf > 1) {
      const int m = subtree_prims(c.nchild, v, c.max_leaf, prims);
      lcount[s] = m <= c.max_leaf ? m : 0;
    }
    if (lcount[s] == 0) {
      imask |= uint8_t(1u << s);
      ++internal;
    } else {
      leaves += uint32_t(lcount[s]);
    }
  }
  uint32_t child_base = 0, tri_base = 0;
  if (internal)
    child_base = atomicAdd(&c.counters[0], internal);
  if (leaves)
    tri_base = atomicAdd(&c.counters[1], leaves);
  if (child_base + internal > c.node_cap) {
    atomicExch(&c.counters[3], 1u);
    return;
  }
  uint32_t q_out_base = 0;
  if (internal)
    q_out_base = atomicAdd(&c.counters[2], internal);
  uint8_t meta[8] = {}, q[6][8] = {};
  uint32_t next_child = child_base, tri_off = 0, qo = q_out_base;
  for (int s = 0; s < 8; ++s) {
    const int v = child_at[s];
    if (v < 0)
      continue;
    const float *b = c.nbox + 6 * size_t(v);
    for (int a = 0; a < 3; ++a) {
      double lo = 0.0, hi = 0.0;
      if (scale[a] > 0.0) {
        lo = floor((double(b[a]) - double(nlo[a])) / scale[a]);
        hi = ceil((double(b[3 + a]) - double(nlo[a])) / scale[a]);
      }
      q[a][s] = uint8_t(fmin(fmax(lo, 0.0), 255.0));
      q[3 + a][s] = uint8_t(fmin(fmax(hi, 0.0), 255.0));
    }
    if (lcount[s] == 0) {
      meta[s] = 0x80;
      qout[qo++] = make_uint2(next_child++, uint32_t(v));
    } else {
      meta[s] = uint8_t((uint32_t(lcount[s]) << 5) | tri_off);
      if (c.nchild[v].x < 0)
        prims[0] = c.nchild[v].y;
      else
        subtree_prims(c.nchild, v, c.max_leaf, prims);
      for (int j = 0; j < lcount[s]; ++j) {
        const uint32_t prim = uint32_t(prims[j]);
        const uint4 vi = c.vidx[prim];
        const float4 v0 = c.pos[vi.x], v1 = c.pos[vi.y], v2 = c.pos[vi.z];
        float4 *r = c.tris + 3 * size_t(tri_base + tri_off);
        r[0] = make_float4(v0.x, v0.y, v0.z, __uint_as_float(prim));
        r[1] = make_float4(v1.x - v0.x, v1.y - v0.y, v1.z - v0.z, 0.f);
        r[2] = make_float4(v2.x - v0.x, v2.y - v0.y, v2.z - v0.z, 0.f);
        ++tri_off;
      }
    }
  }
  uint32_t *w = c.nodes + size_t(ni) * 20;
  w[0] = __float_as_uint(nlo[0]);
  w[1] = __float_as_uint(nlo[1]);
  w[2] = __float_as_uint(nlo[2]);
  w[3] = uint32_t(e[0]) | (uint32_t(e[1]) << 8) | (uint32_t(e[2]) << 16) | (uint32_t(imask) << 24);
  w[4] = child_base;
  w[5] = tri_base;
  w[6] = uint32_t(meta[0]) | (uint32_t(meta[1]) << 8) | (uint32_t(meta[2]) << 16) | (uint32_t(meta[3]) << 24);
  w[7] = uint32_t(meta[4]) | (uint32_t(meta[5]) << 8) | (uint32_t(meta[6]) << 16) | (uint32_t(meta[7]) << 24);
  for (int r = 0; r < 6; ++r) {
    w[8 + 2 * r] = uint32_t(q[r][0]) | (uint32_t(q[r][1]) << 8) | (uint32_t(q[r][2]) << 16) |
        (uint32_t(q[r][3]) << 24);
    w[9 + 2 * r] = uint32_t(q[r][4]) | (uint32_t(q[r][5]) << 8) | (uint32_t(q[r][6]) << 16) |
        (uint32_t(q[r][7]) << 24);
  }
}

// ---------------------------------------------------------------- stage 4a
// The collapse's surface-area program (bvh_collapse.cuh), one launch per
// clustering iteration's new nodes: their children come from earlier
// iterations, so their entries are final.
__global__ void __launch_bounds__(128) k_collapse_dp(CollapseDp d, const float *__restrict__ nbox,
    const int2 *__restrict__ nchild, uint32_t n, uint32_t lo, uint32_t hi, float ct, int max_leaf)
{
  for (uint32_t v = lo + blockIdx.x * blockDim.x + threadIdx.x; v < hi; v += gridDim.x * blockDim.x)
    if (v >= n)
      collapse_dp_node(d, nbox, nchild, n, v, ct, max_leaf);
}

// One wide node from its k candidates ch[i] (lc[i] primitives as a leaf
// child, 0 for an inner node): octant slots, quantised child boxes, the leaf
// records and the queue entries of the inner children, as k_collapse does.
// k_collapse keeps its own copy of these steps: a build that ran both rules
// in one kernel, choosing by a flag, lost leaf children on the device while
// its host compilation built correct nodes.
__device__ void write_wide_node(const Collapse &c, uint32_t ni, const int *ch, const int *lc, int k, uint2 *qout)
{
  int prims[3];
  float nlo[3] = {3.4e38f, 3.4e38f, 3.4e38f}, nhi[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
  for (int i = 0; i < k; ++i)
    for (int a = 0; a < 3; ++a) {
      nlo[a] = fminf(nlo[a], c.nbox[6 * size_t(ch[i]) + a]);
      nhi[a] = fmaxf(nhi[a], c.nbox[6 * size_t(ch[i]) + 3 + a]);
    }
  // octant slots, greedily by the smallest cost (the host builder's rule)
  float pc[3];
  for (int a = 0; a < 3; ++a)
    pc[a] = 0.5f * (nlo[a] + nhi[a]);
  float cost[8][8];
  for (int i = 0; i < k; ++i) {
    float cc[3];
    for (int a = 0; a < 3; ++a)
      cc[a] = 0.5f * (c.nbox[6 * size_t(ch[i]) + a] + c.nbox[6 * size_t(ch[i]) + 3 + a]) - pc[a];
    for (int s = 0; s < 8; ++s) {
      const float dx = (s & 4) ? -1.f : 1.f, dy = (s & 2) ? -1.f : 1.f, dz = (s & 1) ? -1.f : 1.f;
      cost[i][s] = cc[0] * dx + cc[1] * dy + cc[2] * dz;
    }
  }
  int child_at[8], cand_at[8];
  for (int s = 0; s < 8; ++s)
    child_at[s] = cand_at[s] = -1;
  uint32_t used_c = 0u, used_s = 0u;
  for (int it = 0; it < k; ++it) {
    float best = 3.4e38f;
    int bc = -1, bs = -1;
    for (int i = 0; i < k; ++i) {
      if (used_c & (1u << i))
        continue;
      for (int s = 0; s < 8; ++s) {
        if (used_s & (1u << s))
          continue;
        if (cost[i][s] < best || bc < 0) {
          best = cost[i][s];
          bc = i;
          bs = s;
        }
      }
    }
    used_c |= 1u << bc;
    used_s |= 1u << bs;
    child_at[bs] = ch[bc];
    cand_at[bs] = bc;
  }
  // quantisation grid (double, exact powers of two: outward rounding)
  uint8_t e[3];
  double scale[3];
  for (int a = 0; a < 3; ++a) {
    const double ext = double(nhi[a]) - double(nlo[a]);
    int ex = -127;
    if (ext > 0.0) {
      ex = int(ceil(log2(ext / 255.0)));
      while (ldexp(255.0, ex) < ext)
        ++ex;
      while (ex > -127 && ldexp(255.0, ex - 1) >= ext)
        --ex;
    }
    ex = min(max(ex, -127), 127);
    e[a] = uint8_t(ex + 127);
    scale[a] = ex == -127 ? 0.0 : ldexp(1.0, ex);
  }
  // leaf children: single primitives, and internal children of at most
  // max_leaf primitives (lcount[s] primitives each)
  uint32_t internal = 0, leaves = 0;
  uint8_t imask = 0;
  int lcount[8];
  for (int s = 0; s < 8; ++s) {
    lcount[s] = 0;
    if (child_at[s] < 0)
      continue;
    lcount[s] = lc[cand_at[s]];
    if (lcount[s] == 0) {
      imask |= uint8_t(1u << s);
      ++internal;
    } else {
      leaves += uint32_t(lcount[s]);
    }
  }
  uint32_t child_base = 0, tri_base = 0;
  if (internal)
    child_base = atomicAdd(&c.counters[0], internal);
  if (leaves)
    tri_base = atomicAdd(&c.counters[1], leaves);
  if (child_base + internal > c.node_cap) {
    atomicExch(&c.counters[3], 1u);
    return;
  }
  uint32_t q_out_base = 0;
  if (internal)
    q_out_base = atomicAdd(&c.counters[2], internal);
  uint8_t meta[8] = {}, q[6][8] = {};
  uint32_t next_child = child_base, tri_off = 0, qo = q_out_base;
  for (int s = 0; s < 8; ++s) {
    const int v = child_at[s];
    if (v < 0)
      continue;
    const float *b = c.nbox + 6 * size_t(v);
    for (int a = 0; a < 3; ++a) {
      double lo = 0.0, hi = 0.0;
      if (scale[a] > 0.0) {
        lo = floor((double(b[a]) - double(nlo[a])) / scale[a]);
        hi = ceil((double(b[3 + a]) - double(nlo[a])) / scale[a]);
      }
      q[a][s] = uint8_t(fmin(fmax(lo, 0.0), 255.0));
      q[3 + a][s] = uint8_t(fmin(fmax(hi, 0.0), 255.0));
    }
    if (lcount[s] == 0) {
      meta[s] = 0x80;
      qout[qo++] = make_uint2(next_child++, uint32_t(v));
    } else {
      meta[s] = uint8_t((uint32_t(lcount[s]) << 5) | tri_off);
      if (c.nchild[v].x < 0) {
        prims[0] = c.nchild[v].y;
      } else if (subtree_prims(c.nchild, v, c.max_leaf, prims) != lcount[s]) { // cannot happen
        atomicExch(&c.counters[3], 2u);
        return;
      }
      for (int j = 0; j < lcount[s]; ++j) {
        const uint32_t prim = uint32_t(prims[j]);
        const uint4 vi = c.vidx[prim];
        const float4 v0 = c.pos[vi.x], v1 = c.pos[vi.y], v2 = c.pos[vi.z];
        float4 *r = c.tris + 3 * size_t(tri_base + tri_off);
        r[0] = make_float4(v0.x, v0.y, v0.z, __uint_as_float(prim));
        r[1] = make_float4(v1.x - v0.x, v1.y - v0.y, v1.z - v0.z, 0.f);
        r[2] = make_float4(v2.x - v0.x, v2.y - v0.y, v2.z - v0.z, 0.f);
        ++tri_off;
      }
    }
  }
  uint32_t *w = c.nodes + size_t(ni) * 20;
  w[0] = __float_as_uint(nlo[0]);
  w[1] = __float_as_uint(nlo[1]);
  w[2] = __float_as_uint(nlo[2]);
  w[3] = uint32_t(e[0]) | (uint32_t(e[1]) << 8) | (uint32_t(e[2]) << 16) | (uint32_t(imask) << 24);
  w[4] = child_base;
  w[5] = tri_base;
  w[6] = uint32_t(meta[0]) | (uint32_t(meta[1]) << 8) | (uint32_t(meta[2]) << 16) | (uint32_t(meta[3]) << 24);
  w[7] = uint32_t(meta[4]) | (uint32_t(meta[5]) << 8) | (uint32_t(meta[6]) << 16) | (uint32_t(meta[7]) << 24);
  for (int r = 0; r < 6; ++r) {
    w[8 + 2 * r] = uint32_t(q[r][0]) | (uint32_t(q[r][1]) << 8) | (uint32_t(q[r][2]) << 16) |
        (uint32_t(q[r][3]) << 24);
    w[9 + 2 * r] = uint32_t(q[r][4]) | (uint32_t(q[r][5]) << 8) | (uint32_t(q[r][6]) << 16) |
        (uint32_t(q[r][7]) << 24);
  }
}

// One wide node per thread, its children chosen by the surface-area program
// (k_collapse_dp, then sah_children).
struct CollapseSah {
  const uint8_t *split; // CollapseDp::split
  const uchar4 *info;   // CollapseDp::info
  uint32_t n;           // primitives (the binary leaves 0..n-1)
};

__global__ void __launch_bounds__(128) k_collapse_sah(Collapse c, CollapseSah p, const uint2 *__restrict__ qin,
    uint32_t nq, uint2 *__restrict__ qout)
{
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nq)
    return;
  const uint32_t ni = qin[t].x;
  const int root = int(qin[t].y);
  int ch[8], lc[8];
  for (int i = 0; i < 8; ++i)
    ch[i] = lc[i] = 0;
  int k = 1;
  if (uint32_t(root) < p.n) { // a leaf root: one leaf child
    ch[0] = root;
    lc[0] = 1;
  } else {
    k = sah_children(c.nchild, p.split, p.info, p.n, root, ch, lc);
  }
  if (k < 0) {
    atomicExch(&c.counters[3], 2u);
    return;
  }
  write_wide_node(c, ni, ch, lc, k, qout);
}

struct DevBuf {
  void *p{nullptr};
  ~DevBuf()
  {
    if (p)
      cudaFree(p);
  }
  template <class T> T *as() { return static_cast<T *>(p); }
};

void ck(cudaError_t e, const char *what)
{
  if (e != cudaSuccess)
    throw std::runtime_error(std::string("gpu bvh build: ") + what + ": " + cudaGetErrorString(e));
}

void alloc(DevBuf &b, size_t bytes, const char *what)
{
  ck(cudaMalloc(&b.p, bytes ? bytes : 16), what);
}

uint32_t grid_of(uint32_t n, uint32_t block) { return std::max<uint32_t>(1u, std::min<uint32_t>((n + block - 1) / block, 1u << 20)); }

} // namespace

size_t scan_u32_scratch(uint32_t n) { return (size_t(n) + SCAN_TILE - 1) / SCAN_TILE; }

void scan_u32(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *total, uint32_t *scratch, cudaStream_t s)
{
  if (n == 0)
    return;
  const uint32_t tiles = uint32_t(scan_u32_scratch(n));
  k_tile_sums<<<tiles, SCAN_T, 0, s>>>(in, n, scratch);
  k_scan_inplace<<<1, 1024, 0, s>>>(scratch, tiles, total);
  k_tile_scan<<<tiles, SCAN_T, 0, s>>>(in, n, scratch, out);
}

GpuBvh8 build_bvh8_gpu(const float4 *positions, const uint4 *prim_vidx, uint32_t n, cudaStream_t s, int max_leaf,
    int radius, float tri_cost)
{
  if (n == 0)
    throw std::runtime_error("gpu bvh build: no triangles");
  if (n > (1u << 30))
    throw std::runtime_error("gpu bvh build: too many triangles");
  DevBuf boxes, cb, keys[2], vals[2], hist, total;
  alloc(boxes, size_t(n) * 24, "boxes");
  alloc(cb, 6 * 4, "bounds");
  for (int k = 0; k < 2; ++k) {
    alloc(keys[k], size_t(n) * 4, "keys");
    alloc(vals[k], size_t(n) * 4, "values");
  }
  const uint32_t nb = (n + SORT_BLOCK - 1) / SORT_BLOCK;
  alloc(hist, size_t(nb) * 256 * 4, "histogram");
  DevBuf scan_tmp;
  alloc(scan_tmp, std::max(scan_u32_scratch(nb * 256), scan_u32_scratch(n)) * 4, "scan tile sums");
  alloc(total, 16, "total");
  // scene centroid bounds start at (+max, -max) in the ordered encoding
  const uint32_t init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
  ck(cudaMemcpyAsync(cb.p, init, sizeof(init), cudaMemcpyHostToDevice, s), "bounds init");
  k_prim_boxes<<<grid_of(n, 256), 256, 0, s>>>(positions, prim_vidx, n, boxes.as<float>(), cb.as<uint32_t>());
  k_morton<<<grid_of(n, 256), 256, 0, s>>>(boxes.as<float>(), n, cb.as<uint32_t>(), keys[0].as<uint32_t>(),
      vals[0].as<uint32_t>());
  int cur = 0;
  for (int shift = 0; shift < 32; shift += 8) {
    k_digit_hist<<<nb, SORT_BLOCK, 0, s>>>(keys[cur].as<uint32_t>(), n, shift, hist.as<uint32_t>(), nb);
    scan_u32(hist.as<uint32_t>(), hist.as<uint32_t>(), nb * 256, nullptr, scan_tmp.as<uint32_t>(), s);
    k_digit_scatter<<<nb, SORT_BLOCK, 0, s>>>(keys[cur].as<uint32_t>(), vals[cur].as<uint32_t>(), n, shift,
        hist.as<uint32_t>(), nb, keys[cur ^ 1].as<uint32_t>(), vals[cur ^ 1].as<uint32_t>());
    cur ^= 1;
  }
  const uint32_t *sorted = vals[cur].as<uint32_t>();

  // PLOC
  const uint32_t nodes2 = 2 * n - 1;
  DevBuf nbox, nchild, cid[2], cbox[2], nn, mflag, mrank, kflag, krank;
  alloc(nbox, size_t(nodes2) * 24, "bvh2 boxes");
  alloc(nchild, size_t(nodes2) * 8, "bvh2 children");
  for (int k = 0; k < 2; ++k) {
    alloc(cid[k], size_t(n) * 4, "cluster ids");
    alloc(cbox[k], size_t(n) * 24, "cluster boxes");
  }
  alloc(nn, size_t(n) * 4, "neighbours");
  alloc(mflag, size_t(n) * 4, "merge flags");
  alloc(mrank, size_t(n) * 4, "merge ranks");
  alloc(kflag, size_t(n) * 4, "keep flags");
  alloc(krank, size_t(n) * 4, "keep ranks");
  k_leaves<<<grid_of(n, 256), 256, 0, s>>>(boxes.as<float>(), sorted, n, nbox.as<float>(), nchild.as<int2>(),
      cid[0].as<uint32_t>(), cbox[0].as<float>());
  uint32_t count = n, node_base = n;
  int c = 0;
  uint32_t counts[4];
  std::vector<uint32_t> iter_base{n}; // the internal nodes each iteration made: [base[i], base[i + 1])
  for (int iter = 0; count > 1; ++iter) {
    const unsigned nb = (count + TILE - 1) / TILE;
    if (radius <= 2)
      k_ploc_nn<2><<<nb, TILE, 0, s>>>(cbox[c].as<float>(), count, nn.as<uint32_t>());
    else if (radius <= 4)
      k_ploc_nn<4><<<nb, TILE, 0, s>>>(cbox[c].as<float>(), count, nn.as<uint32_t>());
    else if (radius <= 8)
      k_ploc_nn<8><<<nb, TILE, 0, s>>>(cbox[c].as<float>(), count, nn.as<uint32_t>());
    else if (radius <= 16)
      k_ploc_nn<16><<<nb, TILE, 0, s>>>(cbox[c].as<float>(), count, nn.as<uint32_t>());
    else
      k_ploc_nn<32><<<nb, TILE, 0, s>>>(cbox[c].as<float>(), count, nn.as<uint32_t>());
    k_ploc_flags<<<grid_of(count, 256), 256, 0, s>>>(nn.as<uint32_t>(), count, mflag.as<uint32_t>(),
        kflag.as<uint32_t>());
    scan_u32(mflag.as<uint32_t>(), mrank.as<uint32_t>(), count, total.as<uint32_t>(), scan_tmp.as<uint32_t>(), s);
    scan_u32(kflag.as<uint32_t>(), krank.as<uint32_t>(), count, total.as<uint32_t>() + 1, scan_tmp.as<uint32_t>(), s);
    k_ploc_write<<<grid_of(count, 256), 256, 0, s>>>(nn.as<uint32_t>(), count, mflag.as<uint32_t>(),
        mrank.as<uint32_t>(), kflag.as<uint32_t>(), krank.as<uint32_t>(), node_base, cid[c].as<uint32_t>(),
        cbox[c].as<float>(), cid[c ^ 1].as<uint32_t>(), cbox[c ^ 1].as<float>(), nbox.as<float>(),
        nchild.as<int2>());
    ck(cudaMemcpyAsync(counts, total.p, 8, cudaMemcpyDeviceToHost, s), "read counts");
    ck(cudaStreamSynchronize(s), "ploc iteration");
    if (counts[0] == 0 || counts[1] >= count)
      throw std::runtime_error("gpu bvh build: clustering made no progress");
    node_base += counts[0];
    iter_base.push_back(node_base);
    count = counts[1];
    c ^= 1;
  }
  uint32_t root = 0;
  ck(cudaMemcpyAsync(&root, cid[c].p, 4, cudaMemcpyDeviceToHost, s), "read root");
  ck(cudaStreamSynchronize(s), "root");

  // collapse into BVH8 nodes, level by level
  GpuBvh8 out;
  out.node_cap = n; // a BVH8 over n leaves with >= 2 children per inner node has fewer nodes
  DevBuf nodes_buf, tris_buf; // owned here until the build succeeds
  alloc(nodes_buf, size_t(out.node_cap) * 80, "bvh8 nodes");
  alloc(tris_buf, size_t(n) * 48, "bvh8 triangles");
  out.nodes = nodes_buf.p;
  out.tris = tris_buf.p;
  DevBuf q[2], ctr;
  alloc(q[0], size_t(n) * 8, "queue");
  alloc(q[1], size_t(n) * 8, "queue");
  alloc(ctr, 16, "collapse counters");
  const uint32_t c0[4] = {1u, 0u, 0u, 0u};
  ck(cudaMemcpyAsync(ctr.p, c0, sizeof(c0), cudaMemcpyHostToDevice, s), "collapse counters");
  const uint2 first = make_uint2(0u, root);
  ck(cudaMemcpyAsync(q[0].p, &first, sizeof(first), cudaMemcpyHostToDevice, s), "first queue entry");
  const int leaf_max = std::min(std::max(max_leaf, 1), 3);
  // the surface-area program, bottom-up one clustering iteration at a time
  DevBuf dp_cost, dp_split, dp_info;
  const uint32_t inner = node_base - n;
  if (tri_cost > 0.f && inner > 0) {
    alloc(dp_cost, size_t(inner) * 8 * 4, "collapse costs");
    alloc(dp_split, size_t(inner) * 8, "collapse splits");
    alloc(dp_info, size_t(inner) * 4, "collapse choices");
    const CollapseDp d{dp_cost.as<float>(), dp_split.as<uint8_t>(), dp_info.as<uchar4>()};
    for (size_t i = 0; i + 1 < iter_base.size(); ++i) {
      const uint32_t lo = iter_base[i], hi = iter_base[i + 1];
      k_collapse_dp<<<grid_of(hi - lo, 128), 128, 0, s>>>(d, nbox.as<float>(), nchild.as<int2>(), n, lo, hi,
          tri_cost, leaf_max);
    }
    ck(cudaGetLastError(), "collapse program");
  }
  Collapse col{nbox.as<float>(), nchild.as<int2>(), positions, prim_vidx, nodes_buf.as<uint32_t>(),
      tris_buf.as<float4>(), ctr.as<uint32_t>(), out.node_cap, leaf_max};
  const CollapseSah sah{dp_split.as<uint8_t>(), dp_info.as<uchar4>(), n};
  uint32_t nq = 1, depth = 0;
  int qc = 0;
  while (nq > 0) {
    ++depth;
    if (depth > 1000)
      throw std::runtime_error("gpu bvh build: collapse did not end");
    if (dp_split.p)
      k_collapse_sah<<<(nq + 127) / 128, 128, 0, s>>>(col, sah, q[qc].as<uint2>(), nq, q[qc ^ 1].as<uint2>());
    else
      k_collapse<<<(nq + 127) / 128, 128, 0, s>>>(col, q[qc].as<uint2>(), nq, q[qc ^ 1].as<uint2>());
    ck(cudaGetLastError(), "collapse launch");
    uint32_t cc[4];
    ck(cudaMemcpyAsync(cc, ctr.p, 16, cudaMemcpyDeviceToHost, s), "read collapse counters");
    ck(cudaStreamSynchronize(s), "collapse level");
    if (cc[3] == 2)
      throw std::runtime_error("gpu bvh build: the collapse's surface-area choices are inconsistent");
    if (cc[3])
      throw std::runtime_error("gpu bvh build: node capacity exceeded");
    nq = cc[2];
    const uint32_t zero = 0u;
    ck(cudaMemcpyAsync(ctr.as<uint32_t>() + 2, &zero, 4, cudaMemcpyHostToDevice, s), "reset queue length");
    qc ^= 1;
    out.node_count = cc[0];
    out.tri_count = cc[1];
  }
  ck(cudaStreamSynchronize(s), "bvh8 build");
  if (out.tri_count != n)
    throw std::runtime_error("gpu bvh build: leaf records do not cover the triangles");
  out.max_depth = depth;
  // trim the node array from its worst-case size to the nodes made
  DevBuf exact;
  if (out.node_count < out.node_cap && cudaMalloc(&exact.p, size_t(out.node_count) * 80) == cudaSuccess) {
    ck(cudaMemcpyAsync(exact.p, nodes_buf.p, size_t(out.node_count) * 80, cudaMemcpyDeviceToDevice, s),
        "trim nodes");
    ck(cudaStreamSynchronize(s), "trim nodes");
    std::swap(exact.p, nodes_buf.p); // the worst-case array is freed with `exact`
    out.node_cap = out.node_count;
  }
  out.nodes = nodes_buf.p;
  out.tris = tris_buf.p;
  nodes_buf.p = tris_buf.p = nullptr; // ownership passes to the caller
  return out;
}

} // namespace phc
