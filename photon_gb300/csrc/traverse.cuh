// BVH8 traversal on the SMs (GB300 has no RT cores).
//
// Closest-hit and any-hit queries over the quantised BVH8 of bvh8.h.  The
// traversal keeps the current node group (child base, hit mask, internal
// mask) in registers and pushes only groups with children left, so the stack
// holds one 8-byte entry per tree level (a short stack, after Ylitie et al.
// 2017).  Child boxes are tested with one FMA per plane from the 8-bit grid;
// the far distance is widened by 4e-7 relative so the outward-rounded boxes
// never cull a triangle the exact test would hit.
//
// The triangle test is the reference's Möller–Trumbore
// (include/photon/pt/geom/triangle_intersect.h:18-52) with the same operation
// order and the same e1/e2 roundings (precomputed on the host), compiled
// without FMA contraction, so t, u, v and the accept/reject decisions are
// bit-identical to the reference's for the same ray and triangle; the closest
// hit therefore equals the reference's except for exact ties in t, which the
// reference breaks by its own traversal order (mesh_intersector.h:92).
//
// The functions are __host__ __device__ so host-side tests can run the very
// same traversal on the CPU against the oracle.
#pragma once

#include "pt_math.cuh"
#include "scene_types.h"

namespace phc {

#ifndef PHC_STACK_SIZE
#define PHC_STACK_SIZE 64
#endif

struct RayHit {
  float t;
  uint32_t prim; // 0xffffffff: miss
  float u, v;
};

struct TravCounters {
  uint32_t nodes;
  uint32_t tris;
};

PHC_HD uint4 ldg4(const uint4 *p)
{
#ifdef __CUDA_ARCH__
  return __ldg(p);
#else
  return *p;
#endif
}
PHC_HD float4 ldg4(const float4 *p)
{
#ifdef __CUDA_ARCH__
  return __ldg(p);
#else
  return *p;
#endif
}

PHC_HD float safe_inv(float x) { return 1.f / (fabsf(x) > 1e-20f ? x : (x < 0.f ? -1e-20f : 1e-20f)); }

// Möller–Trumbore exactly as triangle_intersect.h:18-52.
PHC_HD bool tri_test(V3 o, V3 d, float4 r0, float4 r1, float4 r2, float tmin, float tmax, float &t, float &u, float &v)
{
  const V3 v0 = v3(r0), e1 = v3(r1), e2 = v3(r2);
  const V3 p = cross(d, e2);
  const float det = dot(e1, p);
  if (fabsf(det) < 1e-30f)
    return false;
  const float inv_det = 1.f / det;
  const V3 tv = o - v0;
  u = dot(tv, p) * inv_det;
  if (u < 0.f || u > 1.f)
    return false;
  const V3 q = cross(tv, e1);
  v = dot(d, q) * inv_det;
  if (v < 0.f || (u + v) > 1.f)
    return false;
  t = dot(e2, q) * inv_det;
  if (t < tmin || t > tmax)
    return false;
  return true;
}

// Byte j of w as a float, exactly: the byte becomes the low mantissa bits of
// 2^23 (one byte permute) and 2^23 is subtracted (one add), which avoids the
// integer-to-float conversion unit that throttled the box tests.
PHC_HD float byte_f(uint32_t w, int j)
{
#ifdef __CUDA_ARCH__
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + uint32_t(j))) - 8388608.f;
#else
  return u2f(0x4B000000u | ((w >> (8 * j)) & 0xffu)) - 8388608.f;
#endif
}

#ifdef __CUDA_ARCH__
// Paired fp32 arithmetic (sm_100+ FADD2 / FFMA2 through __fadd2_rn /
// __ffma2_rn on float2): each element is rounded exactly as the scalar
// instruction would round it, so the box tests below make the same
// decisions as the host restatement with half the issue slots.  Three-input
// min / max in one instruction:
__device__ __forceinline__ float max3f(float a, float b, float c)
{
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float min3f(float a, float b, float c)
{
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
// 2^23 + byte j of w, as float bits (one byte permute)
__device__ __forceinline__ float byte_f23(uint32_t w, int j)
{
  return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7540u + uint32_t(j)));
}
#endif

// Intersects the 8 child boxes of one node; returns the k-ordered hit mask of
// internal children (bit k = slot k ^ oct) and the triangle mask.  SLOTS
// collects the box hits as one slot-order mask first and decodes the leaf
// meta bytes only for hit leaves (fewer instructions per node when leaf hits
// are rare, as for closest-hit rays); the masks are the same either way.
template <bool SLOTS = false>
PHC_HD void intersect_node(const uint4 *__restrict__ nodes, uint32_t ni, V3 o, V3 idir, uint32_t oct, float tmin,
    float tmax, uint32_t &child_base, uint32_t &hits, uint32_t &imask, uint32_t &tri_base, uint32_t &tri_hits)
{
  const uint4 w0 = ldg4(nodes + 5 * size_t(ni) + 0);
  const uint4 w1 = ldg4(nodes + 5 * size_t(ni) + 1);
  const uint4 w2 = ldg4(nodes + 5 * size_t(ni) + 2);
  const uint4 w3 = ldg4(nodes + 5 * size_t(ni) + 3);
  const uint4 w4 = ldg4(nodes + 5 * size_t(ni) + 4);
  const float px = u2f(w0.x), py = u2f(w0.y), pz = u2f(w0.z);
  const float sx = u2f((w0.w & 0xffu) << 23);
  const float sy = u2f(((w0.w >> 8) & 0xffu) << 23);
  const float sz = u2f(((w0.w >> 16) & 0xffu) << 23);
  imask = w0.w >> 24;
  child_base = w1.x;
  tri_base = w1.y;
  const float ax = sx * idir.x, ay = sy * idir.y, az = sz * idir.z;
  const float bx = (px - o.x) * idir.x, by = (py - o.y) * idir.y, bz = (pz - o.z) * idir.z;
  // near/far byte rows per axis (qlo for a positive direction component)
  const bool nxl = idir.x >= 0.f, nyl = idir.y >= 0.f, nzl = idir.z >= 0.f;
  const uint32_t nx0 = nxl ? w2.x : w3.z, nx1 = nxl ? w2.y : w3.w;
  const uint32_t fx0 = nxl ? w3.z : w2.x, fx1 = nxl ? w3.w : w2.y;
  const uint32_t ny0 = nyl ? w2.z : w4.x, ny1 = nyl ? w2.w : w4.y;
  const uint32_t fy0 = nyl ? w4.x : w2.z, fy1 = nyl ? w4.y : w2.w;
  const uint32_t nz0 = nzl ? w3.x : w4.z, nz1 = nzl ? w3.y : w4.w;
  const uint32_t fz0 = nzl ? w4.z : w3.x, fz1 = nzl ? w4.w : w3.y;
  hits = 0u;
  tri_hits = 0u;
  uint32_t slots = 0u; // SLOTS: bit s set when the ray overlaps child box s
#ifdef __CUDA_ARCH__
  // (near, far) of one axis as a float2: q = (2^23 + byte) - 2^23 exactly,
  // then t = fma(q, a, b) per element.
  const float2 m23 = make_float2(-8388608.f, -8388608.f);
  const float2 ax2 = make_float2(ax, ax), ay2 = make_float2(ay, ay), az2 = make_float2(az, az);
  const float2 bx2 = make_float2(bx, bx), by2 = make_float2(by, by), bz2 = make_float2(bz, bz);
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const uint32_t m4 = h ? w1.w : w1.z;
    const uint32_t nxw = h ? nx1 : nx0, fxw = h ? fx1 : fx0;
    const uint32_t nyw = h ? ny1 : ny0, fyw = h ? fy1 : fy0;
    const uint32_t nzw = h ? nz1 : nz0, fzw = h ? fz1 : fz0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t mb = (m4 >> (8 * j)) & 0xffu;
      const float2 tx = __ffma2_rn(__fadd2_rn(make_float2(byte_f23(nxw, j), byte_f23(fxw, j)), m23), ax2, bx2);
      const float2 ty = __ffma2_rn(__fadd2_rn(make_float2(byte_f23(nyw, j), byte_f23(fyw, j)), m23), ay2, by2);
      const float2 tz = __ffma2_rn(__fadd2_rn(make_float2(byte_f23(nzw, j), byte_f23(fzw, j)), m23), az2, bz2);
      const float tnx = tx.x, tfx = tx.y, tny = ty.x, tfy = ty.y, tnz = tz.x, tfz = tz.y;
      const float t0 = fmaxf(max3f(tnx, tny, tnz), tmin);
      const float t1 = fminf(min3f(tfx, tfy, tfz), tmax);
      if constexpr (SLOTS) {
        slots |= (t0 <= t1 * 1.0000004f ? 1u : 0u) << (4 * h + j);
      } else if (t0 <= t1 * 1.0000004f) { // an empty slot (mb 0) adds nothing
        const int s = 4 * h + j;
        if (mb & 0x80u)
          hits |= 1u << (uint32_t(s) ^ oct);
        else
          tri_hits |= ((1u << (mb >> 5)) - 1u) << (mb & 31u);
      }
    }
  }
#else
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const uint32_t m4 = h ? w1.w : w1.z;
    const uint32_t nxw = h ? nx1 : nx0, fxw = h ? fx1 : fx0;
    const uint32_t nyw = h ? ny1 : ny0, fyw = h ? fy1 : fy0;
    const uint32_t nzw = h ? nz1 : nz0, fzw = h ? fz1 : fz0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t mb = (m4 >> (8 * j)) & 0xffu;
      const float tnx = fmaf(byte_f(nxw, j), ax, bx);
      const float tny = fmaf(byte_f(nyw, j), ay, by);
      const float tnz = fmaf(byte_f(nzw, j), az, bz);
      const float tfx = fmaf(byte_f(fxw, j), ax, bx);
      const float tfy = fmaf(byte_f(fyw, j), ay, by);
      const float tfz = fmaf(byte_f(fzw, j), az, bz);
      const float t0 = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
      const float t1 = fminf(fminf(tfx, tfy), fminf(tfz, tmax));
      if constexpr (SLOTS) {
        slots |= (t0 <= t1 * 1.0000004f ? 1u : 0u) << (4 * h + j);
      } else if (t0 <= t1 * 1.0000004f) { // an empty slot (mb 0) adds nothing
        const int s = 4 * h + j;
        if (mb & 0x80u)
          hits |= 1u << (uint32_t(s) ^ oct);
        else
          tri_hits |= ((1u << (mb >> 5)) - 1u) << (mb & 31u);
      }
    }
  }
#endif
  if constexpr (SLOTS) {
    // internal children: slot order -> visiting order (bit k = slot k ^ oct),
    // one swap stage per octant bit
    uint32_t m = slots & imask;
    if (oct & 1u)
      m = ((m << 1) & 0xaau) | ((m >> 1) & 0x55u);
    if (oct & 2u)
      m = ((m << 2) & 0xccu) | ((m >> 2) & 0x33u);
    if (oct & 4u)
      m = ((m << 4) & 0xf0u) | ((m >> 4) & 0x0fu);
    hits = m;
    // leaf children: their triangle ranges from the meta bytes (an empty slot,
    // meta 0, adds nothing)
    uint32_t lm = slots & ~imask;
    while (lm) {
      const uint32_t sl = ffs32(lm) - 1u;
      lm &= lm - 1u;
      const uint32_t mb = ((sl < 4u ? w1.z : w1.w) >> (8u * (sl & 3u))) & 0xffu;
      tri_hits |= ((1u << (mb >> 5)) - 1u) << (mb & 31u);
    }
  }
}

// Resumable traversal state of one ray: the current node group (child base,
// k-ordered hit mask, internal mask) and the stack depth; the stack itself
// is a per-thread array owned by the caller.
struct TravState {
  V3 o, d, idir;
  uint32_t oct;
  float tmin;
  RayHit best;
  uint32_t g_base, g_hits, g_imask;
  int sp;
};

PHC_HD void trav_init(TravState &s, V3 o, V3 d, float tmin, float tmax)
{
  s.o = o;
  s.d = d;
  s.idir = V3{safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
  s.oct = (d.x < 0.f ? 4u : 0u) | (d.y < 0.f ? 2u : 0u) | (d.z < 0.f ? 1u : 0u);
  s.tmin = tmin;
  s.best = RayHit{tmax, 0xffffffffu, 0.f, 0.f};
  s.g_base = 0u;
  s.g_hits = (tmax > tmin) ? 1u << s.oct : 0u; // the root, or nothing for an empty ray
  s.g_imask = 1u;
  s.sp = 0;
}

// One step: the next node of the current group (or of the stack), its box
// tests and the triangles of its hit leaves.  Returns false when the ray is
// finished (nothing left, or an any-hit query found a hit).
template <bool ANY, bool COUNT>
PHC_HD bool trav_step(const uint4 *__restrict__ nodes, const float4 *__restrict__ tris, TravState &s, uint2 *stack,
    TravCounters *ctr)
{
  if (s.g_hits == 0u) {
    if (s.sp == 0)
      return false;
    const uint2 e = stack[--s.sp];
    s.g_base = e.x;
    s.g_hits = e.y & 0xffu;
    s.g_imask = e.y >> 8;
  }
  const uint32_t k = ffs32(s.g_hits) - 1u;
  s.g_hits &= s.g_hits - 1u;
  const uint32_t slot = k ^ s.oct;
  const uint32_t ni = s.g_base + popc32(s.g_imask & ((1u << slot) - 1u));
  if (s.g_hits != 0u && s.sp < PHC_STACK_SIZE) {
    stack[s.sp].x = s.g_base;
    stack[s.sp].y = s.g_hits | (s.g_imask << 8);
    ++s.sp;
  }
  uint32_t tri_base, tri_hits;
  intersect_node<!ANY>(nodes, ni, s.o, s.idir, s.oct, s.tmin, s.best.t, s.g_base, s.g_hits, s.g_imask, tri_base,
      tri_hits);
  if (COUNT)
    ctr->nodes++;
  while (tri_hits) {
    const uint32_t b = ffs32(tri_hits) - 1u;
    tri_hits &= tri_hits - 1u;
    const float4 *r = tris + 3 * size_t(tri_base + b);
    const float4 r0 = ldg4(r), r1 = ldg4(r + 1), r2 = ldg4(r + 2);
    if (COUNT)
      ctr->tris++;
    float t, u, v;
    if (tri_test(s.o, s.d, r0, r1, r2, s.tmin, s.best.t, t, u, v)) {
      s.best.t = t;
      s.best.prim = f2u(r0.w);
      s.best.u = u;
      s.best.v = v;
      if (ANY)
        return false;
    }
  }
  return s.g_hits != 0u || s.sp != 0;
}

// ------------------------------------------------------- two levels
// Traversal of a scene with instances (SCENE_INSTANCES): the top level's
// leaves are instance slots.  A top-level node visit that reaches leaves
// queues their slots (in registers); each queued slot is entered in turn by
// carrying the ray into the object's space (origin and direction through
// the world-to-object rows, the direction not renormalised so that t keeps
// its meaning) and traversing the object's bottom level from its root.  The
// stack depth at entry marks where the bottom level's entries end: when the
// bottom level has no group left above it, the world ray comes back and the
// next queued slot (or the top level's stack) continues.  The stack holds
// the top level's groups below the bottom level's; the scene build keeps the
// two depths' sum below its size.
struct TravState2 : TravState {
  V3 wo, wd, widir; // the world ray
  uint32_t woct;
  uint32_t inst;      // current instance slot, INST_NONE on the top level
  uint32_t inst_hit;  // what a hit in it records: the slot, or INST_NONE for
                      // the scene's own triangles (an identity placement)
  uint32_t best_inst; // instance slot of the closest hit so far
  uint32_t pend_base, pend_mask; // queued instance slots of a top-level node
  int blas_sp;        // stack depth where the current bottom level began
};

PHC_HD void trav_init2(TravState2 &s, V3 o, V3 d, float tmin, float tmax)
{
  trav_init(s, o, d, tmin, tmax);
  s.wo = s.o;
  s.wd = s.d;
  s.widir = s.idir;
  s.woct = s.oct;
  s.inst = INST_NONE;
  s.inst_hit = INST_NONE;
  s.best_inst = INST_NONE;
  s.pend_base = 0u;
  s.pend_mask = 0u;
  s.blas_sp = 0;
}

// p' = M p (rows r0..r2 of a 3x4 matrix); d' = M d without the translation
PHC_HD V3 xf_point3(float4 r0, float4 r1, float4 r2, V3 p)
{
  return V3{r0.x * p.x + r0.y * p.y + r0.z * p.z + r0.w, r1.x * p.x + r1.y * p.y + r1.z * p.z + r1.w,
      r2.x * p.x + r2.y * p.y + r2.z * p.z + r2.w};
}
PHC_HD V3 xf_dir3(float4 r0, float4 r1, float4 r2, V3 d)
{
  return V3{r0.x * d.x + r0.y * d.y + r0.z * d.z, r1.x * d.x + r1.y * d.y + r1.z * d.z,
      r2.x * d.x + r2.y * d.y + r2.z * d.z};
}

PHC_HD void stack_push(uint2 *stack, int &sp, uint32_t x, uint32_t y)
{
  if (sp < PHC_STACK_SIZE) {
    stack[sp].x = x;
    stack[sp].y = y;
    ++sp;
  }
}

template <bool ANY, bool COUNT>
PHC_HD bool trav_step2(const uint4 *__restrict__ nodes, const float4 *__restrict__ tris,
    const float4 *__restrict__ inst_w2o, const uint4 *__restrict__ inst_info, TravState2 &s, uint2 *stack,
    TravCounters *ctr)
{
  // bookkeeping (popping a group, leaving a bottom level, entering a queued
  // instance) runs in the same step as the next node visit, so that every
  // step of a busy lane visits one node.  The loop has no return: all its
  // exits meet before the node visit, where the warp's lanes reconverge.
  bool alive = true;
  for (int guard = 0; guard < 2 * PHC_STACK_SIZE + 66; ++guard) {
    if (s.inst != INST_NONE) { // in a bottom level
      if (s.g_hits != 0u)
        break;
      if (s.sp > s.blas_sp) {
        const uint2 e = stack[--s.sp];
        s.g_base = e.x;
        s.g_hits = e.y & 0xffu;
        s.g_imask = e.y >> 8;
        continue;
      }
      s.o = s.wo; // the bottom level is done: back to the world ray
      s.d = s.wd;
      s.idir = s.widir;
      s.oct = s.woct;
      s.inst = INST_NONE;
      continue;
    }
    if (s.pend_mask != 0u) { // enter the next queued instance
      if (s.g_hits != 0u) {
        stack_push(stack, s.sp, s.g_base, s.g_hits | (s.g_imask << 8));
        s.g_hits = 0u;
      }
      const uint32_t k = ffs32(s.pend_mask) - 1u;
      s.pend_mask &= s.pend_mask - 1u;
      const uint32_t j = s.pend_base + k;
      const uint4 info = ldg4(inst_info + j);
      s.inst = j;
      s.inst_hit = (info.z & INST_IDENTITY) ? INST_NONE : j;
      if (!(info.z & INST_IDENTITY)) {
        const float4 r0 = ldg4(inst_w2o + 3 * size_t(j)), r1 = ldg4(inst_w2o + 3 * size_t(j) + 1);
        const float4 r2 = ldg4(inst_w2o + 3 * size_t(j) + 2);
        s.o = xf_point3(r0, r1, r2, s.wo);
        s.d = xf_dir3(r0, r1, r2, s.wd);
        s.idir = V3{safe_inv(s.d.x), safe_inv(s.d.y), safe_inv(s.d.z)};
        s.oct = (s.d.x < 0.f ? 4u : 0u) | (s.d.y < 0.f ? 2u : 0u) | (s.d.z < 0.f ? 1u : 0u);
      }
      s.blas_sp = s.sp;
      s.g_base = info.x; // the bottom level's root as a one-child group
      s.g_hits = 1u << s.oct;
      s.g_imask = 1u;
      break;
    }
    if (s.g_hits != 0u)
      break;
    if (s.sp == 0) {
      alive = false;
      break;
    }
    const uint2 e = stack[--s.sp];
    s.g_base = e.x;
    s.g_hits = e.y & 0xffu;
    s.g_imask = e.y >> 8;
  }
  if (!alive || s.g_hits == 0u) // (g_hits 0 with alive: not reached, the loop always ends on a group)
    return false;
  const uint32_t k = ffs32(s.g_hits) - 1u;
  s.g_hits &= s.g_hits - 1u;
  const uint32_t slot = k ^ s.oct;
  const uint32_t ni = s.g_base + popc32(s.g_imask & ((1u << slot) - 1u));
  if (s.g_hits != 0u)
    stack_push(stack, s.sp, s.g_base, s.g_hits | (s.g_imask << 8));
  uint32_t tri_base, tri_hits;
  intersect_node<!ANY>(nodes, ni, s.o, s.idir, s.oct, s.tmin, s.best.t, s.g_base, s.g_hits, s.g_imask, tri_base,
      tri_hits);
  if (COUNT)
    ctr->nodes++;
  if (s.inst == INST_NONE) { // top level: the leaves are instance slots
    s.pend_base = tri_base;
    s.pend_mask = tri_hits;
    return s.pend_mask != 0u || s.g_hits != 0u || s.sp != 0;
  }
  while (tri_hits) {
    const uint32_t b = ffs32(tri_hits) - 1u;
    tri_hits &= tri_hits - 1u;
    const float4 *r = tris + 3 * size_t(tri_base + b);
    const float4 r0 = ldg4(r), r1 = ldg4(r + 1), r2 = ldg4(r + 2);
    if (COUNT)
      ctr->tris++;
    float t, u, v;
    if (tri_test(s.o, s.d, r0, r1, r2, s.tmin, s.best.t, t, u, v)) {
      s.best.t = t;
      s.best.prim = f2u(r0.w);
      s.best.u = u;
      s.best.v = v;
      s.best_inst = s.inst_hit;
      if (ANY)
        return false;
    }
  }
  return s.g_hits != 0u || s.sp != 0 || s.pend_mask != 0u;
}

// Full traversal of one ray.  ANY: stop at the first hit (occlusion).
template <bool ANY, bool COUNT>
PHC_HD RayHit trace_ray(const DevScene &sc, V3 o, V3 d, float tmin, float tmax, TravCounters *ctr)
{
  TravState s;
  trav_init(s, o, d, tmin, tmax);
  uint2 stack[PHC_STACK_SIZE];
  if (s.g_hits != 0u)
    while (trav_step<ANY, COUNT>(sc.nodes, sc.tris, s, stack, ctr)) {
    }
  return s.best;
}

// Full two-level traversal of one ray; `inst` gets the hit's instance slot
// (INST_NONE: the scene's own triangles, or a miss).
template <bool ANY, bool COUNT>
PHC_HD RayHit trace_ray2(const DevScene &sc, V3 o, V3 d, float tmin, float tmax, TravCounters *ctr, uint32_t &inst)
{
  TravState2 s;
  trav_init2(s, o, d, tmin, tmax);
  uint2 stack[PHC_STACK_SIZE];
  if (s.g_hits != 0u)
    while (trav_step2<ANY, COUNT>(sc.nodes, sc.tris, sc.inst_w2o, sc.inst_info, s, stack, ctr)) {
    }
  inst = s.best_inst;
  return s.best;
}

// Attributes of a hit as intersect_mesh_bvh computes them after the
// traversal (mesh_intersector.h:129-178): position, geometric normal,
// interpolated shading normal, material id.
struct HitAttr {
  V3 p, n, sn;
  uint32_t material_id;
  uint4 vidx;
};
//
// A hit on an instance (inst = its slot, not INST_NONE) is computed in the
// object's space and carried to world space as the reference's instanced
// back-end does (backend/optix/photon_optix.cu:68-99, 183-186): both normals
// through the inverse transpose of the instance transform (the transpose of
// the world-to-object rows), normalised.
PHC_HD HitAttr hit_attributes(const DevScene &sc, V3 o, V3 d, const RayHit &h, uint32_t inst = INST_NONE)
{
  HitAttr a;
  const float4 *g = sc.prim_geo + 3 * size_t(h.prim);
  const V3 e1 = v3(ldg4(g + 1)), e2 = v3(ldg4(g + 2));
#ifdef __CUDA_ARCH__
  a.vidx = __ldg(sc.prim_vidx + h.prim);
#else
  a.vidx = sc.prim_vidx[h.prim];
#endif
  a.p = o + d * h.t;
  const V3 nn = normalize(cross(e1, e2));
  a.n = nn;
  a.sn = nn;
  uint32_t flags = sc.scene_normals ? INST_NORMALS : 0u;
  if (inst != INST_NONE)
    flags = ldg4(sc.inst_info + inst).z;
  if (flags & INST_NORMALS) {
    const float w0 = 1.f - h.u - h.v, w1 = h.u, w2 = h.v;
    const V3 n0 = v3(ldg4(sc.normals + a.vidx.x)), n1 = v3(ldg4(sc.normals + a.vidx.y));
    const V3 n2 = v3(ldg4(sc.normals + a.vidx.z));
    a.sn = normalize(n0 * w0 + n1 * w1 + n2 * w2);
    if (dot(a.sn, nn) < 0.f)
      a.sn = a.sn * -1.f;
  }
  if (inst != INST_NONE && !(flags & INST_IDENTITY)) {
    const float4 r0 = ldg4(sc.inst_w2o + 3 * size_t(inst)), r1 = ldg4(sc.inst_w2o + 3 * size_t(inst) + 1);
    const float4 r2 = ldg4(sc.inst_w2o + 3 * size_t(inst) + 2);
    const V3 n = a.n, sn = a.sn;
    a.n = normalize(V3{r0.x * n.x + r1.x * n.y + r2.x * n.z, r0.y * n.x + r1.y * n.y + r2.y * n.z,
        r0.z * n.x + r1.z * n.y + r2.z * n.z});
    a.sn = normalize(V3{r0.x * sn.x + r1.x * sn.y + r2.x * sn.z, r0.y * sn.x + r1.y * sn.y + r2.y * sn.z,
        r0.z * sn.x + r1.z * sn.y + r2.z * sn.z});
  }
  a.material_id = a.vidx.w;
  return a;
}

} // namespace phc
