// Host builder of the quantised BVH8 (layout in bvh8.h).
//
// 1. Binned SAH BVH2 over triangle boxes: 32 bins on each of the three axes,
//    leaf when the SAH prefers it and at most max_leaf triangles remain;
//    subtrees above 8K triangles are built as OpenMP tasks.
// 2. Collapse into 8-wide nodes: starting from the two children of a BVH2
//    node, repeatedly open the internal child with the largest surface area
//    until 8 children are reached.
// 3. Octant slot assignment and outward-rounded 8-bit child boxes.
#include "bvh8.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <stdexcept>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace phc {
namespace {

struct Box {
  float lo[3] = {+INFINITY, +INFINITY, +INFINITY};
  float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  void grow(const float *p)
  {
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], p[a]);
      hi[a] = std::max(hi[a], p[a]);
    }
  }
  void grow(const Box &b)
  {
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], b.lo[a]);
      hi[a] = std::max(hi[a], b.hi[a]);
    }
  }
  double area() const
  {
    if (!(hi[0] >= lo[0]))
      return 0.0;
    const double dx = double(hi[0]) - lo[0], dy = double(hi[1]) - lo[1], dz = double(hi[2]) - lo[2];
    return 2.0 * (dx * dy + dy * dz + dz * dx);
  }
};

struct Ref {
  Box b;
  float c[3];
  uint32_t id;
};

struct Node2 {
  Box b;
  int32_t left{-1}, right{-1};
  uint32_t first{0}, count{0}; // leaf when count > 0
};

struct Builder2 {
  std::vector<Ref> refs;
  std::vector<Node2> nodes;
  std::atomic<uint32_t> next{0};
  int max_leaf{3};
  static constexpr int BINS = 32;

  uint32_t alloc2()
  {
    const uint32_t i = next.fetch_add(2);
    if (i + 2 > nodes.size())
      throw std::runtime_error("bvh2 node pool exhausted");
    return i;
  }

  void make_leaf(uint32_t ni, uint32_t begin, uint32_t end)
  {
    nodes[ni].first = begin;
    nodes[ni].count = end - begin;
  }

  void build(uint32_t ni, uint32_t begin, uint32_t end, int depth)
  {
    Box b, cb;
    for (uint32_t i = begin; i < end; ++i) {
      b.grow(refs[i].b);
      cb.grow(refs[i].c);
    }
    nodes[ni].b = b;
    const uint32_t n = end - begin;
    if (n <= 1) {
      make_leaf(ni, begin, end);
      return;
    }
    // binned SAH over all three axes
    int best_axis = -1, best_split = -1;
    double best_cost = INFINITY;
    const double parent_area = b.area();
    for (int a = 0; a < 3; ++a) {
      const float ext = cb.hi[a] - cb.lo[a];
      if (!(ext > 0.f))
        continue;
      const float k = float(BINS) * (1.f - 1e-6f) / ext;
      Box bb[BINS];
      uint32_t bc[BINS] = {};
      for (uint32_t i = begin; i < end; ++i) {
        int bi = int((refs[i].c[a] - cb.lo[a]) * k);
        bi = std::min(std::max(bi, 0), BINS - 1);
        bb[bi].grow(refs[i].b);
        bc[bi]++;
      }
      double ra[BINS];
      uint32_t rn[BINS];
      Box acc;
      uint32_t cnt = 0;
      for (int i = BINS - 1; i > 0; --i) {
        acc.grow(bb[i]);
        cnt += bc[i];
        ra[i] = acc.area();
        rn[i] = cnt;
      }
      acc = Box{};
      cnt = 0;
      for (int i = 0; i < BINS - 1; ++i) {
        acc.grow(bb[i]);
        cnt += bc[i];
        if (cnt == 0 || rn[i + 1] == 0)
          continue;
        const double cost = acc.area() * cnt + ra[i + 1] * rn[i + 1];
        if (cost < best_cost) {
          best_cost = cost;
          best_axis = a;
          best_split = i;
        }
      }
    }
    // cost units: one triangle test = 1, one node traversal = 1
    const double leaf_cost = double(n);
    const double split_cost = parent_area > 0.0 ? 1.0 + best_cost / parent_area : INFINITY;
    if (n <= uint32_t(max_leaf) && (best_axis < 0 || leaf_cost <= split_cost)) {
      make_leaf(ni, begin, end);
      return;
    }
    uint32_t mid;
    if (best_axis < 0 || depth > 60) {
      mid = begin + n / 2; // identical centroids: split by index
    } else {
      const float ext = cb.hi[best_axis] - cb.lo[best_axis];
      const float k = float(BINS) * (1.f - 1e-6f) / ext;
      auto it = std::partition(refs.begin() + begin, refs.begin() + end, [&](const Ref &r) {
        int bi = int((r.c[best_axis] - cb.lo[best_axis]) * k);
        bi = std::min(std::max(bi, 0), BINS - 1);
        return bi <= best_split;
      });
      mid = uint32_t(it - refs.begin());
      if (mid == begin || mid == end)
        mid = begin + n / 2;
    }
    const uint32_t c = alloc2();
    nodes[ni].left = int32_t(c);
    nodes[ni].right = int32_t(c + 1);
    if (n > 8192) {
#pragma omp task default(shared) firstprivate(c, begin, mid, depth)
      build(c, begin, mid, depth + 1);
#pragma omp task default(shared) firstprivate(c, mid, end, depth)
      build(c + 1, mid, end, depth + 1);
#pragma omp taskwait
    } else {
      build(c, begin, mid, depth + 1);
      build(c + 1, mid, end, depth + 1);
    }
  }
};

// Greedy octant assignment: slot s should hold the child that comes first
// along the sign octant direction d(s) (bit 2: x < 0, bit 1: y < 0, bit 0: z < 0).
void assign_slots(const std::vector<int32_t> &children, const std::vector<Node2> &n2, const Box &parent,
    int32_t slot_of_child[8])
{
  const size_t k = children.size();
  float pc[3];
  for (int a = 0; a < 3; ++a)
    pc[a] = 0.5f * (parent.lo[a] + parent.hi[a]);
  float cost[8][8];
  for (size_t c = 0; c < k; ++c) {
    const Box &b = n2[size_t(children[c])].b;
    float cc[3];
    for (int a = 0; a < 3; ++a)
      cc[a] = 0.5f * (b.lo[a] + b.hi[a]) - pc[a];
    for (int s = 0; s < 8; ++s) {
      const float dx = (s & 4) ? -1.f : 1.f, dy = (s & 2) ? -1.f : 1.f, dz = (s & 1) ? -1.f : 1.f;
      cost[c][s] = cc[0] * dx + cc[1] * dy + cc[2] * dz;
    }
  }
  bool used_c[8] = {}, used_s[8] = {};
  for (size_t it = 0; it < k; ++it) {
    float best = INFINITY;
    int bc = -1, bs = -1;
    for (size_t c = 0; c < k; ++c) {
      if (used_c[c])
        continue;
      for (int s = 0; s < 8; ++s) {
        if (used_s[s])
          continue;
        if (cost[c][s] < best || bc < 0) {
          best = cost[c][s];
          bc = int(c);
          bs = s;
        }
      }
    }
    used_c[bc] = true;
    used_s[bs] = true;
    slot_of_child[bc] = bs;
  }
}

struct Collapse {
  const std::vector<Node2> &n2;
  const std::vector<Ref> &refs;
  const float *pos;
  const uint32_t *idx;
  Bvh8Host &out;
  double sah{0.0};
  double root_area{1.0};

  uint32_t alloc_nodes(uint32_t k)
  {
    const uint32_t first = out.node_count;
    out.node_count += k;
    out.nodes.resize(size_t(out.node_count) * 20, 0u);
    return first;
  }

  void emit_tri(uint32_t prim)
  {
    if (!pos) { // box primitives: the leaf lists primitive ids
      out.leaf_prims.push_back(prim);
      out.tri_count++;
      return;
    }
    const float *v0 = &pos[3 * size_t(idx[3 * size_t(prim) + 0])];
    const float *v1 = &pos[3 * size_t(idx[3 * size_t(prim) + 1])];
    const float *v2 = &pos[3 * size_t(idx[3 * size_t(prim) + 2])];
    float rec[12];
    rec[0] = v0[0];
    rec[1] = v0[1];
    rec[2] = v0[2];
    std::memcpy(&rec[3], &prim, 4);
    // e1 = v1 - v0 and e2 = v2 - v0, one float subtraction each
    rec[4] = v1[0] - v0[0];
    rec[5] = v1[1] - v0[1];
    rec[6] = v1[2] - v0[2];
    rec[7] = 0.f;
    rec[8] = v2[0] - v0[0];
    rec[9] = v2[1] - v0[1];
    rec[10] = v2[2] - v0[2];
    rec[11] = 0.f;
    out.tris.insert(out.tris.end(), rec, rec + 12);
    out.tri_count++;
  }

  // Fills BVH8 node `ni` from BVH2 node `root2` (children gathered by SAH area).
  void fill(uint32_t ni, int32_t root2, uint32_t depth)
  {
    out.max_depth = std::max(out.max_depth, depth);
    std::vector<int32_t> ch;
    const Node2 &r = n2[size_t(root2)];
    if (r.count > 0)
      ch.push_back(root2); // a leaf root: one leaf child
    else {
      ch.push_back(r.left);
      ch.push_back(r.right);
    }
    while (ch.size() < 8) {
      int best = -1;
      double best_area = -1.0;
      for (size_t i = 0; i < ch.size(); ++i) {
        const Node2 &c = n2[size_t(ch[i])];
        if (c.count > 0)
          continue;
        const double a = c.b.area();
        if (a > best_area) {
          best_area = a;
          best = int(i);
        }
      }
      if (best < 0)
        break;
      const Node2 &c = n2[size_t(ch[size_t(best)])];
      ch[size_t(best)] = c.left;
      ch.push_back(c.right);
    }
    Box nb;
    for (int32_t c : ch)
      nb.grow(n2[size_t(c)].b);
    sah += nb.area() / root_area;
    int32_t slot_of[8];
    assign_slots(ch, n2, nb, slot_of);
    int32_t child_at[8];
    for (int s = 0; s < 8; ++s)
      child_at[s] = -1;
    for (size_t i = 0; i < ch.size(); ++i)
      child_at[slot_of[i]] = ch[i];

    // quantisation grid
    float p[3];
    uint8_t e[3];
    double scale[3];
    for (int a = 0; a < 3; ++a) {
      p[a] = nb.lo[a];
      const double ext = double(nb.hi[a]) - double(nb.lo[a]);
      int ex = -127;
      if (ext > 0.0) {
        ex = int(std::ceil(std::log2(ext / 255.0)));
        while (std::ldexp(255.0, ex) < ext)
          ++ex;
      }
      ex = std::min(std::max(ex, -127), 127);
      e[a] = uint8_t(ex + 127);
      scale[a] = ex == -127 ? 0.0 : std::ldexp(1.0, ex);
    }
    uint32_t internal_count = 0, tri_total = 0;
    uint8_t imask = 0;
    for (int s = 0; s < 8; ++s) {
      if (child_at[s] < 0)
        continue;
      const Node2 &c = n2[size_t(child_at[s])];
      if (c.count == 0) {
        imask |= uint8_t(1u << s);
        internal_count++;
      } else {
        tri_total += c.count;
      }
    }
    const uint32_t child_base = internal_count ? alloc_nodes(internal_count) : 0u;
    const uint32_t tri_base = out.tri_count;
    uint8_t meta[8] = {}, q[6][8] = {};
    uint32_t tri_off = 0;
    std::vector<std::pair<uint32_t, int32_t>> recurse;
    uint32_t next_child = child_base;
    for (int s = 0; s < 8; ++s) {
      if (child_at[s] < 0)
        continue;
      const Node2 &c = n2[size_t(child_at[s])];
      for (int a = 0; a < 3; ++a) {
        double lo = 0.0, hi = 0.0;
        if (scale[a] > 0.0) {
          lo = std::floor((double(c.b.lo[a]) - double(p[a])) / scale[a]);
          hi = std::ceil((double(c.b.hi[a]) - double(p[a])) / scale[a]);
        }
        q[a][s] = uint8_t(std::min(std::max(lo, 0.0), 255.0));
        q[3 + a][s] = uint8_t(std::min(std::max(hi, 0.0), 255.0));
      }
      if (c.count == 0) {
        meta[s] = 0x80;
        recurse.emplace_back(next_child++, child_at[s]);
      } else {
        meta[s] = uint8_t((c.count << 5) | tri_off);
        for (uint32_t t = 0; t < c.count; ++t)
          emit_tri(refs[c.first + t].id);
        tri_off += c.count;
      }
    }
    (void)tri_total;
    uint32_t *w = &out.nodes[size_t(ni) * 20];
    std::memcpy(&w[0], &p[0], 4);
    std::memcpy(&w[1], &p[1], 4);
    std::memcpy(&w[2], &p[2], 4);
    w[3] = uint32_t(e[0]) | (uint32_t(e[1]) << 8) | (uint32_t(e[2]) << 16) | (uint32_t(imask) << 24);
    w[4] = child_base;
    w[5] = tri_base;
    std::memcpy(&w[6], meta, 8);
    std::memcpy(&w[8], q, 48); // qlo_x, qlo_y, qlo_z, qhi_x, qhi_y, qhi_z
    for (auto &rc : recurse)
      fill(rc.first, rc.second, depth + 1);
  }
};

} // namespace

namespace {

// SAH BVH2 over the references, collapsed into `out`; triangle records when
// positions is set, leaf primitive ids otherwise.
void build_from_refs(Builder2 &b, const float *positions, const uint32_t *indices, Bvh8Host &out)
{
  const uint32_t n = uint32_t(b.refs.size());
  b.nodes.resize(size_t(n) * 2 + 2);
  b.next = 1;
#pragma omp parallel
#pragma omp single
  b.build(0, 0, n, 0);
  b.nodes.resize(b.next.load());

  Collapse c{b.nodes, b.refs, positions, indices, out};
  c.root_area = std::max(b.nodes[0].b.area(), 1e-30);
  if (positions)
    out.tris.reserve(size_t(n) * 12);
  const uint32_t root = c.alloc_nodes(1);
  c.fill(root, 0, 1);
  out.sah_cost = c.sah;
}

} // namespace

void build_bvh8(const float *positions, uint64_t vertex_count, const uint32_t *indices, uint64_t triangle_count,
    Bvh8Host &out, int max_leaf)
{
  (void)vertex_count;
  out = Bvh8Host{};
  if (triangle_count == 0)
    throw std::runtime_error("build_bvh8: no triangles");
  if (triangle_count > 0x7fffffffull)
    throw std::runtime_error("build_bvh8: too many triangles");
  Builder2 b;
  b.max_leaf = std::min(std::max(max_leaf, 1), 3);
  const uint32_t n = uint32_t(triangle_count);
  b.refs.resize(n);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < int64_t(n); ++i) {
    Ref &r = b.refs[size_t(i)];
    r.b = Box{};
    for (int k = 0; k < 3; ++k)
      r.b.grow(&positions[3 * size_t(indices[3 * size_t(i) + k])]);
    for (int a = 0; a < 3; ++a)
      r.c[a] = 0.5f * (r.b.lo[a] + r.b.hi[a]);
    r.id = uint32_t(i);
  }
  build_from_refs(b, positions, indices, out);
}

void build_bvh8_boxes(const float *boxes, uint64_t count, Bvh8Host &out, int max_leaf)
{
  out = Bvh8Host{};
  if (count == 0)
    throw std::runtime_error("build_bvh8_boxes: no boxes");
  if (count > 0x7fffffffull)
    throw std::runtime_error("build_bvh8_boxes: too many boxes");
  Builder2 b;
  b.max_leaf = std::min(std::max(max_leaf, 1), 3);
  b.refs.resize(size_t(count));
  for (size_t i = 0; i < count; ++i) {
    Ref &r = b.refs[i];
    r.b = Box{};
    r.b.grow(&boxes[6 * i]);
    r.b.grow(&boxes[6 * i + 3]);
    for (int a = 0; a < 3; ++a)
      r.c[a] = 0.5f * (r.b.lo[a] + r.b.hi[a]);
    r.id = uint32_t(i);
  }
  build_from_refs(b, nullptr, nullptr, out);
}

void build_prim_records(const float *positions, const uint32_t *indices, uint64_t triangle_count, float *prim_geo)
{
#pragma omp parallel for schedule(static)
  for (int64_t t = 0; t < int64_t(triangle_count); ++t) {
    const float *v0 = &positions[3 * size_t(indices[3 * size_t(t) + 0])];
    const float *v1 = &positions[3 * size_t(indices[3 * size_t(t) + 1])];
    const float *v2 = &positions[3 * size_t(indices[3 * size_t(t) + 2])];
    float *r = &prim_geo[size_t(t) * 12];
    r[0] = v0[0];
    r[1] = v0[1];
    r[2] = v0[2];
    const uint32_t id = uint32_t(t);
    std::memcpy(&r[3], &id, 4);
    r[4] = v1[0] - v0[0];
    r[5] = v1[1] - v0[1];
    r[6] = v1[2] - v0[2];
    r[7] = 0.f;
    r[8] = v2[0] - v0[0];
    r[9] = v2[1] - v0[1];
    r[10] = v2[2] - v0[2];
    r[11] = 0.f;
  }
}

} // namespace phc
