// Host test of the GPU BVH build's surface-area collapse program
// (photon_gb300/csrc/bvh_collapse.cuh, the code the build's kernels run):
// random binary trees in the build's layout, the program bottom-up, the wide
// tree it chooses expanded from the root and checked (every wide node has
// 2..8 children, leaf children hold at most max_leaf primitives, every
// primitive is in exactly one leaf child, the tree's cost recomputed from its
// nodes equals the program's), and on small trees the program's cost against
// the least cost over every cover enumerated explicitly.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <functional>
#include <random>
#include <vector>

#include "bvh_collapse.cuh"

using namespace phc;

namespace {

struct Tree {
  uint32_t n = 0;
  std::vector<float> nbox;
  std::vector<int2> nchild;
  std::vector<uint32_t> iter_base; // inner nodes made per merge round: [base[i], base[i + 1])
  int root = 0;
};

// n random triangle-sized boxes, then rounds that merge random neighbouring
// clusters (children always made before their parents, as the clustering does)
Tree make_tree(uint32_t n, unsigned seed)
{
  std::mt19937 g(seed);
  std::uniform_real_distribution<float> U(-1.f, 1.f), S(0.001f, 0.3f);
  Tree t;
  t.n = n;
  t.nbox.resize(6 * size_t(2 * n - 1));
  t.nchild.resize(2 * n - 1);
  std::vector<float> cx(n);
  for (uint32_t i = 0; i < n; ++i)
    cx[i] = U(g) * 10.f;
  std::sort(cx.begin(), cx.end());
  for (uint32_t i = 0; i < n; ++i) {
    const float c[3] = {cx[i], U(g) * 10.f, U(g) * 10.f};
    for (int a = 0; a < 3; ++a) {
      const float h = S(g);
      t.nbox[6 * size_t(i) + a] = c[a] - h;
      t.nbox[6 * size_t(i) + 3 + a] = c[a] + h;
    }
    t.nchild[i] = make_int2(-1, int(i));
  }
  std::vector<int> cl(n);
  for (uint32_t i = 0; i < n; ++i)
    cl[i] = int(i);
  uint32_t next = n;
  t.iter_base.push_back(n);
  while (cl.size() > 1) {
    std::vector<int> nc;
    size_t i = 0;
    while (i < cl.size()) {
      if (i + 1 < cl.size() && g() % 3 != 0) {
        const int a = cl[i], b = cl[i + 1], v = int(next++);
        for (int k = 0; k < 3; ++k) {
          t.nbox[6 * size_t(v) + k] = std::min(t.nbox[6 * size_t(a) + k], t.nbox[6 * size_t(b) + k]);
          t.nbox[6 * size_t(v) + 3 + k] = std::max(t.nbox[6 * size_t(a) + 3 + k], t.nbox[6 * size_t(b) + 3 + k]);
        }
        t.nchild[v] = make_int2(a, b);
        nc.push_back(v);
        i += 2;
      } else {
        nc.push_back(cl[i++]);
      }
    }
    if (nc.size() < cl.size())
      t.iter_base.push_back(next);
    cl.swap(nc);
  }
  t.root = cl[0];
  return t;
}

void leaves_of(const Tree &t, int u, std::vector<int> &out)
{
  if (uint32_t(u) < t.n) {
    out.push_back(t.nchild[u].y);
    return;
  }
  leaves_of(t, t.nchild[u].x, out);
  leaves_of(t, t.nchild[u].y, out);
}

double area_d(const Tree &t, int v) { return double(dp_area(t.nbox.data(), uint32_t(v))); }

// least cost of w as one slot (leaf child or wide inner node) and of binary
// inner node v as a wide node, over every cover of its two subtrees by at
// most 8 slots, each cover written out explicitly
struct Brute {
  const Tree &t;
  int max_leaf;
  double ct;
  std::vector<double> inner_memo;
  explicit Brute(const Tree &tr, int ml, double c) : t(tr), max_leaf(ml), ct(c), inner_memo(tr.nchild.size(), -1.0) {}
  void covers(int u, std::vector<std::vector<int>> &out)
  {
    out.push_back({u});
    if (uint32_t(u) < t.n)
      return;
    std::vector<std::vector<int>> a, b;
    covers(t.nchild[u].x, a);
    covers(t.nchild[u].y, b);
    for (const auto &x : a)
      for (const auto &y : b)
        if (x.size() + y.size() <= 8) {
          std::vector<int> z = x;
          z.insert(z.end(), y.begin(), y.end());
          out.push_back(z);
        }
  }
  double slot(int w)
  {
    std::vector<int> p;
    leaves_of(t, w, p);
    double best = 1e300;
    if (int(p.size()) <= max_leaf || uint32_t(w) < t.n)
      best = area_d(t, w) * double(p.size()) * ct;
    if (uint32_t(w) >= t.n)
      best = std::min(best, inner(w));
    return best;
  }
  double inner(int v)
  {
    if (inner_memo[v] >= 0.0)
      return inner_memo[v];
    std::vector<std::vector<int>> a, b;
    covers(t.nchild[v].x, a);
    covers(t.nchild[v].y, b);
    double best = 1e300;
    for (const auto &x : a)
      for (const auto &y : b) {
        if (x.size() + y.size() > 8)
          continue;
        double s = 0.0;
        for (int w : x)
          s += slot(w);
        for (int w : y)
          s += slot(w);
        best = std::min(best, s);
      }
    return inner_memo[v] = area_d(t, v) + best;
  }
};

} // namespace

// 0 when every check passes, else a negative code: -1 inconsistent choices,
// -2 a wide node with fewer than 2 or more than 8 children, -3 a leaf child
// over max_leaf primitives or not matching its subtree, -4 primitives not in
// exactly one leaf child, -5 the recomputed cost differs from the program's,
// -6 the program's cost differs from the enumeration's.
// out: [0] program's cost of the root as a wide node, [1] the same recomputed
// from the wide tree, [2] wide nodes, [3] enumeration's cost (n <= 12, else
// -1), [4] leaf children.
extern "C" int ct_check(uint32_t n, unsigned seed, int max_leaf, float ct, double *out)
{
  if (n < 4 || max_leaf < 1 || max_leaf > 3)
    return -100;
  const Tree t = make_tree(n, seed);
  const uint32_t inner = n - 1;
  std::vector<float> cost(size_t(inner) * 8);
  std::vector<uint8_t> split(size_t(inner) * 8);
  std::vector<uchar4> info(inner);
  const CollapseDp d{cost.data(), split.data(), info.data()};
  for (size_t i = 0; i + 1 < t.iter_base.size(); ++i)
    for (uint32_t v = t.iter_base[i]; v < t.iter_base[i + 1]; ++v)
      collapse_dp_node(d, t.nbox.data(), t.nchild.data(), n, v, ct, max_leaf);
  // expand the wide tree from the root
  std::vector<int> seen(n, 0), queue{t.root};
  double total = 0.0;
  int nodes = 0, leaf_children = 0;
  while (!queue.empty()) {
    const int v = queue.back();
    queue.pop_back();
    ++nodes;
    total += area_d(t, v);
    int ch[8], lc[8];
    const int k = sah_children(t.nchild.data(), split.data(), info.data(), n, v, ch, lc);
    if (k < 0)
      return -1;
    if (k < 2 || k > 8)
      return -2;
    for (int i = 0; i < k; ++i) {
      if (lc[i] == 0) {
        if (uint32_t(ch[i]) < n)
          return -3;
        queue.push_back(ch[i]);
        continue;
      }
      std::vector<int> p;
      leaves_of(t, ch[i], p);
      if (int(p.size()) != lc[i] || (lc[i] > max_leaf && uint32_t(ch[i]) >= n))
        return -3;
      for (int q : p)
        ++seen[q];
      total += area_d(t, ch[i]) * double(lc[i]) * double(ct);
      ++leaf_children;
    }
  }
  for (uint32_t i = 0; i < n; ++i)
    if (seen[i] != 1)
      return -4;
  const double prog = double(cost[8 * size_t(uint32_t(t.root) - n)]);
  out[0] = prog;
  out[1] = total;
  out[2] = nodes;
  out[4] = leaf_children;
  if (std::fabs(total - prog) > 1e-5 * std::max(1.0, prog))
    return -5;
  out[3] = -1.0;
  if (n <= 12) {
    Brute b(t, max_leaf, double(ct));
    out[3] = b.inner(t.root);
    if (std::fabs(out[3] - prog) > 1e-5 * std::max(1.0, prog))
      return -6;
  }
  return 0;
}
