// Minimal host-only stand-in for the parts of the Kokkos 5 API that Photon's
// path-tracing sources use, so that those sources compile unmodified with g++
// into the CPU oracle (oracle/_ref).  This is test infrastructure written for
// this project: it is not Kokkos and carries none of its code.
//
// Semantics kept from Kokkos where the reference depends on them:
//  * View<T*> / View<T**> allocate value-initialised storage and share it on
//    copy (reference counted); extent(r), data(), operator() as in Kokkos.
//  * Every view lives in host memory, so create_mirror_view(v) and
//    create_mirror_view_and_copy(HostSpace, v) return v itself (Kokkos does the
//    same for host-accessible views) and deep_copy between equal views is a
//    no-op.
//  * parallel_for / parallel_reduce run the functor over the index range with
//    OpenMP (static schedule, like Kokkos' OpenMP back-end); reductions are sums.
//  * Math functions forward to <cmath> float/double overloads.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <algorithm>

#ifdef _OPENMP
#include <omp.h>
#endif

#define KOKKOS_FUNCTION
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FORCEINLINE_FUNCTION inline
#define KOKKOS_LAMBDA [=]
#define KOKKOS_CLASS_LAMBDA [ =, *this ]
#define KOKKOS_ENABLE_OPENMP_SHIM 1

namespace Kokkos {

struct HostSpace {};
struct LayoutRight {};
struct LayoutLeft {};
struct OpenMP {
  static const char *name() { return "OpenMP"; }
  int concurrency() const
  {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
  }
};
using DefaultExecutionSpace = OpenMP;
using DefaultHostExecutionSpace = OpenMP;

namespace impl {
template <class T> struct view_rank { using value_type = T; static constexpr int rank = 0; };
template <class T> struct view_rank<T *> {
  using value_type = typename view_rank<T>::value_type;
  static constexpr int rank = view_rank<T>::rank + 1;
};
inline bool &initialized_flag() { static bool f = false; return f; }
inline bool &finalized_flag() { static bool f = false; return f; }
} // namespace impl

template <class DataType, class... Props>
class View
{
public:
  using value_type = typename impl::view_rank<DataType>::value_type;
  static constexpr int rank = impl::view_rank<DataType>::rank;
  static_assert(rank >= 1 && rank <= 3, "shim supports rank 1..3 views");

  View() = default;

  explicit View(const std::string &label, size_t n0 = 0, size_t n1 = 0, size_t n2 = 0) : m_label(label)
  {
    m_ext[0] = n0;
    m_ext[1] = rank > 1 ? n1 : 1;
    m_ext[2] = rank > 2 ? n2 : 1;
    const size_t n = size();
    if (n > 0) {
      m_owner = std::shared_ptr<value_type>(new value_type[n](), std::default_delete<value_type[]>());
      m_data = m_owner.get();
    }
  }

  // Unmanaged/sub view over existing storage (used by subview()).
  View(std::shared_ptr<value_type> owner, value_type *data, size_t n0, size_t n1 = 1, size_t n2 = 1)
      : m_owner(std::move(owner)), m_data(data)
  {
    m_ext[0] = n0;
    m_ext[1] = n1;
    m_ext[2] = n2;
  }

  size_t extent(int r) const { return r < 3 ? (r < rank ? m_ext[r] : 1) : 1; }
  int extent_int(int r) const { return int(extent(r)); }
  size_t size() const { return m_ext[0] * (rank > 1 ? m_ext[1] : 1) * (rank > 2 ? m_ext[2] : 1); }
  size_t span() const { return size(); }
  value_type *data() const { return m_data; }
  const std::string &label() const { return m_label; }
  bool is_allocated() const { return m_data != nullptr; }
  const std::shared_ptr<value_type> &owner() const { return m_owner; }

  template <class I> value_type &operator()(I i) const { return m_data[size_t(i)]; }
  template <class I, class J> value_type &operator()(I i, J j) const { return m_data[size_t(i) * m_ext[1] + size_t(j)]; }
  template <class I, class J, class K> value_type &operator()(I i, J j, K k) const
  {
    return m_data[(size_t(i) * m_ext[1] + size_t(j)) * m_ext[2] + size_t(k)];
  }
  template <class I> value_type &operator[](I i) const { return m_data[size_t(i)]; }

private:
  std::shared_ptr<value_type> m_owner;
  value_type *m_data{nullptr};
  size_t m_ext[3]{0, 1, 1};
  std::string m_label;
};

template <class V> V create_mirror_view(const V &v) { return v; }
template <class V> V create_mirror_view(const HostSpace &, const V &v) { return v; }
template <class V> V create_mirror_view_and_copy(const HostSpace &, const V &v) { return v; }
template <class V> V create_mirror(const V &v)
{
  V out(v.label(), v.extent(0), v.extent(1), v.extent(2));
  if (v.size())
    std::copy(v.data(), v.data() + v.size(), out.data());
  return out;
}

template <class D1, class... P1, class D2, class... P2>
void deep_copy(const View<D1, P1...> &dst, const View<D2, P2...> &src)
{
  if (dst.data() == src.data())
    return;
  const size_t n = dst.size() < src.size() ? dst.size() : src.size();
  for (size_t i = 0; i < n; ++i)
    dst.data()[i] = src.data()[i];
}

template <class D, class... P>
void deep_copy(const View<D, P...> &dst, const typename View<D, P...>::value_type &value)
{
  for (size_t i = 0; i < dst.size(); ++i)
    dst.data()[i] = value;
}

template <class D, class... P, class I>
View<D, P...> subview(const View<D, P...> &v, const std::pair<I, I> &range)
{
  static_assert(View<D, P...>::rank == 1, "shim subview: rank 1 only");
  const size_t b = size_t(range.first), e = size_t(range.second);
  return View<D, P...>(v.owner(), v.data() + b, e - b);
}

// ---- execution policies ---------------------------------------------------

template <class... Args>
struct RangePolicy
{
  int64_t begin{0};
  int64_t end{0};
  RangePolicy() = default;
  RangePolicy(int64_t b, int64_t e) : begin(b), end(e) {}
};

template <unsigned N> struct Rank { static constexpr unsigned rank = N; };

template <class R, class... Args>
struct MDRangePolicy
{
  int64_t lo[2]{0, 0};
  int64_t hi[2]{0, 0};
  MDRangePolicy(std::initializer_list<int64_t> l, std::initializer_list<int64_t> h)
  {
    int k = 0;
    for (auto v : l) lo[k++] = v;
    k = 0;
    for (auto v : h) hi[k++] = v;
  }
};

template <class F, class... A>
void parallel_for(const std::string &, const RangePolicy<A...> &p, const F &f)
{
  const int64_t b = p.begin, e = p.end;
#pragma omp parallel for schedule(static)
  for (int64_t i = b; i < e; ++i)
    f(int(i));
}

template <class F, class Int, typename std::enable_if<std::is_integral<Int>::value, int>::type = 0>
void parallel_for(const std::string &label, Int n, const F &f)
{
  parallel_for(label, RangePolicy<>(0, int64_t(n)), f);
}

template <class F, class R, class... A>
void parallel_for(const std::string &, const MDRangePolicy<R, A...> &p, const F &f)
{
  const int64_t y0 = p.lo[0], y1 = p.hi[0], x0 = p.lo[1], x1 = p.hi[1];
#pragma omp parallel for schedule(static)
  for (int64_t y = y0; y < y1; ++y)
    for (int64_t x = x0; x < x1; ++x)
      f(int(y), int(x));
}

template <class F, class T, class... A>
void parallel_reduce(const std::string &, const RangePolicy<A...> &p, const F &f, T &result)
{
  T total{};
  const int64_t b = p.begin, e = p.end;
#pragma omp parallel
  {
    T local{};
#pragma omp for schedule(static)
    for (int64_t i = b; i < e; ++i)
      f(int(i), local);
#pragma omp critical
    total += local;
  }
  result = total;
}

template <class F, class T, class Int, typename std::enable_if<std::is_integral<Int>::value, int>::type = 0>
void parallel_reduce(const std::string &label, Int n, const F &f, T &result)
{
  parallel_reduce(label, RangePolicy<>(0, int64_t(n)), f, result);
}

inline void fence() {}
inline void fence(const std::string &) {}

// ---- initialisation -------------------------------------------------------

class InitializationSettings
{
public:
  InitializationSettings &set_disable_warnings(bool) { return *this; }
  InitializationSettings &set_num_threads(int n)
  {
    m_threads = n;
    return *this;
  }
  int num_threads() const { return m_threads; }

private:
  int m_threads{0};
};

inline void initialize(const InitializationSettings &s = InitializationSettings())
{
#ifdef _OPENMP
  if (s.num_threads() > 0)
    omp_set_num_threads(s.num_threads());
#else
  (void)s;
#endif
  impl::initialized_flag() = true;
}
inline void initialize(int &, char **) { initialize(); }
inline void finalize()
{
  impl::finalized_flag() = true;
  impl::initialized_flag() = false;
}
inline bool is_initialized() { return impl::initialized_flag(); }
inline bool is_finalized() { return impl::finalized_flag(); }

// ---- math -----------------------------------------------------------------

inline float fmax(float a, float b) { return std::fmax(a, b); }
inline double fmax(double a, double b) { return std::fmax(a, b); }
inline float fmin(float a, float b) { return std::fmin(a, b); }
inline double fmin(double a, double b) { return std::fmin(a, b); }
inline float fabs(float a) { return std::fabs(a); }
inline double fabs(double a) { return std::fabs(a); }
inline float abs(float a) { return std::fabs(a); }
inline float sqrt(float a) { return std::sqrt(a); }
inline double sqrt(double a) { return std::sqrt(a); }
inline float floor(float a) { return std::floor(a); }
inline double floor(double a) { return std::floor(a); }
inline float ceil(float a) { return std::ceil(a); }
inline float sin(float a) { return std::sin(a); }
inline double sin(double a) { return std::sin(a); }
inline float cos(float a) { return std::cos(a); }
inline double cos(double a) { return std::cos(a); }
inline float tan(float a) { return std::tan(a); }
inline double tan(double a) { return std::tan(a); }
inline float pow(float a, float b) { return std::pow(a, b); }
inline double pow(double a, double b) { return std::pow(a, b); }
inline float log(float a) { return std::log(a); }
inline double log(double a) { return std::log(a); }
inline float exp(float a) { return std::exp(a); }
inline float acos(float a) { return std::acos(a); }
inline double acos(double a) { return std::acos(a); }
inline float atan(float a) { return std::atan(a); }
inline float atan2(float a, float b) { return std::atan2(a, b); }
inline double atan2(double a, double b) { return std::atan2(a, b); }
inline bool isfinite(float a) { return std::isfinite(a); }
inline bool isnan(float a) { return std::isnan(a); }
template <class T> inline T clamp(const T &x, const T &lo, const T &hi) { return x < lo ? lo : (hi < x ? hi : x); }
template <class T> inline T max(const T &a, const T &b) { return a < b ? b : a; }
template <class T> inline T min(const T &a, const T &b) { return b < a ? b : a; }

} // namespace Kokkos
