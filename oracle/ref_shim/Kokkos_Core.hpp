// Minimal Kokkos-API shim, written for this project, so that the reference's
// own header-only FMM (src/tree.hpp, traverse.hpp, multipoleKernels.hpp,
// complexify.hpp, arrayReduction.hpp, fmmCalculator.hpp) compiles on the host
// with g++ and no Kokkos installation.  It is test infrastructure only: the
// compiled reference is used to make golden fixtures and to check the oracle
// restatement.  It covers exactly the API surface those headers use.
//
// Backends: serial (bitwise reproducible, used for fixtures) or OpenMP when
// compiled with -fopenmp (parallel_for over ranges/leagues, atomics through
// `#pragma omp atomic`).
#pragma once
#include <algorithm>
#include <cassert>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]

#include "Kokkos_Pair.hpp"
#include "Kokkos_MathematicalConstants.hpp"
#include "Kokkos_NumericTraits.hpp"

namespace Kokkos {

// ---------------------------------------------------------------- spaces
struct HostSpaceExec {};
using DefaultExecutionSpace     = HostSpaceExec;
using DefaultHostExecutionSpace = HostSpaceExec;
struct MemoryUnmanaged {};
struct WithoutInitializing_t {};
static constexpr WithoutInitializing_t WithoutInitializing{};
struct AUTO_t {};
static constexpr AUTO_t AUTO{};

inline void fence() {}
inline void fence(const std::string &) {}

struct ScopeGuard {
  ScopeGuard(int &, char **) {}
  ScopeGuard() {}
};

namespace Profiling {
inline void pushRegion(const std::string &) {}
inline void popRegion() {}
} // namespace Profiling

// ---------------------------------------------------------------- complex
template <class T>
class complex {
  T re_, im_;

public:
  using value_type = T;
  complex() : re_(0), im_(0) {}
  complex(const T &r) : re_(r), im_(0) {}
  complex(const T &r, const T &i) : re_(r), im_(i) {}
  template <class U>
  complex(const complex<U> &o) : re_(T(o.real())), im_(T(o.imag())) {}
  T    real() const { return re_; }
  T    imag() const { return im_; }
  void real(const T &v) { re_ = v; }
  void imag(const T &v) { im_ = v; }
  T   &re_ref() { return re_; }
  T   &im_ref() { return im_; }

  complex &operator+=(const complex &o)
  {
    re_ += o.re_;
    im_ += o.im_;
    return *this;
  }
  complex &operator-=(const complex &o)
  {
    re_ -= o.re_;
    im_ -= o.im_;
    return *this;
  }
  complex &operator*=(const complex &o)
  {
    const T r = re_ * o.re_ - im_ * o.im_;
    const T i = re_ * o.im_ + im_ * o.re_;
    re_       = r;
    im_       = i;
    return *this;
  }
  complex &operator/=(const complex &o)
  {
    *this = *this / o;
    return *this;
  }
  complex &operator+=(const T &v)
  {
    re_ += v;
    return *this;
  }
  complex &operator-=(const T &v)
  {
    re_ -= v;
    return *this;
  }
  complex &operator*=(const T &v)
  {
    re_ *= v;
    im_ *= v;
    return *this;
  }
  complex &operator/=(const T &v)
  {
    re_ /= v;
    im_ /= v;
    return *this;
  }
  friend complex operator/(const complex &a, const complex &b)
  {
    // Smith's algorithm (scaled division), as Kokkos::complex does.
    const T s = std::fabs(b.real()) + std::fabs(b.imag());
    const T ars = a.real() / s, ais = a.imag() / s;
    const T brs = b.real() / s, bis = b.imag() / s;
    const T d   = brs * brs + bis * bis;
    return complex((ars * brs + ais * bis) / d, (ais * brs - ars * bis) / d);
  }
};

template <class T> inline T real(const complex<T> &z) { return z.real(); }
template <class T> inline T imag(const complex<T> &z) { return z.imag(); }
template <class T> inline complex<T> conj(const complex<T> &z) { return complex<T>(z.real(), -z.imag()); }

template <class T> inline complex<T> operator+(const complex<T> &a) { return a; }
template <class T> inline complex<T> operator-(const complex<T> &a) { return complex<T>(-a.real(), -a.imag()); }
template <class T> inline complex<T> operator+(const complex<T> &a, const complex<T> &b) { return complex<T>(a.real() + b.real(), a.imag() + b.imag()); }
template <class T> inline complex<T> operator-(const complex<T> &a, const complex<T> &b) { return complex<T>(a.real() - b.real(), a.imag() - b.imag()); }
template <class T> inline complex<T> operator*(const complex<T> &a, const complex<T> &b)
{
  return complex<T>(a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real());
}
template <class T> inline complex<T> operator+(const complex<T> &a, const T &b) { return complex<T>(a.real() + b, a.imag()); }
template <class T> inline complex<T> operator+(const T &a, const complex<T> &b) { return complex<T>(a + b.real(), b.imag()); }
template <class T> inline complex<T> operator-(const complex<T> &a, const T &b) { return complex<T>(a.real() - b, a.imag()); }
template <class T> inline complex<T> operator-(const T &a, const complex<T> &b) { return complex<T>(a - b.real(), -b.imag()); }
template <class T> inline complex<T> operator*(const complex<T> &a, const T &b) { return complex<T>(a.real() * b, a.imag() * b); }
template <class T> inline complex<T> operator*(const T &a, const complex<T> &b) { return complex<T>(a * b.real(), a * b.imag()); }
template <class T> inline complex<T> operator/(const complex<T> &a, const T &b) { return complex<T>(a.real() / b, a.imag() / b); }
template <class T> inline complex<T> operator/(const T &a, const complex<T> &b) { return complex<T>(a) / b; }
template <class T> inline bool operator==(const complex<T> &a, const complex<T> &b) { return a.real() == b.real() && a.imag() == b.imag(); }

// Elementary functions go through std::complex (libm), one call each.
template <class T> inline std::complex<T> to_std(const complex<T> &z) { return std::complex<T>(z.real(), z.imag()); }
template <class T> inline complex<T> from_std(const std::complex<T> &z) { return complex<T>(z.real(), z.imag()); }
template <class T> inline complex<T> exp(const complex<T> &z) { return from_std(std::exp(to_std(z))); }
template <class T> inline complex<T> log(const complex<T> &z) { return from_std(std::log(to_std(z))); }
template <class T> inline complex<T> sqrt(const complex<T> &z) { return from_std(std::sqrt(to_std(z))); }
template <class T> inline complex<T> sin(const complex<T> &z) { return from_std(std::sin(to_std(z))); }
template <class T> inline complex<T> cos(const complex<T> &z) { return from_std(std::cos(to_std(z))); }
template <class T> inline complex<T> tan(const complex<T> &z) { return from_std(std::tan(to_std(z))); }
template <class T> inline complex<T> sinh(const complex<T> &z) { return from_std(std::sinh(to_std(z))); }
template <class T> inline complex<T> cosh(const complex<T> &z) { return from_std(std::cosh(to_std(z))); }
template <class T> inline complex<T> tanh(const complex<T> &z) { return from_std(std::tanh(to_std(z))); }
template <class T> inline complex<T> log10(const complex<T> &z) { return from_std(std::log10(to_std(z))); }
template <class T> inline complex<T> pow(const complex<T> &a, const complex<T> &b) { return from_std(std::pow(to_std(a), to_std(b))); }
template <class T> inline complex<T> pow(const complex<T> &a, const T &b) { return from_std(std::pow(to_std(a), b)); }
template <class T> inline complex<T> pow(const T &a, const complex<T> &b) { return from_std(std::pow(a, to_std(b))); }
template <class T> inline T abs(const complex<T> &z) { return std::hypot(z.real(), z.imag()); }

// Real math
inline double sqrt(double x) { return std::sqrt(x); }
inline double exp(double x) { return std::exp(x); }
inline double erf(double x) { return std::erf(x); }
inline double sin(double x) { return std::sin(x); }
inline double cos(double x) { return std::cos(x); }
inline double acos(double x) { return std::acos(x); }
inline double atan2(double y, double x) { return std::atan2(y, x); }
inline double abs(double x) { return std::fabs(x); }
inline int    abs(int x) { return x < 0 ? -x : x; }
template <class T> inline T max(const T &a, const T &b) { return a < b ? b : a; }
template <class T> inline T min(const T &a, const T &b) { return b < a ? b : a; }

// ---------------------------------------------------------------- atomics
inline void atomic_add(double *p, double v)
{
#pragma omp atomic
  *p += v;
}
inline void atomic_add(complex<double> *p, const complex<double> &v)
{
  double *q = reinterpret_cast<double *>(p);
#pragma omp atomic
  q[0] += v.real();
#pragma omp atomic
  q[1] += v.imag();
}
inline void atomic_add(int *p, int v)
{
#pragma omp atomic
  *p += v;
}

// ---------------------------------------------------------------- views
namespace impl {
template <class D> struct view_traits;
template <class T> struct view_traits<T *> {
  using value_type                 = T;
  static constexpr std::size_t inner = 1;
  static constexpr int         rank  = 1;
};
template <class T, std::size_t N> struct view_traits<T *[N]> {
  using value_type                 = T;
  static constexpr std::size_t inner = N;
  static constexpr int         rank  = 2;
};
} // namespace impl

template <class DataType, class... Props>
class View {
public:
  using traits     = impl::view_traits<DataType>;
  using value_type = typename traits::value_type;
  using data_type  = DataType;

private:
  std::shared_ptr<value_type> store_;
  value_type                 *ptr_ = nullptr;
  std::size_t                 n0_  = 0;

public:
  View() = default;
  View(const std::string &, std::size_t n0) { allocate(n0, true); }
  View(const WithoutInitializing_t &, const std::string &, std::size_t n0) { allocate(n0, false); }
  View(value_type *p, std::size_t n0) : ptr_(p), n0_(n0) {}
  void allocate(std::size_t n0, bool init)
  {
    n0_                 = n0;
    const std::size_t n = n0 * traits::inner;
    value_type       *p = n ? new value_type[n]() : nullptr; // value-initialised, as Kokkos does
    (void)init;
    store_ = std::shared_ptr<value_type>(p, std::default_delete<value_type[]>());
    ptr_   = p;
  }
  value_type &operator()(std::size_t i) const { return ptr_[i]; }
  value_type &operator()(std::size_t i, std::size_t j) const { return ptr_[i * traits::inner + j]; }
  std::size_t extent(int r) const { return r == 0 ? n0_ : traits::inner; }
  std::size_t size() const { return n0_ * traits::inner; }
  value_type *data() const { return ptr_; }
};

template <class D, class... P>
inline View<D, P...> create_mirror_view(const View<D, P...> &v) { return v; }
template <class D, class... P>
inline View<D, P...> create_mirror_view(const WithoutInitializing_t &, const View<D, P...> &v) { return v; }
template <class D, class... P, class D2, class... P2>
inline void deep_copy(const View<D, P...> &dst, const View<D2, P2...> &src)
{
  if (dst.data() == src.data())
    return;
  std::copy(src.data(), src.data() + src.size(), dst.data());
}
template <class D, class... P>
inline void resize(const WithoutInitializing_t &, View<D, P...> &v, std::size_t n)
{
  View<D, P...> nv(WithoutInitializing, "resized", n);
  const std::size_t keep = std::min(n, v.extent(0)) * View<D, P...>::traits::inner;
  if (keep)
    std::copy(v.data(), v.data() + keep, nv.data());
  v = nv;
}
template <class D, class... P>
inline void resize(View<D, P...> &v, std::size_t n) { resize(WithoutInitializing, v, n); }

// ---------------------------------------------------------------- policies
template <class Space = DefaultExecutionSpace, class Tag = void>
struct RangePolicy {
  std::size_t begin, end;
  RangePolicy(Space, std::size_t b, std::size_t e) : begin(b), end(e) {}
  RangePolicy(std::size_t b, std::size_t e) : begin(b), end(e) {}
};

struct TeamMember {
  std::size_t league;
  std::size_t league_rank() const { return league; }
  int         team_rank() const { return 0; }
  int         team_size() const { return 1; }
};

template <class Space = DefaultExecutionSpace, class Tag = void>
struct TeamPolicy {
  using member_type = TeamMember;
  std::size_t league;
  TeamPolicy(Space, std::size_t l, AUTO_t, int = 1) : league(l) {}
  TeamPolicy(std::size_t l, AUTO_t, int = 1) : league(l) {}
  TeamPolicy(Space, std::size_t l, int, int = 1) : league(l) {}
  static int vector_length_max() { return 1; }
};

struct TeamRange {
  std::size_t begin, end;
};
inline TeamRange TeamThreadRange(const TeamMember &, std::size_t b, std::size_t e) { return {b, e}; }
inline TeamRange ThreadVectorRange(const TeamMember &, std::size_t b, std::size_t e) { return {b, e}; }
struct PerThreadTag {};
inline PerThreadTag PerThread(const TeamMember &) { return {}; }
template <class F> inline void single(PerThreadTag, const F &f) { f(); }

namespace impl {
template <class Tag, class F>
inline void call_range(const F &f, std::size_t i)
{
  if constexpr (std::is_void_v<Tag>)
    f(i);
  else
    f(Tag{}, i);
}
} // namespace impl

template <class Space, class Tag, class F>
inline void parallel_for(const std::string &, const RangePolicy<Space, Tag> &p, const F &f)
{
  const long b = long(p.begin), e = long(p.end);
#pragma omp parallel for schedule(dynamic, 64)
  for (long i = b; i < e; i++)
    impl::call_range<Tag>(f, std::size_t(i));
}
template <class Space, class Tag, class F>
inline void parallel_for(const RangePolicy<Space, Tag> &p, const F &f) { parallel_for(std::string(), p, f); }

template <class Space, class Tag, class F>
inline void parallel_for(const std::string &, const TeamPolicy<Space, Tag> &p, const F &f)
{
  const long n = long(p.league);
#pragma omp parallel for schedule(dynamic, 4)
  for (long l = 0; l < n; l++) {
    TeamMember m{std::size_t(l)};
    if constexpr (std::is_void_v<Tag>)
      f(m);
    else
      f(Tag{}, m);
  }
}

// nested team/vector ranges run serially inside one league member
template <class F>
inline void parallel_for(const TeamRange &r, const F &f)
{
  for (std::size_t i = r.begin; i < r.end; i++)
    f(i);
}
template <class F, class Reducer>
inline void parallel_reduce(const TeamRange &r, const F &f, const Reducer &red)
{
  typename Reducer::value_type tmp;
  red.init(tmp);
  for (std::size_t i = r.begin; i < r.end; i++)
    f(i, tmp);
  red.reference() = tmp;
}

// range reduce into three scalars (used by the reference's CG solver)
template <class Space, class Tag, class F>
inline void parallel_reduce(const std::string &, const RangePolicy<Space, Tag> &p, const F &f, double &r0, double &r1, double &r2)
{
  double s0 = 0, s1 = 0, s2 = 0;
  for (std::size_t i = p.begin; i < p.end; i++) {
    if constexpr (std::is_void_v<Tag>)
      f(i, s0, s1, s2);
    else
      f(Tag{}, i, s0, s1, s2);
  }
  r0 = s0;
  r1 = s1;
  r2 = s2;
}

} // namespace Kokkos
