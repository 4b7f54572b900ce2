// Kokkos::pair for the reference-compiling shim (see Kokkos_Core.hpp).
#pragma once
#include <utility>

namespace Kokkos {
template <class T1, class T2>
struct pair {
  T1 first;
  T2 second;
  pair() : first(), second() {}
  pair(const T1 &a, const T2 &b) : first(a), second(b) {}
  pair(T1 &&a, T2 &&b) : first(std::move(a)), second(std::move(b)) {}
  template <class U1, class U2>
  pair(const pair<U1, U2> &o) : first(T1(o.first)), second(T2(o.second)) {}
};
template <class T1, class T2>
inline pair<T1, T2> make_pair(T1 a, T2 b) { return pair<T1, T2>(a, b); }
} // namespace Kokkos
