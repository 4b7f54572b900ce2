// Kokkos numeric traits for the reference-compiling shim (see Kokkos_Core.hpp).
#pragma once
#include <limits>
namespace Kokkos {
namespace Experimental {
template <class T>
inline constexpr T epsilon_v = std::numeric_limits<T>::epsilon();
} // namespace Experimental
} // namespace Kokkos
