// Kokkos::numbers for the reference-compiling shim (see Kokkos_Core.hpp).
#pragma once
namespace Kokkos {
namespace numbers {
inline constexpr double pi         = 3.141592653589793238462643383279502884;
inline constexpr double inv_pi     = 0.318309886183790671537767526745028724;
inline constexpr double inv_sqrtpi = 0.564189583547756286948079451560772586;
inline constexpr double sqrt2      = 1.414213562373095048801688724209698079;
} // namespace numbers
} // namespace Kokkos
