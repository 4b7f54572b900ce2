// Force-included ahead of the reference's headers when the reference is
// compiled as an oracle.  The reference fixes its expansion order, leaf size
// and MAC as compile-time constants in src/exafmmTypes.hpp:12-15 (P=4,
// ncrit=128, theta=0.3); the configurations checked here need other values,
// so this header restates that file's declarations (same Body and Cell
// layouts, exafmmTypes.hpp:18-46) with the three constants taken from
// -DREF_P / -DREF_NCRIT / -DREF_THETA, and defines the reference's include
// guard so that its own exafmmTypes.hpp is skipped.
#ifndef EXAFMMTYPES_HPP
#define EXAFMMTYPES_HPP
#include <Kokkos_Core.hpp>
#include <vector>

#ifndef REF_P
#define REF_P 4
#endif
#ifndef REF_NCRIT
#define REF_NCRIT 128
#endif
#ifndef REF_THETA
#define REF_THETA 0.3
#endif

namespace exafmm {
typedef double                  real_t;
typedef Kokkos::complex<real_t> complex_t;

static constexpr int    P         = REF_P;
static constexpr int    NTERM     = 3 * (P * (P + 1) / 2);
static constexpr int    ncrit     = REF_NCRIT;
static constexpr real_t MAC_theta = REF_THETA;

struct Body {
  real_t J[3][3]{{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
  real_t X[3]{0.0, 0.0, 0.0};
  real_t alpha[3]{0.0, 0.0, 0.0};
  real_t velocity[3]{0.0, 0.0, 0.0};
  real_t dadt[3]{0.0, 0.0, 0.0};
  real_t velocity_old[3]{0.0, 0.0, 0.0};
  real_t dadt_old[3]{0.0, 0.0, 0.0};
  real_t X_old[3]{0.0, 0.0, 0.0};
  real_t alpha_old[3]{0.0, 0.0, 0.0};
  real_t radius{0.0};
  real_t drdt{0.0};
  real_t radius_old{0.0};
  real_t drdt_old{0.0};
};
typedef std::vector<Body> Bodies;

struct Cell {
  size_t NCHILD;
  size_t NBODY;
  size_t ChildOffset;
  size_t BodyOffset;
  real_t X[3];
  Cell  *CHILD;
  Body  *BODY;
  real_t R;
  size_t level;
};
typedef std::vector<Cell> Cells;
} // namespace exafmm
#endif
