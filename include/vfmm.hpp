// vfmm.hpp — header-only C++ drop-in for the reference's calculator class.
//
// A caller written against kursatyurt/UVLM includes this header instead of
// src/fmmCalculator.hpp (and exafmmTypes.hpp) and keeps its code:
//   Vortex::FMMCalculator<Host, Device, Vortex::RK3, Vortex::Inviscid,
//                         Vortex::cVPM, Vortex::Transposed> calc;
//   calc.advance(bodies, dt);          // fmmCalculator.hpp:919
//   calc.getSensorData(sensors);       // fmmCalculator.hpp:726
// exafmm::Body is byte-compatible with the reference's (exafmmTypes.hpp:18-32)
// and zero-initialised like it.  The reference's compile-time constants P,
// ncrit and MAC_theta (exafmmTypes.hpp:12-15) become the macros VFMM_P,
// VFMM_NCRIT, VFMM_THETA (defaults: the reference's values) or constructor
// arguments.  Host/Device tags are accepted and ignored: the work runs on the
// current CUDA device.  Link with libvfmm.so.
#ifndef VFMM_HPP
#define VFMM_HPP

#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>
#include "vfmm.h"

#ifndef VFMM_P
#define VFMM_P 4
#endif
#ifndef VFMM_NCRIT
#define VFMM_NCRIT 128
#endif
#ifndef VFMM_THETA
#define VFMM_THETA 0.3
#endif

namespace exafmm {
typedef double real_t;
static constexpr int    P         = VFMM_P;
static constexpr int    ncrit     = VFMM_NCRIT;
static constexpr real_t MAC_theta = VFMM_THETA;

struct Body : vfmm_body {
  Body() : vfmm_body{} {}
};
static_assert(sizeof(Body) == 296, "exafmm::Body layout");
typedef std::vector<Body> Bodies;
} // namespace exafmm

namespace Vortex {
struct Inviscid {};
struct PSE {};
struct CSM {};
struct Euler {};
struct RK2 {};
struct RK3 {};
struct RK4 {};
struct cVPM {};
struct rVPM {};
struct Transposed {};
struct Classic {};

class Error : public std::runtime_error {
public:
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

// The particle file of the reference driver's writeTovtk lambda
// (src/main.cpp:127-164), which writes "output" + step + ".vtk"; ASCII is
// byte-identical to it, binary keeps full FP64 values.
inline void writeVTK(const exafmm::Bodies &particles, const std::string &path, bool binary = false)
{
  if (vfmm_write_vtk(particles.data(), particles.size(), path.c_str(), binary ? 1 : 0) != VFMM_OK)
    throw Error(VFMM_ERR_INVALID, "writeVTK: cannot write " + path);
}

template <typename Host, typename Device, typename IntegrationScheme, typename ViscousScheme, typename Formulation, typename Stretching>
struct FMMCalculator {
  // nu: the viscosity of the PSE/CSM schemes, which the reference declares
  // (fmmCalculator.hpp:56) but never sets
  explicit FMMCalculator(int p = exafmm::P, int ncrit = exafmm::ncrit, double theta = exafmm::MAC_theta, int precision = VFMM_FP64,
                         double relax = 0.0, double nu = 0.0)
  {
    vfmm_config c;
    vfmm_default_config(&c);
    c.p           = p;
    c.ncrit       = ncrit;
    c.theta       = theta;
    c.precision   = precision;
    c.relax       = relax;
    c.integrator  = std::is_same<IntegrationScheme, Euler>::value ? VFMM_EULER
                    : std::is_same<IntegrationScheme, RK2>::value ? VFMM_RK2
                    : std::is_same<IntegrationScheme, RK3>::value ? VFMM_RK3
                                                                  : VFMM_RK4;
    c.stretching  = std::is_same<Stretching, Classic>::value ? VFMM_CLASSIC : VFMM_TRANSPOSED;
    c.formulation = std::is_same<Formulation, rVPM>::value ? VFMM_RVPM : VFMM_CVPM;
    c.viscous     = std::is_same<ViscousScheme, PSE>::value ? VFMM_PSE : (std::is_same<ViscousScheme, CSM>::value ? VFMM_CSM : VFMM_INVISCID);
    c.nu          = nu;
    check(vfmm_create(&c, &h_), "vfmm_create");
  }
  ~FMMCalculator()
  {
    if (h_)
      vfmm_destroy(h_);
  }
  FMMCalculator(const FMMCalculator &)            = delete;
  FMMCalculator &operator=(const FMMCalculator &) = delete;

  // fmmCalculator.hpp:282 — tree + lists; permutes `bodies` into tree order
  void init(exafmm::Bodies &bodies) { check(vfmm_init(h_, bodies.data(), bodies.size()), "init"); }
  // fmmCalculator.hpp:420 — velocity, J, dadt on the device
  void calculate() { check(vfmm_calculate(h_), "calculate"); }
  // fmmCalculator.hpp:235
  void copyBodies2Host(exafmm::Bodies &bodies) { check(vfmm_copy_bodies_to_host(h_, bodies.data(), bodies.size()), "copyBodies2Host"); }
  // fmmCalculator.hpp:919 — one step; `bodies` overwritten in tree order
  void advance(exafmm::Bodies &bodies, double dt) { check(vfmm_advance(h_, bodies.data(), bodies.size(), dt), "advance"); }
  // fmmCalculator.hpp:726
  void getSensorData(exafmm::Bodies &sensors) { check(vfmm_get_sensor_data(h_, sensors.data(), sensors.size()), "getSensorData"); }
  // fmmCalculator.hpp:856 — vorticity re-interpolation; newPoints shrinks to the kept points
  void RBF(exafmm::Bodies &particles, exafmm::Bodies &newPoints)
  {
    size_t kept = 0;
    check(vfmm_rbf(h_, particles.data(), particles.size(), newPoints.data(), newPoints.size(), &kept, nullptr), "RBF");
    newPoints.resize(kept);
  }
  // relaxation.hpp:8 (the reference leaves it unwired)
  void relaxation(double f) { check(vfmm_relax(h_, f), "relaxation"); }

  // Gradient of energy * E + impulse . I at the state `steps` steps after
  // `bodies` with respect to their initial positions and strengths (no
  // counterpart in the reference; see vfmm_adjoint).  Returns the objective;
  // gradX and gradAlpha get 3 doubles per body in the order of `bodies`.
  double adjoint(const exafmm::Bodies &bodies, double dt, int steps, int checkpointEvery, double energy, const double impulse[3],
                 std::vector<double> &gradX, std::vector<double> &gradAlpha)
  {
    vfmm_objective o{};
    o.energy = energy;
    for (int d = 0; d < 3; d++)
      o.impulse[d] = impulse[d];
    gradX.resize(3 * bodies.size());
    gradAlpha.resize(3 * bodies.size());
    double v = 0;
    check(vfmm_adjoint(h_, bodies.data(), bodies.size(), dt, steps, checkpointEvery, &o, &v, gradX.data(), gradAlpha.data()), "adjoint");
    return v;
  }

  vfmm_handle handle() const { return h_; }

private:
  vfmm_handle h_ = nullptr;
  void        check(int code, const char *what)
  {
    if (code != VFMM_OK)
      throw Error(code, std::string(what) + ": " + vfmm_last_error(h_));
  }
};
} // namespace Vortex

#endif
