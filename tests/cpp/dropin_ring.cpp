// A caller written against the reference's FMMCalculator API, compiled
// against include/vfmm.hpp and linked with libvfmm.so.  Builds a small ring
// of particles, takes one RK3 step, prints the mean velocity and reads the
// velocity at the ring's centre through getSensorData (Gamma / 2R = 0.5 for
// this ring); with a path argument it writes the particles there as the
// reference driver's VTK file (main.cpp:127-164); exit code 0 on success.
#include <cmath>
#include <cstdio>
#include "vfmm.hpp"

int main(int argc, char **argv)
{
  typedef Vortex::FMMCalculator<int, int, Vortex::RK3, Vortex::Inviscid, Vortex::cVPM, Vortex::Transposed> FMMCalculator;
  exafmm::Bodies particles;
  const int      n  = 2000;
  const double   ds = 2 * M_PI / n;
  for (int i = 0; i < n; i++) {
    exafmm::Body b;
    const double ph = i * ds;
    b.X[0]          = std::cos(ph);
    b.X[1]          = std::sin(ph);
    b.X[2]          = 1e-3 * std::sin(7 * ph);
    b.alpha[0]      = -std::sin(ph) * ds;
    b.alpha[1]      = std::cos(ph) * ds;
    b.radius        = 3 * ds;
    particles.push_back(b);
  }
  exafmm::Bodies      sensors(1);
  std::vector<double> gx, ga;
  double              energy = 0;
  try {
    FMMCalculator calc(8, 32, 0.5);
    const double  wI[3] = {0.0, 0.0, 1.0};
    energy              = calc.adjoint(particles, 0.01, 1, 1, 1.0, wI, gx, ga); // before advance reorders the bodies
    calc.advance(particles, 0.01);
    calc.getSensorData(sensors);
    if (argc > 1)
      Vortex::writeVTK(particles, argv[1]);
  } catch (const Vortex::Error &e) {
    std::fprintf(stderr, "vfmm error %d: %s\n", e.code, e.what());
    return 1;
  }
  double uz = 0;
  for (const auto &b : particles)
    uz += b.velocity[2];
  const double uc = sensors[0].velocity[2];
  double gn = 0;
  for (double g : gx)
    gn += g * g;
  std::printf("mean uz %.6e centre uz %.6e objective %.6e |grad_x| %.6e\n", uz / n, uc, energy, std::sqrt(gn));
  return std::isfinite(uz) && std::fabs(uc - 0.5) < 0.01 && std::isfinite(gn) && gx.size() == 3 * (size_t)n ? 0 : 2;
}
