// C entry points around the reference's own FMM, compiled from its unmodified
// headers (src/fmmCalculator.hpp, tree.hpp, traverse.hpp, multipoleKernels.hpp)
// against the project's Kokkos shim (oracle/ref_shim).  Test infrastructure
// only: it produces golden fixtures and checks the oracle restatement.  It is
// built in this container only (the reference sources are not present on the
// GPU machines) by oracle/Makefile, target `ref`, into oracle/_ref/.
//
// Bodies cross this boundary as raw arrays of the reference's exafmm::Body
// (37 doubles, 296 bytes; exafmmTypes.hpp:18-32).
#include <cstdint>
#include <cstring>
#include "fmmCalculator.hpp"

using exafmm::Bodies;
using exafmm::Body;
using Host   = Kokkos::DefaultHostExecutionSpace;
using Device = Kokkos::DefaultExecutionSpace;

static_assert(sizeof(Body) == 296, "exafmm::Body layout");

struct RefCell {
  uint64_t NCHILD, NBODY, ChildOffset, BodyOffset;
  double   X[3];
  double   R;
  uint64_t level;
};

template <class Scheme, class Stretch, class Form>
using Calc = Vortex::FMMCalculator<Host, Device, Scheme, Vortex::Inviscid, Form, Stretch>;

static Bodies load(const void *p, long n)
{
  Bodies b(n);
  if (n)
    std::memcpy(b.data(), p, sizeof(Body) * n);
  return b;
}
static void store(void *p, const Bodies &b)
{
  if (!b.empty())
    std::memcpy(p, b.data(), sizeof(Body) * b.size());
}
static long export_cells(const exafmm::Cells &cells, RefCell *out, long cap)
{
  for (long i = 0; i < (long)cells.size() && i < cap; i++) {
    out[i].NCHILD      = cells[i].NCHILD;
    out[i].NBODY       = cells[i].NBODY;
    out[i].ChildOffset = cells[i].ChildOffset;
    out[i].BodyOffset  = cells[i].BodyOffset;
    for (int d = 0; d < 3; d++)
      out[i].X[d] = cells[i].X[d];
    out[i].R     = cells[i].R;
    out[i].level = cells[i].level;
  }
  return (long)cells.size();
}

extern "C" {

int    ref_P() { return exafmm::P; }
int    ref_ncrit() { return exafmm::ncrit; }
double ref_theta() { return exafmm::MAC_theta; }

long ref_build_tree(void *bodies, long n, RefCell *cells, long cap)
{
  Bodies b     = load(bodies, n);
  auto   tree  = exafmm::buildTree(b);
  long   count = export_cells(tree, cells, cap);
  store(bodies, b);
  return count;
}

// Raw getList output (traverse.hpp:32-85): P2P in stack order, M2L unsorted.
long ref_lists(void *bodies, long n, uint64_t *p2p, long cap_p2p, long *np2p, uint64_t *m2l, long cap_m2l, long *nm2l)
{
  Bodies b    = load(bodies, n);
  auto   tree = exafmm::buildTree(b);
  auto   x    = exafmm::getList(&tree[0], &tree[0]);
  *np2p       = (long)x.first.size();
  *nm2l       = (long)x.second.size();
  for (long i = 0; i < *np2p && i < cap_p2p; i++) {
    p2p[2 * i]     = x.first[i].first;
    p2p[2 * i + 1] = x.first[i].second;
  }
  for (long i = 0; i < *nm2l && i < cap_m2l; i++) {
    m2l[2 * i]     = x.second[i].first;
    m2l[2 * i + 1] = x.second[i].second;
  }
  store(bodies, b);
  return (long)tree.size();
}

} // extern "C"

template <class C>
static int run_calculate(void *bodies, long n, double *M, double *L, long cap_cells, long *ncells)
{
  Bodies b = load(bodies, n);
  C      calc;
  calc.init(b);
  calc.calculate();
  calc.copyBodies2Host(b);
  store(bodies, b);
  const long nc = (long)calc._cellsView.extent(0);
  *ncells       = nc;
  if (M && L && nc <= cap_cells) {
    for (long c = 0; c < nc; c++)
      for (int t = 0; t < exafmm::NTERM; t++) {
        M[2 * (c * exafmm::NTERM + t)]     = calc._multipoleView(c, t).real();
        M[2 * (c * exafmm::NTERM + t) + 1] = calc._multipoleView(c, t).imag();
        L[2 * (c * exafmm::NTERM + t)]     = calc._localView(c, t).real();
        L[2 * (c * exafmm::NTERM + t) + 1] = calc._localView(c, t).imag();
      }
  }
  return 0;
}

extern "C" {

// FMMCalculator::init + calculate (fmmCalculator.hpp:282, :420); bodies come
// back permuted into tree order with velocity, J and dadt filled.
// stretching: 0 Transposed, 1 Classic.  formulation: 0 cVPM, 1 rVPM.
int ref_calculate(void *bodies, long n, int stretching, int formulation, double *M, double *L, long cap_cells, long *ncells)
{
  if (stretching == 0 && formulation == 0)
    return run_calculate<Calc<Vortex::RK2, Vortex::Transposed, Vortex::cVPM>>(bodies, n, M, L, cap_cells, ncells);
  if (stretching == 1 && formulation == 0)
    return run_calculate<Calc<Vortex::RK2, Vortex::Classic, Vortex::cVPM>>(bodies, n, M, L, cap_cells, ncells);
  if (stretching == 0 && formulation == 1)
    return run_calculate<Calc<Vortex::RK2, Vortex::Transposed, Vortex::rVPM>>(bodies, n, M, L, cap_cells, ncells);
  return run_calculate<Calc<Vortex::RK2, Vortex::Classic, Vortex::rVPM>>(bodies, n, M, L, cap_cells, ncells);
}

} // extern "C"

template <class C>
static int run_advance(void *bodies, long n, double dt, int steps)
{
  Bodies b = load(bodies, n);
  C      calc;
  for (int s = 0; s < steps; s++)
    calc.advance(b, dt);
  store(bodies, b);
  return 0;
}

template <class Scheme>
static int advance_scheme(void *bodies, long n, double dt, int steps, int stretching)
{
  if (stretching == 0)
    return run_advance<Calc<Scheme, Vortex::Transposed, Vortex::cVPM>>(bodies, n, dt, steps);
  return run_advance<Calc<Scheme, Vortex::Classic, Vortex::cVPM>>(bodies, n, dt, steps);
}

extern "C" {

// FMMCalculator::advance (fmmCalculator.hpp:919-1005), `steps` times.
// scheme: 0 Euler, 1 RK2, 2 RK3, 3 RK4.
int ref_advance(void *bodies, long n, double dt, int steps, int scheme, int stretching)
{
  switch (scheme) {
  case 0: return advance_scheme<Vortex::Euler>(bodies, n, dt, steps, stretching);
  case 1: return advance_scheme<Vortex::RK2>(bodies, n, dt, steps, stretching);
  case 2: return advance_scheme<Vortex::RK3>(bodies, n, dt, steps, stretching);
  case 3: return advance_scheme<Vortex::RK4>(bodies, n, dt, steps, stretching);
  }
  return -1;
}

// FMMCalculator::advance with the rVPM formulation (fmmCalculator.hpp:407-418:
// the radii evolve) and transposed stretching, `steps` times; scheme 1 RK2,
// 2 RK3.
int ref_advance_rvpm(void *bodies, long n, double dt, int steps, int scheme)
{
  if (scheme == 1)
    return run_advance<Calc<Vortex::RK2, Vortex::Transposed, Vortex::rVPM>>(bodies, n, dt, steps);
  if (scheme == 2)
    return run_advance<Calc<Vortex::RK3, Vortex::Transposed, Vortex::rVPM>>(bodies, n, dt, steps);
  return -1;
}

// FMMCalculator::advance with a viscous scheme (fmmCalculator.hpp:713-724,
// called after every calculate): viscous 1 = Vortex::PSE (multipoleKernels.hpp:
// 415-450), 2 = Vortex::CSM (fmmCalculator.hpp:334-337).  The reference never
// sets its viscosity member _nu (fmmCalculator.hpp:56); it is set here.
// Transposed stretching, cVPM.
int ref_advance_viscous(void *bodies, long n, double dt, int steps, int scheme, int viscous, double nu)
{
  auto run = [&](auto tag_scheme, auto tag_visc) {
    using S = decltype(tag_scheme);
    using V = decltype(tag_visc);
    Bodies b = load(bodies, n);
    Vortex::FMMCalculator<Host, Device, S, V, Vortex::cVPM, Vortex::Transposed> calc;
    calc._nu = nu;
    for (int s = 0; s < steps; s++)
      calc.advance(b, dt);
    store(bodies, b);
    return 0;
  };
  auto by_scheme = [&](auto tag_visc) {
    switch (scheme) {
    case 0: return run(Vortex::Euler{}, tag_visc);
    case 1: return run(Vortex::RK2{}, tag_visc);
    case 2: return run(Vortex::RK3{}, tag_visc);
    case 3: return run(Vortex::RK4{}, tag_visc);
    }
    return -1;
  };
  if (viscous == 1)
    return by_scheme(Vortex::PSE{});
  if (viscous == 2)
    return by_scheme(Vortex::CSM{});
  return -1;
}

// FMMCalculator::RBF (fmmCalculator.hpp:856-917): vorticity of the particles
// at the new points, points with |omega| < 1e-6 removed, CG for the point
// strengths.  particles and points are permuted as the reference leaves them;
// *m_out = points kept.  The reference prints its CG residuals to stdout.
int ref_rbf(void *particles, long n, void *points, long m, long *m_out)
{
  Bodies p = load(particles, n);
  Bodies q = load(points, m);
  Calc<Vortex::RK2, Vortex::Transposed, Vortex::cVPM> calc;
  calc.RBF(p, q);
  store(particles, p);
  store(points, q);
  *m_out = (long)q.size();
  return 0;
}

// init + calculate on the particles, then getSensorData (fmmCalculator.hpp:726-731).
int ref_sensors(void *bodies, long n, void *sensors, long ns)
{
  Bodies b = load(bodies, n);
  Bodies s = load(sensors, ns);
  Calc<Vortex::RK2, Vortex::Transposed, Vortex::cVPM> calc;
  calc.init(b);
  calc.calculate();
  calc.getSensorData(s);
  store(bodies, b);
  store(sensors, s);
  return 0;
}

// exafmm::direct (traverse.hpp:88-98): host P2P with the classic stretching form.
void ref_direct(void *targets, long nt, void *sources, long ns)
{
  Bodies t = load(targets, nt);
  Bodies s = load(sources, ns);
  exafmm::direct(t, s);
  store(targets, t);
}

} // extern "C"
