// Oracle: a CPU restatement, in plain C++, of the reference's vortex-particle
// FMM (kursatyurt/UVLM, src/*.hpp).  TEST INFRASTRUCTURE ONLY: it is the
// checker for the CUDA library's parity tests and the timed CPU baseline; the
// product never links or calls it.
//
// Pinned by: golden fixtures produced by the reference itself (its headers
// compiled against a Kokkos shim, see oracle/ref_driver.cpp) and committed
// under tests/golden/; tests/test_oracle.py checks this file against them.
//
// Unlike the reference, the expansion order P, leaf size ncrit and MAC theta
// are runtime arguments (reference: compile-time, exafmmTypes.hpp:12-15).
// Parallel loops use OpenMP, organised by target so that no atomics are needed.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace vo {

typedef std::complex<double> cd;

// exafmm::Body layout (exafmmTypes.hpp:18-32), 296 bytes.
struct Body {
  double J[3][3];
  double X[3];
  double alpha[3];
  double velocity[3];
  double dadt[3];
  double velocity_old[3];
  double dadt_old[3];
  double X_old[3];
  double alpha_old[3];
  double radius, drdt, radius_old, drdt_old;
};
static_assert(sizeof(Body) == 296, "Body layout");

// exafmm::Cell without its pointers (exafmmTypes.hpp:36-46).
struct Cell {
  uint64_t NCHILD, NBODY, ChildOffset, BodyOffset;
  double   X[3];
  double   R;
  uint64_t level;
};
static_assert(sizeof(Cell) == 72, "Cell layout");

static const double inv_pi     = 0.318309886183790671537767526745028724;
static const double inv_sqrtpi = 0.564189583547756286948079451560772586;

static inline int oddOrEven(int n) { return (n & 1) ? -1 : 1; }     // multipoleKernels.hpp:16-19
static inline int ipow2n(int n) { return n >= 0 ? 1 : oddOrEven(n); } // multipoleKernels.hpp:22-25

// ---------------------------------------------------------------- tree
// getBounds, tree.hpp:7-26
static void getBounds(const Body *b, long n, double &R0, double X0[3])
{
  double Xmin[3], Xmax[3];
  for (int d = 0; d < 3; d++)
    Xmin[d] = Xmax[d] = b[0].X[d];
  for (long i = 0; i < n; i++) {
    for (int d = 0; d < 3; d++)
      Xmin[d] = std::fmin(b[i].X[d], Xmin[d]);
    for (int d = 0; d < 3; d++)
      Xmax[d] = std::fmax(b[i].X[d], Xmax[d]);
  }
  for (int d = 0; d < 3; d++)
    X0[d] = (Xmax[d] + Xmin[d]) / 2;
  R0 = 0;
  for (int d = 0; d < 3; d++) {
    R0 = std::fmax(X0[d] - Xmin[d], R0);
    R0 = std::fmax(Xmax[d] - X0[d], R0);
  }
  R0 *= 1.00001;
}

struct TreeBuilder {
  std::vector<Cell> cells;
  std::vector<Body> tmp;
  Body             *bodies;
  int               ncrit;
  int               maxLevel;
  bool              depthError = false;

  // buildCells, tree.hpp:29-99: a leaf when NBODY <= ncrit; otherwise a stable
  // octant partition (x > centre, strict) and a contiguous block of children
  // appended at the end of the cell array, then recursion in octant order.
  void build(long cellIndex, long begin, long end, const double X[3], double R0, int level)
  {
    Cell &c  = cells[cellIndex];
    c.NBODY  = end - begin;
    c.NCHILD = 0;
    c.ChildOffset = 0;
    c.BodyOffset  = begin;
    for (int d = 0; d < 3; d++)
      c.X[d] = X[d];
    c.R     = R0 / (1 << level);
    c.level = level;
    if (end - begin <= ncrit)
      return;
    if (level >= maxLevel) {
      depthError = true;
      return;
    }
    long size[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    auto octant  = [&](const Body &b) { return (b.X[0] > X[0]) + ((b.X[1] > X[1]) << 1) + ((b.X[2] > X[2]) << 2); };
    for (long i = begin; i < end; i++)
      size[octant(bodies[i])]++;
    long offsets[8], counter[8], off = begin;
    int  nchild = 0;
    for (int i = 0; i < 8; i++) {
      offsets[i] = off;
      off += size[i];
      if (size[i])
        nchild++;
    }
    for (int i = 0; i < 8; i++)
      counter[i] = offsets[i];
    for (long i = begin; i < end; i++)
      tmp[counter[octant(bodies[i])]++] = bodies[i];
    for (long i = begin; i < end; i++)
      bodies[i] = tmp[i];
    const long first = (long)cells.size();
    cells.resize(cells.size() + nchild);
    cells[cellIndex].NCHILD      = nchild;
    cells[cellIndex].ChildOffset = first;
    const double r = R0 / (1 << (level + 1));
    int          k = 0;
    for (int i = 0; i < 8; i++) {
      double Xc[3];
      for (int d = 0; d < 3; d++)
        Xc[d] = X[d] + r * (((i & 1 << d) >> d) * 2 - 1);
      if (size[i]) {
        build(first + k, offsets[i], offsets[i] + size[i], Xc, R0, level + 1);
        k++;
      }
    }
  }
};

// buildTree, tree.hpp:101-113.  Returns false if a cell deeper than maxLevel
// would still hold more than ncrit bodies (the reference recurses forever).
static bool buildTree(Body *bodies, long n, int ncrit, std::vector<Cell> &cells, int maxLevel = 40)
{
  double R0, X0[3];
  getBounds(bodies, n, R0, X0);
  TreeBuilder tb;
  tb.bodies   = bodies;
  tb.ncrit    = ncrit;
  tb.maxLevel = maxLevel;
  tb.tmp.resize(n);
  tb.cells.reserve(n / std::max(ncrit, 1) * 3 + 16);
  tb.cells.resize(1);
  tb.build(0, 0, n, X0, R0, 0);
  cells.swap(tb.cells);
  return !tb.depthError;
}

typedef std::pair<uint64_t, uint64_t> Pair;

// getList, traverse.hpp:32-85: explicit-stack dual-tree traversal.  The MAC
// is |dX|^2 theta^2 < (Ri+Rj)^2 -> near; near leaf pairs -> P2P, near
// non-leaf pairs are split (the target when the source is a leaf or the
// target is at least as large and not a leaf, else the source); far -> M2L.
static void getList(const Cell *tcells, const Cell *scells, double theta, std::vector<Pair> &p2p, std::vector<Pair> &m2l)
{
  p2p.clear();
  m2l.clear();
  if (tcells[0].NCHILD == 0 && scells[0].NCHILD == 0) {
    p2p.push_back(Pair(0, 0));
    return;
  }
  std::vector<Pair> stack;
  stack.push_back(Pair(0, 0));
  auto interact = [&](uint64_t i, uint64_t j) {
    const Cell &Ci = tcells[i], &Cj = scells[j];
    double      dX[3];
    for (int d = 0; d < 3; d++)
      dX[d] = Ci.X[d] - Cj.X[d];
    const double R2 = (dX[0] * dX[0] + dX[1] * dX[1] + dX[2] * dX[2]) * theta * theta;
    if (R2 < (Ci.R + Cj.R) * (Ci.R + Cj.R)) {
      if (Ci.NCHILD == 0 && Cj.NCHILD == 0)
        p2p.push_back(Pair(i, j));
      else
        stack.push_back(Pair(i, j));
    } else {
      m2l.push_back(Pair(i, j));
    }
  };
  while (!stack.empty()) {
    Pair pr = stack.back();
    stack.pop_back();
    const Cell &T = tcells[pr.first], &S = scells[pr.second];
    if (S.NCHILD == 0 || (T.R >= S.R && T.NCHILD != 0)) {
      for (uint64_t c = T.ChildOffset; c < T.ChildOffset + T.NCHILD; c++)
        interact(c, pr.second);
    } else {
      for (uint64_t c = S.ChildOffset; c < S.ChildOffset + S.NCHILD; c++)
        interact(pr.first, c);
    }
  }
}

// ---------------------------------------------------------------- harmonics
static void cart2sph(const double dX[3], double &r, double &theta, double &phi)
{ // multipoleKernels.hpp:27-32
  r     = std::sqrt(dX[0] * dX[0] + dX[1] * dX[1] + dX[2] * dX[2]);
  theta = r == 0.0 ? 0.0 : std::acos(dX[2] / r);
  phi   = std::atan2(dX[1], dX[0]);
}

// evalMultipole (real form), multipoleKernels.hpp:53-92: regular solid
// harmonics rho^n P_n^m(cos a) e^{i m b} / ((-1)^n (n+m)!) at index n^2+n+m,
// with their conjugates at n^2+n-m.
static void evalMultipole(int P, double rho, double alpha, double beta, cd *Ynm)
{
  const double x = std::cos(alpha), y = std::sin(alpha);
  double       fact = 1, pn = 1, rhom = 1;
  const cd     ei = std::exp(cd(0, 1) * beta);
  cd           eim = 1.0;
  for (int m = 0; m < P; m++) {
    double p     = pn;
    const int npn = m * m + 2 * m, nmn = m * m;
    Ynm[npn]     = rhom * p * eim;
    Ynm[nmn]     = std::conj(Ynm[npn]);
    double p1    = p;
    p            = x * (2 * m + 1) * p1;
    rhom *= rho;
    double rhon = rhom;
    for (int n = m + 1; n < P; n++) {
      const int npm = n * n + n + m, nmm = n * n + n - m;
      rhon /= -(n + m);
      Ynm[npm]  = rhon * p * eim;
      Ynm[nmm]  = std::conj(Ynm[npm]);
      double p2 = p1;
      p1        = p;
      p         = (x * (2 * n + 1) * p1 - (n + m) * p2) / (n - m + 1);
      rhon *= rho;
    }
    rhom /= -(2 * m + 2) * (2 * m + 1);
    pn = -pn * fact * y;
    fact += 2;
    eim *= ei;
  }
}

// evalLocal, multipoleKernels.hpp:137-172: singular harmonics
// (-1)^n (n-m)! P_n^m(cos a) e^{i m b} / rho^{n+1} for n < P; the caller's
// buffer holds 4P^2 entries and those of degree >= P stay zero.
static void evalLocal(int P, double rho, double alpha, double beta, cd *Ynm)
{
  const double x = std::cos(alpha), y = std::sin(alpha);
  double       fact = 1, pn = 1;
  const double invR = -1.0 / rho;
  double       rhom = -invR;
  const cd     ei   = std::exp(cd(0, 1) * beta);
  cd           eim  = 1.0;
  for (int m = 0; m < P; m++) {
    double p      = pn;
    const int npn = m * m + 2 * m, nmn = m * m;
    Ynm[npn]      = rhom * p * eim;
    Ynm[nmn]      = std::conj(Ynm[npn]);
    double p1     = p;
    p             = x * (2 * m + 1) * p1;
    rhom *= invR;
    double rhon = rhom;
    for (int n = m + 1; n < P; n++) {
      const int npm = n * n + n + m, nmm = n * n + n - m;
      Ynm[npm]  = rhon * p * eim;
      Ynm[nmm]  = std::conj(Ynm[npm]);
      double p2 = p1;
      p1        = p;
      p         = (x * (2 * n + 1) * p1 - (n + m) * p2) / (n - m + 1);
      rhon *= invR * (n - m + 1);
    }
    pn = -pn * fact * y;
    fact += 2;
    eim *= ei;
  }
}

// ---------------------------------------------------------------- complex step
// The reference's L2P (multipoleKernels.hpp:631-742) differentiates the local
// expansion with a complex step of 1e-32 through the `cplx` scalar
// (complexify.hpp) and a bicomplex `multicomplex` for e^{i m phi}.  This
// restates those rules: comparisons on the real part, acos/atan2 with the
// derivative-correct imaginary parts of complexify.hpp:430-453.
typedef std::complex<double> cs; // value + i*h*derivative
struct mc {                      // multicomplex A + j B, complexify.hpp:470-473
  cs A, B;
};
static inline mc mprod(const mc &V, const mc &W) { return {V.A * W.A - V.B * W.B, V.A * W.B + V.B * W.A}; }
static inline mc mprod(const mc &V, const cs &x) { return {V.A * x, V.B * x}; }
static inline mc mconj(const mc &V) { return {V.A, -V.B}; }
static inline cs cs_acos(const cs &z)
{
  return cs(std::acos(z.real()), -z.imag() / std::sqrt(1.0 - z.real() * z.real() + 1.e-24));
}
static inline cs cs_atan2(const cs &z1, const cs &z2)
{
  return cs(std::atan2(z1.real(), z2.real()),
            (z2.real() * z1.imag() - z1.real() * z2.imag()) / (z1.real() * z1.real() + z2.real() * z2.real()));
}

// evalMultipole (complex-step form), multipoleKernels.hpp:94-134
static void evalMultipoleCS(int P, cs rho, cs alpha, cs beta, mc *Ynm, mc *YnmTheta)
{
  const double EPS  = 1e-16;
  const cs     x    = std::cos(alpha);
  const cs     y    = std::sin(alpha);
  const cs     invY = (std::sin(alpha).real() <= EPS) ? cs(0, 0) : 1.0 / y;
  cs           fact = 1, pn = 1, rhom = 1;
  const mc     ei  = {std::cos(beta), std::sin(beta)};
  mc           eim = {1.0, 0.0};
  for (int m = 0; m < P; m++) {
    cs        p   = pn;
    const int npn = m * m + 2 * m, nmn = m * m;
    Ynm[npn]      = mprod(eim, rhom * p);
    Ynm[nmn]      = mconj(Ynm[npn]);
    cs p1         = p;
    p             = x * double(2 * m + 1) * p1;
    YnmTheta[npn] = mprod(eim, rhom * (p - double(m + 1) * x * p1) * invY);
    rhom *= rho;
    cs rhon = rhom;
    for (int n = m + 1; n < P; n++) {
      const int npm = n * n + n + m, nmm = n * n + n - m;
      rhon /= double(-(n + m));
      Ynm[npm]      = mprod(eim, rhon * p);
      Ynm[nmm]      = mconj(Ynm[npm]);
      cs p2         = p1;
      p1            = p;
      p             = (x * double(2 * n + 1) * p1 - double(n + m) * p2) / double(n - m + 1);
      YnmTheta[npm] = mprod(eim, rhon * (double(n - m + 1) * p - double(n + 1) * x * p1) * invY);
      rhon *= rho;
    }
    rhom /= double(-(2 * m + 2) * (2 * m + 1));
    pn = -pn * fact * y;
    fact += 2.0;
    eim = mprod(eim, ei);
  }
}

// sph2cart, multipoleKernels.hpp:41-50
static void sph2cart(cs r, cs theta, cs phi, const cs *sp, cs *c)
{
  const cs st = std::sin(theta), ct = std::cos(theta), sp_ = std::sin(phi), cp = std::cos(phi);
  c[0] = st * cp * sp[0] + ct * cp / r * sp[1] - sp_ / r / st * sp[2];
  c[1] = st * sp_ * sp[0] + ct * sp_ / r * sp[1] + cp / r / st * sp[2];
  c[2] = ct * sp[0] - st / r * sp[1];
}

// ---------------------------------------------------------------- FMM
struct FMM {
  int    P, ncrit, K; // K = P(P+1)/2 harmonics per component; NTERM = 3K
  double theta;
  int    stretching  = 0; // 0 Transposed, 1 Classic (fmmCalculator.hpp:391-405)
  int    formulation = 0; // 0 cVPM, 1 rVPM (fmmCalculator.hpp:407-418)
  std::vector<Cell> cells;
  std::vector<Pair> p2p, m2l;
  std::vector<cd>   M, L; // [cell][3*nms + d], multipoleKernels.hpp:468-471
  bool              ok = true;

  FMM(int P_, int ncrit_, double theta_) : P(P_), ncrit(ncrit_), K(P_ * (P_ + 1) / 2), theta(theta_) {}

  // FMMCalculator::createTree / init, fmmCalculator.hpp:71-115, 282-288
  void init(Body *b, long n)
  {
    ok = buildTree(b, n, ncrit, cells);
    getList(cells.data(), cells.data(), theta, p2p, m2l);
    M.assign(cells.size() * 3 * K, cd(0, 0));
    L.assign(cells.size() * 3 * K, cd(0, 0));
  }

  // calculateViscosity (fmmCalculator.hpp:713-724), after calculate.
  // kind 1, PSE (multipoleKernels.hpp:415-450): over the P2P pairs, per target i
  // and source leaf, sum (vol_i alpha_j - vol_j alpha_i) e^{-R^2/(2 s^2)} / s^5 with
  // s^2 = sigma_i^2 + sigma_j^2 over R^2 != 0, and add it times
  // nu / sqrt(2) / pi / sqrt(pi) to dadt_i.  kind 2, CSM (fmmCalculator.hpp:334-337):
  // drdt += (sqrt(sigma^2 + 2 nu dt) - sigma) / dt.
  void viscosity(Body *b, long n, int kind, double nu, double dt)
  {
    if (kind == 2) {
#pragma omp parallel for
      for (long i = 0; i < n; i++)
        b[i].drdt += (std::sqrt((b[i].radius * b[i].radius) + (2.0 * nu * dt)) - b[i].radius) / dt;
      return;
    }
    if (kind != 1)
      return;
    const long        nc = (long)cells.size();
    std::vector<long> start(nc + 1, 0);
    for (auto &pr : p2p)
      start[pr.first + 1]++;
    for (long c = 0; c < nc; c++)
      start[c + 1] += start[c];
    std::vector<long> src(p2p.size()), fill(start.begin(), start.end() - 1);
    for (auto &pr : p2p)
      src[fill[pr.first]++] = (long)pr.second;
    const double sqrt2  = 1.41421356237309504880168872420969808;
    const double pi     = 3.14159265358979323846264338327950288;
    const double prefix = nu / sqrt2 * inv_pi * inv_sqrtpi;
#pragma omp parallel for schedule(dynamic, 4)
    for (long c = 0; c < nc; c++)
      for (long q = start[c]; q < start[c + 1]; q++) {
        const Cell &S = cells[src[q]];
        for (uint64_t i = cells[c].BodyOffset; i < cells[c].BodyOffset + cells[c].NBODY; i++) {
          double sum[3] = {0, 0, 0};
          for (uint64_t j = S.BodyOffset; j < S.BodyOffset + S.NBODY; j++) {
            double dX[3];
            for (int d = 0; d < 3; d++)
              dX[d] = b[i].X[d] - b[j].X[d];
            const double R2 = dX[0] * dX[0] + dX[1] * dX[1] + dX[2] * dX[2];
            if (R2 != 0) {
              const double oo    = 1. / (b[i].radius * b[i].radius + b[j].radius * b[j].radius);
              const double s5    = oo * oo * std::sqrt(oo);
              const double vol_i = 4. / 3. * pi * b[i].radius * b[i].radius * b[i].radius;
              const double vol_j = 4. / 3. * pi * b[j].radius * b[j].radius * b[j].radius;
              const double e     = std::exp(-0.5 * R2 * oo);
              for (int d = 0; d < 3; d++)
                sum[d] += (vol_i * b[j].alpha[d] - vol_j * b[i].alpha[d]) * e * s5;
            }
          }
          for (int d = 0; d < 3; d++)
            b[i].dadt[d] += sum[d] * prefix;
        }
      }
  }

  // P2M, multipoleKernels.hpp:452-477
  void P2M(long c, const Body *b)
  {
    std::vector<cd> Ynm(P * P);
    const Cell     &C = cells[c];
    for (uint64_t i = C.BodyOffset; i < C.BodyOffset + C.NBODY; i++) {
      double dX[3];
      for (int d = 0; d < 3; d++)
        dX[d] = b[i].X[d] - C.X[d];
      double rho, al, be;
      cart2sph(dX, rho, al, be);
      evalMultipole(P, rho, al, be, Ynm.data());
      for (int n = 0; n < P; n++)
        for (int m = 0; m <= n; m++) {
          const int nm = n * n + n - m, nms = n * (n + 1) / 2 + m;
          for (int d = 0; d < 3; d++)
            M[(c * K + nms) * 3 + d] += b[i].alpha[d] * Ynm[nm];
        }
    }
  }

  // M2M, multipoleKernels.hpp:479-516 (parent pulls from its children)
  void M2M(long c)
  {
    std::vector<cd> Ynm(P * P);
    const Cell     &C = cells[c];
    for (uint64_t ch = C.ChildOffset; ch < C.ChildOffset + C.NCHILD; ch++) {
      double dX[3];
      for (int d = 0; d < 3; d++)
        dX[d] = C.X[d] - cells[ch].X[d];
      double rho, al, be;
      cart2sph(dX, rho, al, be);
      evalMultipole(P, rho, al, be, Ynm.data());
      const cd *Mc = &M[ch * K * 3];
      for (int j = 0; j < P; j++)
        for (int k = 0; k <= j; k++) {
          const int jks = j * (j + 1) / 2 + k;
          cd        acc[3];
          for (int n = 0; n <= j; n++) {
            for (int m = std::max(-n, -j + k + n); m <= std::min(k - 1, n); m++) {
              const int jnkms = (j - n) * (j - n + 1) / 2 + k - m, nm = n * n + n - m;
              for (int d = 0; d < 3; d++)
                acc[d] += Mc[jnkms * 3 + d] * Ynm[nm] * double(ipow2n(m) * oddOrEven(n));
            }
            for (int m = k; m <= std::min(n, j + k - n); m++) {
              const int jnkms = (j - n) * (j - n + 1) / 2 - k + m, nm = n * n + n - m;
              for (int d = 0; d < 3; d++)
                acc[d] += std::conj(Mc[jnkms * 3 + d]) * Ynm[nm] * double(oddOrEven(k + n + m));
            }
          }
          for (int d = 0; d < 3; d++)
            M[(c * K + jks) * 3 + d] += acc[d];
        }
    }
  }

  // M2L, multipoleKernels.hpp:518-552.  Singular harmonics of degree >= P are
  // zero (evalLocal fills n < P only), so the sum runs over j + n <= P-1.
  void M2L(cd *Lt, const Cell &Ct, const cd *Ms, const Cell &Cs)
  {
    std::vector<cd> Y2(4 * P * P);
    double          dX[3];
    for (int d = 0; d < 3; d++)
      dX[d] = Ct.X[d] - Cs.X[d];
    double rho, al, be;
    cart2sph(dX, rho, al, be);
    evalLocal(P, rho, al, be, Y2.data());
    for (int j = 0; j < P; j++) {
      const double Cnm = oddOrEven(j);
      for (int k = 0; k <= j; k++) {
        const int jks = j * (j + 1) / 2 + k;
        cd        acc[3];
        for (int n = 0; n < P - j; n++) {
          for (int m = -n; m < 0; m++) {
            const int nms = n * (n + 1) / 2 - m, jnkm = (j + n) * (j + n) + j + n + m - k;
            for (int d = 0; d < 3; d++)
              acc[d] += std::conj(Ms[nms * 3 + d]) * Cnm * Y2[jnkm];
          }
          for (int m = 0; m <= n; m++) {
            const int    nms = n * (n + 1) / 2 + m, jnkm = (j + n) * (j + n) + j + n + m - k;
            const double Cnm2 = Cnm * oddOrEven((k - m) * (k < m) + m);
            for (int d = 0; d < 3; d++)
              acc[d] += Ms[nms * 3 + d] * Cnm2 * Y2[jnkm];
          }
        }
        for (int d = 0; d < 3; d++)
          Lt[jks * 3 + d] += acc[d];
      }
    }
  }

  // L2L, multipoleKernels.hpp:591-628 (parent pushes to child; here the child pulls)
  void L2L(long child, long parent)
  {
    std::vector<cd> Ynm(P * P);
    double          dX[3];
    for (int d = 0; d < 3; d++)
      dX[d] = cells[child].X[d] - cells[parent].X[d];
    double rho, al, be;
    cart2sph(dX, rho, al, be);
    evalMultipole(P, rho, al, be, Ynm.data());
    const cd *Lp = &L[parent * K * 3];
    for (int j = 0; j < P; j++)
      for (int k = 0; k <= j; k++) {
        const int jks = j * (j + 1) / 2 + k;
        cd        acc[3];
        for (int n = j; n < P; n++) {
          for (int m = j + k - n; m < 0; m++) {
            const int jnkm = (n - j) * (n - j) + n - j + m - k, nms = n * (n + 1) / 2 - m;
            for (int d = 0; d < 3; d++)
              acc[d] += std::conj(Lp[nms * 3 + d]) * Ynm[jnkm] * double(oddOrEven(k));
          }
          for (int m = 0; m <= n; m++) {
            if (n - j >= std::abs(m - k)) {
              const int jnkm = (n - j) * (n - j) + n - j + m - k, nms = n * (n + 1) / 2 + m;
              for (int d = 0; d < 3; d++)
                acc[d] += Lp[nms * 3 + d] * Ynm[jnkm] * double(oddOrEven((m - k) * (m < k)));
            }
          }
        }
        for (int d = 0; d < 3; d++)
          L[(child * K + jks) * 3 + d] += acc[d];
      }
  }

  // L2P with the complex-step gradient, multipoleKernels.hpp:630-742
  void L2P_body(const cd *Lc, const Cell &C, Body &b)
  {
    std::vector<mc> Ynm(P * P), YnmT(P * P);
    const double    h = 1e-32;
    double          vel[3] = {0, 0, 0}, J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int H = 0; H < 3; H++) {
      cs dX[3];
      for (int d = 0; d < 3; d++)
        dX[d] = b.X[d] - C.X[d];
      dX[H] += cs(0, h);
      cs sph[3][3];
      for (int a = 0; a < 3; a++)
        for (int d = 0; d < 3; d++)
          sph[a][d] = 0;
      const cs r  = std::sqrt(dX[0] * dX[0] + dX[1] * dX[1] + dX[2] * dX[2]);
      const cs th = r.real() == 0.0 ? cs(0) : cs_acos(dX[2] / r);
      const cs ph = cs_atan2(dX[1], dX[0]);
      evalMultipoleCS(P, r, th, ph, Ynm.data(), YnmT.data());
      for (int n = 0; n < P; n++) {
        int nm = n * n + n, nms = n * (n + 1) / 2;
        for (int a = 0; a < 3; a++) {
          const cd  l = Lc[nms * 3 + a];
          const cs  lr(l.real(), 0), li(l.imag(), 0);
          const mc &Y = Ynm[nm], &YT = YnmT[nm];
          sph[a][0] += (lr * Y.A - li * Y.B) / r * double(n);
          sph[a][1] += (lr * YT.A - li * YT.B);
        }
        for (int m = 1; m <= n; m++) {
          nm  = n * n + n + m;
          nms = n * (n + 1) / 2 + m;
          for (int a = 0; a < 3; a++) {
            const cd  l = Lc[nms * 3 + a];
            const cs  lr(l.real(), 0), li(l.imag(), 0);
            const mc &Y = Ynm[nm], &YT = YnmT[nm];
            sph[a][0] += 2.0 * (lr * Y.A - li * Y.B) / r * double(n);
            sph[a][1] += 2.0 * (lr * YT.A - li * YT.B);
            sph[a][2] += 2.0 * (-(lr * Y.B + li * Y.A)) * double(m);
          }
        }
      }
      cs c[3];
      // grad psi_x -> u_z -= d/dy, u_y += d/dz
      sph2cart(r, th, ph, sph[0], c);
      if (H == 0) {
        vel[2] -= c[1].real();
        vel[1] += c[2].real();
      }
      J[1][H] += c[2].imag() / h;
      J[2][H] -= c[1].imag() / h;
      sph2cart(r, th, ph, sph[1], c);
      if (H == 0) {
        vel[2] += c[0].real();
        vel[0] -= c[2].real();
      }
      J[0][H] -= c[2].imag() / h;
      J[2][H] += c[0].imag() / h;
      sph2cart(r, th, ph, sph[2], c);
      if (H == 0) {
        vel[1] -= c[0].real();
        vel[0] += c[1].real();
      }
      J[0][H] += c[1].imag() / h;
      J[1][H] -= c[0].imag() / h;
    }
    for (int d = 0; d < 3; d++)
      b.velocity[d] += 0.25 * inv_pi * vel[d];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
        b.J[i][j] += 0.25 * inv_pi * J[i][j];
  }

  // P2P team kernel (velocity + gradient), multipoleKernels.hpp:223-301
  static void P2P_target(Body &bi, const Body *src, uint64_t j0, uint64_t j1)
  {
    double s[12] = {0};
    for (uint64_t j = j0; j < j1; j++) {
      const Body &bj = src[j];
      double      dX[3];
      for (int d = 0; d < 3; d++)
        dX[d] = bi.X[d] - bj.X[d];
      const double R2 = dX[0] * dX[0] + dX[1] * dX[1] + dX[2] * dX[2];
      if (R2 != 0) {
        const double S2 = bj.radius * bj.radius, RS = R2 / S2 / 2.0, sqrtRS = std::sqrt(RS);
        const double erfS = std::erf(sqrtRS), expm = std::exp(-RS), invSqrtR2 = 1.0 / std::sqrt(R2);
        const double t2 = 2.0 * inv_sqrtpi * sqrtRS * expm, c4 = 0.25 * inv_pi / R2 * invSqrtR2;
        const double cr[3] = {c4 * (dX[1] * bj.alpha[2] - dX[2] * bj.alpha[1]), c4 * (dX[2] * bj.alpha[0] - dX[0] * bj.alpha[2]),
                              c4 * (dX[0] * bj.alpha[1] - dX[1] * bj.alpha[0])};
        const double g = erfS - t2;
        for (int a = 0; a < 3; a++)
          s[a] += cr[a] * g;
        double aux = t2 / S2 - 3.0 * g / R2;
        for (int a = 0; a < 3; a++)
          for (int b = 0; b < 3; b++)
            s[3 + 3 * a + b] += aux * cr[a] * dX[b];
        aux = g * c4;
        s[6] -= aux * bj.alpha[2];
        s[9] += aux * bj.alpha[1];
        s[4] += aux * bj.alpha[2];
        s[10] -= aux * bj.alpha[0];
        s[5] -= aux * bj.alpha[1];
        s[8] += aux * bj.alpha[0];
      }
    }
    for (int a = 0; a < 3; a++)
      bi.velocity[a] -= s[a];
    for (int a = 0; a < 3; a++)
      for (int b = 0; b < 3; b++)
        bi.J[a][b] -= s[3 + 3 * a + b];
  }

  // FMMCalculator::calculate, fmmCalculator.hpp:420-467
  void calculate(Body *b, long n)
  {
    const long nc = (long)cells.size();
    std::fill(M.begin(), M.end(), cd(0, 0));
    std::fill(L.begin(), L.end(), cd(0, 0));
    for (long i = 0; i < n; i++) { // "Reset The Rates"
      for (int d = 0; d < 3; d++)
        b[i].velocity[d] = b[i].dadt[d] = 0;
      for (int a = 0; a < 3; a++)
        for (int c = 0; c < 3; c++)
          b[i].J[a][c] = 0;
      b[i].drdt = 0;
    }
    int maxLevel = 0;
    for (long c = 0; c < nc; c++)
      maxLevel = std::max(maxLevel, (int)cells[c].level);
    std::vector<std::vector<long>> byLevel(maxLevel + 1);
    std::vector<long>              parent(nc, -1);
    for (long c = 0; c < nc; c++) {
      byLevel[cells[c].level].push_back(c);
      for (uint64_t ch = cells[c].ChildOffset; ch < cells[c].ChildOffset + cells[c].NCHILD; ch++)
        parent[ch] = c;
    }
    // upward pass, levels maxLevel..1 (the root is skipped, fmmCalculator.hpp:427)
    for (int lev = maxLevel; lev > 0; lev--) {
      const std::vector<long> &ids = byLevel[lev];
#pragma omp parallel for schedule(dynamic, 4)
      for (long t = 0; t < (long)ids.size(); t++) {
        if (cells[ids[t]].NCHILD == 0)
          P2M(ids[t], b);
        M2M(ids[t]);
      }
    }
    // M2L, grouped by target so that each target is written by one thread
    {
      std::vector<long> start(nc + 1, 0);
      for (auto &pr : m2l)
        start[pr.first + 1]++;
      for (long c = 0; c < nc; c++)
        start[c + 1] += start[c];
      std::vector<long> src(m2l.size()), fill(start.begin(), start.end() - 1);
      for (auto &pr : m2l)
        src[fill[pr.first]++] = (long)pr.second;
#pragma omp parallel for schedule(dynamic, 4)
      for (long c = 0; c < nc; c++)
        for (long q = start[c]; q < start[c + 1]; q++)
          M2L(&L[c * K * 3], cells[c], &M[src[q] * K * 3], cells[src[q]]);
    }
    // P2P, grouped by target leaf
    {
      std::vector<long> start(nc + 1, 0);
      for (auto &pr : p2p)
        start[pr.first + 1]++;
      for (long c = 0; c < nc; c++)
        start[c + 1] += start[c];
      std::vector<long> src(p2p.size()), fill(start.begin(), start.end() - 1);
      for (auto &pr : p2p)
        src[fill[pr.first]++] = (long)pr.second;
      // the sums accumulate per source leaf, as the reference's team reduce does
#pragma omp parallel for schedule(dynamic, 4)
      for (long c = 0; c < nc; c++)
        for (long q = start[c]; q < start[c + 1]; q++) {
          const Cell &S = cells[src[q]];
          for (uint64_t i = cells[c].BodyOffset; i < cells[c].BodyOffset + cells[c].NBODY; i++)
            P2P_target(b[i], b, S.BodyOffset, S.BodyOffset + S.NBODY);
        }
    }
    // downward pass, levels 0..maxLevel: L2L into children, then L2P at leaves
    for (int lev = 0; lev <= maxLevel; lev++) {
      const std::vector<long> &ids = byLevel[lev];
#pragma omp parallel for schedule(dynamic, 4)
      for (long t = 0; t < (long)ids.size(); t++) {
        const long c = ids[t];
        if (parent[c] >= 0)
          L2L(c, parent[c]);
        if (cells[c].NCHILD == 0)
          for (uint64_t i = cells[c].BodyOffset; i < cells[c].BodyOffset + cells[c].NBODY; i++)
            L2P_body(&L[c * K * 3], cells[c], b[i]);
      }
    }
    // stretching (fmmCalculator.hpp:391-405) and rVPM terms (:407-418)
#pragma omp parallel for
    for (long i = 0; i < n; i++) {
      Body &q = b[i];
      for (int a = 0; a < 3; a++)
        for (int c = 0; c < 3; c++)
          q.dadt[a] += (stretching == 0 ? q.J[c][a] : q.J[a][c]) * q.alpha[c];
      if (formulation == 1) {
        const double na = std::sqrt(q.alpha[0] * q.alpha[0] + q.alpha[1] * q.alpha[1] + q.alpha[2] * q.alpha[2]);
        const double ah[3] = {q.alpha[0] / na, q.alpha[1] / na, q.alpha[2] / na};
        const double dot   = q.dadt[0] * ah[0] + q.dadt[1] * ah[1] + q.dadt[2] * ah[2];
        for (int a = 0; a < 3; a++)
          q.dadt[a] -= 3. / 5. * dot * ah[a];
        q.drdt -= 1.0 / 5.0 * q.radius / na * dot;
      }
    }
  }
};

// ---------------------------------------------------------------- time stepping
// Stage updates of fmmCalculator.hpp:493-711.  `h` is the step size dt.
static void storeInitialState(Body &q)
{
  for (int d = 0; d < 3; d++) {
    q.velocity_old[d] = 0;
    q.dadt_old[d]     = 0;
    q.X_old[d]        = q.X[d];
    q.alpha_old[d]    = q.alpha[d];
  }
  q.radius_old = q.radius;
}
static void stepEuler(Body &q, double h)
{
  for (int d = 0; d < 3; d++) {
    q.X[d] += q.velocity[d] * h;
    q.alpha[d] += q.dadt[d] * h;
  }
  q.radius += q.drdt * h;
}
static void stepRK21(Body &q, double h)
{
  for (int d = 0; d < 3; d++) {
    q.velocity_old[d] = q.velocity[d];
    q.dadt_old[d]     = q.dadt[d];
  }
  q.drdt_old = q.drdt;
  for (int d = 0; d < 3; d++) {
    q.X[d] += h * q.velocity_old[d];
    q.alpha[d] += h * q.dadt_old[d];
  }
  q.radius += h * q.drdt_old;
}
static void stepRK22(Body &q, double h)
{
  for (int d = 0; d < 3; d++) {
    q.velocity_old[d] = 0.5 * q.velocity[d] + 0.5 * q.velocity_old[d];
    q.dadt_old[d]     = 0.5 * q.dadt[d] + 0.5 * q.dadt_old[d];
  }
  q.drdt_old = 0.5 * q.drdt + 0.5 * q.drdt_old;
  for (int d = 0; d < 3; d++) {
    q.X[d]     = q.X_old[d] + h * q.velocity_old[d];
    q.alpha[d] = q.alpha_old[d] + h * q.dadt_old[d];
  }
  q.radius = q.radius_old + h * q.drdt_old;
}
// Williamson low-storage RK3: z = A z + dt f; y += B z
static void stepRK3(Body &q, double h, double A, double B, bool first)
{
  for (int d = 0; d < 3; d++) {
    q.velocity_old[d] = first ? h * q.velocity[d] : A * q.velocity_old[d] + h * q.velocity[d];
    q.dadt_old[d]     = first ? h * q.dadt[d] : A * q.dadt_old[d] + h * q.dadt[d];
  }
  q.drdt_old = first ? h * q.drdt : A * q.drdt_old + h * q.drdt;
  for (int d = 0; d < 3; d++) {
    q.X[d] += B * q.velocity_old[d];
    q.alpha[d] += B * q.dadt_old[d];
  }
  q.radius += B * q.drdt_old;
}
static void stepRK41(Body &q, double h)
{
  for (int d = 0; d < 3; d++) {
    q.velocity_old[d] = q.velocity[d];
    q.dadt_old[d]     = q.dadt[d];
  }
  q.drdt_old = q.drdt;
  for (int d = 0; d < 3; d++) {
    q.X[d] += 0.5 * h * q.velocity_old[d];
    q.alpha[d] += 0.5 * h * q.dadt_old[d];
  }
  q.radius += 0.5 * h * q.drdt_old;
}
// stages 2 and 3 (fmmCalculator.hpp:648-689); `c` is 0.5 in both stages of the
// reference (its stage 3 should use 1.0: the classical RK4 evaluates k4 at y + dt*k3)
static void stepRK4mid(Body &q, double h, double c)
{
  for (int d = 0; d < 3; d++) {
    q.velocity_old[d] += 2.0 * q.velocity[d];
    q.dadt_old[d] += 2.0 * q.dadt[d];
  }
  q.drdt_old += 2.0 * q.drdt;
  for (int d = 0; d < 3; d++) {
    q.X[d]     = q.X_old[d] + c * h * q.velocity[d];
    q.alpha[d] = q.alpha_old[d] + c * h * q.dadt[d];
  }
  q.radius = q.radius_old + c * h * q.drdt;
}
static void stepRK44(Body &q, double h)
{
  for (int d = 0; d < 3; d++) {
    q.velocity_old[d] += q.velocity[d];
    q.dadt_old[d] += q.dadt[d];
  }
  q.drdt_old += q.drdt;
  for (int d = 0; d < 3; d++) {
    q.X[d]     = q.X_old[d] + (h / 6.0) * q.velocity_old[d];
    q.alpha[d] = q.alpha_old[d] + (h / 6.0) * q.dadt_old[d];
  }
  q.radius = q.radius_old + (h / 6.0) * q.drdt_old;
}

// Pedrizzetti relaxation, the intent of relaxation.hpp:8-19 written 0-based:
// omega = curl u from J (J[a][b] = du_a/dx_b); alpha <- (1-f) alpha + f |alpha| omega/|omega|.
static void relax(Body &q, double f)
{
  const double w[3] = {q.J[2][1] - q.J[1][2], q.J[0][2] - q.J[2][0], q.J[1][0] - q.J[0][1]};
  const double nw   = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  const double na   = std::sqrt(q.alpha[0] * q.alpha[0] + q.alpha[1] * q.alpha[1] + q.alpha[2] * q.alpha[2]);
  if (nw == 0.0)
    return;
  for (int d = 0; d < 3; d++)
    q.alpha[d] = (1 - f) * q.alpha[d] + f * na * w[d] / nw;
}

} // namespace vo

using namespace vo;

extern "C" {

int vo_set_threads(int n)
{
#ifdef _OPENMP
  if (n > 0)
    omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

// Build the tree (bodies permuted into tree order); returns the cell count or -1 on depth overflow.
long vo_build_tree(Body *bodies, long n, int ncrit, Cell *cells, long cap)
{
  std::vector<Cell> c;
  if (!buildTree(bodies, n, ncrit, c))
    return -1;
  for (long i = 0; i < (long)c.size() && i < cap; i++)
    cells[i] = c[i];
  return (long)c.size();
}

// Interaction lists of a tree (target and source trees may differ).
int vo_lists(const Cell *tcells, const Cell *scells, double theta, uint64_t *p2p, long cap_p2p, long *np2p, uint64_t *m2l, long cap_m2l, long *nm2l)
{
  std::vector<Pair> a, b;
  getList(tcells, scells, theta, a, b);
  *np2p = (long)a.size();
  *nm2l = (long)b.size();
  for (long i = 0; i < *np2p && i < cap_p2p; i++) {
    p2p[2 * i]     = a[i].first;
    p2p[2 * i + 1] = a[i].second;
  }
  for (long i = 0; i < *nm2l && i < cap_m2l; i++) {
    m2l[2 * i]     = b[i].first;
    m2l[2 * i + 1] = b[i].second;
  }
  return 0;
}

// init + calculate; bodies are permuted into tree order and get velocity, J, dadt.
// M and L (optional) receive ncells * 3K complex values in the reference's layout.
int vo_calculate(Body *bodies, long n, int P, int ncrit, double theta, int stretching, int formulation, double *M, double *L, long cap_cells,
                 long *ncells)
{
  FMM f(P, ncrit, theta);
  f.stretching  = stretching;
  f.formulation = formulation;
  f.init(bodies, n);
  if (!f.ok)
    return -1;
  f.calculate(bodies, n);
  *ncells = (long)f.cells.size();
  if (M && L && (long)f.cells.size() <= cap_cells) {
    std::memcpy(M, f.M.data(), f.M.size() * sizeof(cd));
    std::memcpy(L, f.L.data(), f.L.size() * sizeof(cd));
  }
  return 0;
}

// FMMCalculator::advance (fmmCalculator.hpp:919-1005) `steps` times; scheme 0
// Euler, 1 RK2, 2 RK3, 3 RK4; rk4_fixed=1 uses dt (not 0.5 dt) in RK4 stage 3;
// relax_f > 0 applies relaxation after each step with the last stage's J;
// viscous 1 PSE / 2 CSM with viscosity nu after every calculate.
int vo_advance(Body *b, long n, int P, int ncrit, double theta, double dt, int steps, int scheme, int stretching, int formulation, double relax_f,
               int rk4_fixed, int viscous, double nu)
{
  FMM f(P, ncrit, theta);
  f.stretching  = stretching;
  f.formulation = formulation;
  auto stage    = [&](auto update) {
    f.init(b, n);
    if (!f.ok)
      return false;
    f.calculate(b, n);
    f.viscosity(b, n, viscous, nu, dt);
#pragma omp parallel for
    for (long i = 0; i < n; i++)
      update(b[i]);
    return true;
  };
  for (int s = 0; s < steps; s++) {
    bool ok = true;
    if (scheme == 0) {
      ok = stage([&](Body &q) { stepEuler(q, dt); });
    } else if (scheme == 1) {
      f.init(b, n);
      if (!f.ok)
        return -1;
      for (long i = 0; i < n; i++)
        storeInitialState(b[i]);
      f.calculate(b, n);
      f.viscosity(b, n, viscous, nu, dt);
      for (long i = 0; i < n; i++)
        stepRK21(b[i], dt);
      ok = stage([&](Body &q) { stepRK22(q, dt); });
    } else if (scheme == 2) {
      ok = stage([&](Body &q) { stepRK3(q, dt, 0.0, 1.0 / 3.0, true); }) && stage([&](Body &q) { stepRK3(q, dt, -5.0 / 9.0, 15.0 / 16.0, false); }) &&
           stage([&](Body &q) { stepRK3(q, dt, -153.0 / 128.0, 8.0 / 15.0, false); });
    } else if (scheme == 3) {
      f.init(b, n);
      if (!f.ok)
        return -1;
      for (long i = 0; i < n; i++)
        storeInitialState(b[i]);
      f.calculate(b, n);
      f.viscosity(b, n, viscous, nu, dt);
      for (long i = 0; i < n; i++)
        stepRK41(b[i], dt);
      ok = stage([&](Body &q) { stepRK4mid(q, dt, 0.5); }) && stage([&](Body &q) { stepRK4mid(q, dt, rk4_fixed ? 1.0 : 0.5); }) &&
           stage([&](Body &q) { stepRK44(q, dt); });
    } else {
      return -2;
    }
    if (!ok)
      return -1;
    if (relax_f > 0)
      for (long i = 0; i < n; i++)
        relax(b[i], relax_f);
  }
  return 0;
}

// init + calculate on the particles, then getSensorData (fmmCalculator.hpp:
// 117-161, 469-491, 726-731): a second tree over the sensors, traversal
// sensor-tree x particle-tree, M2L into sensor locals, velocity-only P2P
// (multipoleKernels.hpp:303-341), then the sensor downward pass (L2L + L2P,
// which also adds the far-field J).  Sensors come back permuted into their
// tree order; their velocity and dadt are reset first, J is not
// (fmmCalculator.hpp:380-389).
int vo_sensors(Body *b, long n, Body *s, long ns, int P, int ncrit, double theta)
{
  FMM f(P, ncrit, theta);
  f.init(b, n);
  if (!f.ok)
    return -1;
  f.calculate(b, n);
  FMM g(P, ncrit, theta);
  if (!buildTree(s, ns, ncrit, g.cells))
    return -1;
  getList(g.cells.data(), f.cells.data(), theta, g.p2p, g.m2l);
  g.L.assign(g.cells.size() * 3 * g.K, cd(0, 0));
  for (long i = 0; i < ns; i++)
    for (int d = 0; d < 3; d++)
      s[i].velocity[d] = s[i].dadt[d] = 0;
  const long nc = (long)g.cells.size();
  for (auto &pr : g.m2l)
    f.M2L(&g.L[pr.first * g.K * 3], g.cells[pr.first], &f.M[pr.second * f.K * 3], f.cells[pr.second]);
  for (auto &pr : g.p2p) {
    const Cell &T = g.cells[pr.first], &S = f.cells[pr.second];
    for (uint64_t i = T.BodyOffset; i < T.BodyOffset + T.NBODY; i++) {
      double sum[3] = {0, 0, 0};
      for (uint64_t j = S.BodyOffset; j < S.BodyOffset + S.NBODY; j++) {
        double dX[3];
        for (int d = 0; d < 3; d++)
          dX[d] = s[i].X[d] - b[j].X[d];
        const double R2 = dX[0] * dX[0] + dX[1] * dX[1] + dX[2] * dX[2];
        if (R2 != 0) {
          const double S2 = 2.0 * b[j].radius * b[j].radius, RS = R2 / S2, sq = std::sqrt(RS);
          const double t2 = 2.0 * inv_sqrtpi * sq * std::exp(-RS);
          const double cut = 0.25 * inv_pi / R2 * (1.0 / std::sqrt(R2)) * (std::erf(sq) - t2);
          sum[0] += (dX[1] * b[j].alpha[2] - dX[2] * b[j].alpha[1]) * cut;
          sum[1] += (dX[2] * b[j].alpha[0] - dX[0] * b[j].alpha[2]) * cut;
          sum[2] += (dX[0] * b[j].alpha[1] - dX[1] * b[j].alpha[0]) * cut;
        }
      }
      for (int d = 0; d < 3; d++)
        s[i].velocity[d] -= sum[d];
    }
  }
  int maxLevel = 0;
  for (long c = 0; c < nc; c++)
    maxLevel = std::max(maxLevel, (int)g.cells[c].level);
  std::vector<long> parent(nc, -1);
  for (long c = 0; c < nc; c++)
    for (uint64_t ch = g.cells[c].ChildOffset; ch < g.cells[c].ChildOffset + g.cells[c].NCHILD; ch++)
      parent[ch] = c;
  for (int lev = 0; lev <= maxLevel; lev++)
    for (long c = 0; c < nc; c++) {
      if ((int)g.cells[c].level != lev)
        continue;
      if (parent[c] >= 0)
        g.L2L(c, parent[c]);
      if (g.cells[c].NCHILD == 0)
        for (uint64_t i = g.cells[c].BodyOffset; i < g.cells[c].BodyOffset + g.cells[c].NBODY; i++)
          g.L2P_body(&g.L[c * g.K * 3], g.cells[c], s[i]);
    }
  return 0;
}

// FP64 all-pairs sum with the team-P2P formula (multipoleKernels.hpp:239-283):
// velocity and J for `nt` targets (each a copy of a body; X and radius read)
// from all `ns` sources; outputs overwrite the targets' velocity and J.
void vo_direct(Body *t, long nt, const Body *s, long ns)
{
#pragma omp parallel for schedule(dynamic, 16)
  for (long i = 0; i < nt; i++) {
    for (int d = 0; d < 3; d++)
      t[i].velocity[d] = 0;
    for (int a = 0; a < 3; a++)
      for (int c = 0; c < 3; c++)
        t[i].J[a][c] = 0;
    FMM::P2P_target(t[i], s, 0, (uint64_t)ns);
  }
}

// Model-consistent direct sum (the accuracy yardstick of the FMM): for each
// target body (index into the tree-order bodies), every other body
// contributes through the regularised kernel (multipoleKernels.hpp:239-283)
// when its leaf is on the target leaf's P2P list, else through the singular
// Biot-Savart kernel that the expansions represent (multipoleKernels.hpp:
// 519-552, :631-742).  out: nt records of 12 (velocity, J row-major).
void vo_direct_model(const Body *b, long n, const Cell *cells, long nc, const uint64_t *p2p, long np2p, const uint32_t *tgt, long nt,
                     double *out)
{
  std::vector<long> leaf_of(n, -1);
  for (long c = 0; c < nc; c++)
    if (cells[c].NCHILD == 0)
      for (uint64_t i = cells[c].BodyOffset; i < cells[c].BodyOffset + cells[c].NBODY; i++)
        leaf_of[i] = c;
#pragma omp parallel for schedule(dynamic, 4)
  for (long t = 0; t < nt; t++) {
    const Body       &bi = b[tgt[t]];
    const long        ct = leaf_of[tgt[t]];
    std::vector<char> near(nc, 0);
    for (long q = 0; q < np2p; q++)
      if ((long)p2p[2 * q] == ct)
        near[p2p[2 * q + 1]] = 1;
    double s[12] = {0};
    for (long j = 0; j < n; j++) {
      const Body &bj = b[j];
      double      dX[3];
      for (int d = 0; d < 3; d++)
        dX[d] = bi.X[d] - bj.X[d];
      const double R2 = dX[0] * dX[0] + dX[1] * dX[1] + dX[2] * dX[2];
      if (R2 == 0)
        continue;
      const double c4 = 0.25 * inv_pi / R2 / std::sqrt(R2);
      double       g = 1.0, aux = -3.0 / R2;
      if (near[leaf_of[j]]) {
        const double S2 = bj.radius * bj.radius, RS = R2 / S2 / 2.0, sq = std::sqrt(RS);
        const double t2 = 2.0 * inv_sqrtpi * sq * std::exp(-RS);
        g   = std::erf(sq) - t2;
        aux = t2 / S2 - 3.0 * g / R2;
      }
      const double cr[3] = {c4 * (dX[1] * bj.alpha[2] - dX[2] * bj.alpha[1]), c4 * (dX[2] * bj.alpha[0] - dX[0] * bj.alpha[2]),
                            c4 * (dX[0] * bj.alpha[1] - dX[1] * bj.alpha[0])};
      for (int a = 0; a < 3; a++)
        s[a] += cr[a] * g;
      for (int a = 0; a < 3; a++)
        for (int c = 0; c < 3; c++)
          s[3 + 3 * a + c] += aux * cr[a] * dX[c];
      const double a2 = g * c4;
      s[6] -= a2 * bj.alpha[2];
      s[9] += a2 * bj.alpha[1];
      s[4] += a2 * bj.alpha[2];
      s[10] -= a2 * bj.alpha[0];
      s[5] -= a2 * bj.alpha[1];
      s[8] += a2 * bj.alpha[0];
    }
    for (int k = 0; k < 12; k++)
      out[12 * t + k] = -s[k];
  }
}

// Time-step relaxation alone (on J already present in the bodies).
void vo_relax(Body *b, long n, double f)
{
  for (long i = 0; i < n; i++)
    relax(b[i], f);
}

} // extern "C"

extern "C" {
// L2P alone (complex-step form of multipoleKernels.hpp:630-742) for one body:
// local expansion Lc (3K complex, reference layout) about centre C, body at X;
// adds the far-field velocity (3) and J (9, row-major) into out[12].
void vo_l2p_body(int P, const double *Lc, const double *C, const double *X, double *out)
{
  vo::FMM f(P, 1, 0.5);
  vo::Cell c{};
  for (int d = 0; d < 3; d++)
    c.X[d] = C[d];
  vo::Body b{};
  for (int d = 0; d < 3; d++)
    b.X[d] = X[d];
  f.L2P_body(reinterpret_cast<const vo::cd *>(Lc), c, b);
  for (int d = 0; d < 3; d++)
    out[d] = b.velocity[d];
  for (int k = 0; k < 9; k++)
    out[3 + k] = b.J[k / 3][k % 3];
}
}

#include "complex_step.hpp"
