// Whole-step complex-step derivatives.  TEST INFRASTRUCTURE ONLY: the
// independent checker of the CUDA library's reverse-mode adjoint
// (vfmm_adjoint); the product never links or calls it.  Included at the end of
// vfmm_oracle.cpp, whose tree build and traversal it reuses.
//
// The reference differentiates by complex step only inside L2P (a step of
// 1e-32 through its `cplx` scalar, multipoleKernels.hpp:630-742,
// complexify.hpp).  Here the whole of advance (fmmCalculator.hpp:919-1005)
// and the objective run on a complex-step scalar following complexify.hpp's
// rules: arithmetic and sqrt/exp analytic, comparisons on the real part
// (complexify.hpp:130-218), and erf, which complexify lacks, to first order,
//   erf(a + i b) = erf(a) + i b (2 / sqrt(pi)) e^{-a^2}.
// A run from x0 + i h v (h = 1e-30) gives d objective / dv = Im / h with no
// truncation or cancellation error, and, unlike a finite difference, the
// real part (so every tree, list and MAC decision) is exactly the
// unperturbed run's.
//
// The evaluation is templated on the scalar: with T = double it is an FMM
// step whose tree and lists are the reference's (buildTree, getList above),
// with the expansions written in Cartesian form (regular and singular solid
// harmonics by recurrence, L2P derivatives as exact operators on the
// coefficients, the same M2L truncation j + n <= P - 1); vo_cs_advance
// exposes it for the check against vo_advance.  Cell centres and the
// bounding box are complex-step values: the box's extremes are chosen on
// real parts and carry their bodies' imaginary parts.

namespace vo {
namespace cstep {

struct CS {
  double r, i;
  CS() : r(0), i(0) {}
  CS(double a) : r(a), i(0) {}
  CS(double a, double b) : r(a), i(b) {}
};
inline CS  operator+(CS a, CS b) { return {a.r + b.r, a.i + b.i}; }
inline CS  operator-(CS a, CS b) { return {a.r - b.r, a.i - b.i}; }
inline CS  operator-(CS a) { return {-a.r, -a.i}; }
inline CS  operator*(CS a, CS b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
inline CS  operator/(CS a, CS b)
{
  const double d = b.r * b.r + b.i * b.i;
  return {(a.r * b.r + a.i * b.i) / d, (a.i * b.r - a.r * b.i) / d};
}
inline CS &operator+=(CS &a, CS b) { return a = a + b; }
inline CS &operator-=(CS &a, CS b) { return a = a - b; }
inline CS &operator*=(CS &a, CS b) { return a = a * b; }

inline double re(double x) { return x; }
inline double re(const CS &x) { return x.r; }
inline double sqrt_(double x) { return std::sqrt(x); }
inline CS     sqrt_(CS x)
{
  const std::complex<double> z = std::sqrt(std::complex<double>(x.r, x.i));
  return {z.real(), z.imag()};
}
inline double exp_(double x) { return std::exp(x); }
inline CS     exp_(CS x)
{
  const std::complex<double> z = std::exp(std::complex<double>(x.r, x.i));
  return {z.real(), z.imag()};
}
inline double erf_(double x) { return std::erf(x); }
inline CS     erf_(CS x) { return {std::erf(x.r), x.i * 2.0 * inv_sqrtpi * std::exp(-x.r * x.r)}; }

template <class T>
struct Cx {
  T a, b; // real, imaginary
};
template <class T> inline Cx<T> operator+(const Cx<T> &x, const Cx<T> &y) { return {x.a + y.a, x.b + y.b}; }
template <class T> inline Cx<T> operator*(const Cx<T> &x, const Cx<T> &y) { return {x.a * y.a - x.b * y.b, x.a * y.b + x.b * y.a}; }
template <class T> inline Cx<T> conj(const Cx<T> &x) { return {x.a, -x.b}; }
template <class T> inline Cx<T> neg_if(const Cx<T> &x, bool n) { return n ? Cx<T>{-x.a, -x.b} : x; }
template <class T> inline Cx<T> scale(const T &s, const Cx<T> &x) { return {s * x.a, s * x.b}; }

inline int tri(int n, int m) { return n * (n + 1) / 2 + m; }

// Regular solid harmonics Y_n^m (n < N, m >= 0) at tri(n, m): the reference's
// evalMultipole (multipoleKernels.hpp:53-92) by the recurrences
//   Y_m^m = Y_{m-1}^{m-1} (x + iy) / (2m),
//   Y_{n+1}^m = -((2n+1) z Y_n^m + r^2 Y_{n-1}^m) / ((n+m+1)(n-m+1)).
template <class T>
void regular(int N, T x, T y, T z, Cx<T> *Y)
{
  const T r2 = x * x + y * y + z * z;
  Cx<T>   dg{T(1.0), T(0.0)};
  for (int m = 0; m < N; m++) {
    if (m > 0) {
      const double s = 1.0 / (2.0 * m);
      dg             = {(dg.a * x - dg.b * y) * s, (dg.a * y + dg.b * x) * s};
    }
    Cx<T> a = dg, b{T(0.0), T(0.0)};
    Y[tri(m, m)] = a;
    for (int n = m; n + 1 < N; n++) {
      const double c  = -1.0 / double((n + m + 1) * (n - m + 1));
      const T      zz = double(2 * n + 1) * z;
      const Cx<T>  nx{c * (zz * a.a + r2 * b.a), c * (zz * a.b + r2 * b.b)};
      Y[tri(n + 1, m)] = nx;
      b                = a;
      a                = nx;
    }
  }
}

// Singular solid harmonics S_n^m (n < N, m >= 0): the reference's evalLocal
// (multipoleKernels.hpp:137-172) by S_0^0 = 1/r,
//   S_m^m = S_{m-1}^{m-1} (2m-1)(x + iy) / r^2,
//   S_{n+1}^m = -((2n+1) z S_n^m + (n+m)(n-m) S_{n-1}^m) / r^2.
template <class T>
void singular(int N, T x, T y, T z, Cx<T> *S)
{
  const T r2 = x * x + y * y + z * z, ir2 = T(1.0) / r2, s00 = sqrt_(ir2);
  for (int m = 0; m < N; m++) {
    Cx<T> d{s00, T(0.0)};
    for (int k = 1; k <= m; k++) {
      const T s = double(2 * k - 1) * ir2;
      d         = {(d.a * x - d.b * y) * s, (d.a * y + d.b * x) * s};
    }
    Cx<T> a = d, b{T(0.0), T(0.0)};
    S[tri(m, m)] = a;
    for (int n = m; n + 1 < N; n++) {
      const T      zz = double(2 * n + 1) * z;
      const double c2 = double((n + m) * (n - m));
      const Cx<T>  nx{-(zz * a.a + c2 * b.a) * ir2, -(zz * a.b + c2 * b.b) * ir2};
      S[tri(n + 1, m)] = nx;
      b                = a;
      a                = nx;
    }
  }
}

// Full-range coefficient of a real expansion stored for m >= 0, and the
// coefficient (n, mu) of its derivative along `axis`, from
//   dY_n^m/dz = -Y_{n-1}^m, (d/dx + i d/dy) Y_n^m = -Y_{n-1}^{m+1} (m >= 0),
//   (d/dx - i d/dy) Y_n^m = +-Y_{n-1}^{m-1}.
template <class T>
Cx<T> coef_full(const Cx<T> *c, int n, int m, int stride, int comp)
{
  if (m > 0)
    return c[tri(n, m) * stride + comp];
  if (m == 0)
    return {c[tri(n, 0) * stride + comp].a, T(0.0)};
  return conj(c[tri(n, -m) * stride + comp]);
}
template <class T>
Cx<T> deriv_coef(const Cx<T> *c, int n, int mu, int axis, int stride, int comp)
{
  if (axis == 2)
    return neg_if(coef_full(c, n + 1, mu, stride, comp), true);
  const double s = (mu - 1 >= 0) ? -1.0 : 1.0, t = (mu + 1 >= 1) ? 1.0 : -1.0;
  const Cx<T>  A = scale(T(s), coef_full(c, n + 1, mu - 1, stride, comp)), B = scale(T(t), coef_full(c, n + 1, mu + 1, stride, comp));
  if (axis == 0)
    return {0.5 * (A.a + B.a), 0.5 * (A.b + B.b)};
  return {0.5 * (A.b - B.b), -0.5 * (A.a - B.a)};
}

template <class T>
struct BodyT {
  T X[3], A[3], R, U[3], J[9], D[3], VO[3], DO[3], XO[3], AO[3], DR, RO, DRO;
};

template <class T>
struct Stepper {
  int                 P, ncrit, K, stretching, formulation = 0; // formulation 1: rVPM
  int                 viscous = 0;                              // 1 PSE, 2 CSM, with viscosity nu
  double              nu      = 0.0;
  double              theta;
  long                n;
  std::vector<BodyT<T>> b;
  std::vector<Cell>   cells;
  std::vector<Pair>   p2p, m2l;
  std::vector<T>      cx, cy, cz; // cell centres
  std::vector<Cx<T>>  M, L;
  std::vector<long>   parent;
  int                 maxLevel = 0;
  bool                ok       = true;

  // Tree of the real parts (buildTree permutes a real copy, whose order the
  // scalar state follows), lists by getList, complex-step cell centres.
  void tree()
  {
    std::vector<Body> rb(n);
    for (long i = 0; i < n; i++) {
      std::memset(&rb[i], 0, sizeof(Body));
      for (int d = 0; d < 3; d++) {
        rb[i].X[d]     = re(b[i].X[d]);
        rb[i].alpha[d] = re(b[i].A[d]);
      }
      rb[i].radius   = re(b[i].R);
      rb[i].drdt_old = (double)i;
    }
    // getBounds on the scalar state (tree.hpp:7-26), extremes chosen on real parts
    T mn[3], mx[3];
    for (int d = 0; d < 3; d++)
      mn[d] = mx[d] = b[0].X[d];
    for (long i = 0; i < n; i++)
      for (int d = 0; d < 3; d++) {
        if (re(b[i].X[d]) < re(mn[d]))
          mn[d] = b[i].X[d];
        if (re(b[i].X[d]) > re(mx[d]))
          mx[d] = b[i].X[d];
      }
    T X0[3], R0 = T(0.0);
    for (int d = 0; d < 3; d++)
      X0[d] = (mx[d] + mn[d]) / T(2.0);
    for (int d = 0; d < 3; d++) {
      if (re(X0[d] - mn[d]) > re(R0))
        R0 = X0[d] - mn[d];
      if (re(mx[d] - X0[d]) > re(R0))
        R0 = mx[d] - X0[d];
    }
    R0 = R0 * T(1.00001);
    ok = buildTree(rb.data(), n, ncrit, cells);
    if (!ok)
      return;
    std::vector<BodyT<T>> nb(n);
    for (long i = 0; i < n; i++)
      nb[i] = b[(long)rb[i].drdt_old];
    b.swap(nb);
    getList(cells.data(), cells.data(), theta, p2p, m2l);
    const long nc = (long)cells.size();
    cx.assign(nc, T(0.0));
    cy.assign(nc, T(0.0));
    cz.assign(nc, T(0.0));
    parent.assign(nc, -1);
    cx[0]    = X0[0];
    cy[0]    = X0[1];
    cz[0]    = X0[2];
    maxLevel = 0;
    for (long c = 0; c < nc; c++) { // children follow their parent in the cell array
      maxLevel = std::max(maxLevel, (int)cells[c].level);
      const T r = R0 * T(1.0 / double(1 << (cells[c].level + 1)));
      for (uint64_t ch = cells[c].ChildOffset; ch < cells[c].ChildOffset + cells[c].NCHILD; ch++) {
        parent[ch] = c;
        cx[ch]     = cx[c] + (cells[ch].X[0] > cells[c].X[0] ? r : -r);
        cy[ch]     = cy[c] + (cells[ch].X[1] > cells[c].X[1] ? r : -r);
        cz[ch]     = cz[c] + (cells[ch].X[2] > cells[c].X[2] ? r : -r);
      }
    }
  }

  // u, J and dalpha/dt of every body (fmmCalculator.hpp:420-467, 391-405).
  void evaluate()
  {
    const long nc = (long)cells.size();
    M.assign(nc * 3 * K, Cx<T>{T(0.0), T(0.0)});
    L.assign(nc * 3 * K, Cx<T>{T(0.0), T(0.0)});
    std::vector<std::vector<long>> byLevel(maxLevel + 1);
    for (long c = 0; c < nc; c++)
      byLevel[cells[c].level].push_back(c);
    // P2M (leaves below the root), multipoleKernels.hpp:452-477
#pragma omp parallel for schedule(dynamic, 4)
    for (long c = 0; c < nc; c++) {
      if (cells[c].NCHILD != 0 || cells[c].level == 0)
        continue;
      std::vector<Cx<T>> Y(K);
      for (uint64_t i = cells[c].BodyOffset; i < cells[c].BodyOffset + cells[c].NBODY; i++) {
        regular(P, b[i].X[0] - cx[c], b[i].X[1] - cy[c], b[i].X[2] - cz[c], Y.data());
        for (int t = 0; t < K; t++)
          for (int d = 0; d < 3; d++) {
            Cx<T> &o = M[(c * K + t) * 3 + d];
            o.a += b[i].A[d] * Y[t].a;
            o.b -= b[i].A[d] * Y[t].b;
          }
      }
    }
    // M2M into parents at levels maxLevel-1 .. 1, multipoleKernels.hpp:479-516
    for (int lev = maxLevel - 1; lev >= 1; lev--) {
      const std::vector<long> &ids = byLevel[lev];
#pragma omp parallel for schedule(dynamic, 4)
      for (long t = 0; t < (long)ids.size(); t++) {
        const long c = ids[t];
        std::vector<Cx<T>> Y(K);
        for (uint64_t ch = cells[c].ChildOffset; ch < cells[c].ChildOffset + cells[c].NCHILD; ch++) {
          regular(P, cx[c] - cx[ch], cy[c] - cy[ch], cz[c] - cz[ch], Y.data());
          const Cx<T> *Mc = &M[ch * 3 * K];
          for (int j = 0; j < P; j++)
            for (int k = 0; k <= j; k++)
              for (int d = 0; d < 3; d++) {
                Cx<T> acc{T(0.0), T(0.0)};
                for (int nn = 0; nn <= j; nn++) {
                  for (int m = std::max(-nn, -j + k + nn); m <= std::min(k - 1, nn); m++) {
                    const Cx<T> y   = Y[tri(nn, m > 0 ? m : -m)];
                    const bool  neg = ((m < 0 ? (m & 1) : 0) ^ (nn & 1)) != 0;
                    acc             = acc + neg_if(Mc[tri(j - nn, k - m) * 3 + d], neg) * (m > 0 ? conj(y) : y);
                  }
                  for (int m = k; m <= std::min(nn, j + k - nn); m++)
                    acc = acc + neg_if(conj(Mc[tri(j - nn, m - k) * 3 + d]), ((k + nn + m) & 1) != 0) * conj(Y[tri(nn, m)]);
                }
                Cx<T> &o = M[(c * K + tri(j, k)) * 3 + d];
                o        = o + acc;
              }
        }
      }
    }
    // M2L, multipoleKernels.hpp:518-552, truncated at j + n <= P - 1: with
    // M'_n^m = (-1)^m M_n^m (m >= 0), conj(M_n^|m|) (m < 0) and
    // S'_q^u = (-1)^u S_q^u (u >= 0), conj(S_q^|u|) (u < 0),
    //   L_j^k = (-1)^j sum_s sum_{n <= P-1-j} sum_m M'_n^m S'_{j+n}^{m-k}.
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
      for (long t = 0; t < nc; t++) {
        std::vector<Cx<T>> S(K), Sp(P * P), Mp(P * P * 3);
        for (long q = start[t]; q < start[t + 1]; q++) {
          const long s = src[q];
          singular(P, cx[t] - cx[s], cy[t] - cy[s], cz[t] - cz[s], S.data());
          for (int qq = 0; qq < P; qq++)
            for (int u = -qq; u <= qq; u++)
              Sp[qq * qq + qq + u] = u >= 0 ? neg_if(S[tri(qq, u)], u & 1) : conj(S[tri(qq, -u)]);
          for (int nn = 0; nn < P; nn++)
            for (int m = -nn; m <= nn; m++)
              for (int d = 0; d < 3; d++)
                Mp[(nn * nn + nn + m) * 3 + d] = m >= 0 ? neg_if(M[(s * K + tri(nn, m)) * 3 + d], m & 1) : conj(M[(s * K + tri(nn, -m)) * 3 + d]);
          for (int j = 0; j < P; j++)
            for (int k = 0; k <= j; k++)
              for (int d = 0; d < 3; d++) {
                Cx<T> acc{T(0.0), T(0.0)};
                for (int nn = 0; nn <= P - 1 - j; nn++) {
                  const int qq = j + nn;
                  for (int m = -nn; m <= nn; m++)
                    acc = acc + Mp[(nn * nn + nn + m) * 3 + d] * Sp[qq * qq + qq + m - k];
                }
                Cx<T> &o = L[(t * K + tri(j, k)) * 3 + d];
                o        = o + neg_if(acc, j & 1);
              }
        }
      }
    }
    // L2L from parents at levels 0 .. maxLevel-1, multipoleKernels.hpp:591-628
    for (int lev = 1; lev <= maxLevel; lev++) {
      const std::vector<long> &ids = byLevel[lev];
#pragma omp parallel for schedule(dynamic, 4)
      for (long t = 0; t < (long)ids.size(); t++) {
        const long   c = ids[t], p = parent[c];
        std::vector<Cx<T>> Y(K);
        regular(P, cx[c] - cx[p], cy[c] - cy[p], cz[c] - cz[p], Y.data());
        const Cx<T> *Lp = &L[p * 3 * K];
        for (int j = 0; j < P; j++)
          for (int k = 0; k <= j; k++)
            for (int d = 0; d < 3; d++) {
              Cx<T> acc{T(0.0), T(0.0)};
              for (int nn = j; nn < P; nn++) {
                for (int m = j + k - nn; m < 0; m++)
                  acc = acc + neg_if(conj(Lp[tri(nn, -m) * 3 + d]), k & 1) * conj(Y[tri(nn - j, k - m)]);
                for (int m = std::max(0, k - (nn - j)); m <= std::min(nn, k + (nn - j)); m++) {
                  const bool neg = m < k && ((k - m) & 1);
                  const Cx<T> y  = Y[tri(nn - j, m >= k ? m - k : k - m)];
                  acc            = acc + neg_if(Lp[tri(nn, m) * 3 + d], neg) * (m >= k ? y : conj(y));
                }
              }
              Cx<T> &o = L[(c * K + tri(j, k)) * 3 + d];
              o        = o + acc;
            }
      }
    }
    // L2P (u = curl psi / 4pi, J = grad u, exact derivative operators) and the
    // P2P near field (multipoleKernels.hpp:223-301), then the stretching term
    std::vector<long> start(nc + 1, 0);
    for (auto &pr : p2p)
      start[pr.first + 1]++;
    for (long c = 0; c < nc; c++)
      start[c + 1] += start[c];
    std::vector<long> src(p2p.size()), fill(start.begin(), start.end() - 1);
    for (auto &pr : p2p)
      src[fill[pr.first]++] = (long)pr.second;
    const double inv4pi = 0.25 * inv_pi;
    const int    N1 = P * (P - 1) / 2, N2 = P >= 3 ? (P - 1) * (P - 2) / 2 : 0;
#pragma omp parallel for schedule(dynamic, 4)
    for (long c = 0; c < nc; c++) {
      if (cells[c].NCHILD != 0)
        continue;
      const Cx<T>       *Lc = &L[c * 3 * K];
      std::vector<Cx<T>> U(3 * std::max(N1, 1)), JJ(9 * std::max(N2, 1)), Y(std::max(N1, 1));
      for (int nn = 0; nn <= P - 2; nn++)
        for (int mu = 0; mu <= nn; mu++)
          for (int ax = 0; ax < 3; ax++) {
            const int   b1 = (ax + 1) % 3, c1 = (ax + 2) % 3;
            const Cx<T> p = deriv_coef(Lc, nn, mu, b1, 3, c1), q = deriv_coef(Lc, nn, mu, c1, 3, b1);
            U[tri(nn, mu) * 3 + ax] = {inv4pi * (p.a - q.a), inv4pi * (p.b - q.b)};
          }
      for (int nn = 0; nn <= P - 3; nn++)
        for (int mu = 0; mu <= nn; mu++)
          for (int ae = 0; ae < 9; ae++)
            JJ[tri(nn, mu) * 9 + ae] = deriv_coef(U.data(), nn, mu, ae % 3, 3, ae / 3);
      for (uint64_t i = cells[c].BodyOffset; i < cells[c].BodyOffset + cells[c].NBODY; i++) {
        BodyT<T> &q = b[i];
        T         f[12];
        for (int k = 0; k < 12; k++)
          f[k] = T(0.0);
        if (P >= 2) {
          regular(P - 1, q.X[0] - cx[c], q.X[1] - cy[c], q.X[2] - cz[c], Y.data());
          for (int nn = 0; nn <= P - 2; nn++)
            for (int m = 0; m <= nn; m++) {
              const int    t = tri(nn, m);
              const double w = m == 0 ? 1.0 : 2.0;
              for (int ax = 0; ax < 3; ax++)
                f[ax] += w * (U[t * 3 + ax].a * Y[t].a - U[t * 3 + ax].b * Y[t].b);
              if (nn <= P - 3)
                for (int ae = 0; ae < 9; ae++)
                  f[3 + ae] += w * (JJ[t * 9 + ae].a * Y[t].a - JJ[t * 9 + ae].b * Y[t].b);
            }
        }
        T s[12];
        for (int k = 0; k < 12; k++)
          s[k] = T(0.0);
        for (long qq = start[c]; qq < start[c + 1]; qq++) {
          const Cell &S = cells[src[qq]];
          for (uint64_t j = S.BodyOffset; j < S.BodyOffset + S.NBODY; j++) {
            const BodyT<T> &bj = b[j];
            T               dX[3];
            for (int d = 0; d < 3; d++)
              dX[d] = q.X[d] - bj.X[d];
            const T R2 = dX[0] * dX[0] + dX[1] * dX[1] + dX[2] * dX[2];
            if (re(R2) != 0) {
              const T S2 = bj.R * bj.R, RS = R2 / S2 / T(2.0), sqrtRS = sqrt_(RS);
              const T erfS = erf_(sqrtRS), expm = exp_(-RS), invSqrtR2 = T(1.0) / sqrt_(R2);
              const T t2 = 2.0 * inv_sqrtpi * sqrtRS * expm, c4 = 0.25 * inv_pi / R2 * invSqrtR2;
              const T cr[3] = {c4 * (dX[1] * bj.A[2] - dX[2] * bj.A[1]), c4 * (dX[2] * bj.A[0] - dX[0] * bj.A[2]),
                               c4 * (dX[0] * bj.A[1] - dX[1] * bj.A[0])};
              const T g = erfS - t2;
              for (int a = 0; a < 3; a++)
                s[a] += cr[a] * g;
              T aux = t2 / S2 - 3.0 * g / R2;
              for (int a = 0; a < 3; a++)
                for (int bb = 0; bb < 3; bb++)
                  s[3 + 3 * a + bb] += aux * cr[a] * dX[bb];
              aux = g * c4;
              s[6] -= aux * bj.A[2];
              s[9] += aux * bj.A[1];
              s[4] += aux * bj.A[2];
              s[10] -= aux * bj.A[0];
              s[5] -= aux * bj.A[1];
              s[8] += aux * bj.A[0];
            }
          }
        }
        for (int a = 0; a < 3; a++)
          q.U[a] = f[a] - s[a];
        for (int k = 0; k < 9; k++)
          q.J[k] = f[3 + k] - s[3 + k];
      }
    }
#pragma omp parallel for
    for (long i = 0; i < n; i++) {
      BodyT<T> &q = b[i];
      for (int a = 0; a < 3; a++) {
        T v = T(0.0);
        for (int c = 0; c < 3; c++)
          v += (stretching == 0 ? q.J[3 * c + a] : q.J[3 * a + c]) * q.A[c];
        q.D[a] = v;
      }
      q.DR = T(0.0);
      if (formulation == 1) { // rVPM terms, fmmCalculator.hpp:407-418
        const T na    = sqrt_(q.A[0] * q.A[0] + q.A[1] * q.A[1] + q.A[2] * q.A[2]);
        const T ah[3] = {q.A[0] / na, q.A[1] / na, q.A[2] / na};
        const T dot   = q.D[0] * ah[0] + q.D[1] * ah[1] + q.D[2] * ah[2];
        for (int a = 0; a < 3; a++)
          q.D[a] -= T(3. / 5.) * dot * ah[a];
        q.DR -= T(1.0 / 5.0) * q.R / na * dot;
      }
    }
  }

  // The radius's share of the stage updates (as the strengths', with drdt).
  static void update_radius(BodyT<T> &q, int scheme, int stage, double h)
  {
    if (scheme == 0)
      q.R += q.DR * T(h);
    else if (scheme == 1 && stage == 0) {
      q.RO  = q.R;
      q.DRO = q.DR;
      q.R += T(h) * q.DRO;
    } else if (scheme == 1) {
      q.DRO = T(0.5) * q.DR + T(0.5) * q.DRO;
      q.R   = q.RO + T(h) * q.DRO;
    } else if (scheme >= 3 && stage == 0) {
      q.RO  = q.R;
      q.DRO = q.DR;
      q.R += T(0.5 * h) * q.DRO;
    } else if (scheme >= 3 && stage < 3) {
      const double c = (stage == 2 && scheme == 4) ? 1.0 : 0.5;
      q.DRO += T(2.0) * q.DR;
      q.R = q.RO + T(c * h) * q.DR;
    } else if (scheme >= 3) {
      q.DRO += q.DR;
      q.R = q.RO + T(h / 6.0) * q.DRO;
    } else {
      const double A = stage == 0 ? 0.0 : (stage == 1 ? -5.0 / 9.0 : -153.0 / 128.0);
      const double B = stage == 0 ? 1.0 / 3.0 : (stage == 1 ? 15.0 / 16.0 : 8.0 / 15.0);
      q.DRO          = stage == 0 ? T(h) * q.DR : T(A) * q.DRO + T(h) * q.DR;
      q.R += T(B) * q.DRO;
    }
  }

  // Stage updates of fmmCalculator.hpp:493-711: scheme 0 Euler, 1 RK2 Heun,
  // 2 RK3 low storage, 3 RK4 as the reference (its third stage steps by
  // 0.5*dt, :683-689), 4 RK4 with that stage stepping by dt.
  void update(int scheme, int stage, double h)
  {
#pragma omp parallel for
    for (long i = 0; i < n; i++) {
      BodyT<T> &q = b[i];
      update_radius(q, scheme, stage, h);
      for (int d = 0; d < 3; d++) {
        if (scheme == 0) {
          q.X[d] += q.U[d] * T(h);
          q.A[d] += q.D[d] * T(h);
        } else if (scheme == 1 && stage == 0) {
          q.XO[d] = q.X[d];
          q.AO[d] = q.A[d];
          q.VO[d] = q.U[d];
          q.DO[d] = q.D[d];
          q.X[d] += T(h) * q.VO[d];
          q.A[d] += T(h) * q.DO[d];
        } else if (scheme == 1) {
          q.VO[d] = T(0.5) * q.U[d] + T(0.5) * q.VO[d];
          q.DO[d] = T(0.5) * q.D[d] + T(0.5) * q.DO[d];
          q.X[d]  = q.XO[d] + T(h) * q.VO[d];
          q.A[d]  = q.AO[d] + T(h) * q.DO[d];
        } else if (scheme >= 3 && stage == 0) { // stepRK41 :629-649
          q.XO[d] = q.X[d];
          q.AO[d] = q.A[d];
          q.VO[d] = q.U[d];
          q.DO[d] = q.D[d];
          q.X[d] += T(0.5 * h) * q.VO[d];
          q.A[d] += T(0.5 * h) * q.DO[d];
        } else if (scheme >= 3 && stage < 3) { // stepRK42/43 :650-691
          const double c = (stage == 2 && scheme == 4) ? 1.0 : 0.5;
          q.VO[d] += T(2.0) * q.U[d];
          q.DO[d] += T(2.0) * q.D[d];
          q.X[d] = q.XO[d] + T(c * h) * q.U[d];
          q.A[d] = q.AO[d] + T(c * h) * q.D[d];
        } else if (scheme >= 3) { // stepRK44 :692-711
          q.VO[d] += q.U[d];
          q.DO[d] += q.D[d];
          q.X[d] = q.XO[d] + T(h / 6.0) * q.VO[d];
          q.A[d] = q.AO[d] + T(h / 6.0) * q.DO[d];
        } else {
          const double A = stage == 0 ? 0.0 : (stage == 1 ? -5.0 / 9.0 : -153.0 / 128.0);
          const double B = stage == 0 ? 1.0 / 3.0 : (stage == 1 ? 15.0 / 16.0 : 8.0 / 15.0);
          q.VO[d]        = stage == 0 ? T(h) * q.U[d] : T(A) * q.VO[d] + T(h) * q.U[d];
          q.DO[d]        = stage == 0 ? T(h) * q.D[d] : T(A) * q.DO[d] + T(h) * q.D[d];
          q.X[d] += T(B) * q.VO[d];
          q.A[d] += T(B) * q.DO[d];
        }
      }
    }
  }

  // Relaxation (relaxation.hpp:8-19, applied after the last stage as the
  // restatement does): alpha = (1 - f) alpha + f |alpha| w / |w| with
  // w = (J21 - J12, J02 - J20, J10 - J01); bodies with w = 0 keep alpha.
  void relax_all(double f)
  {
#pragma omp parallel for
    for (long i = 0; i < n; i++) {
      BodyT<T> &q    = b[i];
      const T   w[3] = {q.J[7] - q.J[5], q.J[2] - q.J[6], q.J[3] - q.J[1]};
      const T   nw2  = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
      if (re(nw2) == 0.0)
        continue;
      const T nw = sqrt_(nw2), na = sqrt_(q.A[0] * q.A[0] + q.A[1] * q.A[1] + q.A[2] * q.A[2]);
      for (int d = 0; d < 3; d++)
        q.A[d] = T(1 - f) * q.A[d] + T(f) * na * w[d] / nw;
    }
  }

  // calculateViscosity after an evaluation (fmmCalculator.hpp:713-724), as
  // the restatement does it: PSE (multipoleKernels.hpp:415-450) over the P2P
  // pairs, per target and source leaf sum (vol_i alpha_j - vol_j alpha_i)
  // e^{-R^2/(2 s^2)} / s^5, s^2 = sigma_i^2 + sigma_j^2, times nu / sqrt(2) /
  // pi / sqrt(pi) into dalpha/dt; CSM (fmmCalculator.hpp:334-337) adds
  // (sqrt(sigma^2 + 2 nu dt) - sigma) / dt to dr/dt.
  void viscosity(double dt)
  {
    if (viscous == 2) {
#pragma omp parallel for
      for (long i = 0; i < n; i++)
        b[i].DR += (sqrt_(b[i].R * b[i].R + T(2.0 * nu * dt)) - b[i].R) / T(dt);
      return;
    }
    if (viscous != 1)
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
    const double pi     = 3.14159265358979323846264338327950288;
    const double prefix = nu / 1.41421356237309504880168872420969808 * inv_pi * inv_sqrtpi;
#pragma omp parallel for schedule(dynamic, 4)
    for (long c = 0; c < nc; c++)
      for (long qq = start[c]; qq < start[c + 1]; qq++) {
        const Cell &S = cells[src[qq]];
        for (uint64_t i = cells[c].BodyOffset; i < cells[c].BodyOffset + cells[c].NBODY; i++) {
          T sum[3] = {T(0.0), T(0.0), T(0.0)};
          for (uint64_t j = S.BodyOffset; j < S.BodyOffset + S.NBODY; j++) {
            T dX[3];
            for (int d = 0; d < 3; d++)
              dX[d] = b[i].X[d] - b[j].X[d];
            const T R2 = dX[0] * dX[0] + dX[1] * dX[1] + dX[2] * dX[2];
            if (re(R2) != 0) {
              const T oo    = T(1.0) / (b[i].R * b[i].R + b[j].R * b[j].R);
              const T s5    = oo * oo * sqrt_(oo);
              const T vol_i = T(4. / 3. * pi) * b[i].R * b[i].R * b[i].R;
              const T vol_j = T(4. / 3. * pi) * b[j].R * b[j].R * b[j].R;
              const T e     = exp_(T(-0.5) * R2 * oo);
              for (int d = 0; d < 3; d++)
                sum[d] += (vol_i * b[j].A[d] - vol_j * b[i].A[d]) * e * s5;
            }
          }
          for (int d = 0; d < 3; d++)
            b[i].D[d] += sum[d] * T(prefix);
        }
      }
  }

  bool advance(int scheme, double dt, int steps, double relax = 0.0)
  {
    const int S = scheme == 0 ? 1 : (scheme == 1 ? 2 : (scheme == 2 ? 3 : 4));
    for (int st = 0; st < steps; st++)
      for (int k = 0; k < S; k++) {
        tree();
        if (!ok)
          return false;
        evaluate();
        viscosity(dt);
        update(scheme, k, dt);
        if (k == S - 1 && relax > 0)
          relax_all(relax);
      }
    return true;
  }

  // energy * sum u.(x cross alpha) + impulse . 1/2 sum x cross alpha on a fresh evaluation
  T objective(double wE, const double *wI)
  {
    tree();
    if (!ok)
      return T(0.0);
    evaluate();
    T v = T(0.0);
    for (long i = 0; i < n; i++) {
      const BodyT<T> &q = b[i];
      const T xa[3] = {q.X[1] * q.A[2] - q.X[2] * q.A[1], q.X[2] * q.A[0] - q.X[0] * q.A[2], q.X[0] * q.A[1] - q.X[1] * q.A[0]};
      for (int d = 0; d < 3; d++)
        v += T(wE) * q.U[d] * xa[d] + T(0.5 * wI[d]) * xa[d];
    }
    return v;
  }
};

template <class T>
void load(Stepper<T> &s, const Body *src, long n)
{
  s.n = n;
  s.b.assign(n, BodyT<T>{});
  for (long i = 0; i < n; i++) {
    for (int d = 0; d < 3; d++) {
      s.b[i].X[d] = T(src[i].X[d]);
      s.b[i].A[d] = T(src[i].alpha[d]);
    }
    s.b[i].R = T(src[i].radius);
  }
}

} // namespace cstep
} // namespace vo

extern "C" {

// The templated FMM step with T = double: `steps` steps of scheme 0 Euler,
// 1 RK2, 2 RK3, 3 RK4, 4 RK4 with a full-dt third stage (stretching 0
// transposed, 1 classic; formulation 0 cVPM, 1 rVPM; viscous 0 none, 1 PSE,
// 2 CSM with viscosity nu), relaxation factor `relax` after each step's last
// stage (0: none); b receives X, alpha, radius, drdt,
// velocity, J, dadt of the last stage in its tree order.  For the check
// against vo_advance.
int vo_cs_advance(Body *b, long n, int P, int ncrit, double theta, int scheme, int stretching, double dt, int steps, double relax, int formulation,
                  int viscous, double nu)
{
  using namespace vo::cstep;
  Stepper<double> s;
  s.P = P, s.ncrit = ncrit, s.K = P * (P + 1) / 2, s.stretching = stretching, s.theta = theta, s.formulation = formulation;
  s.viscous = viscous, s.nu = nu;
  load(s, b, n);
  if (!s.advance(scheme, dt, steps, relax))
    return -1;
  for (long i = 0; i < n; i++) {
    b[i].radius = s.b[i].R;
    b[i].drdt   = s.b[i].DR;
    for (int d = 0; d < 3; d++) {
      b[i].X[d]        = s.b[i].X[d];
      b[i].alpha[d]    = s.b[i].A[d];
      b[i].velocity[d] = s.b[i].U[d];
      b[i].dadt[d]     = s.b[i].D[d];
    }
    for (int k = 0; k < 9; k++)
      b[i].J[k / 3][k % 3] = s.b[i].J[k];
  }
  return 0;
}

// Objective after `steps` steps (see Stepper::objective) and, for each of nd
// directions (dirs_x, dirs_a: nd x n x 3, in the order of b), its directional
// derivative by complex step, with relaxation factor `relax` after each
// step's last stage (0: none), formulation and viscosity as vo_cs_advance.
// value gets the real objective.
int vo_cs_objective(const Body *b, long n, int P, int ncrit, double theta, int scheme, int stretching, double dt, int steps, double wE,
                    const double *wI, const double *dirs_x, const double *dirs_a, int nd, double *value, double *deriv, double relax,
                    int formulation, int viscous, double nu)
{
  using namespace vo::cstep;
  const double h = 1e-30;
  {
    Stepper<double> s;
    s.P = P, s.ncrit = ncrit, s.K = P * (P + 1) / 2, s.stretching = stretching, s.theta = theta, s.formulation = formulation;
    s.viscous = viscous, s.nu = nu;
    load(s, b, n);
    if (!s.advance(scheme, dt, steps, relax))
      return -1;
    *value = s.objective(wE, wI);
    if (!s.ok)
      return -1;
  }
  for (int k = 0; k < nd; k++) {
    Stepper<CS> s;
    s.P = P, s.ncrit = ncrit, s.K = P * (P + 1) / 2, s.stretching = stretching, s.theta = theta, s.formulation = formulation;
    s.viscous = viscous, s.nu = nu;
    load(s, b, n);
    for (long i = 0; i < n; i++)
      for (int d = 0; d < 3; d++) {
        s.b[i].X[d].i = h * dirs_x[((size_t)k * n + i) * 3 + d];
        s.b[i].A[d].i = h * dirs_a[((size_t)k * n + i) * 3 + d];
      }
    if (!s.advance(scheme, dt, steps, relax))
      return -1;
    const CS v = s.objective(wE, wI);
    if (!s.ok)
      return -1;
    deriv[k] = v.i / h;
  }
  return 0;
}
}
