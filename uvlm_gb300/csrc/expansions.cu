// FP64 expansion kernels: P2M, M2M, M2L, L2L and the fused L2P + P2P +
// stretching pass, restating src/multipoleKernels.hpp:223-742 and the
// stretching / rVPM functors of src/fmmCalculator.hpp:391-418.
//
// Layout: M and L are [cell][3*(n(n+1)/2+m) + d] complex doubles, as the
// reference stores them (multipoleKernels.hpp:468-471), n < P, 0 <= m <= n.
// Every kernel writes only what it owns (a leaf, a parent, a target cell or
// a target body); no atomics.
#include <algorithm>
#include "harmonics.cuh"
#include "vfmm_internal.cuh"

namespace vfmm {

typedef cx<double> zd;

static __constant__ HarmRecip<double> kHarmRecipD = make_harm_recip<double>();

__device__ __forceinline__ zd ldz(const double2 *p)
{
  const double2 v = *p;
  return {v.x, v.y};
}
__device__ __forceinline__ void stz(double2 *p, zd v) { *p = make_double2(v.r, v.i); }
__device__ __forceinline__ int  sgn_odd(int n) { return (n & 1) ? -1 : 1; } // oddOrEven, multipoleKernels.hpp:16-19
__device__ __forceinline__ int  ipow2n(int n) { return n >= 0 ? 1 : sgn_odd(n); }
__device__ __forceinline__ void jk_of(int jks, int &j, int &k)
{
  j = 0;
  while ((j + 1) * (j + 2) / 2 <= jks)
    j++;
  k = jks - j * (j + 1) / 2;
}

struct DevExp {
  CellsView     cv;  // target cells (L, L2P bodies)
  CellsView     scv; // source cells (M2L sources, P2P source leaves); cv except for sensors
  const double *soa;
  size_t        cap;
  const double *ssoa; // source bodies of P2P; soa except for sensors
  size_t        scap;
  const double2 *srcw; // per source body: 1/(2 sigma^2), 1/(sqrt(2) sigma)
  double2      *M, *L, *Mprep;
  const int    *leaf_cells;
  int           nleaves;
  const int    *m2l_start, *m2l_src;
  const int    *p2p_start, *p2p_src;
  const int4   *items;
  int           stretching, formulation;
};

// ------------------------------------------------------------------ P2M
// M_n^m += alpha_d conj(Y_n^m(x_b - X_c)) over the leaf's bodies
// (multipoleKernels.hpp:452-477).  Block of 64 threads per leaf; bodies in
// chunks of 32 whose harmonics are staged in shared memory.
template <int P>
__global__ void __launch_bounds__(64) k_p2m(DevExp a)
{
  constexpr int K = nterms(P), NO = (3 * K + 63) / 64;
  extern __shared__ double2 smem_raw[];
  zd     *Ys = reinterpret_cast<zd *>(smem_raw);
  double *As = reinterpret_cast<double *>(Ys + 32 * K);
  for (int li = blockIdx.x; li < a.nleaves; li += gridDim.x) {
    const int c = a.leaf_cells[li];
    if (a.cv.level[c] == 0)
      continue; // the reference's upward pass skips level 0 (fmmCalculator.hpp:427)
    const int    b0 = a.cv.body[c], nb = a.cv.nbody[c];
    const double cxx = a.cv.x[c], cyy = a.cv.y[c], czz = a.cv.z[c];
    zd           acc[NO];
#pragma unroll
    for (int i = 0; i < NO; i++)
      acc[i] = {0, 0};
    for (int c0 = 0; c0 < nb; c0 += 32) {
      const int nbc = min(32, nb - c0);
      const int t   = threadIdx.x;
      if (t < nbc) {
        const int b = b0 + c0 + t;
        regular_harmonics<double, P>(a.soa[F_X * a.cap + b] - cxx, a.soa[(F_X + 1) * a.cap + b] - cyy, a.soa[(F_X + 2) * a.cap + b] - czz,
                                     Ys + t * K);
        for (int d = 0; d < 3; d++)
          As[t * 3 + d] = a.soa[(F_A + d) * a.cap + b];
      }
      __syncthreads();
#pragma unroll
      for (int i = 0; i < NO; i++) {
        const int o = threadIdx.x + 64 * i;
        if (o < 3 * K) {
          const int nms = o / 3, d = o % 3;
          for (int tt = 0; tt < nbc; tt++) {
            const zd     y  = Ys[tt * K + nms];
            const double al = As[tt * 3 + d];
            acc[i].r        = fma(al, y.r, acc[i].r);
            acc[i].i        = fma(-al, y.i, acc[i].i);
          }
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < NO; i++) {
      const int o = threadIdx.x + 64 * i;
      if (o < 3 * K)
        stz(a.M + (size_t)c * 3 * K + o, acc[i]);
    }
  }
}

// ------------------------------------------------------------------ M2M
// Parent pulls its children's multipoles (multipoleKernels.hpp:479-516),
// dX = X_parent - X_child.  Block of 128 threads per parent: all children's
// multipoles (contiguous, the children form one block of cells) and their
// harmonics are staged once; each thread then sums its outputs over all
// children without further synchronisation.
template <int P>
__global__ void __launch_bounds__(128) k_m2m(DevExp a, const int *cells, int count)
{
  constexpr int K = nterms(P);
  extern __shared__ double2 smem_raw[];
  zd *Ms = reinterpret_cast<zd *>(smem_raw); // [8][3K]
  zd *Ys = Ms + 8 * 3 * K;                   // [8][K]
  for (int pi = blockIdx.x; pi < count; pi += gridDim.x) {
    const int c = cells[pi], nch = a.cv.nchild[c], ch0 = a.cv.child[c];
    if (nch == 0)
      continue;
    __syncthreads();
    for (int e = threadIdx.x; e < nch * 3 * K; e += blockDim.x)
      Ms[e] = ldz(a.M + (size_t)ch0 * 3 * K + e);
    if (threadIdx.x < nch) {
      const int ch = ch0 + threadIdx.x;
      regular_harmonics<double, P>(a.cv.x[c] - a.cv.x[ch], a.cv.y[c] - a.cv.y[ch], a.cv.z[c] - a.cv.z[ch], Ys + threadIdx.x * K);
    }
    __syncthreads();
    for (int o = threadIdx.x; o < 3 * K; o += blockDim.x) {
      const int jks = o / 3, d = o % 3;
      int       j, k;
      jk_of(jks, j, k);
      zd acc[4] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
      for (int t0 = 0; t0 < nch; t0 += 4)
        m2m_term_sum<P, 4>(j, k, d, Ms, Ys, t0, nch, acc);
      double2 *p = a.M + (size_t)c * 3 * K + o;
      stz(p, ldz(p) + ((acc[0] + acc[1]) + (acc[2] + acc[3])));
    }
  }
}

// ------------------------------------------------------------------ M2L
// Prepared multipoles for M2L: M'_n^m = (-1)^m M_n^m (m >= 0),
// conj(M_n^|m|) (m < 0), at [cell][n^2+n+m][d].  With the singular harmonics
// folded the same way, S'_q^u = (-1)^u S_q^u (u > 0), conj(S_q^|u|) (u <= 0),
// the reference's M2L (multipoleKernels.hpp:518-552) reads
//   L_j^k = (-1)^j sum_{n <= P-1-j} sum_{m=-n..n} M'_n^m S'_{j+n}^{m-k}.
template <int P>
__global__ void k_mprep(const double2 *__restrict__ M, double2 *__restrict__ Mp, int ncells)
{
  constexpr int K = nterms(P), PP = P * P;
  const long    total = (long)ncells * PP * 3;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const int  c = (int)(e / (PP * 3)), r = (int)(e % (PP * 3)), idx = r / 3, d = r % 3;
    int        n = 0;
    while ((n + 1) * (n + 1) <= idx)
      n++;
    const int m = idx - n * n - n;
    zd        v = ldz(M + (size_t)c * 3 * K + tri(n, m >= 0 ? m : -m) * 3 + d);
    if (m >= 0) {
      if (m & 1)
        v = {-v.r, -v.i};
    } else
      v = conj(v);
    stz(Mp + e, v);
  }
}

// One warp per target cell, 4 warps per block.  Each lane owns up to MAXI
// work items (j, k0..k0+kb-1, n0..n1) from a balanced static schedule and
// keeps their partial sums for all 3 components in registers across the
// target's whole source list; partials are combined once per target.
template <int P, int KB, int MAXI>
__global__ void __launch_bounds__(128) k_m2l(DevExp a, int ncells)
{
  constexpr int K = nterms(P), PP = P * P;
  extern __shared__ double2 smem_raw[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  zd       *Ms = reinterpret_cast<zd *>(smem_raw) + w * (4 * PP);
  zd       *Ys = Ms + 3 * PP;
  int4      it[MAXI];
#pragma unroll
  for (int i = 0; i < MAXI; i++)
    it[i] = a.items[i * 32 + lane];
  for (int t = blockIdx.x * 4 + w; t < ncells; t += gridDim.x * 4) {
    zd acc[MAXI][KB][3];
#pragma unroll
    for (int i = 0; i < MAXI; i++)
#pragma unroll
      for (int kk = 0; kk < KB; kk++)
#pragma unroll
        for (int d = 0; d < 3; d++)
          acc[i][kk][d] = {0, 0};
    const int    q0 = a.m2l_start[t], q1 = a.m2l_start[t + 1];
    const double tx = a.cv.x[t], ty = a.cv.y[t], tz = a.cv.z[t];
    for (int q = q0; q < q1; q++) {
      const int s = a.m2l_src[q];
      __syncwarp();
      for (int e = lane; e < 3 * PP; e += 32)
        Ms[e] = ldz(a.Mprep + (size_t)s * 3 * PP + e);
      if (lane < P) {
        const double dx = tx - a.scv.x[s], dy = ty - a.scv.y[s], dz = tz - a.scv.z[s];
        const double r2 = dx * dx + dy * dy + dz * dz, ir2 = 1.0 / r2, S00 = sqrt(ir2);
        zd           col[P];
        singular_column<double, P>(lane, dx, dy, dz, ir2, S00, col);
        const int m = lane;
        for (int n = m; n < P; n++) {
          const zd v = col[n];
          Ys[n * n + n + m] = (m & 1) ? zd{-v.r, -v.i} : v;
          if (m > 0)
            Ys[n * n + n - m] = conj(v);
        }
      }
      __syncwarp();
#pragma unroll
      for (int i = 0; i < MAXI; i++) {
        const int j = it[i].x;
        if (j < 0)
          continue;
        const int k0 = it[i].y & 255, kb = it[i].y >> 8, n0 = it[i].z, n1 = it[i].w;
        for (int n = n0; n <= n1; n++) {
          const int base = (j + n) * (j + n) + (j + n) - k0;
          for (int m = -n; m <= n; m++) {
            const zd m0 = Ms[(n * n + n + m) * 3 + 0], m1 = Ms[(n * n + n + m) * 3 + 1], m2 = Ms[(n * n + n + m) * 3 + 2];
#pragma unroll
            for (int kk = 0; kk < KB; kk++) {
              if (kk < kb) {
                const zd y = Ys[base + m - kk];
                cfma(acc[i][kk][0], m0, y);
                cfma(acc[i][kk][1], m1, y);
                cfma(acc[i][kk][2], m2, y);
              }
            }
          }
        }
      }
    }
    // combine partials in a fixed lane order (deterministic), then store
    __syncwarp();
    zd *Lr = Ms;
    for (int e = lane; e < 3 * K; e += 32)
      Lr[e] = {0, 0};
    __syncwarp();
    for (int src = 0; src < 32; src++) {
      if (lane == src) {
#pragma unroll
        for (int i = 0; i < MAXI; i++) {
          const int j = it[i].x;
          if (j < 0)
            continue;
          const int k0 = it[i].y & 255, kb = it[i].y >> 8;
#pragma unroll
          for (int kk = 0; kk < KB; kk++)
            if (kk < kb)
              for (int d = 0; d < 3; d++) {
                zd &o = Lr[tri(j, k0 + kk) * 3 + d];
                o     = o + acc[i][kk][d];
              }
        }
      }
      __syncwarp();
    }
    for (int e = lane; e < 3 * K; e += 32) {
      int j, k;
      jk_of(e / 3, j, k);
      zd v = Lr[e];
      if (j & 1)
        v = {-v.r, -v.i};
      stz(a.L + (size_t)t * 3 * K + e, v);
    }
  }
}

// ------------------------------------------------------------------ L2L
// Children pull their parent's local expansion (multipoleKernels.hpp:591-628),
// dX = X_child - X_parent.  Block of 128 threads per parent: the parent's L
// and all children's harmonics are staged once; threads own (child, output).
template <int P>
__global__ void __launch_bounds__(128) k_l2l(DevExp a, const int *cells, int count)
{
  constexpr int K = nterms(P);
  extern __shared__ double2 smem_raw[];
  zd *Ls = reinterpret_cast<zd *>(smem_raw); // [3K]
  zd *Ys = Ls + 3 * K;                       // [8][K]
  for (int pi = blockIdx.x; pi < count; pi += gridDim.x) {
    const int p = cells[pi], nch = a.cv.nchild[p], ch0 = a.cv.child[p];
    if (nch == 0)
      continue;
    __syncthreads();
    for (int e = threadIdx.x; e < 3 * K; e += blockDim.x)
      Ls[e] = ldz(a.L + (size_t)p * 3 * K + e);
    if (threadIdx.x < nch) {
      const int ch = ch0 + threadIdx.x;
      regular_harmonics<double, P>(a.cv.x[ch] - a.cv.x[p], a.cv.y[ch] - a.cv.y[p], a.cv.z[ch] - a.cv.z[p], Ys + threadIdx.x * K);
    }
    __syncthreads();
    const int ngroups = (nch + 3) / 4;
    for (int o = threadIdx.x; o < ngroups * 3 * K; o += blockDim.x) {
      const int t0 = (o / (3 * K)) * 4, r = o % (3 * K), jks = r / 3, d = r % 3;
      int       j, k;
      jk_of(jks, j, k);
      zd acc[4] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
      l2l_term_sum<P, 4>(j, k, d, Ls, Ys, t0, nch, acc);
#pragma unroll
      for (int c = 0; c < 4; c++)
        if (t0 + c < nch) {
          double2 *q = a.L + (size_t)(ch0 + t0 + c) * 3 * K + r;
          stz(q, ldz(q) + acc[c]);
        }
    }
  }
}

// ------------------------------------------------------------------ L2P + P2P
// Far field: u = (1/4pi) curl psi and J = grad u from the leaf's local
// expansion psi (the reference's L2P, multipoleKernels.hpp:630-742, which takes
// the gradient by a complex step).  Here the derivatives are exact operators
// on the coefficients (see harmonics.cuh): U_a = (1/4pi) eps_abc D_b psi_c
// (degree P-2) and J_ae = D_e U_a (degree P-3) are formed once per leaf and
// evaluated at each body.
// Near field: the regularised Biot-Savart sums of the reference's team P2P
// (multipoleKernels.hpp:223-301) over the leaf's P2P list.
// Then the stretching term (fmmCalculator.hpp:391-405) and rVPM terms
// (:407-418) from the complete u and J.

template <int P>
struct L2PSizes {
  static constexpr int K  = nterms(P);
  static constexpr int K1 = nterms(P - 1) > 0 ? nterms(P - 1) : 1; // degree <= P-2
  static constexpr int K2 = nterms(P - 2) > 0 ? nterms(P - 2) : 1; // degree <= P-3
  static constexpr size_t bytes = (size_t)(3 * K + 3 * K1 + 9 * K2) * sizeof(zd) + 2 * 128 * 12 * sizeof(double);
};

// SENS = false: the bodies' own evaluation; velocity and J are overwritten
// and dadt/drdt completed by the stretching (and rVPM) functors.
// SENS = true: sensor points (fmmCalculator.hpp:469-491): the near field is
// the velocity-only P2P of multipoleKernels.hpp:304-338 against the particle
// leaves, the far field is L2P (multipoleKernels.hpp:631-742), which adds to
// J; velocity and dadt start from zero (resetSensors, fmmCalculator.hpp:380-
// 389), J and drdt keep their input values.
template <int P, bool SENS>
__global__ void __launch_bounds__(128) k_l2p_p2p(DevExp a, double *out)
{
  using S = L2PSizes<P>;
  constexpr int K = S::K, K1 = S::K1, K2 = S::K2;
  constexpr int D1 = P - 1; // degrees of U: 0..P-2
  constexpr int D2 = P - 2; // degrees of J: 0..P-3
  extern __shared__ double2 smem_raw[];
  zd     *Lc  = reinterpret_cast<zd *>(smem_raw);
  zd     *U   = Lc + 3 * K;  // [tri][3]
  zd     *JJ  = U + 3 * K1;  // [tri][9]
  double *far = reinterpret_cast<double *>(JJ + 9 * K2);
  double *red = far + 128 * 12;
  const double inv4pi = 0.25 * 0.318309886183790671537767526745028724;
  const double inv_sqrtpi = 0.564189583547756286948079451560772586;
  const double inv_pi     = 0.318309886183790671537767526745028724;

  for (int li = blockIdx.x; li < a.nleaves; li += gridDim.x) {
    const int    c = a.leaf_cells[li];
    const int    b0 = a.cv.body[c], nb = a.cv.nbody[c];
    const double cxx = a.cv.x[c], cyy = a.cv.y[c], czz = a.cv.z[c];
    __syncthreads();
    for (int e = threadIdx.x; e < 3 * K; e += 128)
      Lc[e] = ldz(a.L + (size_t)c * 3 * K + e);
    __syncthreads();
    // U_a = inv4pi * eps_abc D_b psi_c
    if (D1 > 0)
      for (int e = threadIdx.x; e < 3 * nterms(D1); e += 128) {
        const int idx = e / 3, ax = e % 3;
        int       n, mu;
        jk_of(idx, n, mu);
        const int b1 = (ax + 1) % 3, c1 = (ax + 2) % 3; // u_a = D_{a+1} psi_{a+2} - D_{a+2} psi_{a+1}
        const zd  p = deriv_coef(Lc, n, mu, b1, 3, c1), q = deriv_coef(Lc, n, mu, c1, 3, b1);
        U[idx * 3 + ax] = {inv4pi * (p.r - q.r), inv4pi * (p.i - q.i)};
      }
    __syncthreads();
    if (D2 > 0)
      for (int e = threadIdx.x; e < 9 * nterms(D2); e += 128) {
        const int idx = e / 9, ae = e % 9, ax = ae / 3, ex = ae % 3;
        int       n, mu;
        jk_of(idx, n, mu);
        JJ[idx * 9 + ae] = deriv_coef(U, n, mu, ex, 3, ax);
      }
    __syncthreads();

    for (int tc = 0; tc < nb; tc += 128) {
      const int nbc = min(128, nb - tc);
      // far field at each target of the chunk
      if (threadIdx.x < nbc) {
        const int b = b0 + tc + threadIdx.x;
        const double x = a.soa[F_X * a.cap + b] - cxx, y = a.soa[(F_X + 1) * a.cap + b] - cyy, z = a.soa[(F_X + 2) * a.cap + b] - czz;
        const double r2 = x * x + y * y + z * z;
        double       f[12];
        for (int k = 0; k < 12; k++)
          f[k] = 0;
        zd diag{1.0, 0.0};
        for (int m = 0; m < D1; m++) {
          if (m > 0) {
            const double s = kHarmRecipD.s[m];
            diag           = {(diag.r * x - diag.i * y) * s, (diag.r * y + diag.i * x) * s};
          }
          const double w  = m == 0 ? 1.0 : 2.0;
          zd           ya = diag, yb{0, 0};
          double       tn = double(2 * m + 1); // 2n + 1
          for (int n = m; n < D1; n++, tn += 2.0) {
            const int t = tri(n, m);
            for (int ax = 0; ax < 3; ax++) {
              const zd u = U[t * 3 + ax];
              f[ax] += w * (u.r * ya.r - u.i * ya.i);
            }
            if (n < D2)
              for (int ae = 0; ae < 9; ae++) {
                const zd u = JJ[t * 9 + ae];
                f[3 + ae] += w * (u.r * ya.r - u.i * ya.i);
              }
            const double cc = kHarmRecipD.c[t];
            const double zz = tn * z;
            const zd     nx = {cc * (zz * ya.r + r2 * yb.r), cc * (zz * ya.i + r2 * yb.i)};
            yb              = ya;
            ya              = nx;
          }
        }
        for (int k = 0; k < 12; k++)
          far[threadIdx.x * 12 + k] = f[k];
      }
      // near field: 128 threads = G groups x TG targets
      const int TG = nbc <= 32 ? 32 : (nbc <= 64 ? 64 : 128), G = 128 / TG;
      const int tt = threadIdx.x % TG, g = threadIdx.x / TG;
      double    s[12];
      for (int k = 0; k < 12; k++)
        s[k] = 0;
      if (tt < nbc) {
        const int    i  = b0 + tc + tt;
        const double xi = a.soa[F_X * a.cap + i], yi = a.soa[(F_X + 1) * a.cap + i], zi = a.soa[(F_X + 2) * a.cap + i];
        const int    q0 = a.p2p_start[c], q1 = a.p2p_start[c + 1];
        for (int q = q0 + g; q < q1; q += G) {
          const int sc = a.p2p_src[q], sb = a.scv.body[sc], sn = a.scv.nbody[sc];
          const double *__restrict__ src = a.ssoa;
          const size_t scap = a.scap;
          for (int jb = sb; jb < sb + sn; jb++) {
            const double dx = xi - src[F_X * scap + jb], dy = yi - src[(F_X + 1) * scap + jb], dz = zi - src[(F_X + 2) * scap + jb];
            const double R2 = dx * dx + dy * dy + dz * dz;
            if (R2 != 0) {
              const double ax = src[F_A * scap + jb], ay = src[(F_A + 1) * scap + jb], az = src[(F_A + 2) * scap + jb];
              // the source's w2 = 1/(2 sigma^2) and s = sqrt(w2) made once per
              // evaluation (k_src_weights): no FP64 division or square root per
              // pair on GB300's narrow FP64 pipe, only one reciprocal square root
              const double2 ws = a.srcw[jb];
              const double  w2 = ws.x, RS = R2 * w2, invSqrtR2 = rsqrt(R2), iR2 = invSqrtR2 * invSqrtR2;
              const double  sqrtRS = R2 * invSqrtR2 * ws.y;
              const double  erfS = erf(sqrtRS), expm = exp(-RS);
              const double t2 = 2.0 * inv_sqrtpi * sqrtRS * expm, c4 = 0.25 * inv_pi * iR2 * invSqrtR2;
              const double cr0 = c4 * (dy * az - dz * ay), cr1 = c4 * (dz * ax - dx * az), cr2 = c4 * (dx * ay - dy * ax);
              const double gg  = erfS - t2;
              s[0] += cr0 * gg;
              s[1] += cr1 * gg;
              s[2] += cr2 * gg;
              if (SENS)
                continue;
              double aux = t2 * (2.0 * w2) - 3.0 * gg * iR2;
              s[3] += aux * cr0 * dx;
              s[4] += aux * cr0 * dy;
              s[5] += aux * cr0 * dz;
              s[6] += aux * cr1 * dx;
              s[7] += aux * cr1 * dy;
              s[8] += aux * cr1 * dz;
              s[9] += aux * cr2 * dx;
              s[10] += aux * cr2 * dy;
              s[11] += aux * cr2 * dz;
              aux = gg * c4;
              s[6] -= aux * az;
              s[9] += aux * ay;
              s[4] += aux * az;
              s[10] -= aux * ax;
              s[5] -= aux * ay;
              s[8] += aux * ax;
            }
          }
        }
      }
      for (int k = 0; k < 12; k++)
        red[threadIdx.x * 12 + k] = s[k];
      __syncthreads();
      if (threadIdx.x < nbc) {
        const int t = threadIdx.x, b = b0 + tc + t;
        double    r[12];
        for (int k = 0; k < 12; k++) {
          double nearv = 0;
          for (int gg = 0; gg < G; gg++)
            nearv += red[(gg * TG + t) * 12 + k];
          r[k] = far[t * 12 + k] - nearv;
        }
        if (SENS) {
          for (int d = 0; d < 3; d++) {
            out[(F_U + d) * a.cap + b]    = r[d];
            out[(F_DADT + d) * a.cap + b] = 0.0;
          }
          for (int k = 0; k < 9; k++)
            out[(F_J + k) * a.cap + b] = a.soa[(F_J + k) * a.cap + b] + far[t * 12 + 3 + k];
        } else {
          const double al[3] = {a.soa[F_A * a.cap + b], a.soa[(F_A + 1) * a.cap + b], a.soa[(F_A + 2) * a.cap + b]};
          double       dadt[3];
          for (int aa = 0; aa < 3; aa++) {
            double v = 0;
            for (int cc = 0; cc < 3; cc++)
              v += (a.stretching == VFMM_TRANSPOSED ? r[3 + 3 * cc + aa] : r[3 + 3 * aa + cc]) * al[cc];
            dadt[aa] = v;
          }
          double drdt = 0;
          if (a.formulation == VFMM_RVPM) {
            const double na = sqrt(al[0] * al[0] + al[1] * al[1] + al[2] * al[2]);
            const double ah[3] = {al[0] / na, al[1] / na, al[2] / na};
            const double dot   = dadt[0] * ah[0] + dadt[1] * ah[1] + dadt[2] * ah[2];
            for (int aa = 0; aa < 3; aa++)
              dadt[aa] -= 3. / 5. * dot * ah[aa];
            drdt -= 1.0 / 5.0 * a.soa[F_R * a.cap + b] / na * dot;
          }
          for (int d = 0; d < 3; d++) {
            out[(F_U + d) * a.cap + b]    = r[d];
            out[(F_DADT + d) * a.cap + b] = dadt[d];
          }
          for (int k = 0; k < 9; k++)
            out[(F_J + k) * a.cap + b] = r[3 + k];
          out[F_DRDT * a.cap + b] = drdt;
        }
      }
      __syncthreads();
    }
  }
}

// Per P2P source body: w2 = 1/(2 sigma^2) and s = sqrt(w2) = 1/(sqrt(2) sigma).
__global__ void k_src_weights(const double *__restrict__ soa, size_t cap, int n, double2 *w)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double sg = soa[F_R * cap + i], w2 = 0.5 / (sg * sg);
    w[i]            = make_double2(w2, sqrt(w2));
  }
}

// ------------------------------------------------------------------ host side
static DevExp dev_args(const ExpArgs &e)
{
  DevExp d;
  d.cv          = e.cells;
  d.scv         = e.src_soa ? e.src_cells : e.cells;
  d.soa         = e.soa;
  d.cap         = e.cap;
  d.ssoa        = e.src_soa ? e.src_soa : e.soa;
  d.scap        = e.src_soa ? e.src_cap : e.cap;
  d.srcw        = e.srcw;
  d.M           = e.M;
  d.L           = e.L;
  d.Mprep       = e.Mprep;
  d.leaf_cells  = e.leaf_cells;
  d.nleaves     = e.nleaves;
  d.m2l_start   = e.m2l_start;
  d.m2l_src     = e.m2l_src;
  d.p2p_start   = e.p2p_start;
  d.p2p_src     = e.p2p_src;
  d.items       = e.m2l_items;
  d.stretching  = e.stretching;
  d.formulation = e.formulation;
  return d;
}

#define VFMM_FOR_EACH_P(X) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) X(16)

// M2M into parents at levels maxLevel-1 .. 1 (the root is skipped, as the
// reference's upward pass skips level 0, fmmCalculator.hpp:427).
template <int P>
static void m2m_levels(cudaStream_t s, const ExpArgs &e, const DevExp &d)
{
  const size_t bytes = (size_t)(8 * 3 + 8) * nterms(P) * sizeof(zd);
  VFMM_SMEM_ONCE(bytes, k_m2m<P>);
  for (int l = e.maxLevel - 1; l >= 1; l--) {
    const int n0 = e.level_start_host[l], n1 = e.level_start_host[l + 1];
    if (n1 > n0) {
      k_m2m<P><<<std::min(n1 - n0, 152 * 16), 128, bytes, s>>>(d, e.level_cells + n0, n1 - n0);
      count_launch();
    }
  }
  VFMM_LAUNCH_CHECK();
}

template <int P>
static void upward_P(cudaStream_t s, const ExpArgs &e)
{
  DevExp       d     = dev_args(e);
  const size_t bytes = (size_t)32 * nterms(P) * sizeof(zd) + 32 * 3 * sizeof(double);
  VFMM_SMEM_ONCE(bytes, k_p2m<P>);
  if (e.nleaves > 0) {
    k_p2m<P><<<std::min(e.nleaves, 152 * 16), 64, bytes, s>>>(d);
    count_launch();
  }
  m2m_levels<P>(s, e, d);
}

template <int P>
static void m2m_P(cudaStream_t s, const ExpArgs &e)
{
  DevExp d = dev_args(e);
  m2m_levels<P>(s, e, d);
}

template <int P>
static void mprep_P(cudaStream_t s, const ExpArgs &e)
{
  k_mprep<P><<<grid_for((long)e.ncells * P * P * 3, 256), 256, 0, s>>>(e.M, e.Mprep, e.ncells);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

// M2L into every target cell of e.cells; with prep, the sign-folded source
// multipoles are made first from e.M (same tree as the targets).
template <int P>
static void m2l_P(cudaStream_t s, const ExpArgs &e, bool prep)
{
  DevExp    d  = dev_args(e);
  const int PP = P * P;
  if (prep)
    mprep_P<P>(s, e);
  const size_t bytes = (size_t)4 * 4 * PP * sizeof(zd);
  VFMM_SMEM_ONCE(bytes, k_m2l<P, 2, 4>);
  k_m2l<P, 2, 4><<<grid_for(e.ncells, 4, 152 * 32), 128, bytes, s>>>(d, e.ncells);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

// L2L from parents at levels 0 .. maxLevel-1 into their children.
template <int P>
static void l2l_P(cudaStream_t s, const ExpArgs &e)
{
  DevExp       d     = dev_args(e);
  const size_t bytes = (size_t)(3 + 8) * nterms(P) * sizeof(zd);
  VFMM_SMEM_ONCE(bytes, k_l2l<P>);
  for (int l = 0; l < e.maxLevel; l++) {
    const int n0 = e.level_start_host[l], n1 = e.level_start_host[l + 1];
    if (n1 > n0) {
      k_l2l<P><<<std::min(n1 - n0, 152 * 16), 128, bytes, s>>>(d, e.level_cells + n0, n1 - n0);
      count_launch();
    }
  }
  VFMM_LAUNCH_CHECK();
}

template <int P, bool SENS>
static void l2p_P(cudaStream_t s, const ExpArgs &e, double *out)
{
  DevExp       d     = dev_args(e);
  const size_t bytes = L2PSizes<P>::bytes;
  VFMM_SMEM_ONCE(bytes, k_l2p_p2p<P, SENS>);
  if (e.nsrc > 0) {
    k_src_weights<<<grid_for(e.nsrc, 256), 256, 0, s>>>(d.ssoa, d.scap, e.nsrc, e.srcw);
    count_launch();
  }
  if (e.nleaves > 0) {
    k_l2p_p2p<P, SENS><<<std::min(e.nleaves, 152 * 16), 128, bytes, s>>>(d, out);
    count_launch();
  }
  VFMM_LAUNCH_CHECK();
}

template <int P>
static void l2p_bodies_P(cudaStream_t s, const ExpArgs &e, double *out) { l2p_P<P, false>(s, e, out); }
template <int P>
static void l2p_sensors_P(cudaStream_t s, const ExpArgs &e, double *out) { l2p_P<P, true>(s, e, out); }

#define VFMM_DISPATCH(fn, ...)                                                                                                   \
  switch (e.P) {                                                                                                                \
  case 2: fn<2>(__VA_ARGS__); break;                                                                                            \
  case 3: fn<3>(__VA_ARGS__); break;                                                                                            \
  case 4: fn<4>(__VA_ARGS__); break;                                                                                            \
  case 5: fn<5>(__VA_ARGS__); break;                                                                                            \
  case 6: fn<6>(__VA_ARGS__); break;                                                                                            \
  case 7: fn<7>(__VA_ARGS__); break;                                                                                            \
  case 8: fn<8>(__VA_ARGS__); break;                                                                                            \
  case 9: fn<9>(__VA_ARGS__); break;                                                                                            \
  case 10: fn<10>(__VA_ARGS__); break;                                                                                          \
  case 11: fn<11>(__VA_ARGS__); break;                                                                                          \
  case 12: fn<12>(__VA_ARGS__); break;                                                                                          \
  case 13: fn<13>(__VA_ARGS__); break;                                                                                          \
  case 14: fn<14>(__VA_ARGS__); break;                                                                                          \
  case 15: fn<15>(__VA_ARGS__); break;                                                                                          \
  case 16: fn<16>(__VA_ARGS__); break;                                                                                          \
  default: throw Error(VFMM_ERR_UNSUPPORTED, "expansion order p must be in 2..16");                                            \
  }

void upward_pass(cudaStream_t s, const ExpArgs &e) { VFMM_DISPATCH(upward_P, s, e) }
void m2m_pass(cudaStream_t s, const ExpArgs &e) { VFMM_DISPATCH(m2m_P, s, e) }
void m2l_pass(cudaStream_t s, const ExpArgs &e) { VFMM_DISPATCH(m2l_P, s, e, true) }
void mprep_pass(cudaStream_t s, const ExpArgs &e) { VFMM_DISPATCH(mprep_P, s, e) }
void m2l_sensor_pass(cudaStream_t s, const ExpArgs &e) { VFMM_DISPATCH(m2l_P, s, e, false) }
void downward_l2l(cudaStream_t s, const ExpArgs &e) { VFMM_DISPATCH(l2l_P, s, e) }
void l2p_p2p_pass(cudaStream_t s, const ExpArgs &e, double *out) { VFMM_DISPATCH(l2p_bodies_P, s, e, out) }
void l2p_sensor_pass(cudaStream_t s, const ExpArgs &e, double *out) { VFMM_DISPATCH(l2p_sensors_P, s, e, out) }

// Lane table of the lockstep M2L (k_m2l32v2).  For degree n the outputs
// (j, k), j <= P-1-n, 0 <= k <= j, are cut into half-tiles of kh consecutive
// columns of one row; two half-tiles (any rows) form a lane tile, so short
// rows waste few multiply-adds.  With T tiles, R = min(32 / T, sb) replicas
// take turns over the batch's sources.  Entry [n * 32 + lane] =
// {jA | k0A << 8 | kwA << 16, jB | k0B << 8 | kwB << 16, replica, R | T << 8};
// a missing second half has kwB = 0 (and repeats the first's row/column);
// x = -1 marks an idle lane.
std::vector<int4> m2l_lane_table(int P, int kh, int sb)
{
  std::vector<int4> tab((size_t)P * 32, make_int4(-1, 0, 0, 1));
  for (int n = 0; n < P; n++) {
    std::vector<int> halves;
    for (int j = 0; j <= P - 1 - n; j++)
      for (int k0 = 0; k0 <= j; k0 += kh)
        halves.push_back(j | (k0 << 8) | (std::min(kh, j + 1 - k0) << 16));
    std::vector<int2> tiles;
    for (size_t i = 0; i < halves.size(); i += 2)
      tiles.push_back(make_int2(halves[i], i + 1 < halves.size() ? halves[i + 1] : (halves[i] & 0xffff)));
    const int T = (int)tiles.size();
    if (T > 32)
      throw Error(VFMM_ERR_UNSUPPORTED, "M2L lane table: more than 32 tiles for one degree");
    const int R = std::max(1, std::min(32 / T, sb));
    for (int l = 0; l < 32; l++) {
      int4 e = make_int4(-1, 0, 0, R | (T << 8));
      if (l < T * R)
        e = make_int4(tiles[l % T].x, tiles[l % T].y, l / T, R | (T << 8));
      tab[(size_t)n * 32 + l] = e;
    }
  }
  return tab;
}

// Balanced static schedule for k_m2l: items (j, k0..k0+kb-1, n0..n1) whose
// cost is kb * sum_{n0..n1}(2n+1) complex multiply-adds per component, packed
// onto `lanes` lanes with at most `maxItems` each (longest-processing-time
// first).  Returned as int4 {j, k0 | kb << 8, n0, n1} at [slot * lanes + lane];
// unused slots have j = -1.
std::vector<int4> m2l_schedule(int P, int lanes, int kb, int maxItems, int *itemsPerLane)
{
  struct It {
    int  j, k0, kbn, n0, n1;
    long cost;
  };
  long total = 0;
  for (int j = 0; j < P; j++)
    total += (long)(j + 1) * (P - j) * (P - j);
  std::vector<int4> best;
  double            bestLoad = 1e300;
  for (int div = 1; div <= 64; div *= 2) {
    const long        cap = std::max<long>(1, (total + lanes - 1) / lanes / div);
    std::vector<It>   items;
    for (int j = 0; j < P; j++)
      for (int k0 = 0; k0 <= j; k0 += kb) {
        const int kbn = std::min(kb, j + 1 - k0), nmax = P - 1 - j;
        int       n0  = 0;
        while (n0 <= nmax) {
          int  n1 = n0;
          long c  = (long)kbn * (2 * n0 + 1);
          while (n1 + 1 <= nmax && c + (long)kbn * (2 * (n1 + 1) + 1) <= cap) {
            n1++;
            c += (long)kbn * (2 * n1 + 1);
          }
          items.push_back({j, k0, kbn, n0, n1, c});
          n0 = n1 + 1;
        }
      }
    std::sort(items.begin(), items.end(), [](const It &a, const It &b) { return a.cost > b.cost; });
    std::vector<long> load(lanes, 0);
    std::vector<int>  cnt(lanes, 0);
    std::vector<int4> tab((size_t)maxItems * lanes, make_int4(-1, 0, 0, 0));
    bool              ok = true;
    for (const It &it : items) {
      int bestLane = -1;
      for (int l = 0; l < lanes; l++)
        if (cnt[l] < maxItems && (bestLane < 0 || load[l] < load[bestLane]))
          bestLane = l;
      if (bestLane < 0) {
        ok = false;
        break;
      }
      tab[(size_t)cnt[bestLane] * lanes + bestLane] = make_int4(it.j, it.k0 | (it.kbn << 8), it.n0, it.n1);
      cnt[bestLane]++;
      load[bestLane] += it.cost;
    }
    if (!ok)
      continue;
    const double mx = (double)*std::max_element(load.begin(), load.end());
    if (mx < bestLoad) {
      bestLoad = mx;
      best     = tab;
    }
  }
  if (best.empty())
    throw Error(VFMM_ERR_UNSUPPORTED, "no M2L schedule for this order");
  *itemsPerLane = maxItems;
  return best;
}

} // namespace vfmm
