// Reverse mode of the FP64 evaluation and of the RK stage updates: the
// building blocks of vfmm_adjoint, the adjoint of advance
// (fmmCalculator.hpp:919-1005) for the inviscid cVPM path.
//
// One evaluation maps the bodies (x, alpha, sigma) to u and J through the
// expansion passes P2M -> M2M -> M2L -> L2L -> L2P and the P2P near field
// (multipoleKernels.hpp:223-742), then the stage adds the stretching term
// dalpha/dt = J^T alpha (or J alpha, fmmCalculator.hpp:391-405).  Given the
// adjoints (ubar, Jbar) of u and J, the passes run backwards as their exact
// transposes: L2P^T leaf by leaf, L2L^T up the levels, M2L^T gathered per
// source cell over the transposed lists, M2M^T down the levels, P2M^T leaf
// by leaf, and the pair terms of P2P differentiated in closed form, once per
// target and once per source, so every output has a single writer and the
// sums run in a fixed order.
//
// The tree is a piecewise-constant function of the positions; the cell
// centres are X0 + R0 o_c with X0, R0 the bounding box of getBounds
// (tree.hpp:7-26).  Their derivatives follow from two exact invariances of
// the evaluation: a common translation of bodies and X0 changes nothing, and
// a dilation about X0 of bodies, R0 and sigma scales u by s^-2 and J by s^-3.
// So, with xbar_far the far-field partial adjoints at fixed geometry,
//   X0bar = -sum xbar_far,   R0 R0bar = sum(-2 ubar.u_far - 3 Jbar:J_far)
//                                         - sum xbar_far . (x - X0),
// passed to the bodies that set the bounding box.
#include <algorithm>
#include <vector>
#include "harmonics.cuh"
#include "vfmm_internal.cuh"

namespace vfmm {

namespace {

typedef cx<double> zd;

static __constant__ HarmRecip<double> kHR  = make_harm_recip<double>();
static __constant__ HarmRecip<float>  kHRf = make_harm_recip<float>();
template <class T> __device__ __forceinline__ const HarmRecip<T> &harm_recip();
template <> __device__ __forceinline__ const HarmRecip<double> &harm_recip<double>() { return kHR; }
template <> __device__ __forceinline__ const HarmRecip<float> &harm_recip<float>() { return kHRf; }

constexpr double kInvPi     = 0.318309886183790671537767526745028724;
constexpr double kInvSqrtPi = 0.564189583547756286948079451560772586;

__device__ __forceinline__ zd ldz(const double2 *p)
{
  const double2 v = *p;
  return {v.x, v.y};
}
__device__ __forceinline__ void stz(double2 *p, zd v) { *p = make_double2(v.r, v.i); }
template <class T>
__device__ __forceinline__ void cadd(cx<T> &a, cx<T> b)
{
  a.r += b.r;
  a.i += b.i;
}
__device__ __forceinline__ void jk_of(int jks, int &j, int &k)
{
  j = 0;
  while ((j + 1) * (j + 2) / 2 <= jks)
    j++;
  k = jks - j * (j + 1) / 2;
}

struct AdjDev {
  CellsView     cv;
  const double *soa; // bodies in tree order: X, A, R, and U, J of the FP64 evaluation
  size_t        cap;
  const double2 *L;  // local expansions of the evaluation
  double2       *Lb, *Mb;
  const int     *leaf_cells;
  int            nleaves;
  const int     *p2p_start, *p2p_src;   // P2P rows by target leaf
  const int     *p2pT_start, *p2pT_tgt; // P2P rows by source leaf
  const int     *m2lT_start, *m2lT_tgt; // M2L rows by source cell
  double        *w;                     // work fields (AdjW), field-major, capacity cap
  // mixed mode: FP32 body records of the evaluation and the seeds in FP32
  const float4  *pos32, *alp32;         // (x - X_leaf, 1/(2 sigma^2)), (alpha, 1/sigma)
  float4        *seeds32;               // per body 4 x float4: ubar, ct, Jbar (see k_adj_seeds32)
  float2        *Lhat32;                // per cell 3K: scaled adjoint locals for M2L^T (k_adj_lhat32)
  double         R0;
  double         R0pow[PMAX + 2], iR0pow[PMAX + 2];
};

__device__ __forceinline__ double &W(const AdjDev &a, int f, int i) { return a.w[(size_t)f * a.cap + i]; }
__device__ __forceinline__ double B(const AdjDev &a, int f, int i) { return a.soa[(size_t)f * a.cap + i]; }

// ------------------------------------------------------------------ L2P^T
// Far field of the forward pass at a body of leaf c:
//   u_a = sum w_m Re(U_a[n,m] Y_n^m),  U = (1/4pi) curl of the local expansion,
//   J_ae = sum w_m Re(JJ_ae[n,m] Y_n^m),  JJ_ae = D_e U_a.
// Adjoint: Ubar[n,m] = sum_b w_m ubar_b conj(Y(x_b)), likewise JJbar, then the
// transposed derivative operators give Lbar of the leaf.  The body's own
// position adjoint is ubar . dU/dx + Jbar : dJ/dx, with dJ_ae/dx_g evaluated
// from HH = D_g JJ_ae.
template <int P>
struct AdjL2PSizes {
  static constexpr int    K  = nterms(P);
  static constexpr int    N1 = nterms(P - 1);                  // degree <= P-2
  static constexpr int    N2 = P >= 3 ? nterms(P - 2) : 0;     // degree <= P-3
  static constexpr int    N3 = P >= 4 ? nterms(P - 3) : 0;     // degree <= P-4
  static constexpr int    K1 = N1 > 0 ? N1 : 1, K2 = N2 > 0 ? N2 : 1, K3 = N3 > 0 ? N3 : 1;
  static constexpr int    NB = 32; // bodies per staging chunk
  static constexpr size_t zcount = 3 * K + 3 * K1 + 9 * K2 + 27 * K3 + 3 * K1 + 9 * K2 + 3 * K + NB * K1;
  static constexpr size_t bytes  = zcount * sizeof(zd) + (NB * 12 + K1) * sizeof(double);
};

template <int P>
__global__ void __launch_bounds__(128) k_adj_l2p(AdjDev a)
{
  using S = AdjL2PSizes<P>;
  constexpr int K = S::K, K1 = S::K1, K2 = S::K2, K3 = S::K3, N1 = S::N1, N2 = S::N2, N3 = S::N3, NB = S::NB;
  constexpr int NO = (3 * N1 + 9 * N2 + 127) / 128;
  extern __shared__ double2 smem_raw[];
  zd     *Lc  = reinterpret_cast<zd *>(smem_raw);
  zd     *U   = Lc + 3 * K;
  zd     *JJ  = U + 3 * K1;
  zd     *HH  = JJ + 9 * K2;
  zd     *Ub  = HH + 27 * K3;
  zd     *JJb = Ub + 3 * K1;
  zd     *Lb  = JJb + 9 * K2;
  zd     *Ys  = Lb + 3 * K;
  double *Sd  = reinterpret_cast<double *>(Ys + NB * K1);
  double *Wt  = Sd + NB * 12; // w_m of term tri(n, m): 1 for m = 0, else 2
  const double inv4pi = 0.25 * kInvPi;
  for (int idx = threadIdx.x; idx < N1; idx += 128) {
    int n, m;
    jk_of(idx, n, m);
    Wt[idx] = m == 0 ? 1.0 : 2.0;
  }

  for (int li = blockIdx.x; li < a.nleaves; li += gridDim.x) {
    const int    c = a.leaf_cells[li], b0 = a.cv.body[c], nb = a.cv.nbody[c];
    const double cxx = a.cv.x[c], cyy = a.cv.y[c], czz = a.cv.z[c];
    __syncthreads();
    for (int e = threadIdx.x; e < 3 * K; e += 128)
      Lc[e] = ldz(a.L + (size_t)c * 3 * K + e);
    __syncthreads();
    for (int e = threadIdx.x; e < 3 * N1; e += 128) { // as the forward L2P
      const int idx = e / 3, ax = e % 3;
      int       n, mu;
      jk_of(idx, n, mu);
      const int b1 = (ax + 1) % 3, c1 = (ax + 2) % 3;
      const zd  p = deriv_coef(Lc, n, mu, b1, 3, c1), q = deriv_coef(Lc, n, mu, c1, 3, b1);
      U[idx * 3 + ax] = {inv4pi * (p.r - q.r), inv4pi * (p.i - q.i)};
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 9 * N2; e += 128) {
      const int idx = e / 9, ae = e % 9;
      int       n, mu;
      jk_of(idx, n, mu);
      JJ[idx * 9 + ae] = deriv_coef(U, n, mu, ae % 3, 3, ae / 3);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 27 * N3; e += 128) {
      const int idx = e / 27, r = e % 27;
      int       n, mu;
      jk_of(idx, n, mu);
      HH[idx * 27 + r] = deriv_coef(JJ, n, mu, r % 3, 9, r / 3); // D_g JJ_ae at ae * 3 + g
    }
    __syncthreads();

    zd acc[NO > 0 ? NO : 1];
#pragma unroll
    for (int i = 0; i < (NO > 0 ? NO : 1); i++)
      acc[i] = {0, 0};
    for (int c0 = 0; c0 < nb; c0 += NB) {
      const int nbc = min(NB, nb - c0);
      if (threadIdx.x < nbc) {
        const int t = threadIdx.x, b = b0 + c0 + t;
        regular_harmonics<double, P - 1>(B(a, F_X, b) - cxx, B(a, F_X + 1, b) - cyy, B(a, F_X + 2, b) - czz, Ys + t * K1);
        for (int k = 0; k < 12; k++)
          Sd[t * 12 + k] = W(a, W_SU + k, b);
      }
      __syncthreads();
      // far field and its derivatives at each body: four threads per body
      // (adjacent lanes), each summing every fourth term, combined by shuffles
      {
        const int t = threadIdx.x >> 2, part = threadIdx.x & 3;
        double    f[39]; // u (3), J (9), dJ/dx (27)
#pragma unroll
        for (int k = 0; k < 39; k++)
          f[k] = 0;
        if (t < nbc)
          for (int idx = part; idx < N1; idx += 4) {
            const zd     y  = Ys[t * K1 + idx];
            const double wm = Wt[idx];
#pragma unroll
            for (int ax = 0; ax < 3; ax++)
              f[ax] += wm * (U[idx * 3 + ax].r * y.r - U[idx * 3 + ax].i * y.i);
            if (idx < N2)
#pragma unroll
              for (int ae = 0; ae < 9; ae++)
                f[3 + ae] += wm * (JJ[idx * 9 + ae].r * y.r - JJ[idx * 9 + ae].i * y.i);
            if (idx < N3)
#pragma unroll
              for (int r = 0; r < 27; r++)
                f[12 + r] += wm * (HH[idx * 27 + r].r * y.r - HH[idx * 27 + r].i * y.i);
          }
#pragma unroll
        for (int k = 0; k < 39; k++) {
          f[k] += __shfl_xor_sync(0xffffffffu, f[k], 1);
          f[k] += __shfl_xor_sync(0xffffffffu, f[k], 2);
        }
        if (t < nbc && part == 0) {
          const int     b  = b0 + c0 + t;
          const double *sd = Sd + t * 12;
          double        e  = 0;
          for (int ax = 0; ax < 3; ax++)
            e -= 2.0 * sd[ax] * f[ax];
          for (int ae = 0; ae < 9; ae++)
            e -= 3.0 * sd[3 + ae] * f[3 + ae];
          for (int g = 0; g < 3; g++) {
            double xb = 0;
            for (int ax = 0; ax < 3; ax++)
              xb += sd[ax] * f[3 + ax * 3 + g];
            for (int ae = 0; ae < 9; ae++)
              xb += sd[3 + ae] * f[12 + ae * 3 + g];
            W(a, W_XF + g, b) = xb;
          }
          W(a, W_EF, b) = e;
        }
      }
      __syncthreads();
#pragma unroll
      for (int i = 0; i < NO; i++) {
        const int o = threadIdx.x + 128 * i;
        if (o < 3 * N1) {
          const int idx = o / 3, ax = o % 3;
          int       n, m;
          jk_of(idx, n, m);
          const double wm = m == 0 ? 1.0 : 2.0;
          for (int tt = 0; tt < nbc; tt++) {
            const zd     y = Ys[tt * K1 + idx];
            const double s = wm * Sd[tt * 12 + ax];
            acc[i].r += s * y.r;
            acc[i].i -= s * y.i;
          }
        } else if (o < 3 * N1 + 9 * N2) {
          const int o2 = o - 3 * N1, idx = o2 / 9, ae = o2 % 9;
          int       n, m;
          jk_of(idx, n, m);
          const double wm = m == 0 ? 1.0 : 2.0;
          for (int tt = 0; tt < nbc; tt++) {
            const zd     y = Ys[tt * K1 + idx];
            const double s = wm * Sd[tt * 12 + 3 + ae];
            acc[i].r += s * y.r;
            acc[i].i -= s * y.i;
          }
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < NO; i++) {
      const int o = threadIdx.x + 128 * i;
      if (o < 3 * N1)
        Ub[o] = acc[i];
      else if (o < 3 * N1 + 9 * N2)
        JJb[o - 3 * N1] = acc[i];
    }
    for (int e = threadIdx.x; e < 3 * K; e += 128)
      Lb[e] = {0, 0};
    __syncthreads();
    // JJ_ae = D_e U_a, transposed: one thread per component a (fixed order)
    if (threadIdx.x < 3) {
      const int ax = threadIdx.x;
      for (int idx = 0; idx < N2; idx++) {
        int n, mu;
        jk_of(idx, n, mu);
        for (int ex = 0; ex < 3; ex++)
          deriv_coef_adj(Ub, n, mu, ex, 3, ax, JJb[idx * 9 + ax * 3 + ex]);
      }
    }
    __syncthreads();
    // U_a = (1/4pi)(D_{a+1} psi_{a+2} - D_{a+2} psi_{a+1}), transposed: one thread per psi component
    if (threadIdx.x < 3) {
      const int cc = threadIdx.x;
      for (int idx = 0; idx < N1; idx++) {
        int n, mu;
        jk_of(idx, n, mu);
        const zd u1 = Ub[idx * 3 + (cc + 1) % 3], u2 = Ub[idx * 3 + (cc + 2) % 3];
        deriv_coef_adj(Lb, n, mu, (cc + 2) % 3, 3, cc, zd{inv4pi * u1.r, inv4pi * u1.i});
        deriv_coef_adj(Lb, n, mu, (cc + 1) % 3, 3, cc, zd{-inv4pi * u2.r, -inv4pi * u2.i});
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 3 * K; e += 128)
      stz(a.Lb + (size_t)c * 3 * K + e, Lb[e]);
  }
}

// L2P^T for mixed mode, in FP32 throughout on the leaf-scaled expansion
// Lhat[j] = L[j] R_c^j: a derivative operator lowers the degree by one, so
// with coefficients of degree n carried as c_n R_c^n each D becomes D / R_c,
//   U32 = (1/4pi) curl D(Lhat) / R_c,  JJ32 = D(U32) / R_c,  HH32 = D(JJ32) / R_c,
// and sum c_n Y_n(x - X_c) = sum (c_n R_c^n) Y_n(y), y = (x - X_c) / R_c, gives the
// far field and its derivatives unscaled.  Backwards the same holds for the
// adjoints (Ubar32 = Ubar / R_c^n is the FP32 sum over Y(y)), and only the
// final Lbar = R_c^j Lhatbar is formed in FP64.
__device__ __forceinline__ void load_seeds32(const AdjDev &a, int i, float *ub, float *Jb, float *ct); // FP32 seeds, below

template <int P>
struct AdjL2P32Sizes {
  using S                          = AdjL2PSizes<P>;
  static constexpr int    K        = S::K, K1 = S::K1, K2 = S::K2, K3 = S::K3, NB = S::NB;
  static constexpr size_t zf_count = 3 * K + 3 * K1 + 9 * K2 + 27 * K3 + 3 * K1 + 9 * K2 + 3 * K + NB * K1; // Lh, U, JJ, HH, Ub, JJb, Lb, Ys
  static constexpr size_t bytes    = zf_count * sizeof(cx<float>) + (NB * 12 + K1) * sizeof(float);
};

template <int P>
__global__ void __launch_bounds__(128) k_adj_l2p32(AdjDev a)
{
  using S = AdjL2PSizes<P>;
  typedef cx<float> zf;
  constexpr int K = S::K, K1 = S::K1, K2 = S::K2, K3 = S::K3, N1 = S::N1, N2 = S::N2, N3 = S::N3, NB = S::NB;
  constexpr int NO = (3 * N1 + 9 * N2 + 127) / 128;
  extern __shared__ double2 smem_raw[];
  zf    *Lh  = reinterpret_cast<zf *>(smem_raw);
  zf    *U   = Lh + 3 * K;
  zf    *JJ  = U + 3 * K1;
  zf    *HH  = JJ + 9 * K2;
  zf    *Ub  = HH + 27 * K3;
  zf    *JJb = Ub + 3 * K1;
  zf    *Lb  = JJb + 9 * K2;
  zf    *Ys  = Lb + 3 * K;
  float *Sd  = reinterpret_cast<float *>(Ys + NB * K1);
  float *Wt  = Sd + NB * 12;
  const float inv4pi = (float)(0.25 * kInvPi);
  for (int idx = threadIdx.x; idx < N1; idx += 128) {
    int n, m;
    jk_of(idx, n, m);
    Wt[idx] = m == 0 ? 1.f : 2.f;
  }
  for (int li = blockIdx.x; li < a.nleaves; li += gridDim.x) {
    const int    c = a.leaf_cells[li], b0 = a.cv.body[c], nb = a.cv.nbody[c], lev = a.cv.level[c];
    const double cxx = a.cv.x[c], cyy = a.cv.y[c], czz = a.cv.z[c];
    const double iR  = ldexp(1.0 / a.R0, lev);
    const float  iRf = (float)iR;
    __syncthreads();
    for (int e = threadIdx.x; e < 3 * K; e += 128) {
      int j, k;
      jk_of(e / 3, j, k);
      const double2 v  = a.L[(size_t)c * 3 * K + e];
      const double  sc = ldexp(a.R0pow[j], -lev * j); // R_c^j
      Lh[e]            = {(float)(v.x * sc), (float)(v.y * sc)};
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 3 * N1; e += 128) {
      const int idx = e / 3, ax = e % 3;
      int       n, mu;
      jk_of(idx, n, mu);
      const int b1 = (ax + 1) % 3, c1 = (ax + 2) % 3;
      const zf  p = deriv_coef(Lh, n, mu, b1, 3, c1), q = deriv_coef(Lh, n, mu, c1, 3, b1);
      const float sc = inv4pi * iRf;
      U[idx * 3 + ax] = {sc * (p.r - q.r), sc * (p.i - q.i)};
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 9 * N2; e += 128) {
      const int idx = e / 9, ae = e % 9;
      int       n, mu;
      jk_of(idx, n, mu);
      const zf v       = deriv_coef(U, n, mu, ae % 3, 3, ae / 3);
      JJ[idx * 9 + ae] = {v.r * iRf, v.i * iRf};
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 27 * N3; e += 128) {
      const int idx = e / 27, r = e % 27;
      int       n, mu;
      jk_of(idx, n, mu);
      const zf v       = deriv_coef(JJ, n, mu, r % 3, 9, r / 3);
      HH[idx * 27 + r] = {v.r * iRf, v.i * iRf};
    }
    __syncthreads();

    zf acc[NO > 0 ? NO : 1];
#pragma unroll
    for (int i = 0; i < (NO > 0 ? NO : 1); i++)
      acc[i] = {0.f, 0.f};
    for (int c0 = 0; c0 < nb; c0 += NB) {
      const int nbc = min(NB, nb - c0);
      if (threadIdx.x < nbc) {
        const int t = threadIdx.x, b = b0 + c0 + t;
        regular_harmonics<float, P - 1>((float)((B(a, F_X, b) - cxx) * iR), (float)((B(a, F_X + 1, b) - cyy) * iR),
                                        (float)((B(a, F_X + 2, b) - czz) * iR), Ys + t * K1);
        float ub[3], Jb[9], ct[3];
        load_seeds32(a, b, ub, Jb, ct);
        for (int k = 0; k < 3; k++)
          Sd[t * 12 + k] = ub[k];
        for (int k = 0; k < 9; k++)
          Sd[t * 12 + 3 + k] = Jb[k];
      }
      __syncthreads();
      {
        const int t = threadIdx.x >> 2, part = threadIdx.x & 3;
        float     f[39];
#pragma unroll
        for (int k = 0; k < 39; k++)
          f[k] = 0.f;
        if (t < nbc)
          for (int idx = part; idx < N1; idx += 4) {
            const zf    y  = Ys[t * K1 + idx];
            const float wm = Wt[idx];
#pragma unroll
            for (int ax = 0; ax < 3; ax++)
              f[ax] = fmaf(wm, U[idx * 3 + ax].r * y.r - U[idx * 3 + ax].i * y.i, f[ax]);
            if (idx < N2)
#pragma unroll
              for (int ae = 0; ae < 9; ae++)
                f[3 + ae] = fmaf(wm, JJ[idx * 9 + ae].r * y.r - JJ[idx * 9 + ae].i * y.i, f[3 + ae]);
            if (idx < N3)
#pragma unroll
              for (int r = 0; r < 27; r++)
                f[12 + r] = fmaf(wm, HH[idx * 27 + r].r * y.r - HH[idx * 27 + r].i * y.i, f[12 + r]);
          }
#pragma unroll
        for (int k = 0; k < 39; k++) {
          f[k] += __shfl_xor_sync(0xffffffffu, f[k], 1);
          f[k] += __shfl_xor_sync(0xffffffffu, f[k], 2);
        }
        if (t < nbc && part == 0) {
          const int    b  = b0 + c0 + t;
          const float *sd = Sd + t * 12;
          float        e  = 0.f;
          for (int ax = 0; ax < 3; ax++)
            e -= 2.f * sd[ax] * f[ax];
          for (int ae = 0; ae < 9; ae++)
            e -= 3.f * sd[3 + ae] * f[3 + ae];
          for (int g = 0; g < 3; g++) {
            float xb = 0.f;
            for (int ax = 0; ax < 3; ax++)
              xb = fmaf(sd[ax], f[3 + ax * 3 + g], xb);
            for (int ae = 0; ae < 9; ae++)
              xb = fmaf(sd[3 + ae], f[12 + ae * 3 + g], xb);
            W(a, W_XF + g, b) = xb;
          }
          W(a, W_EF, b) = e;
        }
      }
      __syncthreads();
#pragma unroll
      for (int i = 0; i < NO; i++) {
        const int o = threadIdx.x + 128 * i;
        if (o < 3 * N1) {
          const int   idx = o / 3, ax = o % 3;
          const float wm  = Wt[idx];
          for (int tt = 0; tt < nbc; tt++) {
            const zf    y  = Ys[tt * K1 + idx];
            const float sv = wm * Sd[tt * 12 + ax];
            acc[i].r       = fmaf(sv, y.r, acc[i].r);
            acc[i].i       = fmaf(-sv, y.i, acc[i].i);
          }
        } else if (o < 3 * N1 + 9 * N2) {
          const int   o2 = o - 3 * N1, idx = o2 / 9, ae = o2 % 9;
          const float wm = Wt[idx];
          for (int tt = 0; tt < nbc; tt++) {
            const zf    y  = Ys[tt * K1 + idx];
            const float sv = wm * Sd[tt * 12 + 3 + ae];
            acc[i].r       = fmaf(sv, y.r, acc[i].r);
            acc[i].i       = fmaf(-sv, y.i, acc[i].i);
          }
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < NO; i++) {
      const int o = threadIdx.x + 128 * i;
      if (o < 3 * N1)
        Ub[o] = acc[i];
      else if (o < 3 * N1 + 9 * N2)
        JJb[o - 3 * N1] = acc[i];
    }
    for (int e = threadIdx.x; e < 3 * K; e += 128)
      Lb[e] = {0.f, 0.f};
    __syncthreads();
    // JJ32 = D(U32) / R_c, transposed: one thread per component (fixed order)
    if (threadIdx.x < 3) {
      const int ax = threadIdx.x;
      for (int idx = 0; idx < N2; idx++) {
        int n, mu;
        jk_of(idx, n, mu);
        for (int ex = 0; ex < 3; ex++) {
          const zf v = JJb[idx * 9 + ax * 3 + ex];
          deriv_coef_adj(Ub, n, mu, ex, 3, ax, zf{v.r * iRf, v.i * iRf});
        }
      }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
      const int   cc = threadIdx.x;
      const float sc = inv4pi * iRf;
      for (int idx = 0; idx < N1; idx++) {
        int n, mu;
        jk_of(idx, n, mu);
        const zf u1 = Ub[idx * 3 + (cc + 1) % 3], u2 = Ub[idx * 3 + (cc + 2) % 3];
        deriv_coef_adj(Lb, n, mu, (cc + 2) % 3, 3, cc, zf{sc * u1.r, sc * u1.i});
        deriv_coef_adj(Lb, n, mu, (cc + 1) % 3, 3, cc, zf{-sc * u2.r, -sc * u2.i});
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 3 * K; e += 128) {
      int j, k;
      jk_of(e / 3, j, k);
      const double sc = ldexp(a.R0pow[j], -lev * j); // Lbar = R_c^j Lhatbar
      a.Lb[(size_t)c * 3 * K + e] = make_double2((double)Lb[e].r * sc, (double)Lb[e].i * sc);
    }
  }
}

// ------------------------------------------------------------------ L2L^T
// Forward (k_l2l): L_child[j,k] += terms in L_parent[n, +-m] and the regular
// harmonics of X_child - X_parent.  Transposed, per parent coefficient
// (n, mm): for every child and child coefficient (j <= n, k <= j),
//   term A (mm >= 1, k + mm <= n - j): +-conj(Lbar_child[j,k] Y[n-j, k+mm]),
//   term B (|mm - k| <= n - j):        +-Lbar_child[j,k] (conj Y[n-j, mm-k] | Y[n-j, k-mm]).
// T = float (mixed mode) works in the forward's scaled variables, scaled by
// the parent's half-width R_p: Lbar_child[j] / R_p^j in, harmonics at
// (X_child - X_parent) / R_p, Lbar_parent[n] = R_p^n times the FP32 sum.
template <int P, class T>
__global__ void __launch_bounds__(128) k_adj_l2l(AdjDev a, const int *cells, int count)
{
  typedef cx<T> zt;
  constexpr bool MIX = sizeof(T) == 4;
  constexpr int  K   = nterms(P);
  extern __shared__ double2 smem_raw[];
  zt *Lch = reinterpret_cast<zt *>(smem_raw); // [8][3K]
  zt *Ys  = Lch + 8 * 3 * K;                  // [8][K]
  for (int pi = blockIdx.x; pi < count; pi += gridDim.x) {
    const int p = cells[pi], nch = a.cv.nchild[p], ch0 = a.cv.child[p];
    if (nch == 0)
      continue;
    const int    lev = a.cv.level[p];
    const double iRp = MIX ? ldexp(1.0 / a.R0, lev) : 1.0;
    __syncthreads();
    for (int e = threadIdx.x; e < nch * 3 * K; e += blockDim.x) {
      const double2 v = a.Lb[(size_t)ch0 * 3 * K + e];
      double        sc = 1.0;
      if (MIX) {
        int j, k;
        jk_of((e % (3 * K)) / 3, j, k);
        sc = ldexp(a.iR0pow[j], lev * j); // R_p^{-j}
      }
      Lch[e] = {(T)(v.x * sc), (T)(v.y * sc)};
    }
    if (threadIdx.x < nch) {
      const int ch = ch0 + threadIdx.x;
      regular_harmonics<T, P>((T)((a.cv.x[ch] - a.cv.x[p]) * iRp), (T)((a.cv.y[ch] - a.cv.y[p]) * iRp), (T)((a.cv.z[ch] - a.cv.z[p]) * iRp),
                              Ys + threadIdx.x * K);
    }
    __syncthreads();
    for (int o = threadIdx.x; o < 3 * K; o += blockDim.x) {
      const int idx = o / 3, d = o % 3;
      int       n, mm;
      jk_of(idx, n, mm);
      zt acc{T(0), T(0)};
      for (int ci = 0; ci < nch; ci++) {
        const zt *Y = Ys + ci * K, *Lc = Lch + ci * 3 * K;
        for (int j = 0; j <= n; j++) {
          const int nj = n - j;
          for (int k = 0; k <= j; k++) {
            const zt l = Lc[tri(j, k) * 3 + d];
            if (mm >= 1 && k + mm <= nj)
              cadd(acc, neg_if(conj(l * Y[tri(nj, k + mm)]), (k & 1) != 0));
            if (abs(mm - k) <= nj) {
              const bool neg = mm < k && ((k - mm) & 1);
              const zt   wc  = mm >= k ? conj(Y[tri(nj, mm - k)]) : Y[tri(nj, k - mm)];
              cadd(acc, neg_if(l * wc, neg));
            }
          }
        }
      }
      const double sc = MIX ? ldexp(a.R0pow[n], -lev * n) : 1.0; // R_p^n
      a.Lb[(size_t)p * 3 * K + o] = make_double2((double)acc.r * sc, (double)acc.i * sc);
    }
  }
}

// ------------------------------------------------------------------ M2L^T
// Forward (k_m2l): L_t[j,k] = (-1)^j sum_s sum_{n <= P-1-j} sum_m M'_s[n,m] S'_ts[j+n, m-k]
// with M' the sign-folded multipoles (k_mprep).  Transposed, per source s
// over its targets t:  M'bar[n,m] = sum_t sum_{j <= P-1-n} sum_{k <= j}
// (-1)^j Lbar_t[j,k] conj(S'_ts[j+n, m-k]), then
// Mbar[n,m] = (-1)^m M'bar[n,m] + conj(M'bar[n,-m]) (m > 0).
// One warp per source cell; lanes own outputs (n, m, d).
template <int P>
struct AdjM2LSizes {
  static constexpr int    K = nterms(P), PP = P * P, NE = 3 * PP;
  static constexpr int    WS = (3 * K + PP > NE) ? 3 * K + PP : NE; // per warp, zd
  static constexpr size_t bytes = (size_t)4 * WS * sizeof(zd);
};

template <int P>
__global__ void __launch_bounds__(128) k_adj_m2l(AdjDev a, int ncells)
{
  using S = AdjM2LSizes<P>;
  constexpr int K = S::K, NE = S::NE, NA = (NE + 31) / 32, WS = S::WS;
  extern __shared__ double2 smem_raw[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  zd       *Lt = reinterpret_cast<zd *>(smem_raw) + w * WS;
  zd       *Sp = Lt + 3 * K;
  int       on[NA], om[NA];
#pragma unroll
  for (int i = 0; i < NA; i++) {
    const int e = lane + 32 * i, idx = e / 3;
    int       n = 0;
    while ((n + 1) * (n + 1) <= idx)
      n++;
    on[i] = n;
    om[i] = idx - n * n - n;
  }
  for (int s = blockIdx.x * 4 + w; s < ncells; s += gridDim.x * 4) {
    zd acc[NA];
#pragma unroll
    for (int i = 0; i < NA; i++)
      acc[i] = {0, 0};
    const int    q0 = a.m2lT_start[s], q1 = a.m2lT_start[s + 1];
    const double sx = a.cv.x[s], sy = a.cv.y[s], sz = a.cv.z[s];
    for (int q = q0; q < q1; q++) {
      const int t = a.m2lT_tgt[q];
      __syncwarp();
      for (int e = lane; e < 3 * K; e += 32) {
        int j, k;
        jk_of(e / 3, j, k);
        const zd v = ldz(a.Lb + (size_t)t * 3 * K + e);
        Lt[e]      = (j & 1) ? zd{-v.r, -v.i} : v;
      }
      if (lane < P) {
        const double dx = a.cv.x[t] - sx, dy = a.cv.y[t] - sy, dz = a.cv.z[t] - sz;
        const double r2 = dx * dx + dy * dy + dz * dz, ir2 = 1.0 / r2, S00 = sqrt(ir2);
        zd           col[P];
        singular_column<double, P>(lane, dx, dy, dz, ir2, S00, col);
        const int m = lane;
        for (int n = m; n < P; n++) {
          const zd v        = col[n];
          Sp[n * n + n + m] = (m & 1) ? zd{-v.r, -v.i} : v;
          if (m > 0)
            Sp[n * n + n - m] = conj(v);
        }
      }
      __syncwarp();
#pragma unroll
      for (int i = 0; i < NA; i++) {
        const int e = lane + 32 * i;
        if (e < NE) {
          const int d = e % 3, n = on[i], m = om[i];
          for (int j = 0; j <= P - 1 - n; j++) {
            const int qq = j + n, base = qq * qq + qq + m;
            for (int k = 0; k <= j; k++)
              cadd(acc[i], Lt[tri(j, k) * 3 + d] * conj(Sp[base - k]));
          }
        }
      }
    }
    __syncwarp();
    zd *Mpb = Lt; // [n^2+n+m][d]
#pragma unroll
    for (int i = 0; i < NA; i++) {
      const int e = lane + 32 * i;
      if (e < NE)
        Mpb[e] = acc[i];
    }
    __syncwarp();
    for (int e = lane; e < 3 * K; e += 32) {
      const int d = e % 3;
      int       n, mm;
      jk_of(e / 3, n, mm);
      zd v = Mpb[(n * n + n + mm) * 3 + d];
      if (mm & 1)
        v = {-v.r, -v.i};
      if (mm > 0)
        cadd(v, conj(Mpb[(n * n + n - mm) * 3 + d]));
      stz(a.Mb + (size_t)s * 3 * K + e, v);
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------------ M2M^T
// Forward (m2m_term_sum): M_parent[j,k] += terms in M_child[j-n, .] and the
// regular harmonics of X_parent - X_child.  Transposed, per child
// coefficient (j', k'), over n <= P-1-j' and the parent's (j' + n, k):
//   term 1 (k' >= 1, m = k - k', |m| <= n): +-Mbar_p[j,k] (Y[n,m] | conj Y[n,|m|]),
//   term 2 (m = k + k' <= n):               +-conj(Mbar_p[j,k] Y[n,m]).
// T = float: Mbar_parent[j] R_p^j in, harmonics at (X_parent - X_child) / R_p,
// Mbar_child[j'] += the FP32 sum / R_p^{j'} (the forward's k_m2m32 scaling).
template <int P, class T>
__global__ void __launch_bounds__(128) k_adj_m2m(AdjDev a, const int *cells, int count)
{
  typedef cx<T> zt;
  constexpr bool MIX = sizeof(T) == 4;
  constexpr int  K   = nterms(P);
  extern __shared__ double2 smem_raw[];
  zt *Mp = reinterpret_cast<zt *>(smem_raw); // [3K]
  zt *Ys = Mp + 3 * K;                       // [8][K]
  for (int pi = blockIdx.x; pi < count; pi += gridDim.x) {
    const int c = cells[pi], nch = a.cv.nchild[c], ch0 = a.cv.child[c];
    if (nch == 0)
      continue;
    const int    lev = a.cv.level[c];
    const double iRp = MIX ? ldexp(1.0 / a.R0, lev) : 1.0;
    __syncthreads();
    for (int e = threadIdx.x; e < 3 * K; e += blockDim.x) {
      const double2 v  = a.Mb[(size_t)c * 3 * K + e];
      double        sc = 1.0;
      if (MIX) {
        int j, k;
        jk_of(e / 3, j, k);
        sc = ldexp(a.R0pow[j], -lev * j); // R_p^j
      }
      Mp[e] = {(T)(v.x * sc), (T)(v.y * sc)};
    }
    if (threadIdx.x < nch) {
      const int ch = ch0 + threadIdx.x;
      regular_harmonics<T, P>((T)((a.cv.x[c] - a.cv.x[ch]) * iRp), (T)((a.cv.y[c] - a.cv.y[ch]) * iRp), (T)((a.cv.z[c] - a.cv.z[ch]) * iRp),
                              Ys + threadIdx.x * K);
    }
    __syncthreads();
    for (int o = threadIdx.x; o < nch * 3 * K; o += blockDim.x) {
      const int ci = o / (3 * K), r = o % (3 * K), d = r % 3;
      int       jp, kp;
      jk_of(r / 3, jp, kp);
      const zt *Y = Ys + ci * K;
      zt        acc{T(0), T(0)};
      for (int n = 0; n <= P - 1 - jp; n++) {
        const int j = jp + n;
        if (kp >= 1)
          for (int k = max(0, kp - n); k <= min(j, kp + n); k++) {
            const int  m   = k - kp;
            const zt   y   = Y[tri(n, m > 0 ? m : -m)];
            const bool neg = ((m < 0 ? (m & 1) : 0) ^ (n & 1)) != 0;
            cadd(acc, neg_if(Mp[tri(j, k) * 3 + d] * (m > 0 ? y : conj(y)), neg));
          }
        for (int k = 0; k <= n - kp; k++) {
          const int  m   = k + kp;
          const bool neg = ((k + n + m) & 1) != 0;
          cadd(acc, neg_if(conj(Mp[tri(j, k) * 3 + d] * Y[tri(n, m)]), neg));
        }
      }
      const double sc = MIX ? ldexp(a.iR0pow[jp], lev * jp) : 1.0; // R_p^{-j'}
      double2     *q  = a.Mb + (size_t)(ch0 + ci) * 3 * K + r;
      *q              = make_double2(q->x + (double)acc.r * sc, q->y + (double)acc.i * sc);
    }
  }
}

// ------------------------------------------------------------------ P2M^T
// Forward (k_p2m): M_d[n,m] = sum_b alpha_bd conj(Y_n^m(x_b - X_c)).
//   alphabar_bd = sum Re(Mbar_d[n,m] Y_n^m(x_b - X_c)),
//   xbar_b = sum_d alpha_bd grad phi_d,  phi_d(x) = sum Re(Mbar_d[n,m] Y_n^m(x)),
// the gradient from the derivative operators applied to Mbar_d written as a
// full-range real expansion (m > 0 terms halved).
// T = float: at y = (x - X_c) / R_c with Mbar_d[n] R_c^n (the forward's
// k_p2m32 scaling); the position adjoint is the y-gradient over R_c.
template <int P, class T>
struct AdjP2MSizes {
  static constexpr int    K = nterms(P), N1 = nterms(P - 1);
  static constexpr size_t bytes = (size_t)(6 * K + 9 * N1) * sizeof(cx<T>);
};

template <int P, class T>
__global__ void __launch_bounds__(128) k_adj_p2m(AdjDev a)
{
  typedef cx<T> zt;
  constexpr bool MIX = sizeof(T) == 4;
  constexpr int  K = nterms(P), N1 = nterms(P - 1);
  extern __shared__ double2 smem_raw[];
  zt                 *Mb = reinterpret_cast<zt *>(smem_raw); // [K][3]
  zt                 *Cn = Mb + 3 * K;                       // [K][3]
  zt                 *DM = Cn + 3 * K;                       // [N1][9]: D_ax of component d at ax * 3 + d
  const HarmRecip<T> &hr = harm_recip<T>();
  for (int li = blockIdx.x; li < a.nleaves; li += gridDim.x) {
    const int c = a.leaf_cells[li];
    if (a.cv.level[c] == 0)
      continue; // the forward P2M skips level 0
    const int    b0 = a.cv.body[c], nb = a.cv.nbody[c], lev = a.cv.level[c];
    const double cxx = a.cv.x[c], cyy = a.cv.y[c], czz = a.cv.z[c];
    const double iRc = MIX ? ldexp(1.0 / a.R0, lev) : 1.0;
    __syncthreads();
    for (int e = threadIdx.x; e < 3 * K; e += blockDim.x) {
      int n, m;
      jk_of(e / 3, n, m);
      const double2 v  = a.Mb[(size_t)c * 3 * K + e];
      const double  sc = MIX ? ldexp(a.R0pow[n], -lev * n) : 1.0; // R_c^n
      const zt      w  = {(T)(v.x * sc), (T)(v.y * sc)};
      Mb[e]            = w;
      Cn[e]            = m == 0 ? w : zt{T(0.5) * w.r, T(0.5) * w.i};
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 9 * N1; e += blockDim.x) {
      const int idx = e / 9, r = e % 9;
      int       n, mu;
      jk_of(idx, n, mu);
      DM[idx * 9 + r] = deriv_coef(Cn, n, mu, r / 3, 3, r % 3);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
      const int    b = b0 + t;
      const T      x = (T)((B(a, F_X, b) - cxx) * iRc), y = (T)((B(a, F_X + 1, b) - cyy) * iRc), z = (T)((B(a, F_X + 2, b) - czz) * iRc);
      const double al[3] = {B(a, F_A, b), B(a, F_A + 1, b), B(a, F_A + 2, b)};
      const T      r2    = x * x + y * y + z * z;
      T            ab[3] = {T(0), T(0), T(0)}, F[9];
      for (int k = 0; k < 9; k++)
        F[k] = T(0);
      zt diag{T(1), T(0)};
      for (int m = 0; m < P; m++) {
        if (m > 0) {
          const T s = hr.s[m];
          diag      = {(diag.r * x - diag.i * y) * s, (diag.r * y + diag.i * x) * s};
        }
        const T wm = m == 0 ? T(1) : T(2);
        zt      ya = diag, yb{T(0), T(0)};
        T       tn = T(2 * m + 1);
        for (int n = m; n < P; n++, tn += T(2)) {
          const int ti = tri(n, m);
          for (int d = 0; d < 3; d++)
            ab[d] += Mb[ti * 3 + d].r * ya.r - Mb[ti * 3 + d].i * ya.i;
          if (n <= P - 2)
            for (int k = 0; k < 9; k++)
              F[k] += wm * (DM[ti * 9 + k].r * ya.r - DM[ti * 9 + k].i * ya.i);
          if (n + 1 < P) {
            const T  cc = hr.c[ti], zz = tn * z;
            const zt nx = {cc * (zz * ya.r + r2 * yb.r), cc * (zz * ya.i + r2 * yb.i)};
            yb          = ya;
            ya          = nx;
          }
        }
      }
      for (int d = 0; d < 3; d++)
        W(a, W_AP2M + d, b) = (double)ab[d];
      for (int ax = 0; ax < 3; ax++)
        W(a, W_XF + ax, b) += (al[0] * F[ax * 3] + al[1] * F[ax * 3 + 1] + al[2] * F[ax * 3 + 2]) * iRc;
    }
  }
}

// ------------------------------------------------------------------ P2P^T
// One pair of the forward near field (target i, source j, d = x_i - x_j,
// sigma = sigma_j, R^2 != 0): u_i -= q (d x alpha_j), J_i -= grad_d(q (d x alpha_j)),
// q = g / (4 pi r^3), g = erf(sqrt(RS)) - (2/sqrt(pi)) sqrt(RS) e^-RS,
// RS = r^2 / (2 sigma^2).  Its part of S = ubar.u + Jbar:J is
//   s = -q (A + C) - h B,  A = alpha.(ubar x d), B = alpha.((Jbar d) x d),
//   C = alpha.ct,  ct_c = eps_abc Jbar_ab,  h = q'(r)/r,
// and the derivatives below follow with q_{r^2} = h/2 and
//   h_{r^2} = c4 (-2.5 t2/(sigma^2 r^2) - 0.5 t2/sigma^4 + 7.5 g/r^4),
// t2 = (2/sqrt(pi)) sqrt(RS) e^-RS, c4 = 1/(4 pi r^3).
// gd = ds/dd (to x_i; minus to x_j), wa = ds/dalpha_j.
__device__ __forceinline__ void pair_adj(double dx, double dy, double dz, const double *al, double sg, const double *ub, const double *Jb,
                                         const double *ct, double *gd, double *wa, double *sgb = nullptr)
{
  const double R2 = dx * dx + dy * dy + dz * dz;
  const double S2 = sg * sg, RS = R2 / S2 / 2.0, sqrtRS = sqrt(RS);
  const double erfS = erf(sqrtRS), expm = exp(-RS), invR = 1.0 / sqrt(R2);
  const double t2 = 2.0 * kInvSqrtPi * sqrtRS * expm, c4 = 0.25 * kInvPi / R2 * invR, g = erfS - t2;
  const double q   = g * c4;
  const double h   = c4 * (t2 / S2 - 3.0 * g / R2);
  const double hR2 = c4 * (-2.5 * t2 / (S2 * R2) - 0.5 * t2 / (S2 * S2) + 7.5 * g / (R2 * R2));
  const double d[3] = {dx, dy, dz};
  double       m[3];
  for (int r = 0; r < 3; r++)
    m[r] = Jb[3 * r] * dx + Jb[3 * r + 1] * dy + Jb[3 * r + 2] * dz;
  const double uxd[3] = {ub[1] * dz - ub[2] * dy, ub[2] * dx - ub[0] * dz, ub[0] * dy - ub[1] * dx};
  const double mxd[3] = {m[1] * dz - m[2] * dy, m[2] * dx - m[0] * dz, m[0] * dy - m[1] * dx};
  const double A = al[0] * uxd[0] + al[1] * uxd[1] + al[2] * uxd[2];
  const double Bv = al[0] * mxd[0] + al[1] * mxd[1] + al[2] * mxd[2];
  const double C = al[0] * ct[0] + al[1] * ct[1] + al[2] * ct[2];
  const double dxa[3] = {dy * al[2] - dz * al[1], dz * al[0] - dx * al[2], dx * al[1] - dy * al[0]};
  const double axu[3] = {al[1] * ub[2] - al[2] * ub[1], al[2] * ub[0] - al[0] * ub[2], al[0] * ub[1] - al[1] * ub[0]};
  const double axm[3] = {al[1] * m[2] - al[2] * m[1], al[2] * m[0] - al[0] * m[2], al[0] * m[1] - al[1] * m[0]};
  const double fq = -h * (A + C) - 2.0 * hR2 * Bv; // -2 q_{r^2} (A + C) - 2 h_{r^2} B
  for (int k = 0; k < 3; k++) {
    const double jtd = Jb[k] * dxa[0] + Jb[3 + k] * dxa[1] + Jb[6 + k] * dxa[2];
    gd[k]            = fq * d[k] - q * axu[k] - h * (jtd + axm[k]);
    wa[k]            = -q * uxd[k] - h * mxd[k] - q * ct[k];
  }
  // ds/dsigma of the source radius: sigma dq/dsigma = -(3q + R^2 h) and
  // sigma dh/dsigma = -(5h + 2 R^2 h_{r^2}) for s = -q (A + C) - h B
  if (sgb)
    *sgb = ((3.0 * q + R2 * h) * (A + C) + (5.0 * h + 2.0 * R2 * hR2) * Bv) / sg;
}

__device__ __forceinline__ void load_seeds(const AdjDev &a, int i, double *ub, double *Jb, double *ct)
{
  for (int k = 0; k < 3; k++)
    ub[k] = W(a, W_SU + k, i);
  for (int k = 0; k < 9; k++)
    Jb[k] = W(a, W_SJ + k, i);
  ct[0] = Jb[5] - Jb[7];
  ct[1] = Jb[6] - Jb[2];
  ct[2] = Jb[1] - Jb[3];
}

// Per target: xbar_i += sum over its near sources of ds/dd.
__global__ void __launch_bounds__(128) k_adj_p2p_tgt(AdjDev a)
{
  __shared__ double red[128 * 3];
  for (int li = blockIdx.x; li < a.nleaves; li += gridDim.x) {
    const int c = a.leaf_cells[li], b0 = a.cv.body[c], nb = a.cv.nbody[c];
    const int q0 = a.p2p_start[c], q1 = a.p2p_start[c + 1];
    for (int tc = 0; tc < nb; tc += 128) {
      const int nbc = min(128, nb - tc);
      const int TG = nbc <= 32 ? 32 : (nbc <= 64 ? 64 : 128), G = 128 / TG;
      const int tt = threadIdx.x % TG, g = threadIdx.x / TG;
      double    s[3] = {0, 0, 0};
      if (tt < nbc) {
        const int    i  = b0 + tc + tt;
        const double xi = B(a, F_X, i), yi = B(a, F_X + 1, i), zi = B(a, F_X + 2, i);
        double       ub[3], Jb[9], ct[3];
        load_seeds(a, i, ub, Jb, ct);
        for (int q = q0 + g; q < q1; q += G) {
          const int sc = a.p2p_src[q], sb = a.cv.body[sc], sn = a.cv.nbody[sc];
          for (int j = sb; j < sb + sn; j++) {
            const double dx = xi - B(a, F_X, j), dy = yi - B(a, F_X + 1, j), dz = zi - B(a, F_X + 2, j);
            if (dx * dx + dy * dy + dz * dz != 0) {
              const double al[3] = {B(a, F_A, j), B(a, F_A + 1, j), B(a, F_A + 2, j)};
              double       gd[3], wa[3];
              pair_adj(dx, dy, dz, al, B(a, F_R, j), ub, Jb, ct, gd, wa);
              for (int k = 0; k < 3; k++)
                s[k] += gd[k];
            }
          }
        }
      }
      __syncthreads();
      for (int k = 0; k < 3; k++)
        red[threadIdx.x * 3 + k] = s[k];
      __syncthreads();
      if (threadIdx.x < nbc) {
        const int i = b0 + tc + threadIdx.x;
        for (int k = 0; k < 3; k++) {
          double v = 0;
          for (int gg = 0; gg < G; gg++)
            v += red[(gg * TG + threadIdx.x) * 3 + k];
          W(a, W_XNT + k, i) = v;
        }
      }
    }
  }
}

// Per source: xbar_j -= sum over its near targets of ds/dd, alphabar_j += ds/dalpha_j.
__global__ void __launch_bounds__(128) k_adj_p2p_src(AdjDev a)
{
  __shared__ double red[128 * 7];
  for (int li = blockIdx.x; li < a.nleaves; li += gridDim.x) {
    const int c = a.leaf_cells[li], b0 = a.cv.body[c], nb = a.cv.nbody[c];
    const int q0 = a.p2pT_start[c], q1 = a.p2pT_start[c + 1];
    for (int tc = 0; tc < nb; tc += 128) {
      const int nbc = min(128, nb - tc);
      const int TG = nbc <= 32 ? 32 : (nbc <= 64 ? 64 : 128), G = 128 / TG;
      const int tt = threadIdx.x % TG, g = threadIdx.x / TG;
      double    s[7] = {0, 0, 0, 0, 0, 0, 0};
      if (tt < nbc) {
        const int    j  = b0 + tc + tt;
        const double xj = B(a, F_X, j), yj = B(a, F_X + 1, j), zj = B(a, F_X + 2, j);
        const double al[3] = {B(a, F_A, j), B(a, F_A + 1, j), B(a, F_A + 2, j)};
        const double sg    = B(a, F_R, j);
        for (int q = q0 + g; q < q1; q += G) {
          const int tcell = a.p2pT_tgt[q], tb = a.cv.body[tcell], tn = a.cv.nbody[tcell];
          for (int i = tb; i < tb + tn; i++) {
            const double dx = B(a, F_X, i) - xj, dy = B(a, F_X + 1, i) - yj, dz = B(a, F_X + 2, i) - zj;
            if (dx * dx + dy * dy + dz * dz != 0) {
              double ub[3], Jb[9], ct[3], gd[3], wa[3], sgb;
              load_seeds(a, i, ub, Jb, ct);
              pair_adj(dx, dy, dz, al, sg, ub, Jb, ct, gd, wa, &sgb);
              for (int k = 0; k < 3; k++) {
                s[k] -= gd[k];
                s[3 + k] += wa[k];
              }
              s[6] += sgb;
            }
          }
        }
      }
      __syncthreads();
      for (int k = 0; k < 7; k++)
        red[threadIdx.x * 7 + k] = s[k];
      __syncthreads();
      if (threadIdx.x < nbc) {
        const int j = b0 + tc + threadIdx.x;
        for (int k = 0; k < 7; k++) {
          double v = 0;
          for (int gg = 0; gg < G; gg++)
            v += red[(gg * TG + threadIdx.x) * 7 + k];
          W(a, k < 3 ? W_XNS + k : (k < 6 ? W_ANS + k - 3 : W_RNS), j) = v;
        }
      }
    }
  }
}

// ------------------------------------------------------------------ bodies
// Seeds of an evaluation from the stage cotangent (cu, ca) of (u, dalpha/dt):
// ubar = cu and, for dalpha/dt = J^T alpha (transposed) or J alpha
// (classic), Jbar and the direct alphabar.
__global__ void k_adj_seeds(const double *soa, double *w, size_t cap, int n, int stretching, int add_relax, int formulation)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    auto         S  = [&](int f) -> double & { return w[(size_t)f * cap + i]; };
    auto         Bf = [&](int f) { return soa[(size_t)f * cap + i]; };
    double       ca[3] = {S(W_COT + 3), S(W_COT + 4), S(W_COT + 5)};
    const double al[3] = {Bf(F_A), Bf(F_A + 1), Bf(F_A + 2)};
    double       ab_rvpm[3] = {0, 0, 0}, rb_rvpm = 0;
    if (formulation == VFMM_RVPM) {
      // rVPM terms (fmmCalculator.hpp:407-418) with d the stretching term:
      // dalpha/dt = d - 3/5 (d.alpha) alpha / |alpha|^2, dr/dt = -1/5 r (d.alpha) / |alpha|^2.
      // Their cotangents (ca, cr) give d's cotangent (which then seeds the
      // stretching as ca does for cVPM) and direct alpha and r cotangents.
      double ds[3];
      for (int dd = 0; dd < 3; dd++) {
        double v = 0;
        for (int e = 0; e < 3; e++)
          v += (stretching == VFMM_TRANSPOSED ? Bf(F_J + 3 * e + dd) : Bf(F_J + 3 * dd + e)) * al[e];
        ds[dd] = v;
      }
      const double cr = S(W_COT + 6), rr = Bf(F_R);
      const double q2 = al[0] * al[0] + al[1] * al[1] + al[2] * al[2], sd = ds[0] * al[0] + ds[1] * al[1] + ds[2] * al[2];
      const double cal = ca[0] * al[0] + ca[1] * al[1] + ca[2] * al[2];
      for (int dd = 0; dd < 3; dd++)
        ab_rvpm[dd] = -0.6 * (cal * ds[dd] + sd * ca[dd]) / q2 + 1.2 * sd * cal * al[dd] / (q2 * q2) -
                      0.2 * rr * cr * (ds[dd] / q2 - 2.0 * sd * al[dd] / (q2 * q2));
      rb_rvpm = -0.2 * sd * cr / q2;
      for (int dd = 0; dd < 3; dd++)
        ca[dd] -= (0.6 * cal + 0.2 * rr * cr) * al[dd] / q2;
    }
    S(W_RD) = rb_rvpm;
    for (int k = 0; k < 3; k++)
      S(W_SU + k) = S(W_COT + k);
    for (int r = 0; r < 3; r++)
      for (int cc = 0; cc < 3; cc++) {
        // transposed: dadt_c' = sum_r J[r][c'] alpha_r -> Jbar[r][c'] = alpha_r ca_c'
        // classic:    dadt_r  = sum_c J[r][c] alpha_c  -> Jbar[r][c]  = ca_r alpha_c
        S(W_SJ + 3 * r + cc) = stretching == VFMM_TRANSPOSED ? al[r] * ca[cc] : ca[r] * al[cc];
      }
    if (add_relax) { // w = (J21 - J12, J02 - J20, J10 - J01) of the relaxation after this stage
      const double wb[3] = {S(W_WB), S(W_WB + 1), S(W_WB + 2)};
      S(W_SJ + 7) += wb[0];
      S(W_SJ + 5) -= wb[0];
      S(W_SJ + 2) += wb[1];
      S(W_SJ + 6) -= wb[1];
      S(W_SJ + 3) += wb[2];
      S(W_SJ + 1) -= wb[2];
    }
    for (int cc = 0; cc < 3; cc++) {
      double v = 0;
      for (int r = 0; r < 3; r++)
        v += (stretching == VFMM_TRANSPOSED ? Bf(F_J + 3 * cc + r) : Bf(F_J + 3 * r + cc)) * ca[r];
      S(W_ASTR + cc) = v + ab_rvpm[cc];
    }
  }
}

// Transposed relaxation (relaxation.hpp:8-19 as bodies.cu relax_one applies
// it after a step's last stage update): alpha' = (1 - f) alpha_u + f |alpha_u|
// w / |w| with w = (J21 - J12, J02 - J20, J10 - J01) of the stage's
// evaluation.  g[AB] holds the cotangent of alpha' and leaves with that of
// alpha_u; w[W_WB] gets the cotangent of w, which k_adj_seeds adds to the J
// seeds.  Where w = 0 relaxation is the identity.
__global__ void k_adj_relax(double *g, double *w, const double *soa, const double *au, size_t cap, int n, double f)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    auto         J     = [&](int k) { return soa[(size_t)(F_J + k) * cap + i]; };
    const double om[3] = {J(7) - J(5), J(2) - J(6), J(3) - J(1)};
    const double nw    = sqrt(om[0] * om[0] + om[1] * om[1] + om[2] * om[2]);
    double      *wb    = w + (size_t)W_WB * cap + i;
    if (nw == 0.0) {
      wb[0] = wb[cap] = wb[2 * cap] = 0.0;
      continue;
    }
    const double a[3]  = {au[i], au[cap + i], au[2 * cap + i]};
    const double na    = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    double      *ab    = g + (size_t)G_AB * cap + i;
    const double ga[3] = {ab[0], ab[cap], ab[2 * cap]};
    const double wh[3] = {om[0] / nw, om[1] / nw, om[2] / nw};
    const double dot   = wh[0] * ga[0] + wh[1] * ga[1] + wh[2] * ga[2]; // d alpha'/d|alpha_u| . gbar
    for (int d = 0; d < 3; d++) {
      ab[(size_t)d * cap] = (1 - f) * ga[d] + (na > 0 ? f * dot * a[d] / na : 0.0);
      wb[(size_t)d * cap] = f * na / nw * (ga[d] - dot * wh[d]);
    }
  }
}

// The transposed stage update (bodies.cu k_stage_update) in the tree order
// of the stage: the stage's cotangent of (u, dalpha/dt) into W_COT, the
// adjoint state g updated except for the evaluation's own contribution.
__global__ void k_adj_stage_pre(double *g, double *w, size_t cap, int n, int scheme, int stage, double h, int rk4_fixed)
{
  const double A  = stage == 0 ? 0.0 : (stage == 1 ? -5.0 / 9.0 : -153.0 / 128.0);
  const double Bc = stage == 0 ? 1.0 / 3.0 : (stage == 1 ? 15.0 / 16.0 : 8.0 / 15.0);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    auto G  = [&](int f) -> double & { return g[(size_t)f * cap + i]; };
    auto Wc = [&](int f) -> double & { return w[(size_t)(W_COT + f) * cap + i]; };
    for (int k = 0; k < 3; k++) {
      double *xb = &G(G_XB + k), *ab = &G(G_AB + k), *vb = &G(G_VB + k), *db = &G(G_DB + k), *xob = &G(G_XOB + k), *aob = &G(G_AOB + k);
      if (scheme == VFMM_EULER) { // x' = x + h f
        Wc(k)     = h * *xb;
        Wc(3 + k) = h * *ab;
      } else if (scheme == VFMM_RK2 && stage == 0) { // xold = x; v = f; x' = x + h v
        const double vt = *vb + h * *xb, dt_ = *db + h * *ab;
        Wc(k)           = vt;
        Wc(3 + k)       = dt_;
        *xb += *xob;
        *ab += *aob;
        *vb = *db = *xob = *aob = 0;
      } else if (scheme == VFMM_RK2) { // v' = f/2 + v/2; x' = xold + h v'
        const double vt = *vb + h * *xb, dt_ = *db + h * *ab;
        Wc(k)           = 0.5 * vt;
        Wc(3 + k)       = 0.5 * dt_;
        *xob += *xb;
        *aob += *ab;
        *xb = *ab = 0;
        *vb       = 0.5 * vt;
        *db       = 0.5 * dt_;
      } else if (scheme == VFMM_RK4 && stage == 0) { // xold = x; v = f; x' = x + h/2 v
        Wc(k)     = *vb + 0.5 * h * *xb;
        Wc(3 + k) = *db + 0.5 * h * *ab;
        *xb += *xob;
        *ab += *aob;
        *vb = *db = *xob = *aob = 0;
      } else if (scheme == VFMM_RK4 && stage < 3) { // v' = v + 2f; x' = xold + c h f
        const double c = (stage == 2 && rk4_fixed) ? 1.0 : 0.5;
        Wc(k)          = 2.0 * *vb + c * h * *xb;
        Wc(3 + k)      = 2.0 * *db + c * h * *ab;
        *xob += *xb;
        *aob += *ab;
        *xb = *ab = 0;
      } else if (scheme == VFMM_RK4) { // v' = v + f; x' = xold + h/6 v'
        const double vt = *vb + (h / 6.0) * *xb, dt_ = *db + (h / 6.0) * *ab;
        Wc(k)           = vt;
        Wc(3 + k)       = dt_;
        *xob += *xb;
        *aob += *ab;
        *xb = *ab = 0;
        *vb       = vt;
        *db       = dt_;
      } else { // RK3: Q' = A Q + h f; x' = x + B Q'
        const double qx = *vb + Bc * *xb, qa = *db + Bc * *ab;
        Wc(k)           = h * qx;
        Wc(3 + k)       = h * qa;
        *vb             = A * qx;
        *db             = A * qa;
      }
    }
    // the radius with its rate and registers (DRDTOLD, ROLD), as a strength
    // component with dalpha/dt; Wc(6) is the cotangent of dr/dt
    double *rb = &G(G_RB), *rdb = &G(G_RDB), *rob = &G(G_ROB);
    if (scheme == VFMM_EULER)
      Wc(6) = h * *rb;
    else if (scheme == VFMM_RK2 && stage == 0) {
      Wc(6) = *rdb + h * *rb;
      *rb += *rob;
      *rdb = *rob = 0;
    } else if (scheme == VFMM_RK2) {
      const double t = *rdb + h * *rb;
      Wc(6)          = 0.5 * t;
      *rob += *rb;
      *rb  = 0;
      *rdb = 0.5 * t;
    } else if (scheme == VFMM_RK4 && stage == 0) {
      Wc(6) = *rdb + 0.5 * h * *rb;
      *rb += *rob;
      *rdb = *rob = 0;
    } else if (scheme == VFMM_RK4 && stage < 3) {
      const double c = (stage == 2 && rk4_fixed) ? 1.0 : 0.5;
      Wc(6)          = 2.0 * *rdb + c * h * *rb;
      *rob += *rb;
      *rb = 0;
    } else if (scheme == VFMM_RK4) {
      const double t = *rdb + (h / 6.0) * *rb;
      Wc(6)          = t;
      *rob += *rb;
      *rb  = 0;
      *rdb = t;
    } else {
      const double qr = *rdb + Bc * *rb;
      Wc(6)           = h * qr;
      *rdb            = A * qr;
    }
  }
}

// g[XB] += the evaluation's position adjoints, g[AB] += its strength adjoints.
__global__ void k_adj_combine(double *g, const double *w, size_t cap, int n)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    for (int k = 0; k < 3; k++) {
      const size_t o = (size_t)k * cap + i;
      g[(size_t)G_XB * cap + o] += w[(size_t)W_XF * cap + o] + w[(size_t)W_XNT * cap + o] + w[(size_t)W_XNS * cap + o];
      g[(size_t)G_AB * cap + o] += w[(size_t)W_ASTR * cap + o] + w[(size_t)W_AP2M * cap + o] + w[(size_t)W_ANS * cap + o];
    }
    g[(size_t)G_RB * cap + i] += w[(size_t)W_RNS * cap + i] + w[(size_t)W_RD * cap + i];
  }
}

// Bounding-box terms.  Per block: sum xbar_far (3), sum e (1),
// sum xbar_far.(x - X0) (1), then per axis (min, argmin, max, argmax).
constexpr int GEO_BLOCKS = 152 * 2, GEO_THREADS = 256, GEO_FIELDS = 17;
__global__ void __launch_bounds__(GEO_THREADS) k_adj_geom_partial(const double *soa, const double *w, size_t cap, int n, const DevInfo *info,
                                                                   double *part)
{
  __shared__ double red[GEO_THREADS][GEO_FIELDS];
  double            v[GEO_FIELDS];
  for (int k = 0; k < 5; k++)
    v[k] = 0;
  for (int d = 0; d < 3; d++) {
    v[5 + 4 * d] = INFINITY;
    v[6 + 4 * d] = -1;
    v[7 + 4 * d] = -INFINITY;
    v[8 + 4 * d] = -1;
  }
  const double X0[3] = {info->X0[0], info->X0[1], info->X0[2]};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    for (int d = 0; d < 3; d++) {
      const double xf = w[(size_t)(W_XF + d) * cap + i], x = soa[(size_t)(F_X + d) * cap + i];
      v[d] += xf;
      v[4] += xf * (x - X0[d]);
      if (x < v[5 + 4 * d]) {
        v[5 + 4 * d] = x;
        v[6 + 4 * d] = i;
      }
      if (x > v[7 + 4 * d]) {
        v[7 + 4 * d] = x;
        v[8 + 4 * d] = i;
      }
    }
    v[3] += w[(size_t)W_EF * cap + i];
  }
  for (int k = 0; k < GEO_FIELDS; k++)
    red[threadIdx.x][k] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int t = 1; t < GEO_THREADS; t++) {
      for (int k = 0; k < 5; k++)
        v[k] += red[t][k];
      for (int d = 0; d < 3; d++) {
        const double *r = red[t];
        if (r[5 + 4 * d] < v[5 + 4 * d] || (r[5 + 4 * d] == v[5 + 4 * d] && r[6 + 4 * d] >= 0 && r[6 + 4 * d] < v[6 + 4 * d])) {
          v[5 + 4 * d] = r[5 + 4 * d];
          v[6 + 4 * d] = r[6 + 4 * d];
        }
        if (r[7 + 4 * d] > v[7 + 4 * d] || (r[7 + 4 * d] == v[7 + 4 * d] && r[8 + 4 * d] >= 0 && r[8 + 4 * d] < v[8 + 4 * d])) {
          v[7 + 4 * d] = r[7 + 4 * d];
          v[8 + 4 * d] = r[8 + 4 * d];
        }
      }
    }
    for (int k = 0; k < GEO_FIELDS; k++)
      part[blockIdx.x * GEO_FIELDS + k] = v[k];
  }
}

// Combines the block partials: one warp, lane l over blocks l, l+32, ...,
// then a fixed-order combine across lanes in lane 0.
__global__ void k_adj_geom_final(const double *part, int nb, const DevInfo *info, double *g, size_t cap)
{
  __shared__ double red[32][GEO_FIELDS];
  const int         l = threadIdx.x;
  if (blockIdx.x || l >= 32)
    return;
  auto merge = [](double *v, const double *r) {
    for (int k = 0; k < 5; k++)
      v[k] += r[k];
    for (int d = 0; d < 3; d++) {
      if (r[5 + 4 * d] < v[5 + 4 * d] || (r[5 + 4 * d] == v[5 + 4 * d] && r[6 + 4 * d] >= 0 && (v[6 + 4 * d] < 0 || r[6 + 4 * d] < v[6 + 4 * d]))) {
        v[5 + 4 * d] = r[5 + 4 * d];
        v[6 + 4 * d] = r[6 + 4 * d];
      }
      if (r[7 + 4 * d] > v[7 + 4 * d] || (r[7 + 4 * d] == v[7 + 4 * d] && r[8 + 4 * d] >= 0 && (v[8 + 4 * d] < 0 || r[8 + 4 * d] < v[8 + 4 * d]))) {
        v[7 + 4 * d] = r[7 + 4 * d];
        v[8 + 4 * d] = r[8 + 4 * d];
      }
    }
  };
  double v[GEO_FIELDS];
  for (int k = 0; k < 5; k++)
    v[k] = 0;
  for (int d = 0; d < 3; d++) {
    v[5 + 4 * d] = INFINITY;
    v[6 + 4 * d] = -1;
    v[7 + 4 * d] = -INFINITY;
    v[8 + 4 * d] = -1;
  }
  for (int b = l; b < nb; b += 32)
    merge(v, part + b * GEO_FIELDS);
  for (int k = 0; k < GEO_FIELDS; k++)
    red[l][k] = v[k];
  __syncwarp();
  if (l != 0)
    return;
  for (int t = 1; t < 32; t++)
    merge(v, red[t]);
  const double R0 = info->R0;
  if (!(R0 > 0))
    return;
  const double R0b = (v[3] - v[4]) / R0;
  int          ds  = 0;
  for (int d = 1; d < 3; d++)
    if (v[7 + 4 * d] - v[5 + 4 * d] > v[7 + 4 * ds] - v[5 + 4 * ds])
      ds = d;
  for (int d = 0; d < 3; d++) {
    const int    imn = (int)v[6 + 4 * d], imx = (int)v[8 + 4 * d];
    const double X0b = -v[d];
    double       gmn = 0.5 * X0b, gmx = 0.5 * X0b;
    if (d == ds) { // R0 = 1.00001 (max - min) / 2 along the widest axis
      gmx += 0.5 * 1.00001 * R0b;
      gmn -= 0.5 * 1.00001 * R0b;
    }
    if (imn >= 0)
      g[(size_t)(G_XB + d) * cap + imn] += gmn;
    if (imx >= 0)
      g[(size_t)(G_XB + d) * cap + imx] += gmx;
  }
}

// out[f][perm[p]] = in[f][p] for the NG adjoint-state fields.
__global__ void k_adj_scatter(const double *__restrict__ in, double *__restrict__ out, size_t cap, int n, const uint32_t *__restrict__ perm)
{
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const uint32_t q = perm[p];
    for (int f = 0; f < NG; f++)
      out[(size_t)f * cap + q] = in[(size_t)f * cap + p];
  }
}

__global__ void k_orig_update(const int *__restrict__ in, int *__restrict__ out, const uint32_t *__restrict__ perm, int n)
{
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
    out[p] = in[perm[p]];
}

__global__ void k_iota_int(int *a, int n)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    a[i] = i;
}

// Objective at the final state (bodies in the order of their last tree, u
// from an FP64 evaluation; orig = index of each body in the caller's array):
//   value = wE sum u.(x cross alpha) + 1/2 wI.sum x cross alpha + seeds.(x, alpha),
// its direct derivatives into g, the seed of u into W_SU (Jbar = 0).
constexpr int OBJ_BLOCKS = 152 * 2, OBJ_THREADS = 256;
__global__ void __launch_bounds__(OBJ_THREADS) k_adj_objective(const double *soa, size_t cap, int n, const int *orig, const double *seed_x,
                                                                const double *seed_a, double wE, double wI0, double wI1, double wI2, double *g,
                                                                double *w, double *part)
{
  __shared__ double red[OBJ_THREADS];
  const double      wI[3] = {wI0, wI1, wI2};
  double            acc   = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    auto         Bf = [&](int f) { return soa[(size_t)f * cap + i]; };
    const double x[3] = {Bf(F_X), Bf(F_X + 1), Bf(F_X + 2)}, al[3] = {Bf(F_A), Bf(F_A + 1), Bf(F_A + 2)},
                 u[3] = {Bf(F_U), Bf(F_U + 1), Bf(F_U + 2)};
    const double xa[3] = {x[1] * al[2] - x[2] * al[1], x[2] * al[0] - x[0] * al[2], x[0] * al[1] - x[1] * al[0]};
    const double au[3] = {al[1] * u[2] - al[2] * u[1], al[2] * u[0] - al[0] * u[2], al[0] * u[1] - al[1] * u[0]};
    const double ux[3] = {u[1] * x[2] - u[2] * x[1], u[2] * x[0] - u[0] * x[2], u[0] * x[1] - u[1] * x[0]};
    const double aw[3] = {al[1] * wI[2] - al[2] * wI[1], al[2] * wI[0] - al[0] * wI[2], al[0] * wI[1] - al[1] * wI[0]};
    const double wx[3] = {wI[1] * x[2] - wI[2] * x[1], wI[2] * x[0] - wI[0] * x[2], wI[0] * x[1] - wI[1] * x[0]};
    const int    o     = orig[i];
    for (int k = 0; k < 3; k++) {
      const double sx = seed_x ? seed_x[3 * (size_t)o + k] : 0.0, sa = seed_a ? seed_a[3 * (size_t)o + k] : 0.0;
      acc += wE * u[k] * xa[k] + 0.5 * wI[k] * xa[k] + sx * x[k] + sa * al[k];
      g[(size_t)(G_XB + k) * cap + i]  = wE * au[k] + 0.5 * aw[k] + sx;
      g[(size_t)(G_AB + k) * cap + i]  = wE * ux[k] + 0.5 * wx[k] + sa;
      g[(size_t)(G_VB + k) * cap + i]  = 0;
      g[(size_t)(G_DB + k) * cap + i]  = 0;
      g[(size_t)(G_XOB + k) * cap + i] = 0;
      g[(size_t)(G_AOB + k) * cap + i] = 0;
      w[(size_t)(W_SU + k) * cap + i]   = wE * xa[k];
      w[(size_t)(W_ASTR + k) * cap + i] = 0;
    }
    for (int k = 0; k < 9; k++)
      w[(size_t)(W_SJ + k) * cap + i] = 0;
    g[(size_t)G_RB * cap + i] = g[(size_t)G_RDB * cap + i] = g[(size_t)G_ROB * cap + i] = 0;
    w[(size_t)W_RD * cap + i] = 0;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int st = OBJ_THREADS / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      red[threadIdx.x] += red[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    part[blockIdx.x] = red[0];
}

__global__ void k_sum_final(const double *part, int nb, double *out)
{
  if (threadIdx.x || blockIdx.x)
    return;
  double v = 0;
  for (int b = 0; b < nb; b++)
    v += part[b];
  *out = v;
}

__global__ void k_adj_rows(const double *g, size_t cap, int n, int field, double *rows)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int k = 0; k < 3; k++)
      rows[3 * (size_t)i + k] = g[(size_t)(field + k) * cap + i];
}

// ------------------------------------------------------------------ FP32 reverse passes
// Mixed mode runs the two dominant transposes, P2P^T and M2L^T, in FP32.
//
// P2P^T: the radial functions of one pair are written through
//   F(s) = g(s) s^{-3/2},  s = r^2 / (2 sigma^2),
// so that q = c F, h = c F' / sigma^2, h_{r^2} = c F'' / (2 sigma^4) with
// c = 1 / (4 pi 2^{3/2} sigma^3); F and its derivatives come from the series
// F = (2/sqrt(pi)) sum_k (-1)^k s^k / (k! (k + 3/2)) for s < 2 (g' = (2/sqrt(pi))
// sqrt(s) e^-s integrated termwise; no cancellation at small r) and from the
// closed forms in g, g', g'' above.  Positions are the evaluation's
// leaf-relative FP32 records; partial sums per leaf are folded into a
// float-float (two-sum) accumulator.
struct SeriesF {
  float a[17]; // (2/sqrt(pi)) (-1)^k / (k! (k + 3/2))
};
constexpr SeriesF make_series_f()
{
  SeriesF r{};
  double  f = 1.0;
  for (int k = 0; k < 17; k++) {
    if (k > 0)
      f *= k;
    r.a[k] = (float)(1.128379167095512573896158903121545172 * ((k & 1) ? -1.0 : 1.0) / (f * (k + 1.5)));
  }
  return r;
}
static __constant__ SeriesF kSeriesF = make_series_f();

__device__ __forceinline__ void radial_F(float s, float &F, float &F1, float &F2)
{
  if (s < 2.0f) {
    float p = kSeriesF.a[16], p1 = 0.f, p2 = 0.f;
#pragma unroll
    for (int k = 15; k >= 0; k--) {
      p2 = fmaf(p2, s, p1);
      p1 = fmaf(p1, s, p);
      p  = fmaf(p, s, kSeriesF.a[k]);
    }
    F  = p;
    F1 = p1;
    F2 = 2.f * p2;
  } else {
    const float tsp = 1.1283791670955126f; // 2 / sqrt(pi)
    const float rs = sqrtf(s), e = expf(-s), is = 1.f / s, is15 = is / rs;
    const float g1 = tsp * rs * e, g = erff(rs) - g1, g2 = tsp * e * (0.5f / rs - rs);
    F  = g * is15;
    F1 = (g1 - 1.5f * g * is) * is15;
    F2 = (g2 - 3.f * g1 * is + 3.75f * g * is * is) * is15;
  }
}

// ds/dd and ds/dalpha of one pair in FP32 (the algebra of pair_adj).
__device__ __forceinline__ void pair_adj32(float dx, float dy, float dz, float ax, float ay, float az, float isg, float w2, const float *ub,
                                           const float *Jb, const float *ct, float *gd, float *wa, float *sgb = nullptr)
{
  const float R2 = dx * dx + dy * dy + dz * dz;
  float       F, F1, F2;
  radial_F(R2 * w2, F, F1, F2);
  const float is2 = isg * isg, c = is2 * isg * 0.028134884879909f; // 1 / (4 pi 2^{3/2})
  const float q = c * F, h = c * F1 * is2, hR2 = 0.5f * c * F2 * is2 * is2;
  const float m0 = Jb[0] * dx + Jb[1] * dy + Jb[2] * dz, m1 = Jb[3] * dx + Jb[4] * dy + Jb[5] * dz, m2 = Jb[6] * dx + Jb[7] * dy + Jb[8] * dz;
  const float uxd0 = ub[1] * dz - ub[2] * dy, uxd1 = ub[2] * dx - ub[0] * dz, uxd2 = ub[0] * dy - ub[1] * dx;
  const float mxd0 = m1 * dz - m2 * dy, mxd1 = m2 * dx - m0 * dz, mxd2 = m0 * dy - m1 * dx;
  const float A = ax * uxd0 + ay * uxd1 + az * uxd2, Bv = ax * mxd0 + ay * mxd1 + az * mxd2, C = ax * ct[0] + ay * ct[1] + az * ct[2];
  const float dxa0 = dy * az - dz * ay, dxa1 = dz * ax - dx * az, dxa2 = dx * ay - dy * ax;
  const float axu0 = ay * ub[2] - az * ub[1], axu1 = az * ub[0] - ax * ub[2], axu2 = ax * ub[1] - ay * ub[0];
  const float axm0 = ay * m2 - az * m1, axm1 = az * m0 - ax * m2, axm2 = ax * m1 - ay * m0;
  const float fq = -h * (A + C) - 2.f * hR2 * Bv;
  gd[0] = fq * dx - q * axu0 - h * (Jb[0] * dxa0 + Jb[3] * dxa1 + Jb[6] * dxa2 + axm0);
  gd[1] = fq * dy - q * axu1 - h * (Jb[1] * dxa0 + Jb[4] * dxa1 + Jb[7] * dxa2 + axm1);
  gd[2] = fq * dz - q * axu2 - h * (Jb[2] * dxa0 + Jb[5] * dxa1 + Jb[8] * dxa2 + axm2);
  wa[0] = -q * uxd0 - h * mxd0 - q * ct[0];
  wa[1] = -q * uxd1 - h * mxd1 - q * ct[1];
  wa[2] = -q * uxd2 - h * mxd2 - q * ct[2];
  if (sgb) // ds/dsigma of the source radius, as pair_adj
    *sgb = isg * ((3.f * q + R2 * h) * (A + C) + (5.f * h + 2.f * R2 * hR2) * Bv);
}

__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float v)
{
  const float t  = hi + v;
  const float bb = t - hi;
  lo += (hi - (t - bb)) + (v - bb);
  hi = t;
}

// Seeds in FP32: [ubar0..2, ct0], [ct1, ct2, Jbar0, Jbar1], [Jbar2..5], [Jbar6..8, 0].
__global__ void k_adj_seeds32(AdjDev a, int n)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double ub[3], Jb[9], ct[3];
    load_seeds(a, i, ub, Jb, ct);
    float4 *o = a.seeds32 + 4 * (size_t)i;
    o[0]      = make_float4((float)ub[0], (float)ub[1], (float)ub[2], (float)ct[0]);
    o[1]      = make_float4((float)ct[1], (float)ct[2], (float)Jb[0], (float)Jb[1]);
    o[2]      = make_float4((float)Jb[2], (float)Jb[3], (float)Jb[4], (float)Jb[5]);
    o[3]      = make_float4((float)Jb[6], (float)Jb[7], (float)Jb[8], 0.f);
  }
}
__device__ __forceinline__ void load_seeds32(const AdjDev &a, int i, float *ub, float *Jb, float *ct)
{
  const float4 s0 = a.seeds32[4 * (size_t)i], s1 = a.seeds32[4 * (size_t)i + 1], s2 = a.seeds32[4 * (size_t)i + 2],
               s3 = a.seeds32[4 * (size_t)i + 3];
  ub[0] = s0.x, ub[1] = s0.y, ub[2] = s0.z, ct[0] = s0.w;
  ct[1] = s1.x, ct[2] = s1.y, Jb[0] = s1.z, Jb[1] = s1.w;
  Jb[2] = s2.x, Jb[3] = s2.y, Jb[4] = s2.z, Jb[5] = s2.w;
  Jb[6] = s3.x, Jb[7] = s3.y, Jb[8] = s3.z;
}

// Per target: xbar_i += sum of ds/dd (FP32, leaf-relative).  The source
// bodies of the target leaf's P2P row are staged in shared memory in chunks,
// already shifted into the target leaf's frame; every target thread (or group
// of threads) runs over the chunk, whose partial sums fold into a two-sum.
constexpr int ADJ_CH_T = 512, ADJ_CH_S = 384, ADJ_LG = 32;

// Warp 0 stages the leaves list[q .. q + ng - 1] (ng <= 32) of a P2P row:
// Loff[l] = the leaf's centre minus (cx, cy, cz) in FP32, w = its first body
// (int bits); Lpre[0 .. ng] = the exclusive prefix of the leaves' body counts.
// The row's bodies, leaf after leaf, then form one sequence of Lpre[ng].
__device__ __forceinline__ void stage_row_leaves(const AdjDev &a, const int *list, int q, int ng, double cx, double cy, double cz, float4 *Loff,
                                                 int *Lpre)
{
  const int l   = threadIdx.x & 31;
  int       cnt = 0;
  if (l < ng) {
    const int sc = list[q + l];
    cnt          = a.cv.nbody[sc];
    Loff[l]      = make_float4((float)(a.cv.x[sc] - cx), (float)(a.cv.y[sc] - cy), (float)(a.cv.z[sc] - cz), __int_as_float(a.cv.body[sc]));
  }
  int incl = cnt;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, d);
    if (l >= d)
      incl += v;
  }
  if (l < ng)
    Lpre[l] = incl - cnt;
  if (l == ng - 1)
    Lpre[ng] = incl;
}

// The leaf holding element g of that sequence: the last l < ng with Lpre[l] <= g.
__device__ __forceinline__ int row_leaf_of(const int *Lpre, int ng, int g)
{
  int lb = 0, ub = ng - 1;
  while (lb < ub) {
    const int mid = (lb + ub + 1) >> 1;
    if (Lpre[mid] <= g)
      lb = mid;
    else
      ub = mid - 1;
  }
  return lb;
}

// Chunks of a row's bodies are staged by all threads at once: each copies
// its elements e = tid + 128 i with cp.async (in flight together), then
// shifts its own positions into the frame of the block's leaf.
__global__ void __launch_bounds__(128) k_adj_p2p32_tgt(AdjDev a)
{
  __shared__ float4 Sp[ADJ_CH_T], Sa[ADJ_CH_T];
  __shared__ float  red[2][128 * 3];
  __shared__ float4 Loff[ADJ_LG];
  __shared__ int    Lpre[ADJ_LG + 1];
  static_assert(ADJ_CH_T % 128 == 0 && ADJ_CH_S % 128 == 0, "every thread stages the same number of chunk elements");
  for (int li = blockIdx.x; li < a.nleaves; li += gridDim.x) {
    const int    c = a.leaf_cells[li], b0 = a.cv.body[c], nb = a.cv.nbody[c];
    const int    q0 = a.p2p_start[c], q1 = a.p2p_start[c + 1];
    const double cx = a.cv.x[c], cy = a.cv.y[c], cz = a.cv.z[c];
    for (int tc = 0; tc < nb; tc += 128) {
      const int nbc = min(128, nb - tc);
      const int TG = nbc <= 32 ? 32 : (nbc <= 64 ? 64 : 128), G = 128 / TG;
      const int tt = threadIdx.x % TG, g = threadIdx.x / TG;
      float     hi[3] = {0.f, 0.f, 0.f}, lo[3] = {0.f, 0.f, 0.f};
      float4    pi = make_float4(0.f, 0.f, 0.f, 0.f);
      float     ub[3], Jb[9], ct[3];
      if (tt < nbc) {
        pi = a.pos32[b0 + tc + tt];
        load_seeds32(a, b0 + tc + tt, ub, Jb, ct);
      }
      for (int qg = q0; qg < q1; qg += ADJ_LG) {
        const int ng = min(ADJ_LG, q1 - qg);
        __syncthreads();
        if (threadIdx.x < 32)
          stage_row_leaves(a, a.p2p_src, qg, ng, cx, cy, cz, Loff, Lpre);
        __syncthreads();
        const int total = Lpre[ng];
        for (int c0 = 0; c0 < total; c0 += ADJ_CH_T) {
          const int cnt = min(ADJ_CH_T, total - c0);
          if (c0 > 0)
            __syncthreads();
          int lqs[ADJ_CH_T / 128];
#pragma unroll
          for (int i = 0; i < ADJ_CH_T / 128; i++) {
            const int e = threadIdx.x + 128 * i;
            lqs[i]      = e < cnt ? row_leaf_of(Lpre, ng, c0 + e) : -1;
            if (lqs[i] >= 0) {
              const int bi = __float_as_int(Loff[lqs[i]].w) + (c0 + e - Lpre[lqs[i]]);
              cp_async16(Sp + e, a.pos32 + bi);
              cp_async16(Sa + e, a.alp32 + bi);
            }
          }
          cp_async_wait_all();
#pragma unroll
          for (int i = 0; i < ADJ_CH_T / 128; i++)
            if (lqs[i] >= 0) {
              const int    e = threadIdx.x + 128 * i;
              const float4 o = Loff[lqs[i]], p = Sp[e];
              Sp[e]          = make_float4(p.x + o.x, p.y + o.y, p.z + o.z, p.w);
            }
          __syncthreads();
          if (tt < nbc) {
            float s[3] = {0.f, 0.f, 0.f};
            for (int j = g; j < cnt; j += G) {
              const float4 pj = Sp[j], aj = Sa[j];
              const float  dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
              if (dx * dx + dy * dy + dz * dz != 0.f) {
                float gd[3], wa[3];
                pair_adj32(dx, dy, dz, aj.x, aj.y, aj.z, aj.w, pj.w, ub, Jb, ct, gd, wa);
                s[0] += gd[0];
                s[1] += gd[1];
                s[2] += gd[2];
              }
            }
            for (int k = 0; k < 3; k++)
              two_sum_acc(hi[k], lo[k], s[k]);
          }
        }
      }
      __syncthreads();
      for (int k = 0; k < 3; k++) {
        red[0][threadIdx.x * 3 + k] = hi[k];
        red[1][threadIdx.x * 3 + k] = lo[k];
      }
      __syncthreads();
      if (threadIdx.x < nbc) {
        const int i = b0 + tc + threadIdx.x;
        for (int k = 0; k < 3; k++) {
          float h = 0.f, l = 0.f;
          for (int gg = 0; gg < G; gg++) {
            two_sum_acc(h, l, red[0][(gg * TG + threadIdx.x) * 3 + k]);
            l += red[1][(gg * TG + threadIdx.x) * 3 + k];
          }
          W(a, W_XNT + k, i) = (double)h + (double)l;
        }
      }
    }
  }
}

// Per source: xbar_j -= sum of ds/dd, alphabar_j += sum of ds/dalpha_j (FP32).
// The target bodies of the source leaf's transposed row are staged (position
// in the source leaf's frame and FP32 seeds) in chunks.
__global__ void __launch_bounds__(128) k_adj_p2p32_src(AdjDev a)
{
  __shared__ float4 Tp[ADJ_CH_S], Ts[ADJ_CH_S][4];
  __shared__ float4 Loff[ADJ_LG];
  __shared__ int    Lpre[ADJ_LG + 1];
  // partial sums (hi, lo) of the 7 outputs, in the seed staging buffer once a tile's chunks are done
  float *red0 = reinterpret_cast<float *>(&Ts[0][0]), *red1 = red0 + 128 * 7;
  static_assert(sizeof(Ts) >= 2 * 128 * 7 * sizeof(float), "the reduction fits in the staging buffer");
  for (int li = blockIdx.x; li < a.nleaves; li += gridDim.x) {
    const int    c = a.leaf_cells[li], b0 = a.cv.body[c], nb = a.cv.nbody[c];
    const int    q0 = a.p2pT_start[c], q1 = a.p2pT_start[c + 1];
    const double cx = a.cv.x[c], cy = a.cv.y[c], cz = a.cv.z[c];
    for (int tc = 0; tc < nb; tc += 128) {
      const int nbc = min(128, nb - tc);
      const int TG = nbc <= 32 ? 32 : (nbc <= 64 ? 64 : 128), G = 128 / TG;
      const int tt = threadIdx.x % TG, g = threadIdx.x / TG;
      float     hi[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, lo[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      float4    pj = make_float4(0.f, 0.f, 0.f, 0.f), aj = pj;
      if (tt < nbc) {
        pj = a.pos32[b0 + tc + tt];
        aj = a.alp32[b0 + tc + tt];
      }
      for (int qg = q0; qg < q1; qg += ADJ_LG) {
        const int ng = min(ADJ_LG, q1 - qg);
        __syncthreads();
        if (threadIdx.x < 32)
          stage_row_leaves(a, a.p2pT_tgt, qg, ng, cx, cy, cz, Loff, Lpre);
        __syncthreads();
        const int total = Lpre[ng];
        for (int c0 = 0; c0 < total; c0 += ADJ_CH_S) {
          const int cnt = min(ADJ_CH_S, total - c0);
          if (c0 > 0)
            __syncthreads();
          int lqs[ADJ_CH_S / 128];
#pragma unroll
          for (int i = 0; i < ADJ_CH_S / 128; i++) {
            const int e = threadIdx.x + 128 * i;
            lqs[i]      = e < cnt ? row_leaf_of(Lpre, ng, c0 + e) : -1;
            if (lqs[i] >= 0) {
              const int bi = __float_as_int(Loff[lqs[i]].w) + (c0 + e - Lpre[lqs[i]]);
              cp_async16(Tp + e, a.pos32 + bi);
              for (int v = 0; v < 4; v++)
                cp_async16(&Ts[e][v], a.seeds32 + 4 * (size_t)bi + v);
            }
          }
          cp_async_wait_all();
#pragma unroll
          for (int i = 0; i < ADJ_CH_S / 128; i++)
            if (lqs[i] >= 0) {
              const int    e = threadIdx.x + 128 * i;
              const float4 o = Loff[lqs[i]], p = Tp[e];
              Tp[e]          = make_float4(p.x + o.x, p.y + o.y, p.z + o.z, 0.f);
            }
          __syncthreads();
          if (tt < nbc) {
            float s[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            for (int i = g; i < cnt; i += G) {
              const float4 pi = Tp[i];
              const float  dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
              if (dx * dx + dy * dy + dz * dz != 0.f) {
                const float4 s0 = Ts[i][0], s1 = Ts[i][1], s2 = Ts[i][2], s3 = Ts[i][3];
                const float  ub[3] = {s0.x, s0.y, s0.z}, ct[3] = {s0.w, s1.x, s1.y};
                const float  Jb[9] = {s1.z, s1.w, s2.x, s2.y, s2.z, s2.w, s3.x, s3.y, s3.z};
                float        gd[3], wa[3], sgb;
                pair_adj32(dx, dy, dz, aj.x, aj.y, aj.z, aj.w, pj.w, ub, Jb, ct, gd, wa, &sgb);
                for (int k = 0; k < 3; k++) {
                  s[k] -= gd[k];
                  s[3 + k] += wa[k];
                }
                s[6] += sgb;
              }
            }
            for (int k = 0; k < 7; k++)
              two_sum_acc(hi[k], lo[k], s[k]);
          }
        }
      }
      __syncthreads();
      for (int k = 0; k < 7; k++) {
        red0[threadIdx.x * 7 + k] = hi[k];
        red1[threadIdx.x * 7 + k] = lo[k];
      }
      __syncthreads();
      if (threadIdx.x < nbc) {
        const int j = b0 + tc + threadIdx.x;
        for (int k = 0; k < 7; k++) {
          float h = 0.f, l = 0.f;
          for (int gg = 0; gg < G; gg++) {
            two_sum_acc(h, l, red0[(gg * TG + threadIdx.x) * 7 + k]);
            l += red1[(gg * TG + threadIdx.x) * 7 + k];
          }
          W(a, k < 3 ? W_XNS + k : (k < 6 ? W_ANS + k - 3 : W_RNS), j) = (double)h + (double)l;
        }
      }
    }
  }
}

// M2L^T in FP32 with the mixed forward's scaling (R_s = the source cell's
// half-width): with S'(d) = R_s^{-(q+1)} S'(d / R_s),
//   Mbar_s[n] = R_s^{-n} sum_t sum_j Ltil_t[j] conj(S'_{j+n}(d / R_s)),
//   Ltil_t[j,k] = (-1)^j Lbar_t[j,k] R_s^{-(j+1)} = Lhat_t[j,k] 2^{-(l_t - l_s)(j+1)},
//   Lhat_t[j,k] = (-1)^j Lbar_t[j,k] R_t^{-(j+1)},
// Lhat made once per cell (k_adj_lhat32).  When the target is coarser
// (l_t < l_s) the factor 2^{-(l_t - l_s)(j+1)} would grow past FP32's range,
// so that pair uses harmonics at d / R_t instead, with
//   R_s^{-n} conj(...)  ->  R_s^{-n} 2^{(l_t - l_s) n} sum_j Lhat_t[j] conj(S'_{j+n}(d / R_t)):
// every rescaling is then by 2^{-k}, k >= 0, exact or a negligible underflow
// (the MAC keeps |d| >= 2 max(R_s, R_t)).  One warp per source cell.  The outputs (n, m), all three components,
// are packed onto the lanes by term count ((P-n)(P-n+1)/2 terms each) so that
// every lane has nearly the same work (see m2lt_schedule).
__global__ void k_adj_lhat32(AdjDev a, int ncells, int K)
{
  const long total = (long)ncells * 3 * K;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const int c = (int)(e / (3 * K)), r = (int)(e % (3 * K)), lev = a.cv.level[c];
    int       j, k;
    jk_of(r / 3, j, k);
    const double  sc = ((j & 1) ? -1.0 : 1.0) * ldexp(a.iR0pow[j + 1], lev * (j + 1)); // (-1)^j R_t^{-(j+1)}
    const double2 v  = a.Lb[e];
    a.Lhat32[e]      = make_float2((float)(v.x * sc), (float)(v.y * sc));
  }
}

// Pieces of the M2L^T work, one schedule per order P and process: output
// (n, m) has (P-n)(P-n+1)/2 terms (j <= P-1-n, k <= j, in that order); an
// output longer than the mean lane load is cut into near-equal runs, and the
// pieces are packed largest first onto the least loaded of 32 lanes.
// table[lane * nslot + slot] = {n | (m + 16) << 8, j0 | k0 << 8, length,
// piece id} (length 0 past a lane's list); the pieces of output
// o = n^2 + n + m have ids pstart[o] .. pstart[o + 1] - 1; iters = the largest
// lane load.  Made on the device current at first use.
struct M2LTSchedule {
  int4 *table;
  int  *pstart;
  int   nslot, iters, npieces;
};
template <int P>
const M2LTSchedule &m2lt_schedule()
{
  static const M2LTSchedule sched = [] {
    struct Piece {
      int n, m, j0, k0, len, id;
    };
    int total = 0;
    for (int n = 0; n < P; n++)
      total += (2 * n + 1) * (P - n) * (P - n + 1) / 2;
    const int          target = (total + 31) / 32;
    std::vector<Piece> pieces;
    std::vector<int>   pstart(P * P + 1, 0);
    for (int n = 0; n < P; n++)
      for (int m = -n; m <= n; m++) {
        const int T  = (P - n) * (P - n + 1) / 2;
        const int np = (T + target - 1) / target;
        pstart[n * n + n + m] = (int)pieces.size();
        int f = 0;
        for (int q = 0; q < np; q++) {
          const int len = T / np + (q < T % np ? 1 : 0);
          int       j = 0, k = f;
          while (k > j) { // flattened index f -> (j, k)
            k -= j + 1;
            j++;
          }
          pieces.push_back({n, m, j, k, len, (int)pieces.size()});
          f += len;
        }
      }
    pstart[P * P] = (int)pieces.size();
    std::vector<Piece> order = pieces;
    std::stable_sort(order.begin(), order.end(), [](const Piece &x, const Piece &y) { return x.len > y.len; });
    std::vector<std::vector<Piece>> lanes(32);
    std::vector<int>                load(32, 0);
    for (const Piece &pc : order) {
      int l = 0;
      for (int i = 1; i < 32; i++)
        if (load[i] < load[l])
          l = i;
      lanes[l].push_back(pc);
      load[l] += pc.len;
    }
    M2LTSchedule r{};
    r.npieces = (int)pieces.size();
    for (int l = 0; l < 32; l++) {
      r.nslot = std::max(r.nslot, (int)lanes[l].size());
      r.iters = std::max(r.iters, load[l]);
    }
    std::vector<int4> host(32 * r.nslot, make_int4(0, 0, 0, 0));
    for (int l = 0; l < 32; l++)
      for (size_t i = 0; i < lanes[l].size(); i++) {
        const Piece &pc       = lanes[l][i];
        host[l * r.nslot + i] = make_int4(pc.n | ((pc.m + 16) << 8), pc.j0 | (pc.k0 << 8), pc.len, pc.id);
      }
    VFMM_CUDA_TRY(cudaMalloc((void **)&r.table, host.size() * sizeof(int4)));
    VFMM_CUDA_TRY(cudaMemcpy(r.table, host.data(), host.size() * sizeof(int4), cudaMemcpyHostToDevice));
    VFMM_CUDA_TRY(cudaMalloc((void **)&r.pstart, pstart.size() * sizeof(int)));
    VFMM_CUDA_TRY(cudaMemcpy(r.pstart, pstart.data(), pstart.size() * sizeof(int), cudaMemcpyHostToDevice));
    return r;
  }();
  return sched;
}

template <int P>
struct AdjM2L32Sizes {
  static constexpr int K = nterms(P), PP = P * P;
  // per warp: Lt (3K), S' (PP), piece accumulators (3 per piece); plus the degree table
  static size_t bytes(int npieces) { return (size_t)4 * (3 * K + PP + 3 * npieces) * sizeof(cx<float>) + (size_t)3 * K; }
};

template <int P>
__global__ void __launch_bounds__(128) k_adj_m2l32(AdjDev a, int ncells, const int4 *__restrict__ table, const int *__restrict__ pstart, int nslot,
                                                  int iters, int npieces)
{
  typedef cx<float> zf;
  constexpr int K = nterms(P), PP = P * P;
  extern __shared__ double2 smem_raw[];
  const int      WS   = 3 * K + PP + 3 * npieces;
  const int      w    = threadIdx.x >> 5, lane = threadIdx.x & 31;
  zf            *Lt   = reinterpret_cast<zf *>(smem_raw) + w * WS;
  zf            *Sp   = Lt + 3 * K;
  zf            *Pa   = Sp + PP; // [piece][d]
  unsigned char *jtab = reinterpret_cast<unsigned char *>(reinterpret_cast<zf *>(smem_raw) + 4 * WS); // degree j of element e
  for (int e = threadIdx.x; e < 3 * K; e += blockDim.x) {
    int j, k;
    jk_of(e / 3, j, k);
    jtab[e] = (unsigned char)j;
  }
  __syncthreads();
  for (int s = blockIdx.x * 4 + w; s < ncells; s += gridDim.x * 4) {
    for (int e = lane; e < 3 * npieces; e += 32)
      Pa[e] = {0.f, 0.f};
    const int    q0 = a.m2lT_start[s], q1 = a.m2lT_start[s + 1];
    const double sx = a.cv.x[s], sy = a.cv.y[s], sz = a.cv.z[s];
    const int    ls = a.cv.level[s];
    const double iRs = ldexp(1.0 / a.R0, ls); // 1 / R_s
    for (int q = q0; q < q1; q++) {
      const int t = a.m2lT_tgt[q], dl = a.cv.level[t] - ls;
      __syncwarp();
      const float2 *src = a.Lhat32 + (size_t)t * 3 * K;
      if (dl <= 0)
        for (int e = lane; e < 3 * K; e += 32) {
          const float2 v = src[e];
          Lt[e]          = {v.x, v.y};
        }
      else
        for (int e = lane; e < 3 * K; e += 32) {
          const float2 v  = src[e];
          const float  sc = ldexpf(1.f, -dl * (jtab[e] + 1));
          Lt[e]           = {v.x * sc, v.y * sc};
        }
      if (lane < P) {
        const double iRh = dl < 0 ? ldexp(iRs, dl) : iRs; // 1/R_t for a coarser target, else 1/R_s
        const float  dx = (float)((a.cv.x[t] - sx) * iRh), dy = (float)((a.cv.y[t] - sy) * iRh), dz = (float)((a.cv.z[t] - sz) * iRh);
        const float  r2 = dx * dx + dy * dy + dz * dz, ir2 = 1.f / r2, S00 = sqrtf(ir2);
        zf           col[P];
        singular_column<float, P>(lane, dx, dy, dz, ir2, S00, col);
        const int m = lane;
        for (int n = m; n < P; n++) {
          const zf v        = col[n];
          Sp[n * n + n + m] = (m & 1) ? zf{-v.r, -v.i} : v;
          if (m > 0)
            Sp[n * n + n - m] = conj(v);
        }
      }
      __syncwarp();
      int  slot = 0;
      int4 pc   = table[lane * nslot];
      int  n = pc.x & 255, m = (pc.x >> 8) - 16, j = pc.y & 255, k = pc.y >> 8, left = pc.z;
      zf   acc[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
      for (int it = 0; it < iters; it++) {
        if (left > 0) {
          const int qq = j + n;
          const zf  y  = Sp[qq * qq + qq + m - k];
          const zf *lp = Lt + tri(j, k) * 3;
#pragma unroll
          for (int d = 0; d < 3; d++) {
            const zf l = lp[d];
            acc[d].r   = fmaf(l.r, y.r, fmaf(l.i, y.i, acc[d].r)); // l conj(y)
            acc[d].i   = fmaf(l.i, y.r, fmaf(-l.r, y.i, acc[d].i));
          }
          if (++k > j) {
            k = 0;
            j++;
          }
          if (--left == 0) { // piece complete for this target
            zf         *ap = Pa + pc.w * 3;
            const float sc = dl < 0 ? ldexpf(1.f, dl * n) : 1.f;
#pragma unroll
            for (int d = 0; d < 3; d++) {
              ap[d].r = fmaf(sc, acc[d].r, ap[d].r);
              ap[d].i = fmaf(sc, acc[d].i, ap[d].i);
              acc[d]  = {0.f, 0.f};
            }
            if (++slot < nslot) {
              pc   = table[lane * nslot + slot];
              n    = pc.x & 255;
              m    = (pc.x >> 8) - 16;
              j    = pc.y & 255;
              k    = pc.y >> 8;
              left = pc.z;
            }
          }
        }
      }
    }
    __syncwarp();
    for (int e = lane; e < 3 * K; e += 32) {
      const int d = e % 3;
      int       n, mm;
      jk_of(e / 3, n, mm);
      const int o0 = n * n + n + mm, o1 = n * n + n - mm;
      float     ar = 0.f, ai = 0.f, br = 0.f, bi = 0.f;
      for (int pid = pstart[o0]; pid < pstart[o0 + 1]; pid++) {
        ar += Pa[pid * 3 + d].r;
        ai += Pa[pid * 3 + d].i;
      }
      double vr = (mm & 1) ? -(double)ar : (double)ar, vi = (mm & 1) ? -(double)ai : (double)ai;
      if (mm > 0) {
        for (int pid = pstart[o1]; pid < pstart[o1 + 1]; pid++) {
          br += Pa[pid * 3 + d].r;
          bi += Pa[pid * 3 + d].i;
        }
        vr += br;
        vi -= bi;
      }
      const double sc = ldexp(a.iR0pow[n], ls * n); // R_s^{-n}
      a.Mb[(size_t)s * 3 * K + e] = make_double2(vr * sc, vi * sc);
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------------ host side
template <int P>
void eval_adjoint_P(cudaStream_t s, const ExpArgs &e, const AdjDev &d)
{
  constexpr int K = nterms(P);
  if (e.nleaves > 0) {
    if (d.pos32) {
      VFMM_SMEM_ONCE(AdjL2P32Sizes<P>::bytes, k_adj_l2p32<P>);
      k_adj_l2p32<P><<<std::min(e.nleaves, 152 * 8), 128, AdjL2P32Sizes<P>::bytes, s>>>(d);
    } else {
      VFMM_SMEM_ONCE(AdjL2PSizes<P>::bytes, k_adj_l2p<P>);
      k_adj_l2p<P><<<std::min(e.nleaves, 152 * 8), 128, AdjL2PSizes<P>::bytes, s>>>(d);
    }
    count_launch();
  }
  const bool   mix  = d.pos32 != nullptr;
  const size_t bl2l = (size_t)(8 * 3 * K + 8 * K) * (mix ? sizeof(cx<float>) : sizeof(zd));
  if (mix)
    VFMM_SMEM_ONCE(bl2l, k_adj_l2l<P, float>);
  else
    VFMM_SMEM_ONCE(bl2l, k_adj_l2l<P, double>);
  for (int l = e.maxLevel - 1; l >= 0; l--) { // forward L2L runs parents at levels 0 .. maxLevel-1
    const int n0 = e.level_start_host[l], n1 = e.level_start_host[l + 1];
    if (n1 > n0) {
      if (mix)
        k_adj_l2l<P, float><<<std::min(n1 - n0, 152 * 16), 128, bl2l, s>>>(d, e.level_cells + n0, n1 - n0);
      else
        k_adj_l2l<P, double><<<std::min(n1 - n0, 152 * 16), 128, bl2l, s>>>(d, e.level_cells + n0, n1 - n0);
      count_launch();
    }
  }
  if (d.pos32) {
    const M2LTSchedule &sc    = m2lt_schedule<P>();
    const size_t        bytes = AdjM2L32Sizes<P>::bytes(sc.npieces);
    k_adj_lhat32<<<grid_for((long)e.ncells * 3 * K, 256), 256, 0, s>>>(d, e.ncells, K);
    count_launch();
    VFMM_SMEM_ONCE(bytes, k_adj_m2l32<P>);
    k_adj_m2l32<P><<<grid_for(e.ncells, 4, 152 * 16), 128, bytes, s>>>(d, e.ncells, sc.table, sc.pstart, sc.nslot, sc.iters, sc.npieces);
  } else {
    VFMM_SMEM_ONCE(AdjM2LSizes<P>::bytes, k_adj_m2l<P>);
    k_adj_m2l<P><<<grid_for(e.ncells, 4, 152 * 16), 128, AdjM2LSizes<P>::bytes, s>>>(d, e.ncells);
  }
  count_launch();
  const size_t bm2m = (size_t)(3 * K + 8 * K) * (mix ? sizeof(cx<float>) : sizeof(zd));
  if (mix)
    VFMM_SMEM_ONCE(bm2m, k_adj_m2m<P, float>);
  else
    VFMM_SMEM_ONCE(bm2m, k_adj_m2m<P, double>);
  for (int l = 1; l <= e.maxLevel - 1; l++) { // forward M2M runs parents at levels maxLevel-1 .. 1
    const int n0 = e.level_start_host[l], n1 = e.level_start_host[l + 1];
    if (n1 > n0) {
      if (mix)
        k_adj_m2m<P, float><<<std::min(n1 - n0, 152 * 16), 128, bm2m, s>>>(d, e.level_cells + n0, n1 - n0);
      else
        k_adj_m2m<P, double><<<std::min(n1 - n0, 152 * 16), 128, bm2m, s>>>(d, e.level_cells + n0, n1 - n0);
      count_launch();
    }
  }
  if (e.nleaves > 0) {
    if (mix) {
      VFMM_SMEM_ONCE((AdjP2MSizes<P, float>::bytes), k_adj_p2m<P, float>);
      k_adj_p2m<P, float><<<std::min(e.nleaves, 152 * 8), 128, AdjP2MSizes<P, float>::bytes, s>>>(d);
    } else {
      VFMM_SMEM_ONCE((AdjP2MSizes<P, double>::bytes), k_adj_p2m<P, double>);
      k_adj_p2m<P, double><<<std::min(e.nleaves, 152 * 8), 128, AdjP2MSizes<P, double>::bytes, s>>>(d);
    }
    count_launch();
    if (d.pos32) {
      k_adj_p2p32_tgt<<<std::min(e.nleaves, 152 * 16), 128, 0, s>>>(d);
      count_launch();
      k_adj_p2p32_src<<<std::min(e.nleaves, 152 * 16), 128, 0, s>>>(d);
      count_launch();
    } else {
      k_adj_p2p_tgt<<<std::min(e.nleaves, 152 * 16), 128, 0, s>>>(d);
      count_launch();
      k_adj_p2p_src<<<std::min(e.nleaves, 152 * 16), 128, 0, s>>>(d);
      count_launch();
    }
  }
  VFMM_LAUNCH_CHECK();
}

} // namespace

void adjoint_eval(cudaStream_t s, const ExpArgs &e, const AdjBufs &b, const DevInfo *info)
{
  AdjDev d{};
  d.cv         = e.cells;
  d.soa        = e.soa;
  d.cap        = e.cap;
  d.L          = e.L;
  d.Lb         = b.Lb;
  d.Mb         = b.Mb;
  d.leaf_cells = e.leaf_cells;
  d.nleaves    = e.nleaves;
  d.p2p_start  = e.p2p_start;
  d.p2p_src    = e.p2p_src;
  d.p2pT_start = b.p2pT_start;
  d.p2pT_tgt   = b.p2pT_tgt;
  d.m2lT_start = b.m2lT_start;
  d.m2lT_tgt   = b.m2lT_tgt;
  d.w          = b.w;
  d.pos32      = b.pos32;
  d.alp32      = b.alp32;
  d.seeds32    = b.seeds32;
  d.Lhat32     = b.Lhat32;
  d.R0         = b.R0;
  if (b.pos32) {
    double p = 1.0, ip = 1.0;
    for (int k = 0; k <= PMAX + 1; k++) {
      d.R0pow[k]  = p;
      d.iR0pow[k] = ip;
      p *= b.R0;
      ip /= b.R0;
    }
  }
  const int n  = b.n;
  VFMM_CUDA_TRY(cudaMemsetAsync(b.w + (size_t)W_AP2M * e.cap, 0, 3 * e.cap * sizeof(double), s));
  if (b.pos32) {
    k_adj_seeds32<<<grid_for(n, 256), 256, 0, s>>>(d, n);
    count_launch();
  }
  switch (e.P) {
#define VFMM_ADJ_CASE(PP)                                                                                                                 \
  case PP: eval_adjoint_P<PP>(s, e, d); break;
    VFMM_ADJ_CASE(2) VFMM_ADJ_CASE(3) VFMM_ADJ_CASE(4) VFMM_ADJ_CASE(5) VFMM_ADJ_CASE(6) VFMM_ADJ_CASE(7) VFMM_ADJ_CASE(8)
    VFMM_ADJ_CASE(9) VFMM_ADJ_CASE(10) VFMM_ADJ_CASE(11) VFMM_ADJ_CASE(12) VFMM_ADJ_CASE(13) VFMM_ADJ_CASE(14) VFMM_ADJ_CASE(15)
    VFMM_ADJ_CASE(16)
#undef VFMM_ADJ_CASE
  default: throw Error(VFMM_ERR_UNSUPPORTED, "expansion order p must be in 2..16");
  }
  k_adj_combine<<<grid_for(n, 256), 256, 0, s>>>(b.g, b.w, e.cap, n);
  count_launch();
  k_adj_geom_partial<<<GEO_BLOCKS, GEO_THREADS, 0, s>>>(e.soa, b.w, e.cap, n, info, b.part);
  count_launch();
  k_adj_geom_final<<<1, 32, 0, s>>>(b.part, GEO_BLOCKS, info, b.g, e.cap);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

void adjoint_seeds(cudaStream_t s, const double *soa, double *w, size_t cap, int n, int stretching, int add_relax, int formulation)
{
  k_adj_seeds<<<grid_for(n, 256), 256, 0, s>>>(soa, w, cap, n, stretching, add_relax, formulation);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

void adjoint_relax(cudaStream_t s, double *g, double *w, const double *soa, const double *alpha_u, size_t cap, int n, double f)
{
  k_adj_relax<<<grid_for(n, 256), 256, 0, s>>>(g, w, soa, alpha_u, cap, n, f);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

void adjoint_stage_pre(cudaStream_t s, double *g, double *w, size_t cap, int n, int scheme, int stage, double dt, int rk4_fixed)
{
  k_adj_stage_pre<<<grid_for(n, 256), 256, 0, s>>>(g, w, cap, n, scheme, stage, dt, rk4_fixed);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

void adjoint_objective(cudaStream_t s, const double *soa, size_t cap, int n, const int *orig, const double *seed_x, const double *seed_a, double wE,
                       const double wI[3], double *g, double *w, double *part, double *value)
{
  k_adj_objective<<<OBJ_BLOCKS, OBJ_THREADS, 0, s>>>(soa, cap, n, orig, seed_x, seed_a, wE, wI[0], wI[1], wI[2], g, w, part);
  count_launch();
  k_sum_final<<<1, 32, 0, s>>>(part, OBJ_BLOCKS, value);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

void adjoint_scatter(cudaStream_t s, const double *in, double *out, size_t cap, int n, const uint32_t *perm)
{
  k_adj_scatter<<<grid_for(n, 256), 256, 0, s>>>(in, out, cap, n, perm);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

void orig_update(cudaStream_t s, const int *in, int *out, const uint32_t *perm, int n)
{
  k_orig_update<<<grid_for(n, 256), 256, 0, s>>>(in, out, perm, n);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

void iota_int(cudaStream_t s, int *a, int n)
{
  k_iota_int<<<grid_for(n, 256), 256, 0, s>>>(a, n);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

void adjoint_rows(cudaStream_t s, const double *g, size_t cap, int n, int field, double *rows)
{
  k_adj_rows<<<grid_for(n, 256), 256, 0, s>>>(g, cap, n, field, rows);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

} // namespace vfmm
