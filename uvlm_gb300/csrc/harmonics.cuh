// Solid harmonics and complex helpers for the expansion kernels.
//
// The reference's regular harmonics (evalMultipole, multipoleKernels.hpp:53-92)
// are Y_n^m = rho^n P_n^m(cos a) e^{i m b} / ((-1)^n (n+m)!) with the
// Condon-Shortley phase in P_n^m, and its singular harmonics (evalLocal,
// :137-172) are S_n^m = (-1)^n (n-m)! P_n^m(cos a) e^{i m b} / rho^{n+1}.
// Both are computed here from Cartesian offsets by recurrences without
// trigonometry (the same functions, different rounding):
//   Y_0^0 = 1, Y_m^m = Y_{m-1}^{m-1} (x+iy)/(2m), Y_{m+1}^m = -z Y_m^m,
//   Y_{n+1}^m = -((2n+1) z Y_n^m + r^2 Y_{n-1}^m) / ((n+m+1)(n-m+1));
//   S_0^0 = 1/r, S_m^m = S_{m-1}^{m-1} (2m-1)(x+iy)/r^2,
//   S_{n+1}^m = -((2n+1) z S_n^m + (n+m)(n-m) S_{n-1}^m) / r^2.
// Derivatives of the regular harmonics (used by L2P, which the reference
// evaluates by a complex step): with Y_n^{-m} = conj(Y_n^m),
//   dY_n^m/dz = -Y_{n-1}^m,
//   (d/dx + i d/dy) Y_n^m = s(m) Y_{n-1}^{m+1},  s = -1 (m >= 0), +1 (m < 0),
//   (d/dx - i d/dy) Y_n^m = t(m) Y_{n-1}^{m-1},  t = +1 (m >= 1), -1 (m <= 0).
#pragma once
#include <cuda_runtime.h>

namespace vfmm {

template <class T>
struct cx {
  T r, i;
};
template <class T> __host__ __device__ __forceinline__ cx<T> mk(T r, T i) { return cx<T>{r, i}; }
template <class T> __host__ __device__ __forceinline__ cx<T> operator+(cx<T> a, cx<T> b) { return {a.r + b.r, a.i + b.i}; }
template <class T> __host__ __device__ __forceinline__ cx<T> operator-(cx<T> a, cx<T> b) { return {a.r - b.r, a.i - b.i}; }
template <class T> __host__ __device__ __forceinline__ cx<T> operator*(cx<T> a, cx<T> b) { return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r}; }
template <class T> __host__ __device__ __forceinline__ cx<T> operator*(T s, cx<T> a) { return {s * a.r, s * a.i}; }
template <class T> __host__ __device__ __forceinline__ cx<T> conj(cx<T> a) { return {a.r, -a.i}; }
// acc += a * b
template <class T> __device__ __forceinline__ void cfma(cx<T> &acc, cx<T> a, cx<T> b)
{
  acc.r = fma(a.r, b.r, acc.r);
  acc.r = fma(-a.i, b.i, acc.r);
  acc.i = fma(a.r, b.i, acc.i);
  acc.i = fma(a.i, b.r, acc.i);
}

__host__ __device__ constexpr int nterms(int P) { return P * (P + 1) / 2; }
__host__ __device__ constexpr int tri(int n, int m) { return n * (n + 1) / 2 + m; }

// Regular harmonics Y_n^m, n < NDEG, m >= 0, written to Y[tri(n,m)*stride].
template <class T, int NDEG>
__device__ __forceinline__ void regular_harmonics(T x, T y, T z, cx<T> *Y, int stride = 1)
{
  const T r2 = x * x + y * y + z * z;
  cx<T>   diag{T(1), T(0)};
#pragma unroll
  for (int m = 0; m < NDEG; m++) {
    if (m > 0) {
      const T s = T(1) / T(2 * m);
      diag      = mk<T>((diag.r * x - diag.i * y) * s, (diag.r * y + diag.i * x) * s);
    }
    cx<T> a = diag, b{T(0), T(0)};
    Y[tri(m, m) * stride] = a;
#pragma unroll
    for (int n = m; n + 1 < NDEG; n++) {
      const T c  = T(-1) / T((n + m + 1) * (n - m + 1));
      const T zz = T(2 * n + 1) * z;
      cx<T>   nx = mk<T>(c * (zz * a.r + r2 * b.r), c * (zz * a.i + r2 * b.i));
      Y[tri(n + 1, m) * stride] = nx;
      b = a;
      a = nx;
    }
  }
}

// One column m of the singular harmonics S_n^m, n = m..NDEG-1 (lane-parallel
// use: lane m computes column m), handed to emit(n, S_n^m) in order of n.
// inv_r2 = 1/r^2, S00 = 1/r.
template <class T, int NDEG, class F>
__device__ __forceinline__ void singular_column_emit(int m, T x, T y, T z, T inv_r2, T S00, F &&emit)
{
  cx<T> d{S00, T(0)};
  for (int k = 1; k <= m; k++) {
    const T s = T(2 * k - 1) * inv_r2;
    d         = mk<T>((d.r * x - d.i * y) * s, (d.r * y + d.i * x) * s);
  }
  cx<T> a = d, b{T(0), T(0)};
  emit(m, a);
  for (int n = m; n + 1 < NDEG; n++) {
    const T zz = T(2 * n + 1) * z;
    const T c2 = T((n + m) * (n - m));
    cx<T>   nx = mk<T>(-(zz * a.r + c2 * b.r) * inv_r2, -(zz * a.i + c2 * b.i) * inv_r2);
    emit(n + 1, nx);
    b = a;
    a = nx;
  }
}

// The same column written to out[n].
template <class T, int NDEG>
__device__ __forceinline__ void singular_column(int m, T x, T y, T z, T inv_r2, T S00, cx<T> *out /* indexed by n */)
{
  singular_column_emit<T, NDEG>(m, x, y, z, inv_r2, S00, [&](int n, cx<T> v) { out[n] = v; });
}

// Reciprocals used by the regular-harmonic recurrence when it runs with
// runtime indices: c[tri(n, m)] = -1 / ((n+m+1)(n-m+1)) and s[m] = 1 / (2m),
// n < 16.  Correctly rounded like the divisions they replace.
template <class T>
struct HarmRecip {
  T c[nterms(16)];
  T s[17];
};
template <class T>
constexpr HarmRecip<T> make_harm_recip()
{
  HarmRecip<T> r{};
  for (int n = 0; n < 16; n++)
    for (int m = 0; m <= n; m++)
      r.c[tri(n, m)] = T(-1) / T((n + m + 1) * (n - m + 1));
  for (int m = 1; m < 17; m++)
    r.s[m] = T(1) / T(2 * m);
  return r;
}

template <class T>
__device__ __forceinline__ cx<T> neg_if(cx<T> v, bool neg) { return neg ? cx<T>{-v.r, -v.i} : v; }

// Full-range coefficient c_n^m of a real expansion stored for m >= 0:
// c_n^{-m} = conj(c_n^m), and c_n^0 is taken as real.
template <class T>
__device__ __forceinline__ cx<T> coef_full(const cx<T> *c, int n, int m, int stride, int comp)
{
  if (m > 0)
    return c[tri(n, m) * stride + comp];
  if (m == 0)
    return {c[tri(n, 0) * stride + comp].r, T(0)};
  return conj(c[tri(n, -m) * stride + comp]);
}
// Coefficient (n, mu >= 0) of D_axis applied to the expansion c (whose degree
// n + 1 terms are read), from the derivative rules above.
template <class T>
__device__ __forceinline__ cx<T> deriv_coef(const cx<T> *c, int n, int mu, int axis, int stride, int comp)
{
  if (axis == 2) {
    const cx<T> v = coef_full(c, n + 1, mu, stride, comp);
    return {-v.r, -v.i};
  }
  const T     s = (mu - 1 >= 0) ? T(-1) : T(1);
  const T     t = (mu + 1 >= 1) ? T(1) : T(-1);
  const cx<T> A = s * coef_full(c, n + 1, mu - 1, stride, comp);
  const cx<T> B = t * coef_full(c, n + 1, mu + 1, stride, comp);
  if (axis == 0)
    return {T(0.5) * (A.r + B.r), T(0.5) * (A.i + B.i)};
  // -(i/2)(A - B)
  return {T(0.5) * (A.i - B.i), T(-0.5) * (A.r - B.r)};
}

// Transposes for reverse mode.  A complex variable's adjoint is
// dS/dRe + i dS/dIm of the scalar S being differentiated; with that
// convention z = w c (c constant) gives wbar += zbar conj(c), and
// z = conj(w) gives wbar += conj(zbar).
template <class T>
__device__ __forceinline__ void coef_full_adj(cx<T> *cb, int n, int m, int stride, int comp, cx<T> g)
{
  if (m > 0) {
    cx<T> &o = cb[tri(n, m) * stride + comp];
    o.r += g.r;
    o.i += g.i;
  } else if (m == 0)
    cb[tri(n, 0) * stride + comp].r += g.r;
  else {
    cx<T> &o = cb[tri(n, -m) * stride + comp];
    o.r += g.r;
    o.i -= g.i;
  }
}
// Adds to cb the adjoint of deriv_coef(c, n, mu, axis, stride, comp) whose
// result has adjoint vb.
template <class T>
__device__ __forceinline__ void deriv_coef_adj(cx<T> *cb, int n, int mu, int axis, int stride, int comp, cx<T> vb)
{
  if (axis == 2) {
    coef_full_adj(cb, n + 1, mu, stride, comp, cx<T>{-vb.r, -vb.i});
    return;
  }
  const T s = (mu - 1 >= 0) ? T(-1) : T(1);
  const T t = (mu + 1 >= 1) ? T(1) : T(-1);
  cx<T>   Ab, Bb;
  if (axis == 0) {
    Ab = {T(0.5) * vb.r, T(0.5) * vb.i};
    Bb = Ab;
  } else { // v = (-i/2) A + (i/2) B
    Ab = {T(-0.5) * vb.i, T(0.5) * vb.r};
    Bb = {T(0.5) * vb.i, T(-0.5) * vb.r};
  }
  coef_full_adj(cb, n + 1, mu - 1, stride, comp, cx<T>{s * Ab.r, s * Ab.i});
  coef_full_adj(cb, n + 1, mu + 1, stride, comp, cx<T>{t * Bb.r, t * Bb.i});
}

// One output (j, k, d) of M2M for NC children at once (children t0..t0+NC-1
// that exist): the index arithmetic is shared and the NC accumulators are
// independent, which keeps the arithmetic pipe fed.  M2M of
// multipoleKernels.hpp:479-516 with dX = X_parent - X_child.  Signs ipow2n(m) * oddOrEven(n)
// and oddOrEven(k+n+m) negate an operand instead of costing a multiply.
template <int P, int NC, class T>
__device__ __forceinline__ void m2m_term_sum(int j, int k, int d, const cx<T> *Ms, const cx<T> *Ys, int t0, int nch, cx<T> *acc)
{
  constexpr int K = nterms(P);
  for (int n = 0; n <= j; n++) {
    for (int m = max(-n, -j + k + n); m <= min(k - 1, n); m++) {
      const int  yi = tri(n, m > 0 ? m : -m), mi = tri(j - n, k - m) * 3 + d;
      const bool cj = m > 0, neg = ((m < 0 ? (m & 1) : 0) ^ (n & 1)) != 0;
#pragma unroll
      for (int c = 0; c < NC; c++)
        if (t0 + c < nch) {
          const cx<T> y = Ys[(t0 + c) * K + yi];
          cfma(acc[c], neg_if(Ms[(t0 + c) * 3 * K + mi], neg), cj ? conj(y) : y);
        }
    }
    for (int m = k; m <= min(n, j + k - n); m++) {
      const int  yi = tri(n, m), mi = tri(j - n, m - k) * 3 + d;
      const bool neg = ((k + n + m) & 1) != 0;
#pragma unroll
      for (int c = 0; c < NC; c++)
        if (t0 + c < nch)
          cfma(acc[c], neg_if(conj(Ms[(t0 + c) * 3 * K + mi]), neg), conj(Ys[(t0 + c) * K + yi]));
    }
  }
}

// One output (j, k, d) of L2L for NC children at once (shared parent operand
// and index arithmetic, independent accumulators).  L2L of
// multipoleKernels.hpp:591-628 with dX = X_child - X_parent.
template <int P, int NC, class T>
__device__ __forceinline__ void l2l_term_sum(int j, int k, int d, const cx<T> *Lp, const cx<T> *Ys, int t0, int nch, cx<T> *acc)
{
  constexpr int K = nterms(P);
  for (int n = j; n < P; n++) {
    const bool negk = (k & 1) != 0;
    for (int m = j + k - n; m < 0; m++) {
      const cx<T> l  = neg_if(conj(Lp[tri(n, -m) * 3 + d]), negk);
      const int yi = tri(n - j, k - m);
#pragma unroll
      for (int c = 0; c < NC; c++)
        if (t0 + c < nch)
          cfma(acc[c], l, conj(Ys[(t0 + c) * K + yi]));
    }
    const int mlo = max(0, k - (n - j)), mhi = min(n, k + (n - j)); // n - j >= |m - k|
    for (int m = mlo; m <= mhi; m++) {
      const bool neg = m < k && ((k - m) & 1);
      const cx<T> l   = neg_if(Lp[tri(n, m) * 3 + d], neg);
      const int  yi  = tri(n - j, m >= k ? m - k : k - m);
#pragma unroll
      for (int c = 0; c < NC; c++)
        if (t0 + c < nch) {
          const cx<T> y = Ys[(t0 + c) * K + yi];
          cfma(acc[c], l, m >= k ? y : conj(y));
        }
    }
  }
}

} // namespace vfmm
