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
// use: lane m computes column m).  inv_r2 = 1/r^2, S00 = 1/r.
template <class T, int NDEG>
__device__ __forceinline__ void singular_column(int m, T x, T y, T z, T inv_r2, T S00, cx<T> *out /* indexed by n */)
{
  cx<T> d{S00, T(0)};
  for (int k = 1; k <= m; k++) {
    const T s = T(2 * k - 1) * inv_r2;
    d         = mk<T>((d.r * x - d.i * y) * s, (d.r * y + d.i * x) * s);
  }
  cx<T> a = d, b{T(0), T(0)};
  out[m] = a;
  for (int n = m; n + 1 < NDEG; n++) {
    const T zz = T(2 * n + 1) * z;
    const T c2 = T((n + m) * (n - m));
    cx<T>   nx = mk<T>(-(zz * a.r + c2 * b.r) * inv_r2, -(zz * a.i + c2 * b.i) * inv_r2);
    out[n + 1] = nx;
    b = a;
    a = nx;
  }
}

} // namespace vfmm
