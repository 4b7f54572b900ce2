// FP64 all-pairs sum with the reference's regularised kernel (the team P2P
// formula, multipoleKernels.hpp:239-283): velocity and J at targets from all
// sources.  Used for accuracy checks against the FMM, not on the hot path.
#include "vfmm_internal.cuh"

namespace vfmm {

__global__ void __launch_bounds__(256) k_direct(const double *__restrict__ tx, const double *__restrict__ ty, const double *__restrict__ tz, int nt,
                                                const double *__restrict__ src, size_t scap, int ns, double *out)
{
  __shared__ double sh[7][256];
  const double inv_sqrtpi = 0.564189583547756286948079451560772586, inv_pi = 0.318309886183790671537767526745028724;
  for (int t0 = blockIdx.x * 256; t0 < nt; t0 += gridDim.x * 256) {
    const int    i  = t0 + threadIdx.x;
    const bool   ok = i < nt;
    const double xi = ok ? tx[i] : 0, yi = ok ? ty[i] : 0, zi = ok ? tz[i] : 0;
    double       s[12];
    for (int k = 0; k < 12; k++)
      s[k] = 0;
    for (int j0 = 0; j0 < ns; j0 += 256) {
      __syncthreads();
      const int jj = j0 + threadIdx.x;
      if (jj < ns) {
        sh[0][threadIdx.x] = src[F_X * scap + jj];
        sh[1][threadIdx.x] = src[(F_X + 1) * scap + jj];
        sh[2][threadIdx.x] = src[(F_X + 2) * scap + jj];
        sh[3][threadIdx.x] = src[F_A * scap + jj];
        sh[4][threadIdx.x] = src[(F_A + 1) * scap + jj];
        sh[5][threadIdx.x] = src[(F_A + 2) * scap + jj];
        sh[6][threadIdx.x] = src[F_R * scap + jj];
      }
      __syncthreads();
      const int nj = min(256, ns - j0);
      if (!ok)
        continue;
      for (int j = 0; j < nj; j++) {
        const double dx = xi - sh[0][j], dy = yi - sh[1][j], dz = zi - sh[2][j];
        const double R2 = dx * dx + dy * dy + dz * dz;
        if (R2 != 0) {
          const double ax = sh[3][j], ay = sh[4][j], az = sh[5][j], sg = sh[6][j];
          const double S2 = sg * sg, RS = R2 / S2 / 2.0, sqrtRS = sqrt(RS);
          const double erfS = erf(sqrtRS), expm = exp(-RS), invSqrtR2 = 1.0 / sqrt(R2);
          const double t2 = 2.0 * inv_sqrtpi * sqrtRS * expm, c4 = 0.25 * inv_pi / R2 * invSqrtR2;
          const double cr0 = c4 * (dy * az - dz * ay), cr1 = c4 * (dz * ax - dx * az), cr2 = c4 * (dx * ay - dy * ax);
          const double gg  = erfS - t2;
          s[0] += cr0 * gg;
          s[1] += cr1 * gg;
          s[2] += cr2 * gg;
          double aux = t2 / S2 - 3.0 * gg / R2;
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
    if (ok)
      for (int k = 0; k < 12; k++)
        out[(size_t)k * nt + i] = -s[k];
  }
}

// ------------------------------------------------------------------ model-consistent direct sum
// The FMM of the reference evaluates two different kernels: leaf pairs on the
// P2P list interact through the regularised kernel (multipoleKernels.hpp:
// 239-283), every other pair through the multipole/local expansions of the
// singular Biot-Savart kernel, u = -(1/4 pi) sum (x - x_s) x alpha_s / r^3
// (the Laplace harmonics of M2L/L2P, multipoleKernels.hpp:519-552, :631-742).
// The sum below applies the same split exactly, so its difference from the
// FMM is the expansions' truncation error alone:
//   out(t) = sum_{all s != t} singular(t, s)
//          + sum_{s in the P2P source leaves of leaf(t)} [regularised - singular](t, s).
// FP64 throughout; fixed summation order (deterministic).

// The pair terms (12: velocity, J[a][b] at 3 + 3a + b) with g = erf(rho) - t2
// and aux = t2 / sigma^2 - 3 g / R^2 given; the singular kernel is g = 1, t2 = 0.
__device__ __forceinline__ void pair_terms(double dx, double dy, double dz, double ax, double ay, double az, double c4, double gg, double aux,
                                           double *s)
{
  const double cr0 = c4 * (dy * az - dz * ay), cr1 = c4 * (dz * ax - dx * az), cr2 = c4 * (dx * ay - dy * ax);
  s[0] += cr0 * gg;
  s[1] += cr1 * gg;
  s[2] += cr2 * gg;
  s[3] += aux * cr0 * dx;
  s[4] += aux * cr0 * dy;
  s[5] += aux * cr0 * dz;
  s[6] += aux * cr1 * dx;
  s[7] += aux * cr1 * dy;
  s[8] += aux * cr1 * dz;
  s[9] += aux * cr2 * dx;
  s[10] += aux * cr2 * dy;
  s[11] += aux * cr2 * dz;
  const double a2 = gg * c4;
  s[6] -= a2 * az;
  s[9] += a2 * ay;
  s[4] += a2 * az;
  s[10] -= a2 * ax;
  s[5] -= a2 * ay;
  s[8] += a2 * ax;
}

// Singular kernel over a chunk of the sources: block (target tile of 128,
// source chunk); partial sums part[chunk][12][nt].
__global__ void __launch_bounds__(128) k_direct_singular(const double *__restrict__ soa, size_t cap, const uint32_t *__restrict__ tgt, int nt, int ns,
                                                         int chunk, double *part)
{
  __shared__ double sh[6][128];
  const double inv4pi = 0.0795774715459476678844418816862571810;
  const int    i = blockIdx.x * 128 + threadIdx.x;
  const bool   ok = i < nt;
  const int    bt = ok ? (int)tgt[i] : 0;
  const double xi = soa[F_X * cap + bt], yi = soa[(F_X + 1) * cap + bt], zi = soa[(F_X + 2) * cap + bt];
  double       s[12];
  for (int k = 0; k < 12; k++)
    s[k] = 0;
  const int j_begin = blockIdx.y * chunk, j_end = min(ns, j_begin + chunk);
  for (int j0 = j_begin; j0 < j_end; j0 += 128) {
    __syncthreads();
    const int jj = j0 + threadIdx.x;
    if (jj < j_end)
      for (int f = 0; f < 3; f++) {
        sh[f][threadIdx.x]     = soa[(F_X + f) * cap + jj];
        sh[3 + f][threadIdx.x] = soa[(F_A + f) * cap + jj];
      }
    __syncthreads();
    const int nj = min(128, j_end - j0);
    for (int j = 0; j < nj; j++) {
      const double dx = xi - sh[0][j], dy = yi - sh[1][j], dz = zi - sh[2][j];
      const double R2 = dx * dx + dy * dy + dz * dz;
      if (R2 != 0) {
        const double ir = 1.0 / sqrt(R2), c4 = inv4pi * ir * ir * ir;
        pair_terms(dx, dy, dz, sh[3][j], sh[4][j], sh[5][j], c4, 1.0, -3.0 * ir * ir, s);
      }
    }
  }
  if (ok)
    for (int k = 0; k < 12; k++)
      part[((size_t)blockIdx.y * 12 + k) * nt + i] = s[k];
}

// Regularised minus singular over the P2P source leaves of each target's
// leaf: one warp per target, lanes over the sources, a fixed shuffle tree.
__global__ void k_direct_p2p_correction(const double *__restrict__ soa, size_t cap, CellsView cv, const int *__restrict__ leaf_cells, int nleaves,
                                        const int *__restrict__ p2p_start, const int *__restrict__ p2p_src, const uint32_t *__restrict__ tgt, int nt,
                                        double *corr)
{
  const double inv4pi = 0.0795774715459476678844418816862571810, inv_sqrtpi = 0.564189583547756286948079451560772586;
  const int    lane = threadIdx.x & 31;
  const int    i    = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (i >= nt)
    return;
  const int bt = (int)tgt[i];
  // the leaf holding body bt: leaves are in body order
  int lo = 0, hi = nleaves - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (cv.body[leaf_cells[mid]] <= bt)
      lo = mid;
    else
      hi = mid - 1;
  }
  const int    c  = leaf_cells[lo];
  const double xi = soa[F_X * cap + bt], yi = soa[(F_X + 1) * cap + bt], zi = soa[(F_X + 2) * cap + bt];
  double       s[12];
  for (int k = 0; k < 12; k++)
    s[k] = 0;
  for (int q = p2p_start[c]; q < p2p_start[c + 1]; q++) {
    const int sc = p2p_src[q], j0 = cv.body[sc], nj = cv.nbody[sc];
    for (int j = j0 + lane; j < j0 + nj; j += 32) {
      const double dx = xi - soa[F_X * cap + j], dy = yi - soa[(F_X + 1) * cap + j], dz = zi - soa[(F_X + 2) * cap + j];
      const double R2 = dx * dx + dy * dy + dz * dz;
      if (R2 == 0)
        continue;
      const double ax = soa[F_A * cap + j], ay = soa[(F_A + 1) * cap + j], az = soa[(F_A + 2) * cap + j], sg = soa[F_R * cap + j];
      const double S2 = sg * sg, RS = R2 / S2 / 2.0, sqrtRS = sqrt(RS);
      const double ir = 1.0 / sqrt(R2), c4 = inv4pi * ir * ir * ir;
      const double t2 = 2.0 * inv_sqrtpi * sqrtRS * exp(-RS), gg = erf(sqrtRS) - t2;
      double reg[12] = {}, sing[12] = {};
      pair_terms(dx, dy, dz, ax, ay, az, c4, gg, t2 / S2 - 3.0 * gg / R2, reg);
      pair_terms(dx, dy, dz, ax, ay, az, c4, 1.0, -3.0 * ir * ir, sing);
      for (int k = 0; k < 12; k++)
        s[k] += reg[k] - sing[k];
    }
  }
  for (int o = 16; o > 0; o >>= 1)
    for (int k = 0; k < 12; k++)
      s[k] += __shfl_down_sync(0xffffffffu, s[k], o);
  if (lane == 0)
    for (int k = 0; k < 12; k++)
      corr[(size_t)k * nt + i] = s[k];
}

// out[i][12] = -(sum of the chunks in order + correction): the sign of the
// reference's P2P (u -= ..., multipoleKernels.hpp:255-283).
__global__ void k_direct_model_sum(const double *part, int nchunks, const double *corr, int nt, double *out)
{
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 12 * nt; e += gridDim.x * blockDim.x) {
    const int i = e / 12, k = e % 12;
    double    v = 0;
    for (int ch = 0; ch < nchunks; ch++)
      v += part[((size_t)ch * 12 + k) * nt + i];
    v += corr[(size_t)k * nt + i];
    out[e] = -v;
  }
}

void direct_model_sum(cudaStream_t s, const double *soa, size_t cap, int n, CellsView cv, const int *leaf_cells, int nleaves, const int *p2p_start,
                      const int *p2p_src, const uint32_t *tgt, int nt, double *scratch, int nchunks, double *out)
{
  const int chunk = ((n + nchunks - 1) / nchunks + 127) / 128 * 128;
  double   *part  = scratch, *corr = scratch + (size_t)nchunks * 12 * nt;
  k_direct_singular<<<dim3((nt + 127) / 128, nchunks), 128, 0, s>>>(soa, cap, tgt, nt, n, chunk, part);
  count_launch();
  k_direct_p2p_correction<<<(nt + 3) / 4, 128, 0, s>>>(soa, cap, cv, leaf_cells, nleaves, p2p_start, p2p_src, tgt, nt, corr);
  count_launch();
  k_direct_model_sum<<<grid_for(12L * nt, 256), 256, 0, s>>>(part, nchunks, corr, nt, out);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

void direct_sum(cudaStream_t s, const double *tx, const double *ty, const double *tz, int nt, const double *src, size_t scap, int ns, double *out)
{
  k_direct<<<grid_for(nt, 256, 152 * 8), 256, 0, s>>>(tx, ty, tz, nt, src, scap, ns, out);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

} // namespace vfmm
