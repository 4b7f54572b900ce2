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

void direct_sum(cudaStream_t s, const double *tx, const double *ty, const double *tz, int nt, const double *src, size_t scap, int ns, double *out)
{
  k_direct<<<grid_for(nt, 256, 152 * 8), 256, 0, s>>>(tx, ty, tz, nt, src, scap, ns, out);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

} // namespace vfmm
