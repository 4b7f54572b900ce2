// Viscous diffusion by particle strength exchange (PSE): the reference's
// symmetric kernel (multipoleKernels.hpp:415-450, after Zhao & He, J. Am.
// Helicopter Soc. 55, 012007) over the P2P leaf lists.  For a target i and
// each of its P2P source leaves,
//   sum_j (vol_i alpha_j - vol_j alpha_i) exp(-R^2 / (2 s^2)) / s^5,
//   s^2 = sigma_i^2 + sigma_j^2,  vol = 4/3 pi sigma^3,  over R^2 != 0,
// is added to dadt_i times nu / (sqrt(2) pi sqrt(pi)).  It runs after the
// evaluation of a stage, as calculateViscosity does (fmmCalculator.hpp:713-724).
// One block per target leaf; every target owns its dadt, so no atomics.
#include <algorithm>
#include "vfmm_internal.cuh"

namespace vfmm {

namespace {

struct PseArgs {
  CellsView     cv;
  double       *soa;
  size_t        cap;
  const int    *leaf_cells;
  int           nleaves;
  const int    *p2p_start, *p2p_src;
  const float4 *pos32, *alp32; // mixed mode: (x - X_leaf, 1/(2 sigma^2)), (alpha, 1/sigma)
  double        prefix;        // nu / (sqrt(2) pi sqrt(pi))
};

constexpr double kPi = 3.14159265358979323846264338327950288;

// FP64, in the reference's operation order.
__global__ void __launch_bounds__(128) k_pse64(PseArgs a)
{
  double      *s   = a.soa;
  const size_t cap = a.cap;
  for (int li = blockIdx.x; li < a.nleaves; li += gridDim.x) {
    const int c = a.leaf_cells[li], b0 = a.cv.body[c], nb = a.cv.nbody[c];
    const int q0 = a.p2p_start[c], q1 = a.p2p_start[c + 1];
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
      const int    i  = b0 + t;
      const double xi = s[F_X * cap + i], yi = s[(F_X + 1) * cap + i], zi = s[(F_X + 2) * cap + i];
      const double ri = s[F_R * cap + i];
      const double ai[3] = {s[F_A * cap + i], s[(F_A + 1) * cap + i], s[(F_A + 2) * cap + i]};
      const double vol_i = 4. / 3. * kPi * ri * ri * ri;
      double       dadt[3] = {s[F_DADT * cap + i], s[(F_DADT + 1) * cap + i], s[(F_DADT + 2) * cap + i]};
      for (int q = q0; q < q1; q++) {
        const int sc = a.p2p_src[q], sb = a.cv.body[sc], sn = a.cv.nbody[sc];
        double    sum[3] = {0, 0, 0};
        for (int j = sb; j < sb + sn; j++) {
          const double dx = xi - s[F_X * cap + j], dy = yi - s[(F_X + 1) * cap + j], dz = zi - s[(F_X + 2) * cap + j];
          const double R2 = dx * dx + dy * dy + dz * dz;
          if (R2 != 0) {
            const double rj    = s[F_R * cap + j];
            const double oo    = 1. / (ri * ri + rj * rj);
            const double s5    = oo * oo * sqrt(oo);
            const double vol_j = 4. / 3. * kPi * rj * rj * rj;
            const double e     = exp(-0.5 * R2 * oo);
            for (int d = 0; d < 3; d++)
              sum[d] += (vol_i * s[(F_A + d) * cap + j] - vol_j * ai[d]) * e * s5;
          }
        }
        for (int d = 0; d < 3; d++)
          dadt[d] += sum[d] * a.prefix;
      }
      for (int d = 0; d < 3; d++)
        s[(F_DADT + d) * cap + i] = dadt[d];
    }
  }
}

__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float v)
{
  const float t  = hi + v;
  const float bb = t - hi;
  lo += (hi - (t - bb)) + (v - bb);
  hi = t;
}

// FP32 for the mixed mode: sources staged per chunk in coordinates relative to
// the target leaf's centre (the leaf offsets made once in FP64); the targets of
// a chunk of nt bodies get G = 128 / nt members each, which take every G-th
// source; FP32 sums of 16 sources are folded into a two-sum, the members are
// combined in a fixed order, and the result is added to the FP64 dadt.
constexpr int PSE_CH = 1024;
__global__ void __launch_bounds__(128) k_pse32(PseArgs a)
{
  __shared__ float4 Sp[PSE_CH]; // x, y, z (target-leaf frame), sigma^2
  __shared__ float4 Sa[PSE_CH]; // alpha, vol
  __shared__ float  red[2][128][3];
  const float fourpi3 = (float)(4. / 3. * kPi);
  for (int li = blockIdx.x; li < a.nleaves; li += gridDim.x) {
    const int    c = a.leaf_cells[li], b0 = a.cv.body[c], nb = a.cv.nbody[c];
    const int    q0 = a.p2p_start[c], q1 = a.p2p_start[c + 1];
    const double cx = a.cv.x[c], cy = a.cv.y[c], cz = a.cv.z[c];
    for (int tc = 0; tc < nb; tc += 128) {
      const int  nt = min(128, nb - tc), G = 128 / nt;
      const int  tt = threadIdx.x % nt, g = threadIdx.x / nt;
      const bool active = g < G;
      float      hi[3] = {0.f, 0.f, 0.f}, lo[3] = {0.f, 0.f, 0.f};
      float4     pt = make_float4(0.f, 0.f, 0.f, 0.f), at = pt;
      float      s2i = 0.f, voli = 0.f;
      if (active) {
        pt              = a.pos32[b0 + tc + tt];
        at              = a.alp32[b0 + tc + tt];
        const float sgi = 1.f / at.w;
        s2i             = sgi * sgi;
        voli            = fourpi3 * sgi * sgi * sgi;
      }
      // source bodies of the row, staged in chunks of up to PSE_CH
      int q = q0, off = 0;
      while (q < q1) {
        int cnt = 0;
        __syncthreads();
        while (q < q1 && cnt < PSE_CH) {
          const int   sc = a.p2p_src[q], sb = a.cv.body[sc], sn = a.cv.nbody[sc];
          const int   take = min(sn - off, PSE_CH - cnt);
          const float ox = (float)(a.cv.x[sc] - cx), oy = (float)(a.cv.y[sc] - cy), oz = (float)(a.cv.z[sc] - cz);
          for (int k = threadIdx.x; k < take; k += 128) {
            const float4 p  = a.pos32[sb + off + k];
            const float4 al = a.alp32[sb + off + k];
            const float  sg = 1.f / al.w;
            Sp[cnt + k]     = make_float4(p.x + ox, p.y + oy, p.z + oz, sg * sg);
            Sa[cnt + k]     = make_float4(al.x, al.y, al.z, fourpi3 * sg * sg * sg);
          }
          cnt += take;
          off += take;
          if (off == sn) {
            q++;
            off = 0;
          }
        }
        __syncthreads();
        if (active)
          for (int j0 = g; j0 < cnt; j0 += 16 * G) {
            float     sum[3] = {0.f, 0.f, 0.f};
            const int jend   = min(cnt, j0 + 16 * G);
            for (int j = j0; j < jend; j += G) {
              const float4 ps = Sp[j], as = Sa[j];
              const float  dx = pt.x - ps.x, dy = pt.y - ps.y, dz = pt.z - ps.z;
              const float  R2 = dx * dx + dy * dy + dz * dz;
              const float  s2 = s2i + ps.w;
              const float  oo = 1.f / s2;
              const float  w  = (R2 != 0.f) ? __expf(-0.5f * R2 * oo) * oo * oo * rsqrtf(s2) : 0.f;
              sum[0] += (voli * as.x - as.w * at.x) * w;
              sum[1] += (voli * as.y - as.w * at.y) * w;
              sum[2] += (voli * as.z - as.w * at.z) * w;
            }
            for (int d = 0; d < 3; d++)
              two_sum_acc(hi[d], lo[d], sum[d]);
          }
      }
      __syncthreads();
      for (int d = 0; d < 3; d++) {
        red[0][threadIdx.x][d] = hi[d];
        red[1][threadIdx.x][d] = lo[d];
      }
      __syncthreads();
      if (threadIdx.x < nt) {
        const int i = b0 + tc + threadIdx.x;
        for (int d = 0; d < 3; d++) {
          float h = 0.f, l = 0.f;
          for (int m = 0; m < G; m++) {
            two_sum_acc(h, l, red[0][m * nt + threadIdx.x][d]);
            l += red[1][m * nt + threadIdx.x][d];
          }
          a.soa[(F_DADT + d) * a.cap + i] += ((double)h + (double)l) * a.prefix;
        }
      }
    }
  }
}

} // namespace

void pse_pass(cudaStream_t s, const ExpArgs &e, const float4 *pos32, const float4 *alp32, double nu, double *soa)
{
  if (e.nleaves <= 0)
    return;
  PseArgs a{};
  a.cv         = e.cells;
  a.soa        = soa;
  a.cap        = e.cap;
  a.leaf_cells = e.leaf_cells;
  a.nleaves    = e.nleaves;
  a.p2p_start  = e.p2p_start;
  a.p2p_src    = e.p2p_src;
  a.pos32      = pos32;
  a.alp32      = alp32;
  a.prefix     = nu / 1.41421356237309504880168872420969808 * (1.0 / kPi) * 0.564189583547756286948079451560772586;
  const int grid = std::min(e.nleaves, 152 * 16);
  if (pos32)
    k_pse32<<<grid, 128, 0, s>>>(a);
  else
    k_pse64<<<grid, 128, 0, s>>>(a);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

} // namespace vfmm
