// Vorticity re-interpolation onto new points (FMMCalculator::RBF,
// fmmCalculator.hpp:733-917): the Gaussian vorticity of a body set summed over
// P2P leaf lists (P2P_vorticity, multipoleKernels.hpp:340-404),
//   omega_i = -sum_j alpha_j exp(-R^2 / (2 sigma_j^2)) / ((2 pi)^{3/2} sigma_j^3),
// with the pair R = 0 included, and the elementwise steps and reductions of
// the reference's three component-wise conjugate-gradient solves.  FP64 and
// deterministic: one thread per target, reductions over a fixed partition
// summed in a fixed order.
#include <algorithm>
#include "vfmm_internal.cuh"

namespace vfmm {

namespace {

struct VortArgs {
  CellsView     tc;                  // target cells
  const int    *leaf_cells;          // target leaves
  int           nleaves;
  const int    *p2p_start, *p2p_src; // CSR of P2P source leaves per target cell
  CellsView     sc;                  // source cells
  const double *tsoa, *ssoa;
  size_t        tcap, scap;
  double       *out; // target bodies (field-major, capacity tcap)
  int           field;
  int           zero_dadt; // also clear dadt, as resetSensors does (fmmCalculator.hpp:380-389)
};

__global__ void __launch_bounds__(128) k_vorticity(VortArgs a)
{
  const double inv_pi = 0.318309886183790671537767526745028724, inv_sqrtpi = 0.564189583547756286948079451560772586;
  const double sqrt2  = 1.41421356237309504880168872420969808;
  for (int li = blockIdx.x; li < a.nleaves; li += gridDim.x) {
    const int c = a.leaf_cells[li], b0 = a.tc.body[c], nb = a.tc.nbody[c];
    const int q0 = a.p2p_start[c], q1 = a.p2p_start[c + 1];
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
      const int    i  = b0 + t;
      const double xi = a.tsoa[F_X * a.tcap + i], yi = a.tsoa[(F_X + 1) * a.tcap + i], zi = a.tsoa[(F_X + 2) * a.tcap + i];
      double       w[3] = {0, 0, 0};
      for (int q = q0; q < q1; q++) {
        const int sc = a.p2p_src[q], sb = a.sc.body[sc], sn = a.sc.nbody[sc];
        double    sum[3] = {0, 0, 0};
        for (int j = sb; j < sb + sn; j++) {
          const double dx = xi - a.ssoa[F_X * a.scap + j], dy = yi - a.ssoa[(F_X + 1) * a.scap + j], dz = zi - a.ssoa[(F_X + 2) * a.scap + j];
          const double R2   = dx * dx + dy * dy + dz * dz;
          const double r    = a.ssoa[F_R * a.scap + j];
          const double S2   = 2.0 * r * r;
          const double zeta = exp(-R2 / S2) * inv_pi * inv_sqrtpi / sqrt2 / S2 / r;
          for (int d = 0; d < 3; d++)
            sum[d] += a.ssoa[(F_A + d) * a.scap + j] * zeta;
        }
        for (int d = 0; d < 3; d++)
          w[d] += -sum[d];
      }
      for (int d = 0; d < 3; d++) {
        a.out[(a.field + d) * a.tcap + i] = w[d];
        if (a.zero_dadt)
          a.out[(F_DADT + d) * a.tcap + i] = 0.0;
      }
    }
  }
}

constexpr int RBF_BLOCKS = 152 * 2, RBF_THREADS = 256;

// Elementwise steps (fields of the reference: target vorticity in
// velocity_old, A p in velocity, the solution x in dadt_old, the residual r in
// X_old, the search direction p in alpha), with an optional per-component sum.
__global__ void __launch_bounds__(RBF_THREADS) k_rbf_op(int op, double *s, size_t cap, int n, double c0, double c1, double c2, double *partials)
{
  const double c[3] = {c0, c1, c2};
  const double pi   = 3.14159265358979323846264338327950288;
  double       acc[3] = {0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    auto f = [&](int field, int d) -> double & { return s[(size_t)(field + d) * cap + i]; };
    switch (op) {
    case RBF_INIT_ALPHA: { // initAlphaValues, :765-773
      const double r   = s[F_R * cap + i];
      const double vol = (4. / 3. * pi * r * r * r);
      for (int d = 0; d < 3; d++)
        f(F_A, d) = f(F_VOLD, d) * vol;
      break;
    }
    case RBF_INIT_RESIDUAL: // setInitialResidualAndUpdateAlpha, :784-803
      for (int d = 0; d < 3; d++) {
        const double r = f(F_VOLD, d) - f(F_U, d);
        acc[d] += r * r;
        f(F_DOLD, d) = f(F_A, d);
        f(F_A, d)    = r;
        f(F_XOLD, d) = r;
      }
      break;
    case RBF_PAP: // calculatePAP, :805-812
      for (int d = 0; d < 3; d++)
        acc[d] += f(F_A, d) * f(F_U, d);
      break;
    case RBF_UPDATE: // updateAlphasAndResiduals, :814-825
      for (int d = 0; d < 3; d++) {
        f(F_DOLD, d) += c[d] * f(F_A, d);
        f(F_XOLD, d) -= c[d] * f(F_U, d);
      }
      break;
    case RBF_RES_NORM: // calculateResidualNormSquared, :827-833
      for (int d = 0; d < 3; d++)
        acc[d] += f(F_XOLD, d) * f(F_XOLD, d);
      break;
    case RBF_UPDATE_P: // updateP, :835-842
      for (int d = 0; d < 3; d++)
        f(F_A, d) = f(F_XOLD, d) + c[d] * f(F_A, d);
      break;
    case RBF_STORE: // storeAlphaValues, :844-850
      for (int d = 0; d < 3; d++)
        f(F_A, d) = f(F_DOLD, d);
      break;
    }
  }
  if (!partials)
    return;
  __shared__ double red[3][RBF_THREADS];
  for (int d = 0; d < 3; d++)
    red[d][threadIdx.x] = acc[d];
  __syncthreads();
  for (int st = RBF_THREADS / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int d = 0; d < 3; d++)
        red[d][threadIdx.x] += red[d][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x < 3)
    partials[blockIdx.x * 3 + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void k_rbf_final(const double *partials, int nb, double *out)
{
  if (threadIdx.x < 3) {
    double v = 0;
    for (int b = 0; b < nb; b++)
      v += partials[b * 3 + threadIdx.x];
    out[threadIdx.x] = v;
  }
}

} // namespace

void rbf_vorticity(cudaStream_t s, CellsView tc, const int *leaf_cells, int nleaves, const int *p2p_start, const int *p2p_src, const double *tsoa,
                   size_t tcap, CellsView sc, const double *ssoa, size_t scap, double *out, int field, int zero_dadt)
{
  if (nleaves <= 0)
    return;
  VortArgs a{tc, leaf_cells, nleaves, p2p_start, p2p_src, sc, tsoa, ssoa, tcap, scap, out, field, zero_dadt};
  k_vorticity<<<std::min(nleaves, 152 * 16), 128, 0, s>>>(a);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

void rbf_op(cudaStream_t s, int op, double *soa, size_t cap, int n, const double c[3], double *scratch, double *sums)
{
  k_rbf_op<<<RBF_BLOCKS, RBF_THREADS, 0, s>>>(op, soa, cap, n, c ? c[0] : 0.0, c ? c[1] : 0.0, c ? c[2] : 0.0, sums ? scratch : nullptr);
  count_launch();
  if (sums) {
    k_rbf_final<<<1, 32, 0, s>>>(scratch, RBF_BLOCKS, sums);
    count_launch();
  }
  VFMM_LAUNCH_CHECK();
}

} // namespace vfmm
