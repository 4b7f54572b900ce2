// Body-state kernels: AoS <-> SoA transposes of exafmm::Body records,
// reordering into tree order, input checks, and the fused elementwise stage
// update (fmmCalculator.hpp:493-711) with relaxation (relaxation.hpp:8-19).
#include "vfmm_internal.cuh"

namespace vfmm {

// 32 bodies x 37 fields per block, staged through shared memory so that both
// the AoS reads and the SoA writes are coalesced.
__global__ void k_aos_to_soa(const double *__restrict__ aos, double *__restrict__ soa, size_t cap, int n)
{
  __shared__ double t[32 * NFIELD + 1];
  for (int b0 = blockIdx.x * 32; b0 < n; b0 += gridDim.x * 32) {
    const int nb = min(32, n - b0);
    for (int k = threadIdx.x; k < nb * NFIELD; k += blockDim.x)
      t[k] = aos[(size_t)b0 * NFIELD + k];
    __syncthreads();
    for (int k = threadIdx.x; k < nb * NFIELD; k += blockDim.x) {
      const int f = k / nb, i = k % nb;
      soa[(size_t)f * cap + b0 + i] = t[i * NFIELD + f];
    }
    __syncthreads();
  }
}

__global__ void k_soa_to_aos(const double *__restrict__ soa, size_t cap, double *__restrict__ aos, int n)
{
  __shared__ double t[32 * NFIELD + 1];
  for (int b0 = blockIdx.x * 32; b0 < n; b0 += gridDim.x * 32) {
    const int nb = min(32, n - b0);
    for (int k = threadIdx.x; k < nb * NFIELD; k += blockDim.x) {
      const int f = k / nb, i = k % nb;
      t[i * NFIELD + f] = soa[(size_t)f * cap + b0 + i];
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nb * NFIELD; k += blockDim.x)
      aos[(size_t)b0 * NFIELD + k] = t[k];
    __syncthreads();
  }
}

// The fields of `mask` only: the host link moves whole 128-byte lines, so a
// record read in part costs the lines its fields touch (X, alpha and the
// radius of 2^20 records: 0.75 ms against 1.48 ms for whole records).  The
// other fields of each body are set to a quiet NaN, so that a field left out
// that the caller's computation does read shows up in its results.
struct FieldList {
  uint64_t      mask;
  int           n;
  unsigned char f[NFIELD];
};
__global__ void k_aos_to_soa_fields(const double *__restrict__ aos, double *__restrict__ soa, size_t cap, int n, FieldList fl)
{
  __shared__ double t[32 * NFIELD + 1];
  const double      qnan = __longlong_as_double(0x7ff8000000000000LL);
  for (int b0 = blockIdx.x * 32; b0 < n; b0 += gridDim.x * 32) {
    const int nb = min(32, n - b0);
    for (int k = threadIdx.x; k < nb * fl.n; k += blockDim.x) {
      const int i = k / fl.n, f = fl.f[k % fl.n];
      t[i * NFIELD + f] = aos[(size_t)(b0 + i) * NFIELD + f];
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nb * NFIELD; k += blockDim.x) {
      const int f = k / nb, i = k % nb;
      soa[(size_t)f * cap + b0 + i] = ((fl.mask >> f) & 1) ? t[i * NFIELD + f] : qnan;
    }
    __syncthreads();
  }
}

void aos_to_soa(cudaStream_t s, const double *aos, double *soa, size_t cap, int n, uint64_t mask)
{
  mask &= (1ull << NFIELD) - 1;
  if (mask == (1ull << NFIELD) - 1)
    k_aos_to_soa<<<grid_for(n, 32, 152 * 32), 128, 0, s>>>(aos, soa, cap, n);
  else {
    FieldList fl{};
    fl.mask = mask;
    for (int f = 0; f < NFIELD; f++)
      if ((mask >> f) & 1)
        fl.f[fl.n++] = (unsigned char)f;
    if (fl.n == 0)
      throw Error(VFMM_ERR_INVALID, "no body fields to load");
    k_aos_to_soa_fields<<<grid_for(n, 32, 152 * 32), 128, 0, s>>>(aos, soa, cap, n, fl);
  }
  count_launch();
  VFMM_LAUNCH_CHECK();
}
void soa_to_aos(cudaStream_t s, const double *soa, size_t cap, double *aos, int n)
{
  k_soa_to_aos<<<grid_for(n, 32, 152 * 32), 128, 0, s>>>(soa, cap, aos, n);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

// dst[f][p] = src[f][perm[p]] for the fields in fieldMask.
__global__ void k_gather(const double *__restrict__ src, double *__restrict__ dst, size_t cap, const uint32_t *__restrict__ perm, int n,
                         uint64_t mask)
{
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
    const uint32_t q = perm[p];
#pragma unroll 1
    for (int f = 0; f < NFIELD; f++)
      if ((mask >> f) & 1)
        dst[(size_t)f * cap + p] = src[(size_t)f * cap + q];
  }
}
void gather_bodies(cudaStream_t s, const double *src, double *dst, size_t cap, const uint32_t *perm, int n, uint64_t fieldMask)
{
  k_gather<<<grid_for(n, 256), 256, 0, s>>>(src, dst, cap, perm, n, fieldMask);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

__global__ void k_check_finite(const double *__restrict__ soa, size_t cap, int n, DevInfo *info)
{
  bool bad = false;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    for (int f = F_X; f < F_X + 6; f++)
      bad |= !isfinite(soa[(size_t)f * cap + i]);
    bad |= !isfinite(soa[(size_t)F_R * cap + i]);
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0)
    atomicExch(&info->nonfinite, 1);
}
void check_finite(cudaStream_t s, const double *soa, size_t cap, int n, DevInfo *info)
{
  k_check_finite<<<grid_for(n, 256), 256, 0, s>>>(soa, cap, n, info);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

// "Reset The Rates", fmmCalculator.hpp:359-378
__global__ void k_reset_rates(double *soa, size_t cap, int n)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    for (int f = F_J; f < F_J + 9; f++)
      soa[(size_t)f * cap + i] = 0;
    for (int f = F_U; f < F_U + 6; f++)
      soa[(size_t)f * cap + i] = 0;
    soa[(size_t)F_DRDT * cap + i] = 0;
  }
}
void reset_rates(cudaStream_t s, double *soa, size_t cap, int n)
{
  k_reset_rates<<<grid_for(n, 256), 256, 0, s>>>(soa, cap, n);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

struct BodyRef {
  double *b;
  size_t  cap;
  int     i;
  __device__ double &operator()(int f) const { return b[(size_t)f * cap + i]; }
};

__device__ void relax_one(const BodyRef &q, double f)
{
  const double w[3] = {q(F_J + 7) - q(F_J + 5), q(F_J + 2) - q(F_J + 6), q(F_J + 3) - q(F_J + 1)};
  const double nw   = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
  const double na   = sqrt(q(F_A) * q(F_A) + q(F_A + 1) * q(F_A + 1) + q(F_A + 2) * q(F_A + 2));
  if (nw == 0.0)
    return;
  for (int d = 0; d < 3; d++)
    q(F_A + d) = (1 - f) * q(F_A + d) + f * na * w[d] / nw;
}

// One stage update of the configured scheme (fmmCalculator.hpp:493-711), then
// optional relaxation after the last stage.
__global__ void k_stage_update(double *soa, size_t cap, int n, StageArgs a)
{
  const double h = a.dt;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    BodyRef q{soa, cap, i};
    if (a.csm) // core spreading, fmmCalculator.hpp:334-337
      q(F_DRDT) += (sqrt((q(F_R) * q(F_R)) + (2.0 * a.nu * h)) - q(F_R)) / h;
    if (a.do_update) {
      if (a.store_initial) { // storeInitialState, fmmCalculator.hpp:493-509
        for (int d = 0; d < 3; d++) {
          q(F_VOLD + d) = 0;
          q(F_DOLD + d) = 0;
          q(F_XOLD + d) = q(F_X + d);
          q(F_AOLD + d) = q(F_A + d);
        }
        q(F_ROLD) = q(F_R);
      }
      if (a.scheme == VFMM_EULER) { // :511-521
        for (int d = 0; d < 3; d++) {
          q(F_X + d) += q(F_U + d) * h;
          q(F_A + d) += q(F_DADT + d) * h;
        }
        q(F_R) += q(F_DRDT) * h;
      } else if (a.scheme == VFMM_RK2) {
        if (a.stage == 0) { // stepRK21 :523-540
          for (int d = 0; d < 3; d++) {
            q(F_VOLD + d) = q(F_U + d);
            q(F_DOLD + d) = q(F_DADT + d);
          }
          q(F_DRDTOLD) = q(F_DRDT);
          for (int d = 0; d < 3; d++) {
            q(F_X + d) += h * q(F_VOLD + d);
            q(F_A + d) += h * q(F_DOLD + d);
          }
          q(F_R) += h * q(F_DRDTOLD);
        } else { // stepRK22 :542-562
          for (int d = 0; d < 3; d++) {
            q(F_VOLD + d) = 0.5 * q(F_U + d) + 0.5 * q(F_VOLD + d);
            q(F_DOLD + d) = 0.5 * q(F_DADT + d) + 0.5 * q(F_DOLD + d);
          }
          q(F_DRDTOLD) = 0.5 * q(F_DRDT) + 0.5 * q(F_DRDTOLD);
          for (int d = 0; d < 3; d++) {
            q(F_X + d) = q(F_XOLD + d) + h * q(F_VOLD + d);
            q(F_A + d) = q(F_AOLD + d) + h * q(F_DOLD + d);
          }
          q(F_R) = q(F_ROLD) + h * q(F_DRDTOLD);
        }
      } else if (a.scheme == VFMM_RK3) { // Williamson low-storage, :564-627
        const double A = a.stage == 0 ? 0.0 : (a.stage == 1 ? -5.0 / 9.0 : -153.0 / 128.0);
        const double B = a.stage == 0 ? 1.0 / 3.0 : (a.stage == 1 ? 15.0 / 16.0 : 8.0 / 15.0);
        for (int d = 0; d < 3; d++) {
          q(F_VOLD + d) = a.stage == 0 ? h * q(F_U + d) : A * q(F_VOLD + d) + h * q(F_U + d);
          q(F_DOLD + d) = a.stage == 0 ? h * q(F_DADT + d) : A * q(F_DOLD + d) + h * q(F_DADT + d);
        }
        q(F_DRDTOLD) = a.stage == 0 ? h * q(F_DRDT) : A * q(F_DRDTOLD) + h * q(F_DRDT);
        for (int d = 0; d < 3; d++) {
          q(F_X + d) += B * q(F_VOLD + d);
          q(F_A + d) += B * q(F_DOLD + d);
        }
        q(F_R) += B * q(F_DRDTOLD);
      } else if (a.scheme == VFMM_RK4) { // :629-711
        if (a.stage == 0) {
          for (int d = 0; d < 3; d++) {
            q(F_VOLD + d) = q(F_U + d);
            q(F_DOLD + d) = q(F_DADT + d);
          }
          q(F_DRDTOLD) = q(F_DRDT);
          for (int d = 0; d < 3; d++) {
            q(F_X + d) += 0.5 * h * q(F_VOLD + d);
            q(F_A + d) += 0.5 * h * q(F_DOLD + d);
          }
          q(F_R) += 0.5 * h * q(F_DRDTOLD);
        } else if (a.stage < 3) {
          // stage 3 of the reference uses 0.5*dt (fmmCalculator.hpp:683-689); rk4_fixed uses dt
          const double c = (a.stage == 2 && a.rk4_fixed) ? 1.0 : 0.5;
          for (int d = 0; d < 3; d++) {
            q(F_VOLD + d) += 2.0 * q(F_U + d);
            q(F_DOLD + d) += 2.0 * q(F_DADT + d);
          }
          q(F_DRDTOLD) += 2.0 * q(F_DRDT);
          for (int d = 0; d < 3; d++) {
            q(F_X + d) = q(F_XOLD + d) + c * h * q(F_U + d);
            q(F_A + d) = q(F_AOLD + d) + c * h * q(F_DADT + d);
          }
          q(F_R) = q(F_ROLD) + c * h * q(F_DRDT);
        } else {
          for (int d = 0; d < 3; d++) {
            q(F_VOLD + d) += q(F_U + d);
            q(F_DOLD + d) += q(F_DADT + d);
          }
          q(F_DRDTOLD) += q(F_DRDT);
          for (int d = 0; d < 3; d++) {
            q(F_X + d) = q(F_XOLD + d) + (h / 6.0) * q(F_VOLD + d);
            q(F_A + d) = q(F_AOLD + d) + (h / 6.0) * q(F_DOLD + d);
          }
          q(F_R) = q(F_ROLD) + (h / 6.0) * q(F_DRDTOLD);
        }
      }
    }
    if (a.relax > 0)
      relax_one(q, a.relax);
  }
}

void finish_and_update(cudaStream_t s, double *soa, size_t cap, int n, const StageArgs &a)
{
  k_stage_update<<<grid_for(n, 256), 256, 0, s>>>(soa, cap, n, a);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

void relax_bodies(cudaStream_t s, double *soa, size_t cap, int n, double f)
{
  StageArgs a{};
  a.do_update = 0;
  a.relax     = f;
  k_stage_update<<<grid_for(n, 256), 256, 0, s>>>(soa, cap, n, a);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

__global__ void k_fill(uint4 *p, size_t n16, int v)
{
  const uint4 val = make_uint4(v, v, v, v);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
    p[i] = val;
}
void fill_bytes(cudaStream_t s, void *p, size_t bytes, int value)
{
  k_fill<<<152 * 8, 256, 0, s>>>((uint4 *)p, bytes / 16, value);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

// FMA throughput probe: 8 independent chains per thread, 152 x 8 blocks.
template <class T>
__global__ void __launch_bounds__(256) k_fma_probe(T *out, int iters, T a, T b)
{
  T v[8];
#pragma unroll
  for (int k = 0; k < 8; k++)
    v[k] = T(threadIdx.x + k) * T(1e-3);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++)
      v[k] = fma(v[k], a, b);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++)
    s += v[k];
  if (s == T(12345.678))
    out[0] = s;
}

double fma_probe(cudaStream_t s, bool fp64, void *scratch, int iters, float *ms_out, cudaEvent_t e0, cudaEvent_t e1)
{
  const int blocks = 152 * 8, threads = 256;
  VFMM_CUDA_TRY(cudaEventRecord(e0, s));
  if (fp64)
    k_fma_probe<double><<<blocks, threads, 0, s>>>((double *)scratch, iters, 0.999999, 1e-7);
  else
    k_fma_probe<float><<<blocks, threads, 0, s>>>((float *)scratch, iters, 0.999999f, 1e-7f);
  count_launch();
  VFMM_LAUNCH_CHECK();
  VFMM_CUDA_TRY(cudaEventRecord(e1, s));
  VFMM_CUDA_TRY(cudaEventSynchronize(e1));
  VFMM_CUDA_TRY(cudaEventElapsedTime(ms_out, e0, e1));
  return 2.0 * 8.0 * iters * (double)blocks * threads;
}

// Global invariants of the particle field, FP64: circulation sum alpha,
// linear impulse 1/2 sum x cross alpha, angular impulse 1/3 sum x cross (x cross
// alpha).  Fixed partition (DIAG_BLOCKS blocks) and fixed summation order, so
// the sums are reproducible.
constexpr int DIAG_BLOCKS = 152 * 2, DIAG_THREADS = 256;
__global__ void __launch_bounds__(DIAG_THREADS) k_diag(const double *soa, size_t cap, int n, double *partials)
{
  double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double x[3] = {soa[F_X * cap + i], soa[(F_X + 1) * cap + i], soa[(F_X + 2) * cap + i]};
    const double a[3] = {soa[F_A * cap + i], soa[(F_A + 1) * cap + i], soa[(F_A + 2) * cap + i]};
    const double xa[3] = {x[1] * a[2] - x[2] * a[1], x[2] * a[0] - x[0] * a[2], x[0] * a[1] - x[1] * a[0]};
    const double xxa[3] = {x[1] * xa[2] - x[2] * xa[1], x[2] * xa[0] - x[0] * xa[2], x[0] * xa[1] - x[1] * xa[0]};
    for (int d = 0; d < 3; d++) {
      acc[d] += a[d];
      acc[3 + d] += 0.5 * xa[d];
      acc[6 + d] += xxa[d] / 3.0;
    }
  }
  __shared__ double red[9][DIAG_THREADS];
  for (int k = 0; k < 9; k++)
    red[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int st = DIAG_THREADS / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int k = 0; k < 9; k++)
        red[k][threadIdx.x] += red[k][threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x < 9)
    partials[blockIdx.x * 9 + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void k_diag_final(const double *partials, int nb, double *out)
{
  if (threadIdx.x < 9) {
    double v = 0;
    for (int b = 0; b < nb; b++)
      v += partials[b * 9 + threadIdx.x];
    out[threadIdx.x] = v;
  }
}

void diagnostics(cudaStream_t s, const double *soa, size_t cap, int n, double *scratch, double *out)
{
  k_diag<<<DIAG_BLOCKS, DIAG_THREADS, 0, s>>>(soa, cap, n, scratch);
  count_launch();
  k_diag_final<<<1, 32, 0, s>>>(scratch, DIAG_BLOCKS, out);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

} // namespace vfmm
