// vfmm_bounds_noalloc: the root cell of the octree (centre and half-width, as
// exafmm::getBounds computes them) for coordinates already on the device,
// without allocating any memory.
//
// Who needs it: code that may not call cudaMalloc or cudaFree -- for example
// work issued while a CUDA stream is being captured into a graph (allocation
// calls are not allowed there), a host that has handed all device memory to
// its own pool allocator, or a plugin that must not touch the process's
// allocator.  Those callers pass device pointers for the inputs and the output;
// the per-block partial results that the regular path keeps in handle-owned
// scratch live here in a fixed array compiled into the library.
//
// Limits and sharing: the scratch holds NOALLOC_BOUNDS_BLOCKS partial records
// (608 x 6 doubles = 29,184 bytes) on every GPU that loads the library, for as
// long as the library stays loaded.  Any n from 1 to 2^31-1 bodies fits (blocks
// stride over the bodies); larger n is rejected.  Every call uses the same
// array, so two calls whose kernels overlap on the GPU (different streams, or
// different host threads) race and both results are undefined: serialise them.
// Each call overwrites every record it reads, so nothing needs clearing.
//
// Set-up: the first call on each device looks up the array's device address
// (cudaGetSymbolAddress) with that device current; make that first call before
// any stream capture begins.  The address is kept for the life of the process:
// cudaDeviceReset unloads the library's device module, and the array may come
// back elsewhere, so this entry point must not be used after a reset of that
// device.
#include <climits>
#include <mutex>
#include "vfmm_internal.cuh"

namespace vfmm {

constexpr int NOALLOC_BOUNDS_BLOCKS = 152 * 4;
static __device__ __align__(256) double g_bounds_scratch[NOALLOC_BOUNDS_BLOCKS * 6];

// getBounds (tree.hpp:7-26) from the partial records: the same FP64 operations
// as the tree build's final step, written to out[0..2] = centre, out[3] = R0.
__global__ void k_bounds_final_out(const double *part, int nb, double *out)
{
  if (threadIdx.x != 0 || blockIdx.x != 0)
    return;
  double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int b = 0; b < nb; b++)
    for (int d = 0; d < 3; d++) {
      mn[d] = fmin(part[b * 6 + d], mn[d]);
      mx[d] = fmax(part[b * 6 + 3 + d], mx[d]);
    }
  double X0[3], R0 = 0;
  for (int d = 0; d < 3; d++)
    X0[d] = __ddiv_rn(__dadd_rn(mx[d], mn[d]), 2.0);
  for (int d = 0; d < 3; d++) {
    R0 = fmax(__dsub_rn(X0[d], mn[d]), R0);
    R0 = fmax(__dsub_rn(mx[d], X0[d]), R0);
  }
  R0 = __dmul_rn(R0, 1.00001);
  for (int d = 0; d < 3; d++)
    out[d] = X0[d];
  out[3] = R0;
}

namespace {
std::mutex g_scratch_mu;
void      *g_scratch_addr[256] = {};

// Device address of g_bounds_scratch on the current device (looked up once).
int scratch_address(double **out)
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256)
    return VFMM_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_bounds_scratch) != cudaSuccess || !p)
      return VFMM_ERR_CUDA;
    g_scratch_addr[dev] = p;
  }
  *out = static_cast<double *>(g_scratch_addr[dev]);
  return VFMM_OK;
}
} // namespace
} // namespace vfmm

extern "C" int vfmm_bounds_noalloc(const double *x, const double *y, const double *z, size_t n, double *out, void *stream)
{
  using namespace vfmm;
  if (!x || !y || !z || !out || n == 0)
    return VFMM_ERR_INVALID;
  if (n > (size_t)INT_MAX)
    return VFMM_ERR_INVALID;
  double   *scratch = nullptr;
  const int rc      = scratch_address(&scratch);
  if (rc != VFMM_OK)
    return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  bbox_partial_into(s, x, y, z, (int)n, scratch, NOALLOC_BOUNDS_BLOCKS);
  if (cudaGetLastError() != cudaSuccess)
    return VFMM_ERR_CUDA;
  k_bounds_final_out<<<1, 32, 0, s>>>(scratch, NOALLOC_BOUNDS_BLOCKS, out);
  count_launch();
  return cudaGetLastError() == cudaSuccess ? VFMM_OK : VFMM_ERR_CUDA;
}
