// Tensor-core (tcgen05) kernels.
//
// k_tc_selftest: one kind::tf32 MMA, D[128 x 16] = A[128 x 8] B[8 x 16],
// with A in tensor memory and B in shared memory (K-major, no swizzle), on
// small integers (exact in TF32 and FP32), so that the host can check the
// operand layouts the M2L kernel relies on element by element.
#include "tcgen05.cuh"
#include "vfmm_internal.cuh"

namespace vfmm {

__global__ void __launch_bounds__(128) k_tc_selftest(float *out, int swap_offsets, int *err)
{
  __shared__ __align__(1024) float Bs[128]; // K = 8 x N = 16 TF32, 512 bytes
  __shared__ uint32_t             tbase;
  __shared__ __align__(8) uint64_t mbar;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp == 0) {
    tc::tmem_alloc(&tbase, 512);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // element (k, n) of B at (k/4)*256 + (n/8)*128 + (n%8)*16 + (k%4)*4 bytes:
  // core matrices adjacent in K are 256 bytes apart, adjacent in N 128
  {
    const int n = tid / 8, k = tid % 8;
    const int off = (k / 4) * 256 + (n / 8) * 128 + (n % 8) * 16 + (k % 4) * 4;
    Bs[off / 4]   = (float)(((k * 7 + n * 3) % 13) - 6);
  }
  tc::fence_proxy_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t base = tbase;
  constexpr int  ACOL = 128, DCOL = 0;
  {
    const int m = 32 * warp + lane;
    uint32_t  v[8];
#pragma unroll
    for (int k = 0; k < 8; k++)
      v[k] = __float_as_uint((float)(((m * 3 + k * 5) % 11) - 5));
    tc::tmem_st8(tc::tmem_addr(base, 32 * warp, ACOL), v);
  }
  tc::tmem_st_wait();
  tc::fence_before_sync();
  __syncthreads();
  if (tid == 0) {
    tc::fence_after_sync();
    const uint32_t lbo = swap_offsets ? 128 : 256, sbo = swap_offsets ? 256 : 128;
    const uint64_t bd  = tc::smem_desc_noswizzle(tc::smem_u32(Bs), lbo, sbo);
    tc::mma_tf32_ts(tc::tmem_addr(base, 0, DCOL), tc::tmem_addr(base, 0, ACOL), bd, tc::idesc_tf32(128, 16), 0u);
    tc::mma_commit(&mbar);
  }
  const bool done = tc::mbar_wait_bounded(&mbar, 0);
  tc::fence_after_sync();
  if (!done) {
    if (tid == 0)
      atomicExch(err, VFMM_ERR_TIMEOUT);
  } else {
    const int m = 32 * warp + lane;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      uint32_t v[8];
      tc::tmem_ld8(tc::tmem_addr(base, 32 * warp, DCOL + 8 * h), v);
      tc::tmem_ld_wait();
#pragma unroll
      for (int j = 0; j < 8; j++)
        out[m * 16 + 8 * h + j] = __uint_as_float(v[j]);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(base, 512);
  }
}

} // namespace vfmm

extern "C" int vfmm_tcgen05_selftest(int device, int swap_offsets, float *out)
{
  using namespace vfmm;
  if (!out)
    return VFMM_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess)
    return VFMM_ERR_CUDA;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess)
    return VFMM_ERR_CUDA;
  if (prop.major != 10)
    return VFMM_ERR_UNSUPPORTED; // tcgen05 needs a Blackwell datacenter GPU (sm_100 family)
  float *d   = nullptr;
  int   *err = nullptr;
  if (cudaMalloc(&d, 128 * 16 * sizeof(float) + 16) != cudaSuccess)
    return VFMM_ERR_CUDA;
  err    = reinterpret_cast<int *>(d + 128 * 16);
  int rc = VFMM_OK;
  if (cudaMemset(d, 0, 128 * 16 * sizeof(float) + 16) != cudaSuccess)
    rc = VFMM_ERR_CUDA;
  if (rc == VFMM_OK) {
    k_tc_selftest<<<1, 128>>>(d, swap_offsets, err);
    if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess)
      rc = VFMM_ERR_CUDA;
  }
  int herr = 0;
  if (rc == VFMM_OK && (cudaMemcpy(out, d, 128 * 16 * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess ||
                        cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess))
    rc = VFMM_ERR_CUDA;
  if (rc == VFMM_OK && herr)
    rc = herr;
  cudaFree(d);
  return rc;
}
