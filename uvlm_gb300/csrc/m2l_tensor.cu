// Tensor-core (tcgen05) kernels.
//
// k_tc_selftest: one kind::tf32 MMA, D[128 x 16] = A[128 x 8] B[8 x 16],
// with A in tensor memory and B in shared memory (K-major, no swizzle), on
// small integers (exact in TF32 and FP32), so that the host can check the
// operand layouts the M2L kernel relies on element by element; mode bit 1
// runs it as M = 64 with A[m][0] = m + 1 (other K zero) on a zeroed D, which
// shows which TMEM lanes an M = 64 MMA reads and writes.
#include <algorithm>
#include <cub/cub.cuh>
#include "harmonics.cuh"
#include "tcgen05.cuh"
#include "vfmm_internal.cuh"

namespace vfmm {

__global__ void __launch_bounds__(128) k_tc_selftest(float *out, int mode, int *err)
{
  const bool swap_offsets = mode & 1, m64 = mode & 2;
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
      v[k] = __float_as_uint(m64 ? (k == 0 ? (float)(m + 1) : 0.f) : (float)(((m * 3 + k * 5) % 11) - 5));
    tc::tmem_st8(tc::tmem_addr(base, 32 * warp, ACOL), v);
    const uint32_t z[8] = {0, 0, 0, 0, 0, 0, 0, 0}; // D starts at zero: lanes an M = 64 MMA leaves alone read back 0
    tc::tmem_st8(tc::tmem_addr(base, 32 * warp, DCOL), z);
    tc::tmem_st8(tc::tmem_addr(base, 32 * warp, DCOL + 8), z);
  }
  tc::tmem_st_wait();
  tc::fence_before_sync();
  __syncthreads();
  if (tid == 0) {
    tc::fence_after_sync();
    const uint32_t lbo = swap_offsets ? 128 : 256, sbo = swap_offsets ? 256 : 128;
    const uint64_t bd  = tc::smem_desc_noswizzle(tc::smem_u32(Bs), lbo, sbo);
    tc::mma_tf32_ts(tc::tmem_addr(base, 0, DCOL), tc::tmem_addr(base, 0, ACOL), bd, tc::idesc_tf32(m64 ? 64 : 128, 16), 0u);
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

// ============================================================================
// M2L on the tensor cores, by offset class.
//
// In the scaled variables of the mixed path, the M2L of a pair (target t,
// source s) with d = X_t - X_s is a linear map of the source's scaled
// multipole that depends only on the offset in units of the target's
// half-width, o = d / R_t, and on the level difference delta = l_t - l_s:
//   L_j^k(t) = (-1)^j R_t^(-j-1) sum_{n <= p-1-j} sum_{m=-n..n}
//              2^(delta n) M'_n^m(s) S'_{j+n}^{m-k}(o)
// (multipoleKernels.hpp:519-552 with the truncation j + n <= p - 1 that its
// zero-initialised harmonics impose).  On an octree, same-level pairs have
// o = 2 x (integer vector), so the targets of one level share a few hundred
// offset classes, and every class is one operator A(delta, o) applied to many
// multipoles.
//
// Real form.  Inputs per component: Mt_n^0 (real part; the imaginary part of
// an m = 0 coefficient of a real field is zero) and Re/Im Mt_n^m, m = 1..n, in
// the order n^2, n^2 + 2m - 1 (Re), n^2 + 2m (Im): P^2 values, padded to KP.
// Outputs: Re/Im L_j^k, k <= j, row 2 tri(j, k) + (0: Re, 1: Im): P(P+1)
// rows <= 128 for P <= 10.  With M'_n^m = (-1)^m Mt_n^m, M'_n^-m = conj(Mt_n^m)
// and (c1, d1) = S'_q^{m-k}, (c2, d2) = S'_q^{-m-k}, q = j + n:
//   Re L += a [(-1)^m c1 + c2] + b [-(-1)^m d1 + d2]
//   Im L += a [(-1)^m d1 + d2] + b [(-1)^m c1 - c2]      (Mt_n^m = a + i b).
//
// Layout of one tile: 32 targets of one level (the same octant within their
// parents where possible, so that their offset sets coincide), D = A B with
// A (128 rows x KP) in tensor memory and B (KP x 96: target x component) in
// shared memory, one class at a time (see k_m2l_tc).  FP32 is kept by three
// TF32 products, A_hi B_hi + A_hi B_lo + A_lo B_hi, where x_hi is x rounded
// to TF32 and x_lo is x - x_hi rounded to TF32 (x_hi + x_lo is x to ~2^-22).
// ============================================================================

// Class key: bits 0..10 oz + 1024, 11..21 oy + 1024, 22..32 ox + 1024,
// 33..37 delta + 16, offsets in units of the finer cell's half-width; a pair
// outside that range gets the sentinel class and is contracted on its own.
constexpr int      TC_CLASS_BITS = 38;
constexpr uint64_t TC_SENTINEL   = (1ull << TC_CLASS_BITS) - 1;
constexpr int      TC_COL_SHIFT  = 27; // pair value: column << 27 | source cell

template <int P>
struct TcM2L {
  static constexpr int    KR = P * P, KP = (KR + 7) / 8 * 8, NR = P * (P + 1);
  static constexpr int    TT = 32, N = 3 * TT, KC = KP / 4;
  static constexpr int    SBO = 128, LBO = (N / 8) * 128; // bytes: N-adjacent, K-adjacent core matrices
  static constexpr int    BBYTES = KC * LBO;              // one B operand (hi or lo)
  static constexpr int    STAGE  = 2 * BBYTES;            // hi + lo
  static constexpr int    DCOL = 0, ACOL = N, ABUF = 2 * KP;
  static constexpr size_t smem = 2 * (size_t)STAGE + 1024; // two stages + alignment slack
  static_assert(N + 2 * ABUF <= 512, "D and two A buffers fit in the 512 TMEM columns");
  static_assert(NR <= 128, "the output rows fit the 128 TMEM lanes");
  static_assert(KC % 2 == 0, "B rows are gathered 32 bytes at a time");
};

struct TcArgs {
  const unsigned long long *keys; // sorted: tile << 38 | class
  const uint32_t           *vals; // column << 27 | source
  int                       npairs;
  const int                *tile_start; // [ntiles + 1]
  const int                *tile_cells; // [ntiles][32], -1 = none
  const int                *tile_level;
  const int                *ntiles;     // device scalar
  int                      *tile_next;  // tiles handed out beyond the first gridDim.x (zeroed per evaluation)
  const float              *Bhi, *Blo;  // [cell][3][KP]
  const float4             *table;      // operators, see k_tc_class_ops
  const int                *cidq;       // table index of each group, at its first pair
  CellsView                 cv;
  double2                  *L;
  double                    iR0pow[PMAX + 2]; // R0^-n
  int                      *err;
};


// v * 2^e for any e (exact power-of-two scaling, ldexpf outside the normal range)
__device__ __forceinline__ float tc_scale2(float v, int e)
{
  return (e >= -126 && e <= 127) ? v * __int_as_float((e + 127) << 23) : ldexpf(v, e);
}

// Operator classes of one evaluation: an open-addressing hash of the class
// keys (TC_HASH slots) gives each class an index; the operators of the first
// `cap` indices are built once into a table, in the order the M2L kernel
// reads them: [class][hi, lo][chunk of 8 columns][128 rows][8].
constexpr int      TC_HASH  = 1 << 14;
constexpr uint64_t TC_EMPTY = ~0ull;
__device__ __forceinline__ unsigned tc_hash(unsigned long long k) { return (unsigned)((k * 0x9E3779B97F4A7C15ull) >> 50); }

// Value of column `col` of row (j, k, part) of the operator A(delta, o), from
// the folded harmonics Ys = S'(o) (see the derivation above).
template <int P>
__device__ __forceinline__ float tc_op_value(int col, int rj, int rk, int rpart, bool rlive, int dl, const cx<float> *Ys)
{
  if (col >= P * P || !rlive)
    return 0.f;
  int n = 0;
  while ((n + 1) * (n + 1) <= col)
    n++;
  if (n > P - 1 - rj)
    return 0.f;
  const int r = col - n * n, m = (r + 1) / 2, pin = (r > 0 && (r & 1) == 0) ? 1 : 0;
  const int q = rj + n, base = q * q + q - rk;
  float     v;
  if (m == 0) {
    const cx<float> y0 = Ys[base];
    v                  = rpart ? y0.i : y0.r;
  } else {
    const cx<float> y1 = Ys[base + m], y2 = Ys[base - m];
    const float     sg = (m & 1) ? -1.f : 1.f;
    if (rpart == 0)
      v = pin ? fmaf(-sg, y1.i, y2.i) : fmaf(sg, y1.r, y2.r);
    else
      v = pin ? fmaf(sg, y1.r, -y2.r) : fmaf(sg, y1.i, y2.i);
  }
  return tc_scale2(v, dl * n);
}

// Folded singular harmonics S'(o), column m = 0 .. P-1 on threads 0 .. P-1.
template <int P>
__device__ __forceinline__ void tc_harmonics(float4 o, cx<float> *Ys)
{
  if (threadIdx.x < P) {
    const int    m  = threadIdx.x;
    const double r2 = (double)o.x * o.x + (double)o.y * o.y + (double)o.z * o.z;
    singular_column_emit<float, P>(m, o.x, o.y, o.z, (float)(1.0 / r2), (float)(1.0 / sqrt(r2)), [&](int q, cx<float> c) {
      Ys[q * q + q + m] = (m & 1) ? cx<float>{-c.r, -c.i} : c;
      if (m > 0)
        Ys[q * q + q - m] = conj(c);
    });
  }
}

// Row r of a 128-row operator: (j, k, part) of output L_j^k, or not live.
__device__ __forceinline__ void tc_row_of(int r, int NR, int &rj, int &rk, int &rpart, bool &rlive)
{
  rlive = r < NR;
  rj = rk = 0;
  rpart   = r & 1;
  if (rlive) {
    const int jks = r >> 1;
    while ((rj + 1) * (rj + 2) / 2 <= jks)
      rj++;
    rk = jks - rj * (rj + 1) / 2;
  }
}

// Output row held by TMEM lane L.  An M = 64 MMA covers lanes 0-15 of each
// 32-lane quarter; those 64 lanes hold rows 0..63 (j <= 7, the rows that need
// high input degrees), the other 64 lanes rows 64..127 (j >= 7: they need
// only the first two K steps, input degrees n <= P - 1 - 7 < 4).
__host__ __device__ __forceinline__ int tc_lane_row(int L)
{
  const int q = L >> 5, i = L & 31;
  return i < 16 ? 16 * q + i : 64 + 16 * q + (i - 16);
}

// Offset o (target units) and level difference of a class key.
__device__ __forceinline__ float4 tc_class_offset(unsigned long long k0)
{
  const int   dz = (int)(k0 & 2047) - 1024, dy = (int)((k0 >> 11) & 2047) - 1024, dx = (int)((k0 >> 22) & 2047) - 1024;
  const int   dl = (int)((k0 >> 33) & 31) - 16;
  const float f  = dl < 0 ? ldexpf(1.f, dl) : 1.f; // offsets are in units of the finer cell
  return make_float4(dx * f, dy * f, dz * f, __int_as_float(dl));
}

// Insert the class of every (tile, class) group into the hash.
__global__ void k_tc_class_insert(const unsigned long long *__restrict__ keys, int n, unsigned long long *hkeys, int *err)
{
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const unsigned long long c = keys[q] & TC_SENTINEL;
    if (c == TC_SENTINEL || (q > 0 && keys[q - 1] == keys[q]))
      continue;
    unsigned h = tc_hash(c), probes = 0;
    for (;;) {
      const unsigned long long cur = hkeys[h];
      if (cur == c)
        break;
      if (cur == TC_EMPTY) {
        const unsigned long long prev = atomicCAS(&hkeys[h], TC_EMPTY, c);
        if (prev == TC_EMPTY || prev == c)
          break;
      }
      h = (h + 1) & (TC_HASH - 1);
      if (++probes >= TC_HASH) { // full: more classes than slots
        atomicExch(err, VFMM_ERR_CAPACITY);
        break;
      }
    }
  }
}

// Class index per occupied slot (in slot order) and the class count.
__global__ void __launch_bounds__(1024) k_tc_class_ids(const unsigned long long *__restrict__ hkeys, int *hid, unsigned long long *cls_of, int *count)
{
  constexpr int PER = TC_HASH / 1024;
  __shared__ int wsum[32];
  int            c = 0;
  for (int i = 0; i < PER; i++)
    c += hkeys[threadIdx.x * PER + i] != TC_EMPTY;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int       incl = c;
  for (int d = 1; d < 32; d <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d)
      incl += v;
  }
  if (lane == 31)
    wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    const int v = wsum[lane];
    int       iv = v;
    for (int d = 1; d < 32; d <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, iv, d);
      if (lane >= d)
        iv += u;
    }
    wsum[lane] = iv - v;
    if (lane == 31)
      *count = iv;
  }
  __syncthreads();
  int id = wsum[w] + incl - c;
  for (int i = 0; i < PER; i++) {
    const int                slot = threadIdx.x * PER + i;
    const unsigned long long k    = hkeys[slot];
    hid[slot]                     = k != TC_EMPTY ? id : -1;
    if (k != TC_EMPTY)
      cls_of[id++] = k;
  }
}

// Operators of classes 0 .. min(count, cap) - 1: one block of 128 threads (rows) per class.
template <int P>
__global__ void __launch_bounds__(128) k_tc_class_ops(const unsigned long long *__restrict__ cls_of, const int *__restrict__ count, int cap, float4 *table)
{
  using G = TcM2L<P>;
  constexpr int KP = G::KP, NCH = KP / 8;
  __shared__ cx<float> Ys[P * P];
  const int n = min(*count, cap);
  int       rj, rk, rpart;
  bool      rlive;
  tc_row_of(tc_lane_row(threadIdx.x), G::NR, rj, rk, rpart, rlive); // table row = TMEM lane
  for (int id = blockIdx.x; id < n; id += gridDim.x) {
    const float4 o = tc_class_offset(cls_of[id]);
    __syncthreads();
    tc_harmonics<P>(o, Ys);
    __syncthreads();
    const int dl = __float_as_int(o.w);
    for (int c8 = 0; c8 < NCH; c8++) {
      float h[8], l[8];
      for (int i = 0; i < 8; i++) {
        const float v = tc_op_value<P>(8 * c8 + i, rj, rk, rpart, rlive, dl, Ys), vh = tc::tf32_rn(v);
        h[i]          = vh;
        l[i]          = tc::tf32_rn(v - vh);
      }
      float4 *th = table + ((((size_t)id * 2 + 0) * NCH + c8) * 128 + threadIdx.x) * 2;
      float4 *tl = table + ((((size_t)id * 2 + 1) * NCH + c8) * 128 + threadIdx.x) * 2;
      th[0]      = make_float4(h[0], h[1], h[2], h[3]);
      th[1]      = make_float4(h[4], h[5], h[6], h[7]);
      tl[0]      = make_float4(l[0], l[1], l[2], l[3]);
      tl[1]      = make_float4(l[4], l[5], l[6], l[7]);
    }
  }
}

// Table index of each (tile, class) group, at its first pair: -1 for a
// sentinel pair or a class beyond the table (the kernel builds those).
__global__ void k_tc_class_index(const unsigned long long *__restrict__ keys, int n, const unsigned long long *__restrict__ hkeys,
                                 const int *__restrict__ hid, const int *__restrict__ count, int cap, int *cidq)
{
  const int ncls = min(*count, cap);
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const unsigned long long c = keys[q] & TC_SENTINEL;
    if (q > 0 && keys[q - 1] == keys[q] && c != TC_SENTINEL)
      continue;
    int id = -1;
    if (c != TC_SENTINEL)
      for (unsigned h = tc_hash(c), probes = 0; probes < TC_HASH; h = (h + 1) & (TC_HASH - 1), probes++) {
        const unsigned long long k = hkeys[h];
        if (k == c) {
          id = hid[h];
          break;
        }
        if (k == TC_EMPTY)
          break;
      }
    cidq[q] = id < ncls ? id : -1;
  }
}

// Per-class metadata ring of the M2L kernel (three slots: the class whose
// MMAs run, the next one being staged, the one after being decoded).
struct TcMeta {
  float4 off;   // offset o (target units), w = delta (int bits)
  int    cid;   // table index, -1: build here
  int    tile;  // -1: no more classes
  int    last;  // 1: last class of its tile
  int    level; // target level
  int    src[32];
};

// One block (384 threads, one per SM: 512 TMEM columns) walks the classes of
// its tiles in order: tile blockIdx.x first, then the next unclaimed tile
// (an atomic counter), so that blocks finish together.  Warp w writes and reads TMEM lanes 32 (w % 4) .. + 31
// (rows of A and D); warps w, w + 4, w + 8 split each row's A chunks and D
// columns.  Iteration c:
//   1. B(c) and A(c) complete -> barrier -> one thread of warp 3 issues the MMAs of
//      class c into a fresh D (small products first: A_lo B_hi and A_hi B_lo,
//      then A_hi B_hi, each from the highest degrees down), commit;
//   2. warp 2 decodes class c + 2 into the metadata ring;
//   3. all threads stage class c + 1 while the tensor core works: B by
//      cp.async into the other shared-memory stage, the nonzero chunks of
//      their operator rows from the table (L2) into the other TMEM A buffer
//      (classes without a table entry build their operator here);
//   4. the issuing thread waits for class c's MMAs; all threads add D into registers;
//      at the last class of a tile they write its local expansions (FP64).
// A fresh D per class keeps the tensor core's truncating FP32 accumulation
// to a few units in the last place of each class's sum; the classes are
// summed in FP32 in two levels (groups of 8, then the groups).
// 384 threads at 136 registers (52,224 of the SM's 65,536; no spills) and
// 161 KB of shared memory leave room on every SM for one block of the leaf
// kernel's near pass (128 threads x 96 registers, 39 KB), which runs on a
// second stream beside this kernel: at 168 registers the kernel alone is 8%
// faster, but the near field it hides is worth more.
template <int P>
__global__ void __maxnreg__(136) k_m2l_tc(TcArgs a)
{
  using G = TcM2L<P>;
  constexpr int K = nterms(P), KP = G::KP, N = G::N, NCH = KP / 8;
  constexpr int DT = N / 3; // D columns per third
  static_assert(DT % 16 == 0, "each thread drains its D columns 16 at a time");
  extern __shared__ unsigned char tc_smem_raw[];
  unsigned char *sB = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ cx<float> Ys[P * P];
  __shared__ TcMeta    meta[3];
  __shared__ uint32_t  tbase;
  __shared__ __align__(8) uint64_t mbar[2];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int quarter = warp & 3, third = warp >> 2;
  // Roles.  Thread ISSUER (warp 3, whose TMEM quarter holds the lightest
  // operator rows) issues the MMAs, which blocks it for about their duration;
  // its quarter's operator chunks go to warps 7 and 11.  Warp 2 decodes.
  constexpr int ISSUER = 96, DECODER = 2;
  int           c_lo = (NCH * third) / 3, c_hi = (NCH * (third + 1)) / 3; // A chunks of this warp
  if (quarter == 3) {
    c_lo = third == 0 ? 0 : (third == 1 ? 0 : NCH / 2);
    c_hi = third == 0 ? 0 : (third == 1 ? NCH / 2 : NCH);
  }

  if (warp == 0) {
    tc::tmem_alloc(&tbase, 512);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&mbar[0], 1);
    tc::mbar_init(&mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tb = tbase;

  // this thread's output row (TMEM lane) and its nonzero operator chunks
  const int lane_id = 32 * quarter + lane, row = tc_lane_row(lane_id);
  int       rj, rk, rpart;
  bool      rlive;
  tc_row_of(row, G::NR, rj, rk, rpart, rlive);
  const int      nz        = rlive ? ((P - rj) * (P - rj) + 7) / 8 : 0;
  const int      nzw       = __reduce_max_sync(0xffffffffu, nz); // the warp's largest
  const uint32_t lane_base = tc::tmem_addr(tb, 32 * quarter, 0);
  { // zero both A buffers once: chunks beyond a row's nonzero ones stay zero (every chunk of every lane: the warps of a quarter cover [0, NCH))
    const uint32_t z[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int b = 0; b < 2; b++)
      for (int c8 = c_lo; c8 < c_hi; c8++) {
        tc::tmem_st8(lane_base + G::ACOL + b * G::ABUF + 8 * c8, z);
        tc::tmem_st8(lane_base + G::ACOL + b * G::ABUF + KP + 8 * c8, z);
      }
    tc::tmem_st_wait();
  }
  // this thread's B gather: column n (target n / 3, component n % 3) of the
  // hi (which = 0) or lo (1) operand, K chunk pairs [cp_lo, cp_hi)
  constexpr int KC2 = G::KC / 2;
  const int     gcol = tid % N, gwhich = (tid / N) & 1, ghalf = tid / (2 * N); // 384 = 96 x 2 x 2
  const int     cp_lo = ghalf ? KC2 / 2 : 0, cp_hi = ghalf ? KC2 : KC2 / 2;
  const int     gdoff = gwhich * G::BBYTES + (gcol >> 3) * G::SBO + (gcol & 7) * 16;
  const float  *gbase = (gwhich ? a.Blo : a.Bhi) + (gcol % 3) * KP;

  // the decoder warp's walker over this block's tiles and classes
  const int ntiles = *a.ntiles;
  int       wT = blockIdx.x, we = 0, wp1 = 0;
  if (warp == DECODER && wT < ntiles) {
    we  = a.tile_start[wT];
    wp1 = a.tile_start[wT + 1];
  }
  auto decode = [&](TcMeta &M) { // decoder warp: the class at the walker into M
    while (wT < ntiles && we >= wp1) { // next tile: the first gridDim.x by block index, then whoever is free
      int next = 0;
      if (lane == 0)
        next = (int)gridDim.x + atomicAdd(a.tile_next, 1);
      wT = __shfl_sync(0xffffffffu, next, 0);
      if (wT < ntiles) {
        we  = a.tile_start[wT];
        wp1 = a.tile_start[wT + 1];
      }
    }
    if (wT >= ntiles) {
      if (lane == 0)
        M.tile = -1;
      return;
    }
    const unsigned long long k0  = a.keys[we];
    const bool               in  = we + lane < wp1;
    const unsigned long long kl  = in ? a.keys[we + lane] : ~0ull;
    const uint32_t           v   = in ? a.vals[we + lane] : 0u;
    const bool               sen = (k0 & TC_SENTINEL) == TC_SENTINEL;
    const unsigned           eq  = __ballot_sync(0xffffffffu, in && kl == k0);
    const int                cnt = sen ? 1 : __popc(eq); // members are contiguous from lane 0
    M.src[lane]                  = -1;
    __syncwarp();
    if (lane < cnt)
      M.src[v >> TC_COL_SHIFT] = (int)(v & ((1u << TC_COL_SHIFT) - 1));
    if (lane == 0) {
      const int lt = a.tile_level[wT];
      float4    o;
      if (!sen)
        o = tc_class_offset(k0);
      else {
        const int    sc = (int)(v & ((1u << TC_COL_SHIFT) - 1)), t = a.tile_cells[wT * 32 + (v >> TC_COL_SHIFT)];
        const double iR = 1.0 / a.cv.R[t];
        o = make_float4((float)((a.cv.x[t] - a.cv.x[sc]) * iR), (float)((a.cv.y[t] - a.cv.y[sc]) * iR), (float)((a.cv.z[t] - a.cv.z[sc]) * iR),
                        __int_as_float(lt - a.cv.level[sc]));
      }
      M.off   = o;
      M.cid   = a.cidq[we];
      M.tile  = wT;
      M.last  = we + cnt >= wp1;
      M.level = lt;
    }
    we += cnt;
  };

  // stage class M into shared-memory stage / TMEM buffer b (all threads)
  // B of class M into shared-memory stage b (cp.async; all threads)
  auto gather_b = [&](const TcMeta &M, int b) {
    unsigned char *dst = sB + b * G::STAGE + gdoff;
    const int      src = M.src[gcol / 3];
    if (src >= 0) {
      const float *g = gbase + (size_t)src * 3 * KP;
#pragma unroll 4
      for (int cp2 = cp_lo; cp2 < cp_hi; cp2++) {
        cp_async16(dst + (2 * cp2) * G::LBO, g + 8 * cp2);
        cp_async16(dst + (2 * cp2 + 1) * G::LBO, g + 8 * cp2 + 4);
      }
    } else {
      for (int cp2 = cp_lo; cp2 < cp_hi; cp2++) {
        *reinterpret_cast<float4 *>(dst + (2 * cp2) * G::LBO)     = make_float4(0.f, 0.f, 0.f, 0.f);
        *reinterpret_cast<float4 *>(dst + (2 * cp2 + 1) * G::LBO) = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
  };
  // the operator of class M into TMEM buffer b (all threads: a class without
  // a table entry synchronises the block)
  auto stage_a = [&](const TcMeta &M, int b) {
    const uint32_t ahi = lane_base + G::ACOL + b * G::ABUF, alo = ahi + KP;
    const int      cid = M.cid;
    if (cid >= 0) {
      const float4 *th = a.table + ((size_t)cid * 2 * NCH) * 128 * 2;
      const float4 *tl = th + (size_t)NCH * 128 * 2;
      for (int c8 = c_lo; c8 < min(c_hi, nzw); c8++) {
        float4 h0 = make_float4(0.f, 0.f, 0.f, 0.f), h1 = h0, l0 = h0, l1 = h0;
        if (c8 < nz) {
          const size_t o8 = ((size_t)c8 * 128 + lane_id) * 2;
          h0              = __ldg(th + o8);
          h1              = __ldg(th + o8 + 1);
          l0              = __ldg(tl + o8);
          l1              = __ldg(tl + o8 + 1);
        }
        const uint32_t hv[8] = {__float_as_uint(h0.x), __float_as_uint(h0.y), __float_as_uint(h0.z), __float_as_uint(h0.w),
                                __float_as_uint(h1.x), __float_as_uint(h1.y), __float_as_uint(h1.z), __float_as_uint(h1.w)};
        const uint32_t lv[8] = {__float_as_uint(l0.x), __float_as_uint(l0.y), __float_as_uint(l0.z), __float_as_uint(l0.w),
                                __float_as_uint(l1.x), __float_as_uint(l1.y), __float_as_uint(l1.z), __float_as_uint(l1.w)};
        tc::tmem_st8(ahi + 8 * c8, hv);
        tc::tmem_st8(alo + 8 * c8, lv);
      }
    } else { // block-uniform: a class without a table entry builds its operator here
      __syncthreads(); // Ys free
      tc_harmonics<P>(M.off, Ys);
      __syncthreads();
      const int dl = __float_as_int(M.off.w);
      for (int c8 = c_lo; c8 < c_hi; c8++) {
        uint32_t hv[8], lv[8];
#pragma unroll
        for (int i = 0; i < 8; i++) {
          const float v = tc_op_value<P>(8 * c8 + i, rj, rk, rpart, rlive, dl, Ys), vh = tc::tf32_rn(v);
          hv[i]         = __float_as_uint(vh);
          lv[i]         = __float_as_uint(tc::tf32_rn(v - vh));
        }
        tc::tmem_st8(ahi + 8 * c8, hv);
        tc::tmem_st8(alo + 8 * c8, lv);
      }
    }
  };

  float acc[DT], tot[DT]; // sum of the current group of 8 classes, sum of the groups
#pragma unroll
  for (int i = 0; i < DT; i++)
    acc[i] = tot[i] = 0.f;
  int ingroup = 0;

  // prologue: decode classes 0 and 1, stage class 0
  if (warp == DECODER) {
    decode(meta[0]);
    decode(meta[1]);
  }
  __syncthreads();
  if (meta[0].tile >= 0) {
    gather_b(meta[0], 0);
    stage_a(meta[0], 0);
  }
  bool failed = false;
  for (unsigned c = 0; !failed; c++) {
    const TcMeta &M = meta[c % 3];
    if (M.tile < 0)
      break; // block-uniform (read after a barrier)
    const int s = c & 1;
    // 1. operands of class c complete and visible to the tensor core; D drained
    cp_async_wait_all();
    tc::fence_proxy_async_smem();
    tc::tmem_st_wait();
    tc::fence_before_sync();
    __syncthreads();
    const TcMeta &Mn = meta[(c + 1) % 3];
    if (warp == ISSUER / 32 && Mn.tile >= 0) // before its blocking issue: stage s ^ 1 is free (class c - 1 completed)
      gather_b(Mn, s ^ 1);
    if (tid == ISSUER) {
      tc::fence_after_sync();
      const uint32_t     D = tc::tmem_addr(tb, 0, G::DCOL), Ahi = tc::tmem_addr(tb, 0, G::ACOL + s * G::ABUF), Alo = Ahi + KP;
      const uint64_t     dhi = tc::smem_desc_noswizzle(tc::smem_u32(sB + s * G::STAGE), G::LBO, G::SBO);
      const uint64_t     dlo = tc::smem_desc_noswizzle(tc::smem_u32(sB + s * G::STAGE + G::BBYTES), G::LBO, G::SBO);
      constexpr uint64_t dk  = (uint64_t)(2 * G::LBO) >> 4; // descriptor start-address step per K step of 8
      constexpr uint32_t idesc = tc::idesc_tf32(128, N), idesc64 = tc::idesc_tf32(64, N);
      constexpr int      KS128 = 2; // K steps that need all 128 rows
      static_assert((P - 7) * (P - 7) <= 8 * KS128, "rows 64.. (j >= 7) vanish beyond the M = 128 K steps");
      // K steps 0 and 1 at M = 128 (all rows), the others at M = 64 (the rows
      // of the lanes 0-15 of each quarter: the other rows are zero there).
      // The first MMA (M = 128) starts D afresh on every lane; the small
      // products come first, A_hi B_hi from the highest degrees down.
#pragma unroll 1
      for (int kk = KS128 - 1; kk >= 0; kk--) {
        tc::mma_tf32_ts(D, Alo + 8 * kk, dhi + dk * kk, idesc, kk == KS128 - 1 ? 0u : 1u);
        tc::mma_tf32_ts(D, Ahi + 8 * kk, dlo + dk * kk, idesc, 1u);
      }
#pragma unroll 1
      for (int kk = NCH - 1; kk >= KS128; kk--) {
        tc::mma_tf32_ts(D, Alo + 8 * kk, dhi + dk * kk, idesc64, 1u);
        tc::mma_tf32_ts(D, Ahi + 8 * kk, dlo + dk * kk, idesc64, 1u);
      }
#pragma unroll 1
      for (int kk = NCH - 1; kk >= KS128; kk--)
        tc::mma_tf32_ts(D, Ahi + 8 * kk, dhi + dk * kk, idesc64, 1u);
#pragma unroll 1
      for (int kk = KS128 - 1; kk >= 0; kk--)
        tc::mma_tf32_ts(D, Ahi + 8 * kk, dhi + dk * kk, idesc, 1u);
      tc::mma_commit(&mbar[s]);
    }
    // 2. decode class c + 2 (its slot held class c - 1, finished last iteration)
    if (warp == DECODER)
      decode(meta[(c + 2) % 3]);
    // 3. stage class c + 1 into the other stage and A buffer (their last
    // reader, class c - 1, completed before class c was issued)
    if (Mn.tile >= 0) {
      if (warp != ISSUER / 32)
        gather_b(Mn, s ^ 1);
      stage_a(Mn, s ^ 1);
    }
    // 4. class c's D into the accumulators; a tile's last class writes its L
    const bool ok = tid != ISSUER || tc::mbar_wait_bounded(&mbar[s], (c >> 1) & 1);
    if (__syncthreads_or(!ok)) { // block-uniform: every thread leaves together
      if (tid == ISSUER)
        atomicExch(a.err, VFMM_ERR_TIMEOUT);
      failed = true;
      break;
    }
    tc::fence_after_sync();
#pragma unroll
    for (int h = 0; h < DT; h += 16) {
      uint32_t v0[8], v1[8];
      tc::tmem_ld8(lane_base + G::DCOL + DT * third + h, v0);
      tc::tmem_ld8(lane_base + G::DCOL + DT * third + h + 8, v1);
      tc::tmem_ld_wait();
#pragma unroll
      for (int i = 0; i < 8; i++) {
        acc[h + i] += __uint_as_float(v0[i]);
        acc[h + 8 + i] += __uint_as_float(v1[i]);
      }
    }
    if (++ingroup == 8 || M.last) {
#pragma unroll
      for (int i = 0; i < DT; i++) {
        tot[i] += acc[i];
        acc[i] = 0.f;
      }
      ingroup = 0;
    }
    if (M.last) {
      if (rlive) {
        const int    jks = row >> 1, lt = M.level, T = M.tile;
        const double scale = ((rj & 1) ? -1.0 : 1.0) * ldexp(a.iR0pow[rj + 1], lt * (rj + 1));
#pragma unroll
        for (int i = 0; i < DT; i++) {
          const int col = DT * third + i, t = col / 3, d = col - 3 * t, cell = a.tile_cells[T * 32 + t];
          if (cell >= 0)
            reinterpret_cast<double *>(a.L)[2 * ((size_t)cell * 3 * K + 3 * jks + d) + rpart] = (double)tot[i] * scale;
        }
      }
#pragma unroll
      for (int i = 0; i < DT; i++)
        tot[i] = 0.f;
    }
  }
  cp_async_wait_all(); // no copy of this block stays in flight
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tb, 512);
  }
}

// ---------------------------------------------------------------- tiles and classes
// Sort key of a target cell: level, octant within its parent, index; cells
// without M2L sources sort last.
__global__ void k_tc_target_keys(CellsView cv, const int *__restrict__ m2l_start, int ncells, unsigned long long *keys)
{
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += gridDim.x * blockDim.x) {
    unsigned long long k = ~0ull;
    if (m2l_start[c + 1] > m2l_start[c]) {
      const int p   = cv.parent[c];
      unsigned  oct = 0;
      if (p >= 0)
        oct = (cv.x[c] > cv.x[p] ? 1u : 0u) | (cv.y[c] > cv.y[p] ? 2u : 0u) | (cv.z[c] > cv.z[p] ? 4u : 0u);
      k = ((unsigned long long)cv.level[c] << 40) | ((unsigned long long)oct << 32) | (unsigned)c;
    }
    keys[c] = k;
  }
}

// meta: [0, L) first sorted index of each level (-1: none), [L, 2L) one past
// its last, [2L, 3L) its first tile, [3L] the tile count (L = MAXL + 1).
constexpr int TC_L = MAXL + 1;

__global__ void k_tc_level_bounds(const unsigned long long *__restrict__ sk, int n, int *meta)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned long long k = sk[i];
    if (k == ~0ull)
      continue;
    const int l = (int)(k >> 40);
    if (i == 0 || (int)(sk[i - 1] >> 40) != l)
      meta[l] = i;
    if (i == n - 1 || sk[i + 1] == ~0ull || (int)(sk[i + 1] >> 40) != l)
      meta[TC_L + l] = i + 1;
  }
}

__global__ void k_tc_tile_bases(int *meta)
{
  if (threadIdx.x != 0 || blockIdx.x != 0)
    return;
  int base = 0;
  for (int l = 0; l < TC_L; l++) {
    meta[2 * TC_L + l] = base;
    if (meta[l] >= 0)
      base += (meta[TC_L + l] - meta[l] + 31) / 32;
  }
  meta[3 * TC_L] = base;
}

__global__ void k_tc_assign(const unsigned long long *__restrict__ sk, int n, const int *__restrict__ meta, int *tile_cells, int *tile_level,
                            int *tile_of, int *col_of)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned long long k = sk[i];
    if (k == ~0ull)
      continue;
    const int l = (int)(k >> 40), c = (int)(k & 0xffffffffu);
    const int pos = i - meta[l], T = meta[2 * TC_L + l] + pos / 32, col = pos % 32;
    tile_cells[T * 32 + col] = c;
    tile_of[c]               = T;
    col_of[c]                = col;
    if (col == 0)
      tile_level[T] = l;
  }
}

// Lattice coordinates of each cell: (x - x0) / R, an odd integer (2 i + 1 for
// the cell's index i along each axis at its level), with x0 the root cell's
// lower corner; w = level.  The centres come from the reference's FP64 chain,
// so the quotient is an odd integer to within far less than 1/2.
__global__ void k_tc_cell_coords(CellsView cv, int nc, int4 *cc)
{
  const double x0 = cv.x[0] - cv.R[0], y0 = cv.y[0] - cv.R[0], z0 = cv.z[0] - cv.R[0];
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    const double iR = 1.0 / cv.R[c];
    cc[c]           = make_int4((int)llrint((cv.x[c] - x0) * iR), (int)llrint((cv.y[c] - y0) * iR), (int)llrint((cv.z[c] - z0) * iR), cv.level[c]);
  }
}

// Pair (t, s) -> key tile(t) << 38 | class, value column(t) << 27 | s; the
// class offset (x_t - x_s) / R_f in units of the finer cell's half-width R_f,
// from the lattice coordinates in integer arithmetic.
__global__ void k_tc_pair_keys(const unsigned long long *__restrict__ pk, int n, int kb, const int4 *__restrict__ cc, const int *__restrict__ tile_of,
                               const int *__restrict__ col_of, unsigned long long *keys, uint32_t *vals)
{
  const unsigned long long smask = (1ull << kb) - 1;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int          t = (int)(pk[q] >> kb), s = (int)(pk[q] & smask);
    const int4         ct = cc[t], cs = cc[s];
    const int          dl = ct.w - cs.w, lf = max(ct.w, cs.w), st = lf - ct.w, ss = lf - cs.w;
    const long long    ox = ((long long)ct.x << st) - ((long long)cs.x << ss), oy = ((long long)ct.y << st) - ((long long)cs.y << ss),
                    oz = ((long long)ct.z << st) - ((long long)cs.z << ss);
    unsigned long long cls = TC_SENTINEL;
    if (dl >= -14 && dl <= 14 && llabs(ox) <= 1022 && llabs(oy) <= 1022 && llabs(oz) <= 1022)
      cls = ((unsigned long long)(dl + 16) << 33) | ((unsigned long long)(ox + 1024) << 22) | ((unsigned long long)(oy + 1024) << 11) |
            (unsigned long long)(oz + 1024);
    keys[q] = ((unsigned long long)tile_of[t] << TC_CLASS_BITS) | cls;
    vals[q] = ((uint32_t)col_of[t] << TC_COL_SHIFT) | (uint32_t)s;
  }
}

// First sorted pair of each tile; tile_start[ntiles] = n.
__global__ void k_tc_tile_ranges(const unsigned long long *__restrict__ keys, int n, const int *__restrict__ meta, int *tile_start)
{
  const int nt = meta[3 * TC_L];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x) {
    const int T  = i < n ? (int)(keys[i] >> TC_CLASS_BITS) : nt;
    const int Tp = i > 0 ? (int)(keys[i - 1] >> TC_CLASS_BITS) : -1;
    for (int r = Tp + 1; r <= T; r++)
      tile_start[r] = i;
  }
}

// The pre-pass of one evaluation (tiles, pair keys, class table), which needs
// only the tree and the lists; it leaves what the kernel launch needs in S.
template <int P>
static void m2l_tc_prepare_P(cudaStream_t s, const ExpArgs &e, const MixedArgs &m)
{
  using G     = TcM2L<P>;
  TcScratch &S = *m.tc;
  const int  nc = e.ncells, np = m.n_m2l;
  VFMM_CUDA_TRY(cudaMemsetAsync(e.L, 0, sizeof(double2) * (size_t)nc * 3 * nterms(P), s));
  S.launch_tiles = 0;
  if (np == 0 || nc == 0)
    return;
  if (nc >= (1 << TC_COL_SHIFT))
    throw Error(VFMM_ERR_CAPACITY, "tensor-core M2L: more than 2^27 cells");
  const int ntmax = nc / 32 + TC_L + 1; // tiles: per level ceil(count / 32)
  int       tile_bits = 1;
  while ((1ll << tile_bits) <= ntmax)
    tile_bits++;
  if (TC_CLASS_BITS + tile_bits > 64)
    throw Error(VFMM_ERR_CAPACITY, "tensor-core M2L: too many tiles for a 64-bit pair key");
  S.tkeys.reserve(nc);
  S.tkeys_sorted.reserve(nc);
  S.tile_of.reserve(nc);
  S.coords.reserve(nc);
  S.col_of.reserve(nc);
  S.meta.reserve(3 * TC_L + 3);
  S.tile_cells.reserve((size_t)ntmax * 32);
  S.tile_level.reserve(ntmax);
  S.tile_start.reserve(ntmax + 1);
  S.pkeys.reserve(np);
  S.pkeys_sorted.reserve(np);
  S.pvals.reserve(np);
  S.pvals_sorted.reserve(np);
  size_t b1 = 0, b2 = 0;
  VFMM_CUDA_TRY(cub::DeviceRadixSort::SortKeys(nullptr, b1, S.tkeys.p, S.tkeys_sorted.p, nc, 0, 45, s));
  VFMM_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, b2, S.pkeys.p, S.pkeys_sorted.p, S.pvals.p, S.pvals_sorted.p, np, 0,
                                                TC_CLASS_BITS + tile_bits, s));
  S.cub_tmp.reserve(std::max(b1, b2));

  VFMM_CUDA_TRY(cudaMemsetAsync(S.meta.p, 0xFF, sizeof(int) * (3 * TC_L + 2), s));
  VFMM_CUDA_TRY(cudaMemsetAsync(S.meta.p + 3 * TC_L + 2, 0, sizeof(int), s)); // the tile counter
  VFMM_CUDA_TRY(cudaMemsetAsync(S.tile_cells.p, 0xFF, sizeof(int) * (size_t)ntmax * 32, s));
  k_tc_target_keys<<<grid_for(nc, 256), 256, 0, s>>>(e.cells, e.m2l_start, nc, S.tkeys.p);
  count_launch();
  size_t bytes = S.cub_tmp.cap;
  VFMM_CUDA_TRY(cub::DeviceRadixSort::SortKeys(S.cub_tmp.p, bytes, S.tkeys.p, S.tkeys_sorted.p, nc, 0, 45, s));
  count_launch();
  k_tc_level_bounds<<<grid_for(nc, 256), 256, 0, s>>>(S.tkeys_sorted.p, nc, S.meta.p);
  count_launch();
  k_tc_tile_bases<<<1, 32, 0, s>>>(S.meta.p);
  count_launch();
  k_tc_assign<<<grid_for(nc, 256), 256, 0, s>>>(S.tkeys_sorted.p, nc, S.meta.p, S.tile_cells.p, S.tile_level.p, S.tile_of.p, S.col_of.p);
  count_launch();
  k_tc_cell_coords<<<grid_for(nc, 256), 256, 0, s>>>(e.cells, nc, S.coords.p);
  count_launch();
  k_tc_pair_keys<<<grid_for(np, 256), 256, 0, s>>>(m.m2l_keys, np, m.m2l_key_bits, S.coords.p, S.tile_of.p, S.col_of.p, S.pkeys.p, S.pvals.p);
  count_launch();
  bytes = S.cub_tmp.cap;
  VFMM_CUDA_TRY(cub::DeviceRadixSort::SortPairs(S.cub_tmp.p, bytes, S.pkeys.p, S.pkeys_sorted.p, S.pvals.p, S.pvals_sorted.p, np, 0,
                                                TC_CLASS_BITS + tile_bits, s));
  count_launch();
  k_tc_tile_ranges<<<grid_for(np + 1, 256), 256, 0, s>>>(S.pkeys_sorted.p, np, S.meta.p, S.tile_start.p);
  count_launch();

  // operator classes and their table
  int dev = 0, nsm = 0;
  VFMM_CUDA_TRY(cudaGetDevice(&dev));
  VFMM_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  S.hkeys.reserve(TC_HASH);
  S.hid.reserve(TC_HASH);
  S.cls_of.reserve(TC_HASH);
  S.cidq.reserve(np);
  if (!S.ncls_host) {
    VFMM_CUDA_TRY(cudaMallocHost((void **)&S.ncls_host, sizeof(int)));
    *S.ncls_host = 0;
  }
  // table capacity: the last evaluation's class count (its copy completed at
  // the tree build's host synchronisation) with headroom; classes beyond it
  // are built inside the M2L kernel
  const int want = *S.ncls_host + *S.ncls_host / 4 + 64;
  S.cap          = std::min(TC_HASH, std::max(std::max(S.cap, 512), want));
  constexpr int NCH = G::KP / 8;
  S.table.reserve((size_t)S.cap * 2 * NCH * 128 * 2);
  int *count = S.meta.p + 3 * TC_L + 1;
  VFMM_CUDA_TRY(cudaMemsetAsync(S.hkeys.p, 0xFF, sizeof(unsigned long long) * TC_HASH, s));
  k_tc_class_insert<<<grid_for(np, 256), 256, 0, s>>>(S.pkeys_sorted.p, np, S.hkeys.p, m.eval_err);
  count_launch();
  k_tc_class_ids<<<1, 1024, 0, s>>>(S.hkeys.p, S.hid.p, S.cls_of.p, count);
  count_launch();
  k_tc_class_ops<P><<<std::min(S.cap, 2 * nsm), 128, 0, s>>>(S.cls_of.p, count, S.cap, S.table.p);
  count_launch();
  k_tc_class_index<<<grid_for(np, 256), 256, 0, s>>>(S.pkeys_sorted.p, np, S.hkeys.p, S.hid.p, count, S.cap, S.cidq.p);
  count_launch();
  VFMM_CUDA_TRY(cudaMemcpyAsync(S.ncls_host, count, sizeof(int), cudaMemcpyDeviceToHost, s));
  S.launch_tiles = ntmax;
}

// The kernel of one evaluation, after its pre-pass (m2l_tc_prepare_P) and the
// upward pass that wrote the operand rows.
template <int P>
static void m2l_tc_run_P(cudaStream_t s, const ExpArgs &e, const MixedArgs &m)
{
  using G      = TcM2L<P>;
  TcScratch &S = *m.tc;
  const int  np = m.n_m2l, ntmax = S.launch_tiles;
  if (ntmax == 0)
    return;
  int nsm = 0, dev = 0;
  VFMM_CUDA_TRY(cudaGetDevice(&dev));
  VFMM_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  TcArgs a{};
  a.keys       = S.pkeys_sorted.p;
  a.vals       = S.pvals_sorted.p;
  a.npairs     = np;
  a.tile_start = S.tile_start.p;
  a.tile_cells = S.tile_cells.p;
  a.tile_level = S.tile_level.p;
  a.ntiles     = S.meta.p + 3 * TC_L;
  a.tile_next  = S.meta.p + 3 * TC_L + 2;
  a.Bhi        = m.Bhi;
  a.Blo        = m.Blo;
  a.table      = S.table.p;
  a.cidq       = S.cidq.p;
  a.cv         = e.cells;
  a.L          = e.L;
  a.err        = m.eval_err;
  const double iR0 = 1.0 / m.R0;
  a.iR0pow[0]      = 1.0;
  for (int k = 1; k < PMAX + 2; k++)
    a.iR0pow[k] = a.iR0pow[k - 1] * iR0;
  VFMM_SMEM_ONCE(G::smem, k_m2l_tc<P>);
  VFMM_CARVEOUT_MAX_ONCE(k_m2l_tc<P>);
  k_m2l_tc<P><<<std::max(1, std::min(nsm, ntmax)), 384, G::smem, s>>>(a);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

void m2l_tensor_prepare(cudaStream_t s, const ExpArgs &e, const MixedArgs &m)
{
  switch (e.P) {
  case 8: m2l_tc_prepare_P<8>(s, e, m); break;
  case 9: m2l_tc_prepare_P<9>(s, e, m); break;
  case 10: m2l_tc_prepare_P<10>(s, e, m); break;
  default: throw Error(VFMM_ERR_UNSUPPORTED, "tensor-core M2L: order outside 8..10");
  }
}

void m2l_tensor_run(cudaStream_t s, const ExpArgs &e, const MixedArgs &m)
{
  switch (e.P) {
  case 8: m2l_tc_run_P<8>(s, e, m); break;
  case 9: m2l_tc_run_P<9>(s, e, m); break;
  case 10: m2l_tc_run_P<10>(s, e, m); break;
  default: throw Error(VFMM_ERR_UNSUPPORTED, "tensor-core M2L: order outside 8..10");
  }
}

void m2l_tensor(cudaStream_t s, const ExpArgs &e, const MixedArgs &m)
{
  m2l_tensor_prepare(s, e, m);
  m2l_tensor_run(s, e, m);
}

} // namespace vfmm

extern "C" int vfmm_tcgen05_selftest(int device, int mode, float *out)
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
    k_tc_selftest<<<1, 128>>>(d, mode, err);
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

