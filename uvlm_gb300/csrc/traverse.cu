// Dual-tree traversal on the device: the same P2P and M2L pair sets as the
// reference's explicit-stack traversal (src/traverse.hpp:32-85).
//
// The split decision and the MAC depend only on the pair (T, S), so a
// level-synchronous frontier expansion visits exactly the pairs the stack
// traversal visits.  Each step expands every frontier pair: split T when S is
// a leaf or (R_T >= R_S and T is not a leaf), else split S (traverse.hpp:74-
// 82); each child pair is near when |dX|^2 theta^2 < (Ri + Rj)^2, evaluated
// with the reference's operation order and no contraction (traverse.hpp:
// 52-57); near leaf pairs go to P2P, near others to the next frontier, far
// pairs to M2L.  Pairs are then sorted by (target, source) into CSR rows.
#include <algorithm>
#include <cub/cub.cuh>
#include "vfmm_internal.cuh"

namespace vfmm {

__device__ __forceinline__ bool mac_near(const CellsView &a, int i, const CellsView &b, int j, double theta)
{
  const double d0 = __dsub_rn(a.x[i], b.x[j]);
  const double d1 = __dsub_rn(a.y[i], b.y[j]);
  const double d2 = __dsub_rn(a.z[i], b.z[j]);
  const double nrm = __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2));
  const double R2  = __dmul_rn(__dmul_rn(nrm, theta), theta);
  const double s   = __dadd_rn(a.R[i], b.R[j]);
  return R2 < __dmul_rn(s, s);
}

// Warp-aggregated reservation in *ctr: every lane of the warp calls with its
// count c (possibly 0) and receives its start offset; one atomic per warp.
__device__ __forceinline__ int warp_reserve(int *ctr, int c)
{
  const int lane = threadIdx.x & 31;
  int       incl = c;
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o)
      incl += v;
  }
  const int tot  = __shfl_sync(0xffffffffu, incl, 31);
  int       base = 0;
  if (lane == 31 && tot)
    base = atomicAdd(ctr, tot);
  base = __shfl_sync(0xffffffffu, base, 31);
  return base + incl - c;
}

__global__ void k_traverse_init(CellsView tc, CellsView sc, int2 *front, DevInfo *info, unsigned long long *p2p)
{
  if (threadIdx.x || blockIdx.x)
    return;
  info->n_p2p = 0;
  info->n_m2l = 0;
  info->front_n[1] = 0;
  info->front_n[2] = 0;
  if (tc.nchild[0] == 0 && sc.nchild[0] == 0) {
    p2p[0]           = 0ull; // (0, 0)
    info->n_p2p      = 1;
    info->front_n[0] = 0;
  } else {
    front[0]         = make_int2(0, 0);
    info->front_n[0] = 1;
  }
}

// The frontier counters form a ring of three: this step reads n_in, counts
// into n_out (zero since the step before the previous one) and zeroes
// n_next, the next step's output, which no block of this step touches.
__global__ void k_traverse_step(CellsView tc, CellsView sc, const int2 *__restrict__ fin, int *n_in, int cap_in, int2 *fout, int *n_out,
                                int *n_next, int cap_front, unsigned long long *p2p, unsigned long long *m2l, int *np2p, int *nm2l, int cap_p2p,
                                int cap_m2l, double theta, int cell_bits, int *overflow)
{
  if (blockIdx.x == 0 && threadIdx.x == 0)
    *n_next = 0;
  // After an overflow the previous step's counter has run past its buffer and
  // some of its slots were left unwritten: the lists are redone with larger
  // buffers, so the remaining steps do nothing.  The clamp keeps every read of
  // fin inside its buffer regardless.
  if (*(volatile int *)overflow)
    return;
  const int n = min(*n_in, cap_in);
  // warp-uniform trip count (blockDim is a multiple of 32) for the aggregated reservations
  for (int q0 = blockIdx.x * blockDim.x; q0 < n; q0 += gridDim.x * blockDim.x) {
    const int  q     = q0 + threadIdx.x;
    const bool valid = q < n;
    const int2 pr    = valid ? fin[q] : make_int2(0, 0);
    const int  T = pr.x, S = pr.y;
    const bool splitT = sc.nchild[S] == 0 || (tc.R[T] >= sc.R[S] && tc.nchild[T] != 0);
    const int  c0 = splitT ? tc.child[T] : sc.child[S];
    const int  nc = valid ? (splitT ? tc.nchild[T] : sc.nchild[S]) : 0;
    unsigned   kind = 0; // 2 bits per child: 0 m2l, 1 p2p, 2 push
    int        cm = 0, cp = 0, cf = 0;
    for (int k = 0; k < nc; k++) {
      const int i = splitT ? c0 + k : T, j = splitT ? S : c0 + k;
      int       kd;
      if (mac_near(tc, i, sc, j, theta))
        kd = (tc.nchild[i] == 0 && sc.nchild[j] == 0) ? 1 : 2;
      else
        kd = 0;
      kind |= (unsigned)kd << (2 * k);
      cm += kd == 0;
      cp += kd == 1;
      cf += kd == 2;
    }
    int bm = warp_reserve(nm2l, cm);
    int bp = warp_reserve(np2p, cp);
    int bf = warp_reserve(n_out, cf);
    if (bm + cm > cap_m2l || bp + cp > cap_p2p || bf + cf > cap_front) {
      atomicExch(overflow, 1);
      continue;
    }
    for (int k = 0; k < nc; k++) {
      const int i = splitT ? c0 + k : T, j = splitT ? S : c0 + k;
      const int kd = (kind >> (2 * k)) & 3;
      const unsigned long long key = ((unsigned long long)i << cell_bits) | (unsigned long long)j;
      if (kd == 0)
        m2l[bm++] = key;
      else if (kd == 1)
        p2p[bp++] = key;
      else
        fout[bf++] = make_int2(i, j);
    }
  }
}

void traverse(cudaStream_t s, CellsView tc, CellsView sc, int ntc, int nsc, int maxLevelT, int maxLevelS, double theta, DevInfo *info,
              ListScratch &ls, size_t cap_front, size_t cap_p2p, size_t cap_m2l)
{
  ls.front[0].reserve(cap_front);
  ls.front[1].reserve(cap_front);
  ls.p2p_raw.reserve(cap_p2p);
  ls.m2l_raw.reserve(cap_m2l);
  // the kernel's counters and capacities are int
  const size_t int_max = 0x7fffffff;
  if (ls.front[0].cap > int_max || ls.front[1].cap > int_max || ls.p2p_raw.cap > int_max || ls.m2l_raw.cap > int_max)
    throw Error(VFMM_ERR_CAPACITY, "interaction lists exceed 2^31 pairs");
  // pair keys (target << key_bits | source): the sort then covers 2 * key_bits bits
  int cell_bits = 1;
  while ((1ll << cell_bits) < (long long)std::max(ntc, nsc))
    cell_bits++;
  ls.key_bits = cell_bits;
  k_traverse_init<<<1, 32, 0, s>>>(tc, sc, ls.front[0].p, info, ls.p2p_raw.p);
  count_launch();
  const int steps = maxLevelT + maxLevelS + 1;
  for (int it = 0; it < steps; it++) {
    const int a = it & 1, b = a ^ 1; // frontier buffers ping-pong; counters cycle through three
    k_traverse_step<<<152 * 8, 128, 0, s>>>(tc, sc, ls.front[a].p, &info->front_n[it % 3], (int)ls.front[a].cap, ls.front[b].p,
                                            &info->front_n[(it + 1) % 3], &info->front_n[(it + 2) % 3], (int)ls.front[b].cap,
                                            ls.p2p_raw.p, ls.m2l_raw.p, &info->n_p2p, &info->n_m2l, (int)ls.p2p_raw.cap, (int)ls.m2l_raw.cap, theta,
                                            cell_bits, &info->overflow);
    count_launch();
  }
  VFMM_LAUNCH_CHECK();
}

// CSR rows by target from sorted (target << kb | source) keys; also counts
// body-body P2P interactions (self pairs excluded), one atomic per warp.
__global__ void k_csr(const unsigned long long *__restrict__ keys, int n, int kb, int ncells, int *start, int *src, const int *nbody,
                      unsigned long long *interactions)
{
  const unsigned long long smask = (1ull << kb) - 1;
  unsigned long long       local = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x) {
    const int t  = i < n ? (int)(keys[i] >> kb) : ncells;
    const int tp = i > 0 ? (int)(keys[i - 1] >> kb) : -1;
    for (int r = tp + 1; r <= t; r++)
      start[r] = i;
    if (i < n) {
      const int sidx = (int)(keys[i] & smask);
      src[i]         = sidx;
      if (nbody) {
        const unsigned long long a = (unsigned long long)nbody[t], b = (unsigned long long)nbody[sidx];
        local += t == sidx ? a * a - a : a * b;
      }
    }
  }
  if (interactions) {
    for (int o = 16; o > 0; o >>= 1)
      local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local)
      atomicAdd(interactions, local);
  }
}

void lists_to_csr(cudaStream_t s, ListScratch &ls, int n_p2p, int n_m2l, int ncells_t, int cell_bits, int *p2p_start, int *p2p_src, int *m2l_start,
                  int *m2l_src, const int *nbody_t, unsigned long long *interactions)
{
  (void)cell_bits;
  ls.p2p_sorted.reserve(n_p2p + 1);
  ls.m2l_sorted.reserve(n_m2l + 1);
  const int end_bit = 2 * ls.key_bits;
  size_t    b1 = 0, b2 = 0;
  VFMM_CUDA_TRY(cub::DeviceRadixSort::SortKeys(nullptr, b1, ls.p2p_raw.p, ls.p2p_sorted.p, n_p2p, 0, end_bit, s));
  VFMM_CUDA_TRY(cub::DeviceRadixSort::SortKeys(nullptr, b2, ls.m2l_raw.p, ls.m2l_sorted.p, n_m2l, 0, end_bit, s));
  ls.cub_tmp.reserve(b1 > b2 ? b1 : b2);
  if (n_p2p > 0) {
    VFMM_CUDA_TRY(cub::DeviceRadixSort::SortKeys(ls.cub_tmp.p, b1, ls.p2p_raw.p, ls.p2p_sorted.p, n_p2p, 0, end_bit, s));
    count_launch();
  }
  if (n_m2l > 0) {
    VFMM_CUDA_TRY(cub::DeviceRadixSort::SortKeys(ls.cub_tmp.p, b2, ls.m2l_raw.p, ls.m2l_sorted.p, n_m2l, 0, end_bit, s));
    count_launch();
  }
  k_csr<<<grid_for(n_p2p + 1, 256), 256, 0, s>>>(ls.p2p_sorted.p, n_p2p, ls.key_bits, ncells_t, p2p_start, p2p_src, nbody_t, interactions);
  count_launch();
  k_csr<<<grid_for(n_m2l + 1, 256), 256, 0, s>>>(ls.m2l_sorted.p, n_m2l, ls.key_bits, ncells_t, m2l_start, m2l_src, nullptr, nullptr);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

// (target << kb | source) -> (source << kb | target)
__global__ void k_swap_keys(const unsigned long long *__restrict__ in, unsigned long long *__restrict__ out, int n, int kb)
{
  const unsigned long long mask = (1ull << kb) - 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned long long k = in[i];
    out[i]                     = ((k & mask) << kb) | (k >> kb);
  }
}

// Rows by source cell of the sorted pair lists in ls (for the reverse-mode
// passes, which gather per source): targets of source s at
// tgt[start[s] .. start[s+1]).  keys and sorted hold max(n_p2p, n_m2l) keys.
void lists_transpose(cudaStream_t s, ListScratch &ls, int n_p2p, int n_m2l, int ncells_s, unsigned long long *keys, unsigned long long *sorted,
                     int *p2p_start, int *p2p_tgt, int *m2l_start, int *m2l_tgt)
{
  const int end_bit = 2 * ls.key_bits;
  size_t    b1 = 0, b2 = 0;
  VFMM_CUDA_TRY(cub::DeviceRadixSort::SortKeys(nullptr, b1, keys, sorted, n_p2p, 0, end_bit, s));
  VFMM_CUDA_TRY(cub::DeviceRadixSort::SortKeys(nullptr, b2, keys, sorted, n_m2l, 0, end_bit, s));
  ls.cub_tmp.reserve(std::max(b1, b2));
  const unsigned long long *src[2] = {ls.p2p_sorted.p, ls.m2l_sorted.p};
  const int                 cnt[2] = {n_p2p, n_m2l};
  int                      *st[2] = {p2p_start, m2l_start}, *tg[2] = {p2p_tgt, m2l_tgt};
  for (int l = 0; l < 2; l++) {
    const int n = cnt[l];
    if (n > 0) {
      k_swap_keys<<<grid_for(n, 256), 256, 0, s>>>(src[l], keys, n, ls.key_bits);
      count_launch();
      size_t bytes = std::max(b1, b2);
      VFMM_CUDA_TRY(cub::DeviceRadixSort::SortKeys(ls.cub_tmp.p, bytes, keys, sorted, n, 0, end_bit, s));
      count_launch();
    }
    k_csr<<<grid_for(n + 1, 256), 256, 0, s>>>(sorted, n, ls.key_bits, ncells_s, st[l], tg[l], nullptr, nullptr);
    count_launch();
  }
  VFMM_LAUNCH_CHECK();
}

} // namespace vfmm
