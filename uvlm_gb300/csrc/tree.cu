// Octree build on the device, bit-exact with the reference's recursive
// top-down build (src/tree.hpp:7-113).
//
// The reference sorts bodies by a stable octant partition, level by level,
// until a cell holds <= ncrit bodies.  Here:
//   1. bounding box and root (tree.hpp:7-26), same FP64 operations;
//   2. per body, a 63-bit key of 21 octant digits, each digit from the strict
//      comparison x > centre with the centre chain of tree.hpp:86-92
//      (c <- c +/- R0/2^(l+1), one rounded add per level);
//   3. radix sort of the keys (stable);
//   4. per body, its leaf level: the first level whose key prefix is shared by
//      <= ncrit bodies (binary searches in the sorted keys);
//   5. inside each leaf, bodies ordered by their incoming index: that is the
//      order the reference's stable partitions leave them in;
//   6. cells: every (level, prefix) with level <= the leaf level is a cell;
//      enumerated in preorder (sorted by first body, then level), and placed
//      at the index the reference gives them: a node's children form one
//      contiguous block, appended when the node is visited in preorder
//      (tree.hpp:81-84), so block start = 1 + sum of NCHILD over earlier
//      nodes in preorder.
#include <cub/cub.cuh>
#include "vfmm_internal.cuh"

namespace vfmm {

__device__ __forceinline__ int lower_bound_u64(const uint64_t *a, int lo, int hi, uint64_t v)
{
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] < v)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

// ------------------------------------------------------------ bounding box
__global__ void k_bbox_partial(const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z, int n, double *part)
{
  double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  // 64-bit index: n may be close to 2^31 - 1, where i + gridDim.x * blockDim.x
  // would overflow an int
  const long long step = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
    const double v[3] = {x[i], y[i], z[i]};
    for (int d = 0; d < 3; d++) {
      mn[d] = fmin(v[d], mn[d]);
      mx[d] = fmax(v[d], mx[d]);
    }
  }
  for (int o = 16; o > 0; o >>= 1)
    for (int d = 0; d < 3; d++) {
      mn[d] = fmin(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
      mx[d] = fmax(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
    }
  __shared__ double s[32][6];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
    for (int d = 0; d < 3; d++) {
      s[w][d]     = mn[d];
      s[w][3 + d] = mx[d];
    }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); k++)
      for (int d = 0; d < 3; d++) {
        s[0][d]     = fmin(s[0][d], s[k][d]);
        s[0][3 + d] = fmax(s[0][3 + d], s[k][3 + d]);
      }
    for (int k = 0; k < 6; k++)
      part[blockIdx.x * 6 + k] = s[0][k];
  }
}

// getBounds, tree.hpp:7-26: centre = (max+min)/2, R0 = largest half extent
// about the centre, times 1.00001.
// One warp; min/max are exact, so the lane split does not change the result.
__global__ void k_bbox_final(const double *part, int nb, DevInfo *info)
{
  double mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int b = threadIdx.x; b < nb; b += 32)
    for (int d = 0; d < 3; d++) {
      mn[d] = fmin(part[b * 6 + d], mn[d]);
      mx[d] = fmax(part[b * 6 + 3 + d], mx[d]);
    }
  for (int o = 16; o > 0; o >>= 1)
    for (int d = 0; d < 3; d++) {
      mn[d] = fmin(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
      mx[d] = fmax(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
    }
  if (threadIdx.x != 0)
    return;
  double X0[3], R0 = 0;
  for (int d = 0; d < 3; d++)
    X0[d] = __ddiv_rn(__dadd_rn(mx[d], mn[d]), 2.0);
  for (int d = 0; d < 3; d++) {
    R0 = fmax(__dsub_rn(X0[d], mn[d]), R0);
    R0 = fmax(__dsub_rn(mx[d], X0[d]), R0);
  }
  R0 = __dmul_rn(R0, 1.00001);
  for (int d = 0; d < 3; d++)
    info->X0[d] = X0[d];
  info->R0 = R0;
}

// The partial-reduction kernel into caller-provided storage of nb*6 doubles.
void bbox_partial_into(cudaStream_t s, const double *x, const double *y, const double *z, int n, double *part, int nb)
{
  k_bbox_partial<<<nb, 256, 0, s>>>(x, y, z, n, part);
  count_launch();
}

void tree_bounds(cudaStream_t s, const double *X, size_t cap, int n, DevInfo *info, TreeScratch &ts)
{
  const int nb = 152 * 4;
  ts.bbox_part.reserve(nb * 6);
  k_bbox_partial<<<nb, 256, 0, s>>>(X, X + cap, X + 2 * cap, n, ts.bbox_part.p);
  count_launch();
  k_bbox_final<<<1, 32, 0, s>>>(ts.bbox_part.p, nb, info);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

// ------------------------------------------------------------ keys
// a > b for finite doubles, on the integer pipe: the sign-magnitude bit
// patterns, mapped to two's-complement order, compare as the doubles do;
// +0 and -0 compare equal.
__device__ __forceinline__ bool dgreater(double a, double b)
{
  const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
  if (((ia | ib) & 0x7fffffffffffffffll) == 0)
    return false; // both zero
  const long long ka = ia ^ ((ia >> 63) & 0x7fffffffffffffffll), kb = ib ^ ((ib >> 63) & 0x7fffffffffffffffll);
  return ka > kb;
}

// Octant keys of the first `levels` levels (the digit of level l at bits
// 3 (MAXL - 1 - l), deeper digits zero).
__global__ void k_keys(const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z, int n, const DevInfo *info,
                       int levels, uint64_t *keys, uint32_t *idx)
{
  // the centre chain's half-widths R0 / 2^(l+1), the same division for every body
  __shared__ double half[MAXL];
  if (threadIdx.x < MAXL)
    half[threadIdx.x] = __ddiv_rn(info->R0, (double)(1 << (threadIdx.x + 1)));
  __syncthreads();
  // 64-bit index: n may be close to 2^31 - 1, where i + gridDim.x * blockDim.x
  // would overflow an int
  const long long step = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
    const double p[3] = {x[i], y[i], z[i]};
    double       c[3] = {info->X0[0], info->X0[1], info->X0[2]};
    uint64_t     key  = 0;
#pragma unroll 1
    for (int l = 0; l < levels; l++) {
      const int b0 = dgreater(p[0], c[0]), b1 = dgreater(p[1], c[1]), b2 = dgreater(p[2], c[2]);
      key          = (key << 3) | (uint64_t)(b0 | (b1 << 1) | (b2 << 2));
      const double r = half[l];
      c[0]           = __dadd_rn(c[0], b0 ? r : -r);
      c[1]           = __dadd_rn(c[1], b1 ? r : -r);
      c[2]           = __dadd_rn(c[2], b2 ? r : -r);
    }
    keys[i] = levels < MAXL ? key << (3 * (MAXL - levels)) : key;
    idx[i]  = (uint32_t)i;
  }
}

// Leaf level of each sorted body: the shallowest level whose prefix count is
// <= ncrit (tree.hpp:43: a cell with <= ncrit bodies is a leaf).  Keys of
// `levels` < MAXL levels that leave a cell at that depth with more than ncrit
// bodies set info->deeper (the build is redone with full keys).
__global__ void k_leaf_level(const uint64_t *__restrict__ sk, int n, int ncrit, int levels, int *lvl, int *lo, int *hi, DevInfo *info)
{
  // 64-bit index: n may be close to 2^31 - 1, where i + gridDim.x * blockDim.x
  // would overflow an int
  const long long step = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
    const uint64_t key = sk[i];
    int            a = 0, b = n, L = -1;
    for (int l = 0; l <= levels; l++) {
      if (l > 0) {
        const int      sh = 3 * (MAXL - l);
        const uint64_t p  = key >> sh;
        a                 = lower_bound_u64(sk, a, b, p << sh);
        b                 = lower_bound_u64(sk, a, b, (p + 1) << sh);
      }
      if (b - a <= ncrit) {
        L = l;
        break;
      }
    }
    if (L < 0) {
      if (levels < MAXL)
        atomicExch(&info->deeper, 1);
      else
        atomicExch(&info->err, (int)VFMM_ERR_DEPTH);
      L = levels;
    }
    lvl[i] = L;
    lo[i]  = a;
    hi[i]  = b;
  }
}

// Inside a leaf, bodies keep their incoming relative order.
__global__ void k_leaf_perm(const uint32_t *__restrict__ sidx, const int *__restrict__ lo, const int *__restrict__ hi, int n, uint32_t *perm)
{
  // 64-bit index: n may be close to 2^31 - 1, where i + gridDim.x * blockDim.x
  // would overflow an int
  const long long step = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
    const int      a = lo[i], b = hi[i];
    const uint32_t me = sidx[i];
    int            rank = 0;
    for (int j = a; j < b; j++)
      rank += sidx[j] < me;
    perm[a + rank] = me;
  }
}

__device__ __forceinline__ int common_digits(uint64_t a, uint64_t b)
{
  const uint64_t x = a ^ b;
  if (x == 0)
    return MAXL;
  const int hb = 63 - __clzll((long long)x);
  return (62 - hb) / 3;
}

// Number of cells whose first body is sorted body i.
__global__ void k_node_count(const uint64_t *__restrict__ sk, const int *__restrict__ lvl, int n, int *cnt)
{
  // 64-bit index: n may be close to 2^31 - 1, where i + gridDim.x * blockDim.x
  // would overflow an int
  const long long step = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
    const int L = lvl[i];
    if (i == 0)
      cnt[i] = L + 1;
    else {
      const int c = common_digits(sk[i - 1], sk[i]);
      cnt[i]      = L > c ? L - c : 0;
    }
  }
}

__global__ void k_node_write(const uint64_t *__restrict__ sk, const int *__restrict__ lvl, const int *__restrict__ hi, const int *__restrict__ off,
                             const int *__restrict__ cnt, int n, int *nlevel, int *nstart, int *ncount, int ncap, DevInfo *info)
{
  // 64-bit index: n may be close to 2^31 - 1, where i + gridDim.x * blockDim.x
  // would overflow an int
  const long long step = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
    const int c = cnt[i];
    if (c == 0)
      continue;
    const int      L = lvl[i], ls = L - c + 1;
    const uint64_t key = sk[i];
    for (int l = ls; l <= L; l++) {
      const int t = off[i] + (l - ls);
      if (t >= ncap) {
        atomicExch(&info->overflow, 1);
        continue;
      }
      int end;
      if (l == L)
        end = hi[i];
      else if (l == 0)
        end = n;
      else {
        const int      sh = 3 * (MAXL - l);
        const uint64_t p  = key >> sh;
        end               = lower_bound_u64(sk, i, n, (p + 1) << sh);
      }
      nlevel[t] = l;
      nstart[t] = i;
      ncount[t] = end - i;
    }
  }
}

__global__ void k_iota(int *a, int n)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    a[i] = i;
}

// Per-level start offsets into the level-sorted node list; level_start[MAXL+1]
// = nnodes.  Also records nnodes and maxLevel.
__global__ void k_level_start(const int *__restrict__ slvl, int nn, int *level_start, DevInfo *info)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= nn; i += gridDim.x * blockDim.x) {
    const int lp = i == 0 ? -1 : slvl[i - 1];
    const int lc = i == nn ? MAXL + 1 : slvl[i];
    for (int l = lp + 1; l <= lc; l++)
      level_start[l] = i;
    if (i == nn) {
      info->nnodes   = nn;
      info->maxLevel = nn > 0 ? slvl[nn - 1] : 0;
    }
  }
}

__device__ __forceinline__ int lb_start(const int *list, const int *nstart, int a, int b, int v)
{ // first k in [a,b) with nstart[list[k]] >= v
  while (a < b) {
    int m = (a + b) >> 1;
    if (nstart[list[m]] < v)
      a = m + 1;
    else
      b = m;
  }
  return a;
}

__global__ void k_node_links(int nn, const int *__restrict__ nlevel, const int *__restrict__ nstart, const int *__restrict__ ncount,
                             const int *__restrict__ slist, const int *__restrict__ level_start, int ncrit, int *nparent, int *nrank, int *nchild,
                             int *leafflag)
{
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nn; t += gridDim.x * blockDim.x) {
    const int l = nlevel[t], s = nstart[t], c = ncount[t];
    int       parent = -1, rank = 0, nch = 0;
    if (l > 0) {
      const int a = level_start[l - 1], b = level_start[l];
      const int k = lb_start(slist, nstart, a, b, s + 1) - 1; // last with start <= s
      parent      = slist[k];
      const int a2 = level_start[l], b2 = level_start[l + 1];
      const int first = lb_start(slist, nstart, a2, b2, nstart[parent]);
      const int me    = lb_start(slist, nstart, a2, b2, s);
      rank            = me - first;
    }
    if (c > ncrit && l < MAXL) {
      const int a = level_start[l + 1], b = level_start[l + 2];
      nch         = lb_start(slist, nstart, a, b, s + c) - lb_start(slist, nstart, a, b, s);
    }
    nparent[t]  = parent;
    nrank[t]    = rank;
    nchild[t]   = nch;
    leafflag[t] = nch == 0 ? 1 : 0;
  }
}

__global__ void k_node_ref(int nn, const int *__restrict__ nparent, const int *__restrict__ nrank, const int *__restrict__ nbs, int *nref)
{
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nn; t += gridDim.x * blockDim.x)
    nref[t] = t == 0 ? 0 : 1 + nbs[nparent[t]] + nrank[t];
}

__global__ void k_cell_write(int nn, const uint64_t *__restrict__ sk, const int *__restrict__ nlevel, const int *__restrict__ nstart,
                             const int *__restrict__ ncount, const int *__restrict__ nparent, const int *__restrict__ nchild,
                             const int *__restrict__ nbs, const int *__restrict__ nref, const int *__restrict__ leafflag,
                             const int *__restrict__ leafoff, DevInfo *info, CellsView cv, int *leaf_cells)
{
  const double R0 = info->R0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nn; t += gridDim.x * blockDim.x) {
    const int r = nref[t], l = nlevel[t];
    if (r < 0 || r >= nn || (leafflag[t] && (leafoff[t] < 0 || leafoff[t] >= nn))) {
      atomicExch(&info->overflow, 1); // inconsistent tree: never write out of range
      continue;
    }
    const uint64_t key = sk[nstart[t]];
    double         c[3] = {info->X0[0], info->X0[1], info->X0[2]};
    for (int k = 0; k < l; k++) {
      const int    dig = (int)((key >> (3 * (MAXL - 1 - k))) & 7);
      const double rr  = __ddiv_rn(R0, (double)(1 << (k + 1)));
      c[0]             = __dadd_rn(c[0], (dig & 1) ? rr : -rr);
      c[1]             = __dadd_rn(c[1], (dig & 2) ? rr : -rr);
      c[2]             = __dadd_rn(c[2], (dig & 4) ? rr : -rr);
    }
    cv.nchild[r] = nchild[t];
    cv.nbody[r]  = ncount[t];
    cv.child[r]  = nchild[t] ? 1 + nbs[t] : 0;
    cv.body[r]   = nstart[t];
    cv.level[r]  = l;
    cv.parent[r] = nparent[t] < 0 ? -1 : nref[nparent[t]];
    cv.x[r]      = c[0];
    cv.y[r]      = c[1];
    cv.z[r]      = c[2];
    cv.R[r]      = __ddiv_rn(R0, (double)(1 << l));
    if (leafflag[t])
      leaf_cells[leafoff[t]] = r;
  }
}

__global__ void k_map_level_cells(int nn, const int *__restrict__ slist, const int *__restrict__ nref, int *level_cells)
{
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const int t = slist[k];
    level_cells[k] = (t >= 0 && t < nn) ? nref[t] : 0;
  }
}

__global__ void k_set_leaves(const int *leafoff, const int *leafflag, int nn, DevInfo *info)
{
  if (threadIdx.x == 0 && blockIdx.x == 0)
    info->nleaves = nn > 0 ? leafoff[nn - 1] + leafflag[nn - 1] : 0;
}

template <class F>
static void cub_call(TreeScratch &ts, F f)
{
  size_t bytes = 0;
  VFMM_CUDA_TRY(f(nullptr, bytes));
  ts.cub_tmp.reserve(bytes);
  VFMM_CUDA_TRY(f(ts.cub_tmp.p, bytes));
}

// Steps 2-5: keys, sort, leaf levels and the final body permutation
// (ts.perm[p] = incoming index of the body at tree position p).
void tree_sort_bodies(cudaStream_t s, const double *X, size_t cap, int n, int ncrit, int levels, DevInfo *info, TreeScratch &ts)
{
  ts.keys.reserve(n);
  ts.skeys.reserve(n);
  ts.idx.reserve(n);
  ts.sidx.reserve(n);
  ts.perm.reserve(n);
  ts.lvl.reserve(n);
  ts.lo.reserve(n);
  ts.hi.reserve(n);
  ts.cnt.reserve(n);
  ts.off.reserve(n);
  const int g = grid_for(n, 256);
  k_keys<<<g, 256, 0, s>>>(X, X + cap, X + 2 * cap, n, info, levels, ts.keys.p, ts.idx.p);
  count_launch();
  VFMM_LAUNCH_CHECK();
  cub_call(ts, [&](void *tmp, size_t &bytes) {
    return cub::DeviceRadixSort::SortPairs(tmp, bytes, ts.keys.p, ts.skeys.p, ts.idx.p, ts.sidx.p, n, 3 * (MAXL - levels), 3 * MAXL, s);
  });
  count_launch();
  k_leaf_level<<<g, 256, 0, s>>>(ts.skeys.p, n, ncrit, levels, ts.lvl.p, ts.lo.p, ts.hi.p, info);
  count_launch();
  k_leaf_perm<<<g, 256, 0, s>>>(ts.sidx.p, ts.lo.p, ts.hi.p, n, ts.perm.p);
  count_launch();
  VFMM_LAUNCH_CHECK();
}

// Step 6.  `nncap` bounds the node count (n + MAXL*n/(ncrit+1) + 64).
bool tree_build_cells(cudaStream_t s, int n, int ncrit, int nncap, DevInfo *info, TreeScratch &ts, CellsView cv, int *level_cells, int *level_start,
                      int *leaf_cells)
{
  const int g = grid_for(n, 256);
  k_node_count<<<g, 256, 0, s>>>(ts.skeys.p, ts.lvl.p, n, ts.cnt.p);
  count_launch();
  cub_call(ts, [&](void *tmp, size_t &bytes) { return cub::DeviceScan::ExclusiveSum(tmp, bytes, ts.cnt.p, ts.off.p, n, s); });
  count_launch();
  ts.nlevel.reserve(nncap);
  ts.nstart.reserve(nncap);
  ts.ncount.reserve(nncap);
  ts.nparent.reserve(nncap);
  ts.nchild.reserve(nncap);
  ts.nrank.reserve(nncap);
  ts.nref.reserve(nncap);
  ts.nbs.reserve(nncap);
  ts.nsortidx.reserve(nncap);
  ts.nsortlvl.reserve(nncap);
  ts.nflag.reserve(nncap);
  ts.noff.reserve(nncap);
  k_node_write<<<g, 256, 0, s>>>(ts.skeys.p, ts.lvl.p, ts.hi.p, ts.off.p, ts.cnt.p, n, ts.nlevel.p, ts.nstart.p, ts.ncount.p, nncap, info);
  count_launch();
  VFMM_LAUNCH_CHECK();
  // The node count is needed on the host for the radix sort and scans below.
  int h_off = 0, h_cnt = 0, h_deeper = 0;
  VFMM_CUDA_TRY(cudaMemcpyAsync(&h_off, ts.off.p + (n - 1), sizeof(int), cudaMemcpyDeviceToHost, s));
  VFMM_CUDA_TRY(cudaMemcpyAsync(&h_cnt, ts.cnt.p + (n - 1), sizeof(int), cudaMemcpyDeviceToHost, s));
  VFMM_CUDA_TRY(cudaMemcpyAsync(&h_deeper, &info->deeper, sizeof(int), cudaMemcpyDeviceToHost, s));
  VFMM_CUDA_TRY(cudaStreamSynchronize(s));
  if (h_deeper)
    return false;
  const int nn = h_off + h_cnt;
  if (nn > nncap)
    throw Error(VFMM_ERR_CAPACITY, "tree node capacity exceeded");
  const int gn = grid_for(nn, 256);
  int      *iota = ts.nrank.p; // temporary: node ids 0..nn-1, overwritten later
  k_iota<<<gn, 256, 0, s>>>(iota, nn);
  count_launch();
  int *slist = ts.nsortidx.p, *slvl = ts.nsortlvl.p;
  cub_call(ts, [&](void *tmp, size_t &bytes) {
    return cub::DeviceRadixSort::SortPairs(tmp, bytes, ts.nlevel.p, slvl, iota, slist, nn, 0, 5, s);
  });
  count_launch();
  k_level_start<<<grid_for(nn + 1, 256), 256, 0, s>>>(slvl, nn, level_start, info);
  count_launch();
  int *leafflag = ts.nflag.p, *leafoff = ts.noff.p;
  k_node_links<<<gn, 256, 0, s>>>(nn, ts.nlevel.p, ts.nstart.p, ts.ncount.p, slist, level_start, ncrit, ts.nparent.p, ts.nrank.p, ts.nchild.p,
                                  leafflag);
  count_launch();
  cub_call(ts, [&](void *tmp, size_t &bytes) { return cub::DeviceScan::ExclusiveSum(tmp, bytes, ts.nchild.p, ts.nbs.p, nn, s); });
  count_launch();
  cub_call(ts, [&](void *tmp, size_t &bytes) { return cub::DeviceScan::ExclusiveSum(tmp, bytes, leafflag, leafoff, nn, s); });
  count_launch();
  k_node_ref<<<gn, 256, 0, s>>>(nn, ts.nparent.p, ts.nrank.p, ts.nbs.p, ts.nref.p);
  count_launch();
  k_cell_write<<<gn, 256, 0, s>>>(nn, ts.skeys.p, ts.nlevel.p, ts.nstart.p, ts.ncount.p, ts.nparent.p, ts.nchild.p, ts.nbs.p, ts.nref.p, leafflag,
                                  leafoff, info, cv, leaf_cells);
  count_launch();
  k_map_level_cells<<<gn, 256, 0, s>>>(nn, slist, ts.nref.p, level_cells);
  count_launch();
  k_set_leaves<<<1, 32, 0, s>>>(leafoff, leafflag, nn, info);
  count_launch();
  VFMM_LAUNCH_CHECK();
  return true;
}

} // namespace vfmm
