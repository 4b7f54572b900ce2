// Mixed-precision expansion kernels: FP32 P2M, M2M, M2L, L2L, L2P and P2P;
// the tree (tree.cu), the expansion arrays between kernels and the outputs
// stay FP64.
//
// Scaling.  FP32 cannot hold the raw expansions at high order (rho^n/(n+m)!
// and (n-m)!/rho^(n+1) leave its exponent range), so inside these kernels a
// cell c of half-width R_c = R0/2^level carries
//   scaled multipole  Mt_n^m = M_n^m / R_c^n,
//   scaled local      Lt_j^k = L_j^k * R_c^j,
// and harmonics are evaluated at offsets divided by the cell size.  The FP64
// arrays M and L between kernels stay unscaled (the reference's values).
//   P2M:  Mt_n^m(c) = sum_b alpha_b conj(Y_n^m((x_b - X_c)/R_c)).
//   M2L:  Lt_j^k(t) += (R_t/R_s)^j / R_s * (-1)^j sum M't_n^m S'_{j+n}^{m-k}(d/R_s),
//         d = X_t - X_s; (R_t/R_s) is a power of two.
//   M2M, L2L: scaled by the parent's half-width R_p instead (see k_m2m32).
//   L2P:  u = (1/R) sum (D Lt)(y), J = (1/R^2) sum (D D Lt)(y), y = (x - X_c)/R.
// P2P uses leaf-relative FP32 coordinates, a series form of the regularised
// kernel for close pairs (no cancellation), and per-source-leaf FP32 partial
// sums folded into a float-float (two-sum) accumulator.
#include <algorithm>
#include "harmonics.cuh"
#include "tcgen05.cuh"
#include "vfmm_internal.cuh"

namespace vfmm {

typedef cx<float>  zf;
typedef cx<double> zd;

static __constant__ HarmRecip<float> kHarmRecipF = make_harm_recip<float>();

// (n, m) of triangle index tri(n, m) for n <= PMAX: a table read instead of
// jk_of_m's search, whose trip count differs from lane to lane
struct TriNM {
  unsigned char n[nterms(PMAX + 1)], m[nterms(PMAX + 1)];
};
constexpr TriNM make_tri_nm()
{
  TriNM t{};
  for (int n = 0; n <= PMAX; n++)
    for (int m = 0; m <= n; m++) {
      t.n[tri(n, m)] = (unsigned char)n;
      t.m[tri(n, m)] = (unsigned char)m;
    }
  return t;
}
static __device__ const TriNM kTriNM = make_tri_nm();

struct DevMixed {
  CellsView     cv;
  const double *soa;
  size_t        cap;
  double2      *M, *L;
  float2       *Mp;      // prepared scaled multipoles [cell][P*P][3]
  const float4 *pos32;   // per body: (x - X_leaf, y - Y_leaf, z - Z_leaf, 1/(2 sigma^2))
  const float4 *alp32;   // per body: (alpha, 1/sigma)
  const int    *leaf_cells;
  int           nleaves;
  const int    *m2l_start, *m2l_src;
  const int    *p2p_start, *p2p_src;
  const int4   *items;
  double        R0, iR0;
  double        R0pow[PMAX + 1], iR0pow[PMAX + 1]; // R0^n, R0^-n
  int           stretching, formulation;
  float        *Bhi, *Blo; // tensor-core M2L operand rows [cell][3][tc_kp(P)] (null: not used)
  float        *near32;    // near-field sums of the split leaf kernel, [body][hi 12, lo 12]
};

// 2^e as a double built from its exponent field (-1022 <= e <= 1023; here
// |e| <= 21 levels x 16 orders): multiplying by it is exact, like ldexp,
// without ldexp's range handling on GB300's narrow FP64 pipe.
__device__ __forceinline__ double exp2i(int e) { return __longlong_as_double((long long)(1023 + e) << 52); }

// R_c^n and R_c^-n for a cell at `level` (R_c = R0 / 2^level): exact
// power-of-two rescalings of the per-tree tables.
__device__ __forceinline__ double cell_Rpow(const DevMixed &a, int level, int n) { return a.R0pow[n] * exp2i(-level * n); }
__device__ __forceinline__ double cell_iRpow(const DevMixed &a, int level, int n) { return a.iR0pow[n] * exp2i(level * n); }

// Store the scaled multipole Mt_n^m (m >= 0, component d) of cell c in the
// folded FP32 form read by M2L, [cell][n^2+n+m][d]: M'_n^m = (-1)^m Mt_n^m and,
// for m > 0, M'_n^{-m} = conj(Mt_n^m).  Written by P2M and M2M, which hold Mt
// in FP32 already.
__device__ __forceinline__ void store_mfold(const DevMixed &a, int PP, int c, int n, int m, int d, float re, float im)
{
  float2   *row = a.Mp + (size_t)c * 3 * PP;
  const int nn  = n * n + n;
  row[(nn + m) * 3 + d] = (m & 1) ? make_float2(-re, -im) : make_float2(re, im);
  if (m > 0)
    row[(nn - m) * 3 + d] = make_float2(re, -im);
}

// The scaled multipole Mt_n^m (m >= 0, component d) of cell c as a row of
// the tensor-core M2L's B operand: Mt_n^0 (real part) at n^2, Re/Im Mt_n^m at
// n^2 + 2m - 1 and n^2 + 2m, each as TF32 hi and lo parts (rounded to
// nearest); the padding after
// P^2 is zeroed with the (0, 0) term.
template <int P>
__device__ __forceinline__ void store_btc(const DevMixed &a, int c, int n, int m, int d, float re, float im)
{
  constexpr int KP = tc_kp(P);
  float        *hi = a.Bhi + ((size_t)c * 3 + d) * KP, *lo = a.Blo + ((size_t)c * 3 + d) * KP;
  const int     col = n * n + (m ? 2 * m - 1 : 0);
  const float   rh = tc::tf32_rn(re), ih = tc::tf32_rn(im);
  hi[col]          = rh;
  lo[col]          = tc::tf32_rn(re - rh);
  if (m) {
    hi[col + 1] = ih;
    lo[col + 1] = tc::tf32_rn(im - ih);
  }
  if (n == 0)
    for (int k = P * P; k < KP; k++)
      hi[k] = lo[k] = 0.f;
}

__device__ __forceinline__ void jk_of_m(int jks, int &j, int &k)
{
  j = 0;
  while ((j + 1) * (j + 2) / 2 <= jks)
    j++;
  k = jks - j * (j + 1) / 2;
}

// ------------------------------------------------------------------ prep
// Leaf-relative FP32 body data for the P2P sources and targets.
// One warp per leaf (leaves hold ~ncrit/2 bodies).
__global__ void k_prep_bodies(DevMixed a)
{
  const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  for (int li = blockIdx.x * wpb + (threadIdx.x >> 5); li < a.nleaves; li += gridDim.x * wpb) {
    const int    c  = a.leaf_cells[li];
    const int    b0 = a.cv.body[c], nb = a.cv.nbody[c];
    const double cx_ = a.cv.x[c], cy_ = a.cv.y[c], cz_ = a.cv.z[c];
    for (int t = lane; t < nb; t += 32) {
      const int    b  = b0 + t;
      const double sg = a.soa[F_R * a.cap + b];
      float4       p, q;
      p.x = (float)(a.soa[F_X * a.cap + b] - cx_);
      p.y = (float)(a.soa[(F_X + 1) * a.cap + b] - cy_);
      p.z = (float)(a.soa[(F_X + 2) * a.cap + b] - cz_);
      p.w = (float)(0.5 / (sg * sg));
      q.x = (float)a.soa[F_A * a.cap + b];
      q.y = (float)a.soa[(F_A + 1) * a.cap + b];
      q.z = (float)a.soa[(F_A + 2) * a.cap + b];
      q.w = (float)(1.0 / sg);
      const_cast<float4 *>(a.pos32)[b] = p;
      const_cast<float4 *>(a.alp32)[b] = q;
    }
  }
}

// ------------------------------------------------------------------ P2M
template <int P>
__global__ void __launch_bounds__(64) k_p2m32(DevMixed a)
{
  constexpr int K = nterms(P), NO = (3 * K + 63) / 64;
  extern __shared__ float4 smem32[];
  zf    *Ys = reinterpret_cast<zf *>(smem32);
  float *As = reinterpret_cast<float *>(Ys + 32 * K);
  for (int li = blockIdx.x; li < a.nleaves; li += gridDim.x) {
    const int c = a.leaf_cells[li];
    if (a.cv.level[c] == 0)
      continue; // the reference's upward pass skips level 0 (fmmCalculator.hpp:427)
    const int    b0 = a.cv.body[c], nb = a.cv.nbody[c];
    const int   lev = a.cv.level[c];
    const float iR  = (float)(a.iR0 * exp2i(lev)); // = ldexp(iR0, lev), exact
    zf          acc[NO];
#pragma unroll
    for (int i = 0; i < NO; i++)
      acc[i] = {0.f, 0.f};
    for (int c0 = 0; c0 < nb; c0 += 32) {
      const int nbc = min(32, nb - c0);
      const int t   = threadIdx.x;
      if (t < nbc) {
        const float4 p = a.pos32[b0 + c0 + t];
        regular_harmonics<float, P>(p.x * iR, p.y * iR, p.z * iR, Ys + t * K);
        const float4 q = a.alp32[b0 + c0 + t];
        As[t * 3 + 0]  = q.x;
        As[t * 3 + 1]  = q.y;
        As[t * 3 + 2]  = q.z;
      }
      __syncthreads();
#pragma unroll
      for (int i = 0; i < NO; i++) {
        const int o = threadIdx.x + 64 * i;
        if (o < 3 * K) {
          const int nms = o / 3, d = o % 3;
          for (int tt = 0; tt < nbc; tt++) {
            const zf    y  = Ys[tt * K + nms];
            const float al = As[tt * 3 + d];
            acc[i].r       = fmaf(al, y.r, acc[i].r);
            acc[i].i       = fmaf(-al, y.i, acc[i].i);
          }
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < NO; i++) {
      const int o = threadIdx.x + 64 * i;
      if (o < 3 * K) {
        int n, m;
        jk_of_m(o / 3, n, m);
        const double s = cell_Rpow(a, lev, n);
        a.M[(size_t)c * 3 * K + o] = make_double2(acc[i].r * s, acc[i].i * s);
        store_mfold(a, P * P, c, n, m, o % 3, acc[i].r, acc[i].i);
        if (a.Bhi)
          store_btc<P>(a, c, n, m, o % 3, acc[i].r, acc[i].i);
      }
    }
  }
}

// ------------------------------------------------------------------ M2L
// M2M and L2L in FP32 (multipoleKernels.hpp:479-516, :591-628) with every
// operand scaled by the parent's half-width R_p: the child multipoles enter
// as M_c / R_p^n and the parent's local expansion as L_p R_p^n, the offset
// harmonics are Y(dX / R_p), and the outputs are rescaled by R_p^j (M2M) or
// R_p^-j (L2L) in FP64 when they are added to the FP64 expansions.  Block of
// 128 threads per parent, as the FP64 kernels.
template <int P>
__global__ void __launch_bounds__(128) k_m2m32(DevMixed a, const int *cells, int count)
{
  constexpr int K = nterms(P);
  extern __shared__ float4 smem32[];
  zf *Ms = reinterpret_cast<zf *>(smem32); // [8][3K]
  zf *Ys = Ms + 8 * 3 * K;                  // [8][K]
  for (int pi = blockIdx.x; pi < count; pi += gridDim.x) {
    const int c = cells[pi], nch = a.cv.nchild[c], ch0 = a.cv.child[c], lev = a.cv.level[c];
    if (nch == 0)
      continue;
    __syncthreads();
    for (int e = threadIdx.x; e < nch * 3 * K; e += blockDim.x) {
      int n, m;
      jk_of_m((e % (3 * K)) / 3, n, m);
      const double2 v = a.M[(size_t)ch0 * 3 * K + e];
      const double  s = cell_iRpow(a, lev, n);
      Ms[e]           = {(float)(v.x * s), (float)(v.y * s)};
    }
    if (threadIdx.x < nch) {
      const int    ch = ch0 + threadIdx.x;
      const double iR = a.iR0 * exp2i(lev); // = ldexp(iR0, lev), exact
      regular_harmonics<float, P>((float)((a.cv.x[c] - a.cv.x[ch]) * iR), (float)((a.cv.y[c] - a.cv.y[ch]) * iR),
                                  (float)((a.cv.z[c] - a.cv.z[ch]) * iR), Ys + threadIdx.x * K);
    }
    __syncthreads();
    for (int o = threadIdx.x; o < 3 * K; o += blockDim.x) {
      const int jks = o / 3, d = o % 3;
      int       j, k;
      jk_of_m(jks, j, k);
      zf acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
      for (int t0 = 0; t0 < nch; t0 += 4)
        m2m_term_sum<P, 4>(j, k, d, Ms, Ys, t0, nch, acc);
      const zf     sum = (acc[0] + acc[1]) + (acc[2] + acc[3]);
      const double s   = cell_Rpow(a, lev, j);
      double2     *q   = a.M + (size_t)c * 3 * K + o;
      const double2 old = *q;
      *q                = make_double2(old.x + (double)sum.r * s, old.y + (double)sum.i * s);
      store_mfold(a, P * P, c, j, k, d, sum.r, sum.i);
      if (a.Bhi)
        store_btc<P>(a, c, j, k, d, sum.r, sum.i);
    }
  }
}

template <int P>
__global__ void __launch_bounds__(128) k_l2l32(DevMixed a, const int *cells, int count)
{
  constexpr int K = nterms(P);
  extern __shared__ float4 smem32[];
  zf *Ls = reinterpret_cast<zf *>(smem32); // [3K]
  zf *Ys = Ls + 3 * K;                      // [8][K]
  for (int pi = blockIdx.x; pi < count; pi += gridDim.x) {
    const int p = cells[pi], nch = a.cv.nchild[p], ch0 = a.cv.child[p], lev = a.cv.level[p];
    if (nch == 0)
      continue;
    __syncthreads();
    for (int e = threadIdx.x; e < 3 * K; e += blockDim.x) {
      int n, m;
      jk_of_m(e / 3, n, m);
      const double2 v = a.L[(size_t)p * 3 * K + e];
      const double  s = cell_Rpow(a, lev, n);
      Ls[e]           = {(float)(v.x * s), (float)(v.y * s)};
    }
    if (threadIdx.x < nch) {
      const int    ch = ch0 + threadIdx.x;
      const double iR = a.iR0 * exp2i(lev); // = ldexp(iR0, lev), exact
      regular_harmonics<float, P>((float)((a.cv.x[ch] - a.cv.x[p]) * iR), (float)((a.cv.y[ch] - a.cv.y[p]) * iR),
                                  (float)((a.cv.z[ch] - a.cv.z[p]) * iR), Ys + threadIdx.x * K);
    }
    __syncthreads();
    const int ngroups = (nch + 3) / 4;
    for (int o = threadIdx.x; o < ngroups * 3 * K; o += blockDim.x) {
      const int t0 = (o / (3 * K)) * 4, r = o % (3 * K), jks = r / 3, d = r % 3;
      int       j, k;
      jk_of_m(jks, j, k);
      zf acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
      l2l_term_sum<P, 4>(j, k, d, Ls, Ys, t0, nch, acc);
      const double s = cell_iRpow(a, lev, j);
#pragma unroll
      for (int c = 0; c < 4; c++)
        if (t0 + c < nch) {
          double2      *q   = a.L + (size_t)(ch0 + t0 + c) * 3 * K + r;
          const double2 old = *q;
          *q                = make_double2(old.x + (double)acc[c].r * s, old.y + (double)acc[c].i * s);
        }
    }
  }
}

// M2L, lockstep form.  One block per target cell, one warp per input degree
// n (P warps).  Within warp n every lane runs the same m-loop (-n..n), so
// there is no divergence; a lane owns an output tile of two half-tiles (each
// a row j and KH consecutive columns k, all 3 components) and keeps one
// sliding register window per half over the singular harmonics
// S'_{j+n}^{m-k}.  Warps whose degree has few tiles replicate them over
// several sources of the batch.  The per-pair factor (R_t/R_s)^j / R_s is
// split exactly into 2^{(lt-ls) n} on the staged multipole and
// 2^{(ls-lt) q} / R_s on the staged harmonics (q = j + n).  Lane table: see
// m2l_lane_table.
constexpr int M2L_YOFF = 4; // leading pad of each staged harmonic table


// v * 2^e, equal to ldexpf(v, e): a multiply by the exactly built power of
// two inside the normal exponent range, ldexpf outside it.
__device__ __forceinline__ float scale2f(float v, int e)
{
  return (e >= -126 && e <= 127) ? v * __int_as_float((e + 127) << 23) : ldexpf(v, e);
}

template <int P, int SB>
struct M2LV2 {
  static constexpr int KH = m2l_half_width(P); // k columns per half-tile
  static_assert(KH >= 2, "the two-step window update assumes KH >= 2");
  static constexpr int K = nterms(P), PP = P * P;
  static constexpr int MSTR = 3 * PP + 1;            // complex stride of a staged multipole
  static constexpr int YSTR = PP + M2L_YOFF + 1;     // complex stride of a staged harmonic table
  static constexpr size_t bytes = (size_t)(SB * (MSTR + YSTR)) * sizeof(zf); // dynamic: multipoles, harmonics
  static constexpr size_t meta  = 2 * (size_t)SB * (sizeof(float4) + 2 * sizeof(int)) + 16; // static, with the masks and padding
  // per-warp partial locals [P][3K] reuse the staging arrays after the last batch
  static_assert(P * 3 * K <= SB * (MSTR + YSTR), "per-warp partials fit in the staging arrays");
  static_assert(bytes + meta == m2l32_smem_bytes(P, SB), "the host-side size check uses the same layout");
};

template <int P, int SB>
__global__ void __launch_bounds__(P * 32) k_m2l32v2(DevMixed a, const int4 *__restrict__ lanes, int ncells)
{
  using G = M2LV2<P, SB>;
  constexpr int K = G::K, PP = G::PP, MSTR = G::MSTR, YSTR = G::YSTR, KH = G::KH;
  extern __shared__ float4 smem32[];
  zf *Ms = reinterpret_cast<zf *>(smem32);
  zf *Ys = Ms + SB * MSTR;
  zf *Lw = Ms; // [P][3K] after the batches
  // Source metadata of a batch, two buffers: per source (d / R_s, 1 / R_s),
  // index, level, and the mask of sources on another level than the target.
  // Warp 0 (degree 0, the lightest m-loop) stages batch k + 1 into the other
  // buffer after its own compute of batch k, so each batch needs no barrier
  // between staging its metadata and using it beyond the one that ends the
  // previous batch.
  __shared__ float4   OffB[2][SB];
  __shared__ int      SrcB[2][SB], LvlB[2][SB];
  __shared__ unsigned cmaskB[2];
  static_assert(SB <= 32, "one warp stages a batch");
  const int n = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int4 me = lanes[n * 32 + lane];
  const bool busy = me.x >= 0;
  const int  jA = me.x & 255, k0A = (me.x >> 8) & 255, kwA = (me.x >> 16) & 255;
  const int  jB = me.y & 255, k0B = (me.y >> 8) & 255, kwB = (me.y >> 16) & 255;
  const int  rep = me.z, R = me.w & 255;
  const int  nthreads = P * 32;
  for (int t = blockIdx.x; t < ncells; t += gridDim.x) {
    zf accA[KH][3], accB[KH][3];
#pragma unroll
    for (int kk = 0; kk < KH; kk++)
#pragma unroll
      for (int d = 0; d < 3; d++)
        accA[kk][d] = accB[kk][d] = {0.f, 0.f};
    const int    q0 = a.m2l_start[t], q1 = a.m2l_start[t + 1];
    const double tx = a.cv.x[t], ty = a.cv.y[t], tz = a.cv.z[t];
    const int    lt = a.cv.level[t];
    // warp 0 (all 32 lanes, n == 0) stages the sources qb .. qb + cnt - 1 into buffer buf
    auto stage_meta = [&](int buf, int qb, int cnt) {
      bool cl = false;
      if (lane < cnt) {
        const int    s   = a.m2l_src[qb + lane];
        const int    ls  = a.cv.level[s];
        const double iRs = a.iR0 * exp2i(ls); // = ldexp(iR0, ls), exact
        SrcB[buf][lane]  = s;
        LvlB[buf][lane]  = ls;
        OffB[buf][lane]  = make_float4((float)((tx - a.cv.x[s]) * iRs), (float)((ty - a.cv.y[s]) * iRs), (float)((tz - a.cv.z[s]) * iRs),
                                       (float)iRs);
        cl               = ls != lt;
      }
      const unsigned msk = __ballot_sync(0xffffffffu, cl);
      if (lane == 0)
        cmaskB[buf] = msk;
    };
    // buffer 0 was last read before the barriers that ended the previous cell
    if (n == 0 && q0 < q1)
      stage_meta(0, q0, min(SB, q1 - q0));
    for (int qb = q0, k = 0; qb < q1; qb += SB, k ^= 1) {
      const int nb = min(SB, q1 - qb);
      __syncthreads(); // the previous batch's compute is done; this batch's metadata is visible
      const float4 *Off = OffB[k];
      const int    *Src = SrcB[k];
      const int    *Lvl = LvlB[k];
      // stage multipoles: asynchronous copies of Mp32, all in flight at once
      // while the harmonics are made; sources on another level than the
      // target are scaled by 2^{(lt - ls) n} afterwards
      for (int r = threadIdx.x; r < 3 * PP; r += nthreads)
        for (int b = 0; b < nb; b++)
          cp_async8(Ms + b * MSTR + r, a.Mp + (size_t)Src[b] * 3 * PP + r);
      // stage singular harmonics at d / R_s, folded and scaled by 2^{(ls - lt) q} / R_s
      if (threadIdx.x < nb * P) {
        const int    b = threadIdx.x / P, m = threadIdx.x - b * P, ls = Lvl[b];
        const float4 o = Off[b];
        const float  dx = o.x, dy = o.y, dz = o.z;
        const float  r2 = dx * dx + dy * dy + dz * dz, ir2 = 1.0f / r2, S00 = rsqrtf(r2);
        zf          *Y = Ys + b * YSTR + M2L_YOFF;
        singular_column_emit<float, P>(m, dx, dy, dz, ir2, S00, [&](int q, zf c) {
          const float f    = scale2f(o.w, (ls - lt) * q);
          const zf    v    = {c.r * f, c.i * f};
          Y[q * q + q + m] = (m & 1) ? zf{-v.r, -v.i} : v;
          if (m > 0)
            Y[q * q + q - m] = conj(v);
        });
      }
      cp_async_wait_all();
      __syncthreads();
      const unsigned cmask = cmaskB[k];
      if (cmask) { // block-uniform: sources on another level than the target
        for (int r = threadIdx.x; r < 3 * PP; r += nthreads) {
          const int nn = (int)sqrtf((float)(r / 3)); // degree of entry n^2+n+m (exact for these small integers)
          for (unsigned mk = cmask; mk; mk &= mk - 1) {
            const int b  = __ffs(mk) - 1;
            const int sh = (lt - Lvl[b]) * nn;
            zf       &v  = Ms[b * MSTR + r];
            v            = {scale2f(v.r, sh), scale2f(v.i, sh)};
          }
        }
        __syncthreads();
      }
      if (busy) {
        const int qA = jA + n, qB = jB + n;
        const int baseA = M2L_YOFF + qA * qA + qA - k0A, baseB = M2L_YOFF + qB * qB + qB - k0B;
        for (int b = rep; b < nb; b += R) {
          const zf *YA = Ys + b * YSTR + baseA;
          const zf *YB = Ys + b * YSTR + baseB;
          const zf *Mb = Ms + b * MSTR + (n * n + n) * 3;
          // windows ya[kk] = YA[m - kk], yb[kk] = YB[m - kk] of the current m
          zf ya[KH], yb[KH];
#pragma unroll
          for (int kk = 0; kk < KH; kk++) {
            ya[kk] = YA[-n - kk];
            yb[kk] = YB[-n - kk];
          }
          // one step: column kk of each half-tile takes M'_n^m S'_{q}^{m-k0-kk}
          auto step = [&](int m, const zf (&wa)[KH], const zf (&wb)[KH]) {
            const zf m0 = Mb[m * 3 + 0], m1 = Mb[m * 3 + 1], m2 = Mb[m * 3 + 2];
#pragma unroll
            for (int kk = 0; kk < KH; kk++) {
              cfma(accA[kk][0], m0, wa[kk]);
              cfma(accA[kk][1], m1, wa[kk]);
              cfma(accA[kk][2], m2, wa[kk]);
              cfma(accB[kk][0], m0, wb[kk]);
              cfma(accB[kk][1], m1, wb[kk]);
              cfma(accB[kk][2], m2, wb[kk]);
            }
          };
          step(-n, ya, yb);
          // the remaining 2n steps two at a time (m + 1, m + 2)
          for (int m = -n; m < n; m += 2) {
            zf wa1[KH], wb1[KH], wa2[KH], wb2[KH];
            wa1[0] = YA[m + 1];
            wb1[0] = YB[m + 1];
            wa2[0] = YA[m + 2];
            wb2[0] = YB[m + 2];
            wa2[1] = wa1[0];
            wb2[1] = wb1[0];
#pragma unroll
            for (int kk = 1; kk < KH; kk++) {
              wa1[kk] = ya[kk - 1];
              wb1[kk] = yb[kk - 1];
            }
#pragma unroll
            for (int kk = 2; kk < KH; kk++) {
              wa2[kk] = ya[kk - 2];
              wb2[kk] = yb[kk - 2];
            }
            step(m + 1, wa1, wb1);
            step(m + 2, wa2, wb2);
#pragma unroll
            for (int kk = 0; kk < KH; kk++) {
              ya[kk] = wa2[kk];
              yb[kk] = wb2[kk];
            }
          }
        }
      }
      // the other buffer was last read before this batch's first barrier
      if (n == 0 && qb + SB < q1)
        stage_meta(k ^ 1, qb + SB, min(SB, q1 - qb - SB));
    }
    // combine: replicas inside the warp (deterministic tree), then warps in order
    const int T = me.w >> 8;
    for (int st = 1; st < R; st <<= 1) {
#pragma unroll
      for (int kk = 0; kk < KH; kk++)
#pragma unroll
        for (int d = 0; d < 3; d++) {
          const float ar = __shfl_down_sync(0xffffffffu, accA[kk][d].r, T * st);
          const float ai = __shfl_down_sync(0xffffffffu, accA[kk][d].i, T * st);
          const float br = __shfl_down_sync(0xffffffffu, accB[kk][d].r, T * st);
          const float bi = __shfl_down_sync(0xffffffffu, accB[kk][d].i, T * st);
          if (busy && (rep % (2 * st)) == 0 && rep + st < R) {
            accA[kk][d].r += ar;
            accA[kk][d].i += ai;
            accB[kk][d].r += br;
            accB[kk][d].i += bi;
          }
        }
    }
    __syncthreads(); // staging arrays free: per-warp partials Lw[n] (each output of row j
                     // is owned by one lane of each warp n <= P-1-j)
    if (busy && rep == 0) {
#pragma unroll
      for (int kk = 0; kk < KH; kk++)
#pragma unroll
        for (int d = 0; d < 3; d++) {
          if (kk < kwA)
            Lw[n * 3 * K + tri(jA, k0A + kk) * 3 + d] = accA[kk][d];
          if (kk < kwB)
            Lw[n * 3 * K + tri(jB, k0B + kk) * 3 + d] = accB[kk][d];
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 3 * K; e += nthreads) {
      int jj, kk;
      jk_of_m(e / 3, jj, kk);
      zf v = Lw[e];
      for (int w = 1; w <= P - 1 - jj; w++)
        v = v + Lw[w * 3 * K + e];
      const double s = ((jj & 1) ? -1.0 : 1.0) * cell_iRpow(a, lt, jj);
      a.L[(size_t)t * 3 * K + e] = make_double2(v.r * s, v.i * s);
    }
  }
}

// ------------------------------------------------------------------ L2P + P2P
__device__ __forceinline__ zf coef_full32(const zf *c, int n, int m, int stride, int comp)
{
  if (m > 0)
    return c[tri(n, m) * stride + comp];
  if (m == 0)
    return {c[tri(n, 0) * stride + comp].r, 0.f};
  return conj(c[tri(n, -m) * stride + comp]);
}
__device__ __forceinline__ zf deriv_coef32(const zf *c, int n, int mu, int axis, int stride, int comp)
{
  if (axis == 2) {
    zf v = coef_full32(c, n + 1, mu, stride, comp);
    return {-v.r, -v.i};
  }
  const float s = (mu - 1 >= 0) ? -1.f : 1.f;
  const float t = (mu + 1 >= 1) ? 1.f : -1.f;
  const zf    A = s * coef_full32(c, n + 1, mu - 1, stride, comp);
  const zf    B = t * coef_full32(c, n + 1, mu + 1, stride, comp);
  if (axis == 0)
    return {0.5f * (A.r + B.r), 0.5f * (A.i + B.i)};
  return {0.5f * (A.i - B.i), -0.5f * (A.r - B.r)};
}

// CH_: near-field source bodies staged per chunk (the P2P tile): 768 (five
// blocks per SM, 96 registers: the default) or 512 (seven blocks per SM, 72
// registers with a few spilled; vfmm_config.p2p_chunk).  At 2^20 bodies the
// unspilled five-block form is 7% faster than six blocks at 80 registers.
// MODE 2 (the far-field pass of the split kernel) stages no source pairs: its
// first buffer only holds the members' partial sums, and more of its blocks
// fit on an SM to hide the latency of its per-leaf steps.
template <int P, int CH_, int MODE = 0>
struct L2P32Sizes {
  static constexpr int    K  = nterms(P);
  static constexpr int    K1 = nterms(P - 1) > 0 ? nterms(P - 1) : 1;
  static constexpr int    K2 = nterms(P - 2) > 0 ? nterms(P - 2) : 1;
  static constexpr int    CH = CH_;
  static constexpr int    SQ4 = MODE == 2 ? 2 * 128 * 12 / 4 : (CH / 2) * 5; // float4 of the first buffer
  static constexpr int    BLOCKS = MODE == 2 ? 8 : (CH == 512 ? 7 : 5);   // resident blocks per SM the launch bounds ask for
  static constexpr size_t bytes =
      (size_t)SQ4 * sizeof(float4) + 128 * (sizeof(float4) + sizeof(int)) + (size_t)(3 * K + 3 * K1 + 9 * K2) * sizeof(zf);
  static_assert((size_t)SQ4 * sizeof(float4) >= 2 * 128 * 12 * sizeof(float), "the staging buffer holds the reduction");
};

constexpr float kInv4pi = 0.0795774715459476679f;
constexpr float kC2spi  = 1.12837916709551257f; // 2/sqrt(pi)
constexpr float kIsq2   = 0.707106781186547524f;

// ---- packed FP32 (two sources per lane) --------------------------------------
// The near-field loop runs on float2 operands with the f32x2 instructions
// (one instruction, two FP32 FMAs): each lane carries two source bodies.
__device__ __forceinline__ float2 pk(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 add2(float2 x, float2 y) { return __fadd2_rn(x, y); }
__device__ __forceinline__ float2 mul2(float2 x, float2 y) { return __fmul2_rn(x, y); }
__device__ __forceinline__ float2 fma2(float2 x, float2 y, float2 z) { return __ffma2_rn(x, y, z); }
// 1/sqrt(x) and 2^x, the PTX approximations with subnormals flushed (the
// operands here are squared distances between bodies and -rho^2 log2(e))
__device__ __forceinline__ float rsqrt_ftz(float x)
{
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float ex2_ftz(float x)
{
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float rcp_ftz(float x)
{
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// erfcx(rho) = e^(rho^2) erfc(rho) ~ t (c1 + c2 t + c3 t^2 + c4 t^3 + c5 t^4),
// t = 1 / (1 + a rho), for rho >= 0.5: a weighted least-squares fit whose
// error, with these FP32 constants, is below 5e-8 relative to g(rho) below
// (uvlm_gb300/csrc/fit_erfcx.py makes them; tests/test_erfcx_fit.py checks
// them in FP32 arithmetic)
constexpr float kErfcxA = 0.49f;
constexpr float kErfcx1 = 0.26611265540122986f;
constexpr float kErfcx2 = 0.36194512248039246f;
constexpr float kErfcx3 = -0.03765244781970978f;
constexpr float kErfcx4 = 0.6230325698852539f;
constexpr float kErfcx5 = -0.2134859561920166f;

// Weights of the regularised Biot-Savart kernel (multipoleKernels.hpp:239-283)
// for two pairs at once, from R^2, w = 1/(2 sigma^2) and s = 1/(sqrt(2) sigma)
// of the source: velocity G = g(rho) / R^3 and half the gradient weight
// A = (w t2 - 1.5 g / R^2) / R^3 (both without the kernel's 1/(4 pi), which the
// caller applies to its sums), rho = R s, g = erf(rho) - t2,
// t2 = (2/sqrt(pi)) rho e^(-rho^2), evaluated as g = 1 - e^(-rho^2) H(rho),
// H = erfcx(rho) + (2/sqrt(pi)) rho, from the exponential t2 needs and the fit
// above (no erf call).  Pairs with rho^2 < 0.25 take the x^3-scaled series
// instead of the cancelling difference (a branch: about one pair in 250 of a
// uniform cloud), and R^2 = 0 (the body itself) gives zero.
__device__ __forceinline__ void p2p_weights2(float2 R2, float2 w, float2 s, float2 &G, float2 &A)
{
  const float2 RS = mul2(R2, w); // rho^2
  const float2 ri = pk(rsqrt_ftz(R2.x), rsqrt_ftz(R2.y));
  const float2 xs = mul2(mul2(R2, ri), s);
  const float2 ea = mul2(RS, pk(-1.44269504088896341f, -1.44269504088896341f));
  const float2 ex = pk(ex2_ftz(ea.x), ex2_ftz(ea.y));
  const float2 u  = fma2(xs, pk(kErfcxA, kErfcxA), pk(1.f, 1.f));
  const float2 t  = pk(rcp_ftz(u.x), rcp_ftz(u.y));
  float2       q  = fma2(pk(kErfcx5, kErfcx5), t, pk(kErfcx4, kErfcx4));
  q               = fma2(q, t, pk(kErfcx3, kErfcx3));
  q               = fma2(q, t, pk(kErfcx2, kErfcx2));
  q               = fma2(q, t, pk(kErfcx1, kErfcx1));
  const float2 kx = mul2(xs, pk(kC2spi, kC2spi));
  const float2 t2 = mul2(kx, ex);
  const float2 gg = fma2(mul2(ex, fma2(q, t, kx)), pk(-1.f, -1.f), pk(1.f, 1.f)); // erf - t2
  const float2 ri2 = mul2(ri, ri);
  const float2 c4  = mul2(ri2, ri);
  G                = mul2(gg, c4);
  A                = mul2(fma2(mul2(gg, ri2), pk(-1.5f, -1.5f), mul2(t2, w)), c4);
  if (RS.x < 0.25f || RS.y < 0.25f) {
    // g / rho^3 and the gradient's (3 g - rho g') / rho^5 as series in
    // rho^2, times (2/sqrt(pi)) s^3 and (2/sqrt(pi)) s^5
    constexpr float kK3 = kC2spi;
    const float     r2[2] = {RS.x, RS.y}, q2[2] = {R2.x, R2.y}, sv[2] = {s.x, s.y};
    float           g2[2] = {G.x, G.y}, a2[2] = {A.x, A.y};
#pragma unroll
    for (int h = 0; h < 2; h++)
      if (r2[h] < 0.25f) {
        const float x = r2[h];
        const float gpoly = ((((((1.f / 5400.f) * x - 1.f / 780.f) * x + 1.f / 132.f) * x - 1.f / 27.f) * x + 1.f / 7.f) * x - 0.4f) * x + 2.f / 3.f;
        const float hpoly = ((((((-1.f / 6120.f) * x + 1.f / 900.f) * x - 1.f / 156.f) * x + 1.f / 33.f) * x - 1.f / 9.f) * x + 2.f / 7.f) * x - 0.4f;
        const float s3 = sv[h] * sv[h] * sv[h];
        g2[h]          = q2[h] != 0.f ? gpoly * kK3 * s3 : 0.f;
        a2[h]          = q2[h] != 0.f ? hpoly * kK3 * s3 * sv[h] * sv[h] : 0.f;
      }
    G = pk(g2[0], g2[1]);
    A = pk(a2[0], a2[1]);
  }
}

// two-sum: hi + lo accumulates v without losing its low-order bits
__device__ __forceinline__ void two_sum_add(float &hi, float &lo, float v)
{
  const float s  = hi + v;
  const float bb = s - hi;
  const float e  = (hi - (s - bb)) + (v - bb);
  hi             = s;
  lo += e;
}

// One block (128 threads) per target leaf.  Each thread works for one target
// t of the chunk (nt targets) as member g of its G or G - 1 members (G =
// ceil(128 / nt)); lanes are ordered so that a warp serves targets with the
// same member count where it can:
//  * far field: member g evaluates the columns m = g, g+G, ... of the leaf's
//    derivative expansions at the target;
//  * near field: the bodies of the leaf's P2P source leaves are staged in
//    shared memory as one flat sequence of body pairs in coordinates relative
//    to the target leaf's centre (each source leaf's centre offset computed
//    once, in FP64), and member g takes every G-th pair, both bodies at once in
//    packed FP32; groups of 16 pairs are summed in FP32 (per body of a pair).
// Everything is folded into a two-sum (float-float) accumulator, the G members
// are combined in a fixed order, and the result becomes FP64 for the
// stretching epilogue.  All lanes run the same trip counts.
// MODE 0 does both fields.  The split form runs the near field (MODE 1, which
// needs no local expansion) beside the tensor-core M2L and stores each body's
// combined near-field sum as a float-float pair in a.near32; MODE 2 then
// evaluates the far field, adds it to that pair member by member, and runs
// the epilogue.
template <int P, int CH_, int MODE = 0>
__global__ void __launch_bounds__(128, L2P32Sizes<P, CH_, MODE>::BLOCKS) k_l2p_p2p32(DevMixed a, double *out)
{
  using S = L2P32Sizes<P, CH_, MODE>;
  constexpr int K = S::K, K1 = S::K1, K2 = S::K2, CH = S::CH, LG = 128;
  constexpr int D1 = P - 1, D2 = P - 2;
  extern __shared__ float4 smem32[];
  float4 *Sq   = smem32;   // staged source pairs, five float4 per pair of bodies
  float4 *Loff = Sq + S::SQ4;      // per source leaf of the current group: centre offset, w = body start (int bits)
  int    *Lcnt = reinterpret_cast<int *>(Loff + LG);
  __shared__ int Lpre[LG + 1]; // exclusive prefix of Lcnt over the group; Lpre[ng] = the group's bodies
  static_assert(CH % 128 == 0, "every thread stages the same number of chunk elements");
  zf     *Lc   = reinterpret_cast<zf *>(Lcnt + LG);
  zf     *U    = Lc + 3 * K;
  zf     *JJ   = U + 3 * K1;
  float  *rhi  = reinterpret_cast<float *>(Sq); // [128][12] partial sums (hi), reusing the staging buffer
  float  *rlo  = rhi + 128 * 12;                // [128][12] partial sums (lo)
  (void)K1;
  (void)K2;
  const float inv4pi = kInv4pi;

  for (int li = blockIdx.x; li < a.nleaves; li += gridDim.x) {
    const int    c = a.leaf_cells[li];
    const int    b0 = a.cv.body[c], nb = a.cv.nbody[c];
    const int    lev = a.cv.level[c];
    const float  iR  = (float)(a.iR0 * exp2i(lev)); // = ldexp(iR0, lev): a power-of-two scaling, exact
    const int    q0 = MODE == 2 ? 0 : a.p2p_start[c], q1 = MODE == 2 ? 0 : a.p2p_start[c + 1];
    __syncthreads();
    for (int e = threadIdx.x; MODE != 1 && e < 3 * K; e += 128) {
      const int     n = __ldg(&kTriNM.n[e / 3]), m = __ldg(&kTriNM.m[e / 3]);
      const double2 v = a.L[(size_t)c * 3 * K + e];
      const double  s = cell_Rpow(a, lev, n); // scaled local Lt = L R^n
      Lc[e]           = {(float)(v.x * s), (float)(v.y * s)};
    }
    __syncthreads();
    // component-major (a warp's lanes mostly share the derivative axis, and
    // so the branches of deriv_coef32); each entry's arithmetic as before
    if (D1 > 0 && MODE != 1)
      for (int e = threadIdx.x; e < 3 * nterms(D1); e += 128) {
        const int ax = e / K1, idx = e % K1; // K1 = nterms(D1)
        const int n = __ldg(&kTriNM.n[idx]), mu = __ldg(&kTriNM.m[idx]);
        const int b1 = (ax + 1) % 3, c1 = (ax + 2) % 3;
        const zf  p = deriv_coef32(Lc, n, mu, b1, 3, c1), q = deriv_coef32(Lc, n, mu, c1, 3, b1);
        U[idx * 3 + ax] = {inv4pi * (p.r - q.r), inv4pi * (p.i - q.i)};
      }
    __syncthreads();
    if (D2 > 0 && MODE != 1)
      for (int e = threadIdx.x; e < 9 * nterms(D2); e += 128) {
        const int ae = e / K2, idx = e % K2, ax = ae / 3, ex = ae % 3; // K2 = nterms(D2) here
        const int n = __ldg(&kTriNM.n[idx]), mu = __ldg(&kTriNM.m[idx]);
        JJ[idx * 9 + ae] = deriv_coef32(U, n, mu, ex, 3, ax);
      }
    __syncthreads();

    for (int tc = 0; tc < nb; tc += 128) {
      // every thread works: the first `full` targets of the chunk have G members,
      // the others G - 1; member g of target tt takes every Gt-th column / source
      const int nt = min(128, nb - tc);
      const int G = (128 + nt - 1) / nt, full = 128 - (G - 1) * nt;
      // With at most five members per target (26 or more targets), lanes
      // 0 .. full G - 1 serve the targets with G members and the others the
      // targets with G - 1, so that a warp's lanes mostly share a trip count
      // (a 32-body leaf: 96% of the near-field lane slots busy instead of
      // 88%).  With more members per target a warp would then read too many
      // different staged pairs, and lane l serves target l % nt as member
      // l / nt.  Member g of target tt keeps partial-sum slot g nt + tt.
      int tt, g;
      if (G > 5 || full == nt) {
        tt = threadIdx.x % nt;
        g  = threadIdx.x / nt;
      } else if (threadIdx.x < full * G) {
        tt = threadIdx.x % full;
        g  = threadIdx.x / full;
      } else {
        const int l = threadIdx.x - full * G;
        tt          = full + l % (nt - full);
        g           = l / (nt - full);
      }
      const int  Gt = tt < full ? G : G - 1, slot = g * nt + tt;
      const bool active = g < Gt;
      float      hi[12], lo[12];
      for (int k = 0; k < 12; k++)
        hi[k] = lo[k] = 0.f;
      float4 pt = make_float4(0.f, 0.f, 0.f, 0.f);
      if (active)
        pt = a.pos32[b0 + tc + tt];
      if (active && MODE != 1) {
        // far field: columns m = g, g + G, ... (u scaled by 1/R, J by 1/R^2)
        const float x = pt.x * iR, y = pt.y * iR, z = pt.z * iR;
        const float r2 = x * x + y * y + z * z;
        float       f[12];
        for (int k = 0; k < 12; k++)
          f[k] = 0.f;
        zf  diag{1.f, 0.f};
        int turn = g; // this member evaluates the columns m with m = g (mod Gt)
        for (int m = 0; m < D1; m++, turn--) {
          if (m > 0) {
            const float sc = kHarmRecipF.s[m];
            diag           = {(diag.r * x - diag.i * y) * sc, (diag.r * y + diag.i * x) * sc};
          }
          if (turn != 0)
            continue;
          turn          = Gt;
          const float w = m == 0 ? 1.f : 2.f;
          zf          ya = diag, yb{0.f, 0.f};
          float       tn = float(2 * m + 1); // 2n + 1
          for (int n = m; n < D1; n++, tn += 2.f) {
            const int t = tri(n, m);
            for (int ax = 0; ax < 3; ax++) {
              const zf u = U[t * 3 + ax];
              f[ax] += w * (u.r * ya.r - u.i * ya.i);
            }
            if (n < D2)
              for (int ae = 0; ae < 9; ae++) {
                const zf u = JJ[t * 9 + ae];
                f[3 + ae] += w * (u.r * ya.r - u.i * ya.i);
              }
            const float cc = kHarmRecipF.c[t];
            const float zz = tn * z;
            const zf    nx = {cc * (zz * ya.r + r2 * yb.r), cc * (zz * ya.i + r2 * yb.i)};
            yb             = ya;
            ya             = nx;
          }
        }
        for (int k = 0; k < 3; k++)
          two_sum_add(hi[k], lo[k], f[k] * iR);
        for (int k = 3; k < 12; k++)
          two_sum_add(hi[k], lo[k], f[k] * (iR * iR));
      }
      // near field, source leaves in groups of LG
      for (int qg = q0; qg < q1; qg += LG) {
        const int ng = min(LG, q1 - qg);
        __syncthreads();
        if (threadIdx.x < ng) {
          const int sc      = a.p2p_src[qg + threadIdx.x];
          Loff[threadIdx.x] = make_float4((float)(a.cv.x[sc] - a.cv.x[c]), (float)(a.cv.y[sc] - a.cv.y[c]), (float)(a.cv.z[sc] - a.cv.z[c]),
                                          __int_as_float(a.cv.body[sc]));
          Lcnt[threadIdx.x] = a.cv.nbody[sc];
        }
        __syncthreads();
        if (threadIdx.x < 32) { // warp 0: exclusive prefix of the group's body counts, four per lane
          const int l = threadIdx.x;
          int       c[4], sum = 0;
#pragma unroll
          for (int u = 0; u < 4; u++) {
            c[u] = 4 * l + u < ng ? Lcnt[4 * l + u] : 0;
            sum += c[u];
          }
          int incl = sum;
#pragma unroll
          for (int d = 1; d < 32; d <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, d);
            if (l >= d)
              incl += v;
          }
          int run = incl - sum;
#pragma unroll
          for (int u = 0; u < 4; u++) {
            if (4 * l + u < ng)
              Lpre[4 * l + u] = run;
            run += c[u];
          }
          if (l == 31)
            Lpre[ng] = incl;
        }
        __syncthreads();
        // The group's source bodies as one sequence (leaf by leaf) cut into
        // chunks of CH, staged as pairs of consecutive bodies: pair k is four
        // five float4, {-x, -y}, {-z, s}, {alpha_x, alpha_y}, {alpha_z, -alpha_x},
        // {-alpha_y, -alpha_z} of bodies 2k and 2k + 1 (each float2 = the two
        // bodies), positions relative to the target leaf's centre,
        // s = 1/(sqrt(2) sigma) (and 1/(2 sigma^2) = s^2); both signs of alpha
        // make each cross-product component one multiply and one FMA.  Element
        // e = tid + 128 i finds its leaf by binary search over Lpre, loads its
        // body, and swaps words with lane e ^ 1, so that the even lane stores
        // the pair's float4 0, 1, 4 and the odd lane float4 2, 3.  An odd count
        // is padded with a body of zero strength far away, whose terms are
        // exactly zero.
        const int total = Lpre[ng];
        for (int c0 = 0; c0 < total; c0 += CH) {
          const int cnt = min(CH, total - c0), npair = (cnt + 1) >> 1;
          const bool odd = threadIdx.x & 1;
#pragma unroll
          for (int i = 0; i < CH / 128; i++) {
            const int e  = threadIdx.x + 128 * i;
            float     nx = 1e3f, ny = 1e3f, nz = 1e3f, sv = 1.f, ax = 0.f, ay = 0.f, az = 0.f;
            if (e < cnt) {
              const int g = c0 + e;
              int       lb = 0, ub = ng - 1; // the last leaf with Lpre <= g
              while (lb < ub) {
                const int mid = (lb + ub + 1) >> 1;
                if (Lpre[mid] <= g)
                  lb = mid;
                else
                  ub = mid - 1;
              }
              const float4 o  = Loff[lb];
              const int    bi = __float_as_int(o.w) + (g - Lpre[lb]);
              const float4 p = __ldg(a.pos32 + bi), q = __ldg(a.alp32 + bi);
              nx = -(p.x + o.x);
              ny = -(p.y + o.y);
              nz = -(p.z + o.z);
              sv = q.w * kIsq2;
              ax = q.x;
              ay = q.y;
              az = q.z;
            }
            const float v0 = __shfl_xor_sync(0xffffffffu, odd ? nx : ax, 1);
            const float v1 = __shfl_xor_sync(0xffffffffu, odd ? ny : ay, 1);
            const float v2 = __shfl_xor_sync(0xffffffffu, odd ? nz : az, 1);
            const float v3 = __shfl_xor_sync(0xffffffffu, odd ? sv : -ax, 1);
            const float v4 = __shfl_xor_sync(0xffffffffu, -ay, 1);
            const float v5 = __shfl_xor_sync(0xffffffffu, -az, 1);
            const int   k  = e >> 1;
            if (k < npair) {
              if (!odd) {
                Sq[5 * k]     = make_float4(nx, v0, ny, v1);
                Sq[5 * k + 1] = make_float4(nz, v2, sv, v3);
                Sq[5 * k + 4] = make_float4(-ay, v4, -az, v5);
              } else {
                Sq[5 * k + 2] = make_float4(v0, ax, v1, ay);
                Sq[5 * k + 3] = make_float4(v2, az, v3, -ax);
              }
            }
          }
          __syncthreads();
          if (active) {
            const float2 px = pk(pt.x, pt.x), py = pk(pt.y, pt.y), pz = pk(pt.z, pt.z);
            for (int k0 = g; k0 < npair; k0 += 16 * Gt) {
              // velocity V, G alpha (E) and half the gradient's A-part (J),
              // each as two FP32 partial sums (one per body of a pair)
              float2 V0{0.f, 0.f}, V1{0.f, 0.f}, V2{0.f, 0.f}, E0{0.f, 0.f}, E1{0.f, 0.f}, E2{0.f, 0.f};
              float2 J[8];
#pragma unroll
              for (int u = 0; u < 8; u++)
                J[u] = pk(0.f, 0.f);
              const int kend = min(npair, k0 + 16 * Gt);
              for (int k = k0; k < kend; k += Gt) {
                const float4 f0 = Sq[5 * k], f1 = Sq[5 * k + 1], f2 = Sq[5 * k + 2], f3 = Sq[5 * k + 3], f4 = Sq[5 * k + 4];
                const float2 dx = add2(px, pk(f0.x, f0.y)), dy = add2(py, pk(f0.z, f0.w)), dz = add2(pz, pk(f1.x, f1.y));
                const float2 ax = pk(f2.x, f2.y), ay = pk(f2.z, f2.w), az = pk(f3.x, f3.y);
                const float2 R2 = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
                const float2 sv = pk(f1.z, f1.w);
                float2       G, A;
                p2p_weights2(R2, mul2(sv, sv), sv, G, A);
                const float2 c0 = fma2(dz, pk(f4.x, f4.y), mul2(dy, az)); // d x alpha
                const float2 c1 = fma2(dx, pk(f4.z, f4.w), mul2(dz, ax));
                const float2 c2 = fma2(dy, pk(f3.z, f3.w), mul2(dx, ay));
                V0              = fma2(G, c0, V0);
                V1              = fma2(G, c1, V1);
                V2              = fma2(G, c2, V2);
                E0              = fma2(G, ax, E0);
                E1              = fma2(G, ay, E1);
                E2              = fma2(G, az, E2);
                const float2 a0 = mul2(A, c0), a1 = mul2(A, c1), a2 = mul2(A, c2);
                J[0]            = fma2(a0, dx, J[0]);
                J[1]            = fma2(a0, dy, J[1]);
                J[2]            = fma2(a0, dz, J[2]);
                J[3]            = fma2(a1, dx, J[3]);
                J[4]            = fma2(a1, dy, J[4]);
                J[5]            = fma2(a1, dz, J[5]);
                J[6]            = fma2(a2, dx, J[6]);
                J[7]            = fma2(a2, dy, J[7]);
              }
              // velocity (0..2) and gradient (3..11, J[a][b] at 3 + 3a + b):
              // J[a][b] = 2 J_ab + the G alpha terms of the kernel's
              // antisymmetric part, all times 1/(4 pi); the A-part is
              // trace-free ((d x alpha) . d = 0), so J_22 = -(J_00 + J_11); the
              // near field enters with a minus sign
              const float ex = kInv4pi * (E0.x + E0.y), ey = kInv4pi * (E1.x + E1.y), ez = kInv4pi * (E2.x + E2.y);
              float       v[12];
              v[0] = kInv4pi * (V0.x + V0.y);
              v[1] = kInv4pi * (V1.x + V1.y);
              v[2] = kInv4pi * (V2.x + V2.y);
#pragma unroll
              for (int u = 0; u < 8; u++)
                v[3 + u] = (2.f * kInv4pi) * (J[u].x + J[u].y);
              v[11] = -(v[3] + v[7]);
              v[4] += ez;
              v[5] -= ey;
              v[6] -= ez;
              v[8] += ex;
              v[9] += ey;
              v[10] -= ex;
#pragma unroll
              for (int u = 0; u < 12; u++)
                two_sum_add(hi[u], lo[u], -v[u]);
            }
          }
          __syncthreads();
        }
      }
      __syncthreads(); // staging buffer free: reuse it for the partial sums
#pragma unroll
      for (int k = 0; k < 12; k++) {
        rhi[slot * 12 + k] = hi[k];
        rlo[slot * 12 + k] = lo[k];
      }
      __syncthreads();
      if (MODE == 1) { // the members' near-field sums combined in a fixed order, per body and component
        for (int w = threadIdx.x; w < 12 * nt; w += 128) {
          const int t = w / 12, k = w % 12, Gm = t < full ? G : G - 1;
          float     h = 0.f, l = 0.f;
          for (int gg = 0; gg < Gm; gg++) {
            two_sum_add(h, l, rhi[(gg * nt + t) * 12 + k]);
            l += rlo[(gg * nt + t) * 12 + k];
          }
          float *dst = a.near32 + (size_t)(b0 + tc + t) * 24;
          dst[k]      = h;
          dst[12 + k] = l;
        }
      }
      // Four adjacent lanes per target (item w = 4 t + q): q = 0 combines the
      // velocity, q = 1..3 the three gradient entries that make dadt component
      // q - 1 (column q - 1 of J for the transposed scheme, row q - 1 for the
      // classic one) and that component; the rVPM correction's dot product is
      // summed over the four lanes.  Every lane runs the same trip count.
      for (int w0 = 0; MODE != 1 && w0 < 4 * nt; w0 += 128) {
        const int  w = w0 + threadIdx.x, q = w & 3;
        const bool ok = w < 4 * nt;
        const int  t = ok ? w >> 2 : 0, b = b0 + tc + t, Gm = t < full ? G : G - 1;
        int        comp[3];
#pragma unroll
        for (int c = 0; c < 3; c++)
          comp[c] = q == 0 ? c : (a.stretching == VFMM_TRANSPOSED ? 3 + 3 * c + (q - 1) : 3 + 3 * (q - 1) + c);
        double r3[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
          float h = 0.f, l = 0.f;
          if (MODE == 2) { // the body's near-field sum first, then the members' far-field parts
            h = a.near32[(size_t)b * 24 + comp[c]];
            l = a.near32[(size_t)b * 24 + 12 + comp[c]];
          }
          for (int gg = 0; gg < Gm; gg++) {
            two_sum_add(h, l, rhi[(gg * nt + t) * 12 + comp[c]]);
            l += rlo[(gg * nt + t) * 12 + comp[c]];
          }
          r3[c] = (double)h + (double)l;
        }
        const double al[3] = {a.soa[F_A * a.cap + b], a.soa[(F_A + 1) * a.cap + b], a.soa[(F_A + 2) * a.cap + b]};
        double       da    = q == 0 ? 0. : r3[0] * al[0] + r3[1] * al[1] + r3[2] * al[2];
        double       drdt  = 0.;
        if (a.formulation == VFMM_RVPM) { // one reciprocal square root per lane: FP64 is a narrow pipe here
          const double ina = rsqrt(al[0] * al[0] + al[1] * al[1] + al[2] * al[2]);
          const double ah  = q == 0 ? 0. : al[q - 1] * ina;
          double       dot = da * ah;
          dot += __shfl_xor_sync(0xffffffffu, dot, 1);
          dot += __shfl_xor_sync(0xffffffffu, dot, 2);
          if (q == 0)
            drdt = -1.0 / 5.0 * a.soa[F_R * a.cap + b] * ina * dot;
          else
            da -= 3. / 5. * dot * ah;
        }
        if (ok) {
#pragma unroll
          for (int c = 0; c < 3; c++)
            out[((q == 0 ? F_U : F_J) + comp[c] - (q == 0 ? 0 : 3)) * a.cap + b] = r3[c];
          if (q == 0)
            out[F_DRDT * a.cap + b] = drdt;
          else
            out[(F_DADT + q - 1) * a.cap + b] = da;
        }
      }
    }
  }
}

// ------------------------------------------------------------------ host side
static DevMixed dev_mixed(const ExpArgs &e, const MixedArgs &m)
{
  DevMixed d;
  d.cv          = e.cells;
  d.soa         = e.soa;
  d.cap         = e.cap;
  d.M           = e.M;
  d.L           = e.L;
  d.Mp          = m.Mp32;
  d.pos32       = m.pos32;
  d.alp32       = m.alp32;
  d.leaf_cells  = e.leaf_cells;
  d.nleaves     = e.nleaves;
  d.m2l_start   = e.m2l_start;
  d.m2l_src     = e.m2l_src;
  d.p2p_start   = e.p2p_start;
  d.p2p_src     = e.p2p_src;
  d.items       = m.items32;
  (void)m.lanes32;
  d.R0          = m.R0;
  d.iR0         = 1.0 / m.R0;
  d.R0pow[0] = d.iR0pow[0] = 1.0;
  for (int n = 1; n <= PMAX; n++) {
    d.R0pow[n]  = d.R0pow[n - 1] * m.R0;
    d.iR0pow[n] = d.iR0pow[n - 1] * d.iR0;
  }
  d.stretching  = e.stretching;
  d.formulation = e.formulation;
  d.Bhi         = m.Bhi;
  d.Blo         = m.Blo;
  d.near32      = m.near32;
  return d;
}

template <int P>
static void p2m32_P(cudaStream_t s, const ExpArgs &e, const MixedArgs &m)
{
  DevMixed     d     = dev_mixed(e, m);
  const size_t bytes = (size_t)32 * nterms(P) * sizeof(zf) + 32 * 3 * sizeof(float);
  if (e.nleaves > 0) {
    k_prep_bodies<<<std::min((e.nleaves + 3) / 4, 152 * 16), 128, 0, s>>>(d);
    count_launch();
    k_p2m32<P><<<std::min(e.nleaves, 152 * 16), 64, bytes, s>>>(d);
    count_launch();
  }
  VFMM_LAUNCH_CHECK();
}

template <int P, int SB>
static void m2l32_launch(cudaStream_t s, const DevMixed &d, const ExpArgs &e, const MixedArgs &m)
{
  const size_t bytes = M2LV2<P, SB>::bytes;
  VFMM_SMEM_ONCE(bytes, k_m2l32v2<P, SB>);
  if (e.ncells > 0) {
    k_m2l32v2<P, SB><<<std::min(e.ncells, 152 * 8), P * 32, bytes, s>>>(d, m.lanes32, e.ncells);
    count_launch();
  }
}

template <int P>
static void m2l32_P(cudaStream_t s, const ExpArgs &e, const MixedArgs &m)
{
  DevMixed  d  = dev_mixed(e, m);
  const int PP = P * P;
  (void)PP; // the folded FP32 multipoles were written by P2M and M2M
  if (m.m2l_batch == 32)
    m2l32_launch<P, 32>(s, d, e, m);
  else if (m.m2l_batch == 30)
    m2l32_launch<P, 30>(s, d, e, m);
  else if (m.m2l_batch == 24)
    m2l32_launch<P, 24>(s, d, e, m);
  else if (m.m2l_batch == 8)
    m2l32_launch<P, 8>(s, d, e, m);
  else
    m2l32_launch<P, 16>(s, d, e, m);
  VFMM_LAUNCH_CHECK();
}

template <int P, int CH, int MODE = 0>
static void l2p32_launch(cudaStream_t s, const DevMixed &d, const ExpArgs &e, double *out)
{
  const size_t bytes = L2P32Sizes<P, CH, MODE>::bytes;
  VFMM_SMEM_ONCE(bytes, k_l2p_p2p32<P, CH, MODE>);
  if (MODE == 1)
    VFMM_CARVEOUT_MAX_ONCE(k_l2p_p2p32<P, CH, MODE>);
  if (e.nleaves > 0) {
    k_l2p_p2p32<P, CH, MODE><<<std::min(e.nleaves, 152 * 16), 128, bytes, s>>>(d, out);
    count_launch();
  }
}

template <int P>
static void l2p32_P(cudaStream_t s, const ExpArgs &e, const MixedArgs &m, double *out)
{
  DevMixed d = dev_mixed(e, m);
  if (m.p2p_chunk == 512)
    l2p32_launch<P, 512>(s, d, e, out);
  else
    l2p32_launch<P, 768>(s, d, e, out);
  VFMM_LAUNCH_CHECK();
}

// The split leaf kernel (the orders of the tensor-core M2L): MODE 1 near
// field into m.near32, MODE 2 far field plus that sum and the epilogue.
template <int P, int MODE>
static void l2p32_split_P(cudaStream_t s, const ExpArgs &e, const MixedArgs &m, double *out)
{
  DevMixed d = dev_mixed(e, m);
  if (!m.near32)
    throw Error(VFMM_ERR_INVALID, "split leaf kernel without its near-field buffer");
  if (m.p2p_chunk == 512)
    l2p32_launch<P, 512, MODE>(s, d, e, out);
  else
    l2p32_launch<P, 768, MODE>(s, d, e, out);
  VFMM_LAUNCH_CHECK();
}

// M2M into parents at levels maxLevel-1 .. 1 (level 0 skipped as in the
// reference's upward pass, fmmCalculator.hpp:427); L2L from parents at levels
// 0 .. maxLevel-1.
template <int P>
static void m2m32_P(cudaStream_t s, const ExpArgs &e, const MixedArgs &m)
{
  const DevMixed d     = dev_mixed(e, m);
  const size_t   bytes = (size_t)(8 * 3 + 8) * nterms(P) * sizeof(zf);
  VFMM_SMEM_ONCE(bytes, k_m2m32<P>);
  for (int l = e.maxLevel - 1; l >= 1; l--) {
    const int n0 = e.level_start_host[l], n1 = e.level_start_host[l + 1];
    if (n1 > n0) {
      k_m2m32<P><<<std::min(n1 - n0, 152 * 16), 128, bytes, s>>>(d, e.level_cells + n0, n1 - n0);
      count_launch();
    }
  }
  VFMM_LAUNCH_CHECK();
}

template <int P>
static void l2l32_P(cudaStream_t s, const ExpArgs &e, const MixedArgs &m)
{
  const DevMixed d     = dev_mixed(e, m);
  const size_t   bytes = (size_t)(3 + 8) * nterms(P) * sizeof(zf);
  VFMM_SMEM_ONCE(bytes, k_l2l32<P>);
  for (int l = 0; l < e.maxLevel; l++) {
    const int n0 = e.level_start_host[l], n1 = e.level_start_host[l + 1];
    if (n1 > n0) {
      k_l2l32<P><<<std::min(n1 - n0, 152 * 16), 128, bytes, s>>>(d, e.level_cells + n0, n1 - n0);
      count_launch();
    }
  }
  VFMM_LAUNCH_CHECK();
}

#define VFMM_DISPATCH_M(fn, ...)                                                                                                 \
  switch (e.P) {                                                                                                                \
  case 2: fn<2>(__VA_ARGS__); break;                                                                                            \
  case 3: fn<3>(__VA_ARGS__); break;                                                                                            \
  case 4: fn<4>(__VA_ARGS__); break;                                                                                            \
  case 5: fn<5>(__VA_ARGS__); break;                                                                                            \
  case 6: fn<6>(__VA_ARGS__); break;                                                                                            \
  case 7: fn<7>(__VA_ARGS__); break;                                                                                            \
  case 8: fn<8>(__VA_ARGS__); break;                                                                                            \
  case 9: fn<9>(__VA_ARGS__); break;                                                                                            \
  case 10: fn<10>(__VA_ARGS__); break;                                                                                          \
  case 11: fn<11>(__VA_ARGS__); break;                                                                                          \
  case 12: fn<12>(__VA_ARGS__); break;                                                                                          \
  case 13: fn<13>(__VA_ARGS__); break;                                                                                          \
  case 14: fn<14>(__VA_ARGS__); break;                                                                                          \
  case 15: fn<15>(__VA_ARGS__); break;                                                                                          \
  case 16: fn<16>(__VA_ARGS__); break;                                                                                          \
  default: throw Error(VFMM_ERR_UNSUPPORTED, "expansion order p must be in 2..16");                                            \
  }

void p2m_mixed(cudaStream_t s, const ExpArgs &e, const MixedArgs &m) { VFMM_DISPATCH_M(p2m32_P, s, e, m) }
void m2l_mixed(cudaStream_t s, const ExpArgs &e, const MixedArgs &m)
{
  if (m.tc)
    m2l_tensor(s, e, m);
  else
    VFMM_DISPATCH_M(m2l32_P, s, e, m)
}
void m2m_mixed(cudaStream_t s, const ExpArgs &e, const MixedArgs &m) { VFMM_DISPATCH_M(m2m32_P, s, e, m) }
void l2l_mixed(cudaStream_t s, const ExpArgs &e, const MixedArgs &m) { VFMM_DISPATCH_M(l2l32_P, s, e, m) }
void l2p_p2p_mixed(cudaStream_t s, const ExpArgs &e, const MixedArgs &m, double *out) { VFMM_DISPATCH_M(l2p32_P, s, e, m, out) }
void l2p_p2p_mixed_split(cudaStream_t s, const ExpArgs &e, const MixedArgs &m, double *out, int mode)
{
  if (mode != 1 && mode != 2)
    throw Error(VFMM_ERR_INVALID, "split leaf kernel: mode must be 1 (near) or 2 (far)");
  switch (e.P) {
  case 8: mode == 1 ? l2p32_split_P<8, 1>(s, e, m, out) : l2p32_split_P<8, 2>(s, e, m, out); break;
  case 9: mode == 1 ? l2p32_split_P<9, 1>(s, e, m, out) : l2p32_split_P<9, 2>(s, e, m, out); break;
  case 10: mode == 1 ? l2p32_split_P<10, 1>(s, e, m, out) : l2p32_split_P<10, 2>(s, e, m, out); break;
  default: throw Error(VFMM_ERR_UNSUPPORTED, "the split leaf kernel serves p = 8..10");
  }
}

} // namespace vfmm
