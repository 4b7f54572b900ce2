// Internal declarations shared by the vfmm CUDA translation units.
#pragma once
#include <cuda_runtime.h>
#include <atomic>
#include <mutex>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>
#include "../../include/vfmm.h"

namespace vfmm {

// Tree depth limit: a 63-bit key holds 21 octant digits.
constexpr int MAXL = 21;
constexpr int PMIN = 2, PMAX = 16;
constexpr int NCRIT_MAX = 256;

// Body fields in device memory, field-major (field f of body i at
// f*cap + i), in the order of exafmm::Body (exafmmTypes.hpp:18-32) so that the
// 296-byte records transpose directly.
enum BodyField {
  F_J = 0, // 9: J[a][b] at F_J + 3a + b
  F_X = 9,
  F_A = 12,
  F_U = 15,
  F_DADT = 18,
  F_VOLD = 21,
  F_DOLD = 24,
  F_XOLD = 27,
  F_AOLD = 30,
  F_R = 33,
  F_DRDT = 34,
  F_ROLD = 35,
  F_DRDTOLD = 36,
  NFIELD = 37
};

// Device-side scalars of one tree build and evaluation.  Counters are
// written by kernels and read back by the host at the two sync points of a
// stage (after node enumeration, after traversal).
struct DevInfo {
  double   X0[3];
  double   R0;
  int      err;         // VFMM_ERR_* raised by a kernel
  int      nnodes;      // cells of the tree
  int      nleaves;
  int      maxLevel;
  int      front_n[3];  // traversal frontier sizes (ring of three: in, out, next out)
  int      n_p2p, n_m2l;
  int      overflow;    // 1 if a capacity was exceeded
  int      nonfinite;   // 1 if an input was NaN/Inf
  unsigned long long p2p_interactions;
  int      deeper;      // 1 if a cell at the key depth holds more than ncrit bodies (keys too short)
  int      pad[4];
};

// Cells in the reference's order (tree.hpp:29-99), structure of arrays.
struct CellsView {
  int    *nchild, *nbody, *child, *body, *level, *parent;
  double *x, *y, *z, *R;
};

// Launch bookkeeping (kernel count for instrumentation).
extern thread_local unsigned long long *g_launch_counter;
inline void count_launch()
{
  if (g_launch_counter)
    (*g_launch_counter)++;
}

#define VFMM_CUDA_TRY(expr)                                                                            \
  do {                                                                                                 \
    cudaError_t e_ = (expr);                                                                           \
    if (e_ != cudaSuccess) {                                                                           \
      throw ::vfmm::Error(VFMM_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_));         \
    }                                                                                                  \
  } while (0)

#define VFMM_LAUNCH_CHECK() VFMM_CUDA_TRY(cudaGetLastError())

struct Error {
  int         code;
  std::string msg;
  Error(int c, std::string m) : code(c), msg(std::move(m)) {}
};

// Raise a kernel's dynamic shared-memory limit once per device.  The
// attribute belongs to the device that is current when it is set, and handles
// on different GPUs may share a process (vfmm_config.device), so each call
// site keeps one flag per device ordinal; a mutex makes the first setting
// thread-safe (vfmm_advance_batch runs systems on a thread pool).  The kernel
// comes last so that template arguments may contain commas.
struct PerDeviceOnce {
  static constexpr int NDEV = 64;
  std::mutex           mu;
  std::atomic<bool>    done[NDEV] = {};
  template <class F>
  void run(F &&f)
  {
    int dev = 0;
    VFMM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NDEV) { // beyond the table: set it every time (cheap)
      VFMM_CUDA_TRY(f());
      return;
    }
    if (done[dev].load(std::memory_order_acquire))
      return;
    std::lock_guard<std::mutex> lock(mu);
    if (done[dev].load(std::memory_order_relaxed))
      return;
    VFMM_CUDA_TRY(f());
    done[dev].store(true, std::memory_order_release);
  }
};

#define VFMM_SMEM_ONCE(bytes, ...)                                                                              \
  do {                                                                                                          \
    static ::vfmm::PerDeviceOnce vfmm_once_;                                                                    \
    vfmm_once_.run([&]() { return cudaFuncSetAttribute(__VA_ARGS__, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                                       (int)(bytes)); });                                        \
  } while (0)

// The shared-memory carveout of a kernel that shares its SMs with another
// one: the largest shared-memory configuration, so that a tensor M2L block
// and a leaf block fit on one SM together.
#define VFMM_CARVEOUT_MAX_ONCE(...)                                                                              \
  do {                                                                                                          \
    static ::vfmm::PerDeviceOnce vfmm_once_;                                                                    \
    vfmm_once_.run([&]() { return cudaFuncSetAttribute(__VA_ARGS__, cudaFuncAttributePreferredSharedMemoryCarveout, \
                                                       (int)cudaSharedmemCarveoutMaxShared); });                 \
  } while (0)


// Grow-only device buffer.
template <class T>
struct DevBuf {
  T     *p   = nullptr;
  size_t cap = 0;
  void   reserve(size_t n)
  {
    if (n <= cap)
      return;
    if (p)
      cudaFree(p);
    p   = nullptr;
    cap = 0;
    size_t want = n + n / 4 + 64;
    VFMM_CUDA_TRY(cudaMalloc((void **)&p, want * sizeof(T)));
    cap = want;
  }
  void release()
  {
    if (p)
      cudaFree(p);
    p   = nullptr;
    cap = 0;
  }
};

inline int grid_for(long n, int block, int maxBlocks = 152 * 16)
{
  long g = (n + block - 1) / block;
  if (g < 1)
    g = 1;
  if (g > maxBlocks)
    g = maxBlocks;
  return (int)g;
}

// ---- tree.cu
struct TreeScratch {
  DevBuf<uint64_t> keys, skeys;
  DevBuf<uint32_t> idx, sidx, perm;
  DevBuf<int>      lvl, lo, hi, cnt, off;
  DevBuf<int>      nlevel, nstart, ncount, nparent, nchild, nrank, nref, nbs, nsortidx, nsortlvl, nflag, noff;
  DevBuf<double>   bbox_part;
  DevBuf<unsigned char> cub_tmp;
  size_t           cub_bytes = 0;
};
void tree_bounds(cudaStream_t s, const double *X, size_t cap, int n, DevInfo *info, TreeScratch &ts);
void bbox_partial_into(cudaStream_t s, const double *x, const double *y, const double *z, int n, double *part, int nb);
void tree_sort_bodies(cudaStream_t s, const double *X, size_t cap, int n, int ncrit, int levels, DevInfo *info, TreeScratch &ts);
// false (nothing built) when the keys were too short for the tree: a cell at
// their depth holds more than ncrit bodies
bool tree_build_cells(cudaStream_t s, int n, int ncrit, int nnodes, DevInfo *info, TreeScratch &ts, CellsView cv, int *level_cells,
                      int *level_start, int *leaf_cells);

// ---- traverse.cu
struct ListScratch {
  DevBuf<int2>               front[2];
  DevBuf<unsigned long long> p2p_raw, m2l_raw, p2p_sorted, m2l_sorted;
  DevBuf<unsigned char>      cub_tmp;
  size_t                     cub_bytes = 0;
  int                        key_bits  = 32; // pair key = target << key_bits | source
};
void traverse(cudaStream_t s, CellsView tc, CellsView sc, int ntc, int nsc, int maxLevelT, int maxLevelS, double theta, DevInfo *info,
              ListScratch &ls, size_t cap_front, size_t cap_p2p, size_t cap_m2l);
void lists_to_csr(cudaStream_t s, ListScratch &ls, int n_p2p, int n_m2l, int ncells_t, int cell_bits, int *p2p_start, int *p2p_src, int *m2l_start,
                  int *m2l_src, const int *nbody_t, unsigned long long *interactions);
void lists_transpose(cudaStream_t s, ListScratch &ls, int n_p2p, int n_m2l, int ncells_s, unsigned long long *keys, unsigned long long *sorted,
                     int *p2p_start, int *p2p_tgt, int *m2l_start, int *m2l_tgt);

// ---- bodies.cu
// Records to field-major arrays; with a mask, only those fields are read and
// the others are set to NaN.
void aos_to_soa(cudaStream_t s, const double *aos, double *soa, size_t cap, int n, uint64_t mask = ~0ull);
void soa_to_aos(cudaStream_t s, const double *soa, size_t cap, double *aos, int n);
void gather_bodies(cudaStream_t s, const double *src, double *dst, size_t cap, const uint32_t *perm, int n, uint64_t fieldMask);
void check_finite(cudaStream_t s, const double *soa, size_t cap, int n, DevInfo *info);
void reset_rates(cudaStream_t s, double *soa, size_t cap, int n);
// Stage update kernel variants: scheme and stage index select the formula of
// fmmCalculator.hpp:493-711; stretching/formulation complete the rates first.
struct StageArgs {
  int    scheme, stage, stretching, formulation, rk4_fixed, store_initial, do_update;
  int    csm; // add the core-spreading rate before the update (fmmCalculator.hpp:334-337)
  double dt, relax, nu;
};
void finish_and_update(cudaStream_t s, double *soa, size_t cap, int n, const StageArgs &a);
void relax_bodies(cudaStream_t s, double *soa, size_t cap, int n, double f);
void fill_bytes(cudaStream_t s, void *p, size_t bytes, int value);
constexpr int DIAG_SCRATCH = 152 * 2 * 9; // doubles of partial sums for diagnostics()
// out[9] (device) = circulation, linear impulse, angular impulse of the bodies
void diagnostics(cudaStream_t s, const double *soa, size_t cap, int n, double *scratch, double *out);
double fma_probe(cudaStream_t s, bool fp64, void *scratch, int iters, float *ms_out, cudaEvent_t e0, cudaEvent_t e1);

// ---- expansions.cu (FP64 path)
struct ExpArgs {
  int           P;
  CellsView     cells;
  int           ncells;
  const int    *level_cells;
  const int    *level_start_host; // host copy: [MAXL+2]
  int           maxLevel;
  const int    *leaf_cells;
  int           nleaves;
  const double *soa;
  size_t        cap;
  double2      *M, *L, *Mprep;
  const int    *m2l_start, *m2l_src;
  const int    *p2p_start, *p2p_src;
  const int4   *m2l_items; // per-lane schedule, see m2l_schedule
  int           m2l_nitems_per_lane;
  int           stretching, formulation;
  // Sources when they are another tree than the targets (sensors): source
  // cells for M2L and P2P, source bodies for P2P.  src_soa == nullptr means
  // the targets' own cells and bodies.
  CellsView     src_cells;
  const double *src_soa;
  size_t        src_cap;
  // FP64 P2P: per-source-body weights (1/(2 sigma^2), 1/(sqrt(2) sigma)),
  // written by the leaf pass for its nsrc source bodies
  double2      *srcw = nullptr;
  int           nsrc = 0;
};
void upward_pass(cudaStream_t s, const ExpArgs &a); // P2M + M2M (FP64)
void m2m_pass(cudaStream_t s, const ExpArgs &a);    // M2M only (FP64)
void m2l_pass(cudaStream_t s, const ExpArgs &a);
void downward_l2l(cudaStream_t s, const ExpArgs &a);
void l2p_p2p_pass(cudaStream_t s, const ExpArgs &a, double *soa_out);
// Sensor evaluation (FP64): mprep_pass makes the sign-folded multipoles of
// the particle tree (e.M -> e.Mprep over e.ncells); m2l_sensor_pass runs M2L
// into the sensor cells from e.Mprep of e.src_cells; l2p_sensor_pass is the
// sensors' L2P plus velocity-only P2P against e.src_soa.
void mprep_pass(cudaStream_t s, const ExpArgs &a);
void m2l_sensor_pass(cudaStream_t s, const ExpArgs &a);
void l2p_sensor_pass(cudaStream_t s, const ExpArgs &a, double *soa_out);
std::vector<int4> m2l_schedule(int P, int lanes, int kb, int maxItems, int *itemsPerLane);

// ---- mixed.cu (FP32 P2M / M2M / M2L / L2L / L2P+P2P, FP64 expansion arrays)
// Scratch of the tensor-core M2L (m2l_tensor.cu): the sources' multipoles as
// TF32 hi/lo operand rows [cell][3][tc_kp(P)], target tiles and the pairs
// sorted by (tile, offset class).
struct TcScratch {
  DevBuf<float>              B;
  DevBuf<unsigned long long> tkeys, tkeys_sorted, pkeys, pkeys_sorted;
  DevBuf<uint32_t>           pvals, pvals_sorted;
  DevBuf<int>                tile_of, col_of, tile_cells, tile_level, tile_start, meta;
  DevBuf<int4>               coords; // per cell: lattice coordinates (odd integers) and level
  int                        launch_tiles = 0; // tile bound of the prepared evaluation (0: nothing to launch)
  DevBuf<unsigned char>      cub_tmp;
  // operator classes: hash (keys, index per slot), keys by index, index per
  // pair group, operator table for the first `cap` classes; the class count
  // of the last evaluation, copied back asynchronously (pinned), sizes the
  // next table
  DevBuf<unsigned long long> hkeys, cls_of;
  DevBuf<int>                hid, cidq;
  DevBuf<float4>             table;
  int                        cap       = 0;
  int                       *ncls_host = nullptr;
};
// Padded K extent of one component's multipole operand row (P^2 real terms).
__host__ __device__ constexpr int tc_kp(int P) { return (P * P + 7) / 8 * 8; }
// Orders the tensor-core M2L handles: the P(P+1) output rows fit the 128 TMEM lanes.
constexpr int TC_PMIN = 8, TC_PMAX = 10;

struct MixedArgs {
  float2       *Mp32;
  float4       *pos32, *alp32;
  const int4   *items32;
  const int4   *lanes32; // k_m2l32v2 lane table, see m2l_lane_table
  int           m2l_batch; // sources staged per batch in k_m2l32v2 (8, 16 or 32)
  int           p2p_chunk; // near-field sources staged per chunk in the leaf kernel (512 or 768; 0: 768)
  double        R0;
  // tensor-core M2L (null tc: the CUDA-core kernel k_m2l32v2): operand rows
  // written by P2M/M2M, the traversal's sorted (target << key_bits | source)
  // M2L keys, and the device error word of the evaluation
  TcScratch                *tc;
  float                    *Bhi, *Blo;
  const unsigned long long *m2l_keys;
  int                       m2l_key_bits, n_m2l;
  int                      *eval_err;
  float                    *near32 = nullptr; // the split leaf kernel's near-field sums, 24 floats per body
};
// The tensor-core M2L for P in TC_PMIN..TC_PMAX (m2l_tensor.cu): its pre-pass
// (needs the tree and lists only; zeroes the local expansions), the kernel
// (needs the pre-pass and the operand rows of the upward pass), or both.
void m2l_tensor_prepare(cudaStream_t s, const ExpArgs &e, const MixedArgs &m);
void m2l_tensor_run(cudaStream_t s, const ExpArgs &e, const MixedArgs &m);
void m2l_tensor(cudaStream_t s, const ExpArgs &e, const MixedArgs &m);
// Columns per half-tile of the mixed M2L lane tiles: at most 32 tiles per degree.
__host__ __device__ constexpr int m2l_half_width(int P) { return P >= 16 ? 4 : 2; }
// Shared memory of k_m2l32v2<P, SB>: per source of a batch, a staged
// multipole (3P^2 + 1 complex floats) and a harmonic table (P^2 + 5), both
// dynamic; and, static, two buffers of the sources' offsets, indices and
// levels (24 bytes each) with their cross-level masks and alignment (16
// bytes).  A batch fits when the total is at most the 227 KB a block can opt
// in to.
__host__ __device__ constexpr size_t m2l32_smem_bytes(int P, int SB)
{
  return (size_t)SB * ((3 * P * P + 1) + (P * P + 5)) * 8 + 2 * (size_t)SB * 24 + 16;
}
constexpr bool m2l_batch_fits(int P, int SB) { return m2l32_smem_bytes(P, SB) <= (size_t)227 * 1024; }
std::vector<int4> m2l_lane_table(int P, int kh, int sb);
void p2m_mixed(cudaStream_t s, const ExpArgs &e, const MixedArgs &m);
void m2l_mixed(cudaStream_t s, const ExpArgs &e, const MixedArgs &m);
void m2m_mixed(cudaStream_t s, const ExpArgs &e, const MixedArgs &m); // FP32, scaled
void l2l_mixed(cudaStream_t s, const ExpArgs &e, const MixedArgs &m); // FP32, scaled
void l2p_p2p_mixed(cudaStream_t s, const ExpArgs &e, const MixedArgs &m, double *out);
// The leaf kernel in two passes (p = 8..10): mode 1 the near field into
// m.near32, mode 2 the far field, that sum and the epilogue into out.
void l2p_p2p_mixed_split(cudaStream_t s, const ExpArgs &e, const MixedArgs &m, double *out, int mode);

// ---- viscous.cu: PSE over the P2P lists, added to dadt in soa (FP64 from the
// soa fields when pos32 is null, else FP32 from the mixed-mode body records)
void pse_pass(cudaStream_t s, const ExpArgs &e, const float4 *pos32, const float4 *alp32, double nu, double *soa);

// ---- rbf.cu: vorticity re-interpolation (FMMCalculator::RBF)
enum RbfOp { RBF_INIT_ALPHA, RBF_INIT_RESIDUAL, RBF_PAP, RBF_UPDATE, RBF_RES_NORM, RBF_UPDATE_P, RBF_STORE };
constexpr int RBF_PARTIALS = 152 * 2 * 3; // doubles of reduction scratch
// out[field..field+2] of the targets = -(Gaussian vorticity of the sources over the P2P lists)
void rbf_vorticity(cudaStream_t s, CellsView tc, const int *leaf_cells, int nleaves, const int *p2p_start, const int *p2p_src, const double *tsoa,
                   size_t tcap, CellsView sc, const double *ssoa, size_t scap, double *out, int field, int zero_dadt);
// one elementwise step over n bodies; with sums != null also its three component sums (device)
void rbf_op(cudaStream_t s, int op, double *soa, size_t cap, int n, const double c[3], double *scratch, double *sums);

// ---- adjoint.cu: reverse mode of the FP64 evaluation and of the stage updates
// Adjoint state of the bodies, permuted with them between stages: positions,
// strengths and the RK registers (VOLD/DOLD, XOLD/AOLD); radius and its
// registers (DRDTOLD, ROLD).
enum AdjG { G_XB = 0, G_AB = 3, G_VB = 6, G_DB = 9, G_XOB = 12, G_AOB = 15, G_RB = 18, G_RDB = 19, G_ROB = 20, NG = 21 };
// Work fields of one evaluation's adjoint: seeds of u and J, far-field
// position adjoints and dilation terms, near-field position and strength
// adjoints (per target / per source), P2M^T and stretching strength
// adjoints, the stage cotangent of (u, dalpha/dt, dr/dt), the cotangent of
// the relaxation's vorticity w, and radius adjoints (near field per source;
// the rVPM terms).
enum AdjW { W_SU = 0, W_SJ = 3, W_XF = 12, W_EF = 15, W_XNT = 16, W_XNS = 19, W_ANS = 22, W_AP2M = 25, W_ASTR = 28, W_COT = 31, W_WB = 38,
            W_RNS = 41, W_RD = 42, NW = 43 };
struct AdjBufs {
  double    *g; // adjoint state, NG fields
  double    *w; // work, NW fields
  int        n;
  double2   *Mb, *Lb; // adjoint expansions [cell][3K]
  const int *p2pT_start, *p2pT_tgt, *m2lT_start, *m2lT_tgt;
  double    *part; // ADJ_PARTIALS doubles
  // mixed mode (else null): the evaluation's FP32 body records, FP32 seed
  // scratch (4 float4 per body), the tree's R0; P2P^T and M2L^T then run in FP32
  const float4 *pos32, *alp32;
  float4       *seeds32;
  float2       *Lhat32; // ncells * 3K
  double        R0;
};
constexpr int ADJ_PARTIALS = 152 * 2 * 17;
// vjp of the evaluation whose tree, lists and FP64 expansions are in e, with
// the seeds in b.w (W_SU, W_SJ, W_ASTR): adds to g[G_XB], g[G_AB].
void adjoint_eval(cudaStream_t s, const ExpArgs &e, const AdjBufs &b, const DevInfo *info);
void adjoint_seeds(cudaStream_t s, const double *soa, double *w, size_t cap, int n, int stretching, int add_relax, int formulation);
void adjoint_stage_pre(cudaStream_t s, double *g, double *w, size_t cap, int n, int scheme, int stage, double dt, int rk4_fixed);
void adjoint_relax(cudaStream_t s, double *g, double *w, const double *soa, const double *alpha_u, size_t cap, int n, double f);
void adjoint_objective(cudaStream_t s, const double *soa, size_t cap, int n, const int *orig, const double *seed_x, const double *seed_a, double wE,
                       const double wI[3], double *g, double *w, double *part, double *value);
void adjoint_scatter(cudaStream_t s, const double *in, double *out, size_t cap, int n, const uint32_t *perm);
void orig_update(cudaStream_t s, const int *in, int *out, const uint32_t *perm, int n);
void iota_int(cudaStream_t s, int *a, int n);
void adjoint_rows(cudaStream_t s, const double *g, size_t cap, int n, int field, double *rows);

// ---- direct.cu
void direct_sum(cudaStream_t s, const double *tx, const double *ty, const double *tz, int nt, const double *src, size_t scap, int ns, double *out /*12*nt*/);
// Model-consistent FP64 direct sum on a built tree: singular kernel for all
// pairs plus (regularised - singular) over each target leaf's P2P row;
// scratch holds (nchunks + 1) * 12 * nt doubles; out is [nt][12].
void direct_model_sum(cudaStream_t s, const double *soa, size_t cap, int n, CellsView cv, const int *leaf_cells, int nleaves, const int *p2p_start,
                      const int *p2p_src, const uint32_t *tgt, int nt, double *scratch, int nchunks, double *out);

// Asynchronous global -> shared copies (cp.async): 8 bytes through L1, 16
// bytes through L2 (both addresses aligned to the size), and the wait for all
// of this thread's copies.
__device__ __forceinline__ void cp_async8(void *smem, const void *gmem)
{
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

} // namespace vfmm
