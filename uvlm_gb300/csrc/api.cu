// The C ABI (include/vfmm.h): handle, device memory, and the per-stage
// pipeline of the reference's FMMCalculator (src/fmmCalculator.hpp):
//   init      = tree build + lists            (createTree, :71-115)
//   calculate = upward, M2L, downward, L2P+P2P, stretching   (:420-467)
//   advance   = stages of init + calculate + stage update    (:919-1005)
// All work runs on the handle's stream; the host synchronises twice per
// tree build (node counts, pair counts) and at the end of each API call.
#include <climits>
#include <algorithm>
#include <atomic>
#include <thread>
#include <type_traits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <exception>
#include "vfmm_internal.cuh"

namespace vfmm {
thread_local unsigned long long *g_launch_counter = nullptr;

// One octree in the reference's cell order (tree.hpp:29-99) with its
// per-level tables.
struct Tree {
  DevBuf<int>    nchild, nbody, child, body, level, parent;
  DevBuf<double> x, y, z, R;
  DevBuf<int>    level_cells, level_start, leaf_cells;
  int            level_start_host[MAXL + 2]{};
  int            ncells = 0, nleaves = 0, maxLevel = 0;
  double         R0 = 0;

  CellsView view() { return CellsView{nchild.p, nbody.p, child.p, body.p, level.p, parent.p, x.p, y.p, z.p, R.p}; }
  void      release()
  {
    for (auto *b : {&nchild, &nbody, &child, &body, &level, &parent, &level_cells, &level_start, &leaf_cells})
      b->release();
    for (auto *b : {&x, &y, &z, &R})
      b->release();
  }
};

// P2P and M2L lists of a (target tree, source tree) traversal as CSR rows
// over the target cells; the sorted (target << 32 | source) keys stay in ls.
struct Lists {
  DevBuf<int> p2p_start, p2p_src, m2l_start, m2l_src;
  int         n_p2p = 0, n_m2l = 0;
  size_t      cap_front = 0, cap_p2p = 0, cap_m2l = 0;
  ListScratch ls;

  void release()
  {
    for (auto *b : {&p2p_start, &p2p_src, &m2l_start, &m2l_src})
      b->release();
    ls.front[0].release();
    ls.front[1].release();
    for (auto *b : {&ls.p2p_raw, &ls.m2l_raw, &ls.p2p_sorted, &ls.m2l_sorted})
      b->release();
    ls.cub_tmp.release();
  }
};
} // namespace vfmm

using namespace vfmm;

static_assert(sizeof(vfmm_config) == 72, "vfmm_config layout");
static_assert(sizeof(vfmm_body) == 296, "vfmm_body must match exafmm::Body");
static_assert(sizeof(vfmm_cell) == 72, "vfmm_cell layout");
static_assert(sizeof(vfmm_tuning) == 40, "vfmm_tuning layout");
static_assert(sizeof(vfmm_objective) == 48, "vfmm_objective layout");

struct vfmm_handle_s {
  vfmm_config  cfg;
  int          device = 0;
  cudaStream_t stream = nullptr;
  // second stream of the tensor-core M2L's pre-pass, beside the upward pass,
  // and its fork/join events (made on first use)
  cudaStream_t side = nullptr;
  cudaEvent_t  side_go = nullptr, side_done = nullptr;
  // the split leaf kernel: near field on the second stream beside the tensor
  // M2L (VFMM_P2P_OVERLAP=0 keeps the fused kernel), its fork/join events and
  // the per-body near-field sums it hands to the far-field pass
  int            overlap = 1;
  cudaEvent_t    near_go = nullptr, near_done = nullptr;
  DevBuf<float>  near32;
  cudaEvent_t    pn[3]{};           // timing: near pass start and end (second stream), far pass start
  bool           split_ran = false; // the last timed evaluation ran the split leaf kernel
  cudaEvent_t  ev[16]{};
  cudaEvent_t  ph[8]{};
  bool         ph_valid = false;
  bool         timing   = true; // record the phase events (off inside a batch: fewer driver calls)
  std::string  err;
  unsigned long long launches = 0;

  // bodies, field-major SoA, double-buffered for reordering
  size_t         cap = 0;
  int            n   = 0;
  DevBuf<double> soa[2];
  int            cur = 0;
  DevBuf<double> aos; // device staging for 296-byte records

  // particle tree and its self-interaction lists
  DevInfo    *info  = nullptr; // device
  DevInfo    *hinfo = nullptr; // pinned host
  TreeScratch ts;
  Tree        tree;
  Lists       lists;

  // sensor points: bodies (field-major, double-buffered), tree, lists
  // against the particle tree, local expansions
  size_t          scap = 0;
  int             ns = 0, scur = 0;
  DevBuf<double>  ssoa[2];
  DevInfo        *sinfo = nullptr, *shinfo = nullptr;
  Tree            stree;
  Lists           slists;
  DevBuf<double2> sL;

  // expansions
  DevBuf<double2> M, L, Mprep;
  DevBuf<double2> srcw; // FP64 P2P: per particle 1/(2 sigma^2), 1/(sqrt(2) sigma)
  DevBuf<int4>    items, items32, lanes32;
  int             m2l_batch = 16; // sources per mixed-M2L batch (set per p); VFMM_M2L_BATCH = 8, 16, 24, 30 or 32 overrides
  int             items_P = 0, items_per_lane = 0, items_batch = 0;
  DevBuf<float2>  Mp32;
  DevBuf<float4>  pos32, alp32;
  TcScratch       tcs;                // tensor-core M2L (mixed mode, p = 8..10)
  int            *eval_err = nullptr; // device: error raised by an evaluation kernel (bounded waits)
  int            *eval_err_host = nullptr; // pinned: its copy, read after the handle's stream synchronises

  DevBuf<unsigned char> flushbuf;
  DevBuf<double>        dtmp;
  bool                  has_tree = false, has_eval = false;
  bool                  moved    = false; // a stage update moved the bodies after the last tree build

  // reverse mode (vfmm_adjoint): adjoint state (ping-pong for the reorders),
  // work fields, adjoint expansions, lists by source, checkpoints, caller
  // index of each body, seeds
  struct {
    DevBuf<double>             g[2], w, ckpt, seedx, seeda, part, rows, value;
    DevBuf<double2>            Mb, Lb;
    DevBuf<int>                p2pT_start, p2pT_tgt, m2lT_start, m2lT_tgt, orig[2];
    DevBuf<unsigned long long> tkeys, tsorted;
    DevBuf<float4>             seeds32;
    DevBuf<float2>             Lhat32;
    // one recomputed segment's stage evaluations, swapped into the handle
    // for the reverse sweep: tree, lists (CSR and sorted keys), local
    // expansions, FP32 body records, tree permutation, the bodies' J, X,
    // alpha and radius in tree order, and the tree's bounding box (DevInfo)
    struct Ctx {
      Tree                       tree;
      DevBuf<int>                p2p_start, p2p_src, m2l_start, m2l_src;
      DevBuf<unsigned long long> p2p_sorted, m2l_sorted;
      int                        n_p2p = 0, n_m2l = 0, key_bits = 0;
      DevBuf<double2>            L;
      DevBuf<float4>             pos32, alp32;
      DevBuf<uint32_t>           perm;
      DevBuf<double>             body;
      DevBuf<DevInfo>            info;
    };
    std::vector<Ctx> ctx;
  } adj;
};

namespace {

struct LaunchScope {
  unsigned long long *prev;
  explicit LaunchScope(vfmm_handle h) : prev(g_launch_counter) { g_launch_counter = &h->launches; }
  ~LaunchScope() { g_launch_counter = prev; }
};

template <class F>
int guarded(vfmm_handle h, F f)
{
  if (!h)
    return VFMM_ERR_INVALID;
  LaunchScope scope(h);
  try {
    VFMM_CUDA_TRY(cudaSetDevice(h->device));
    f();
    h->err.clear();
    return VFMM_OK;
  } catch (const Error &e) {
    h->err = e.msg;
    return e.code;
  } catch (const std::exception &e) {
    h->err = e.what();
    return VFMM_ERR_CUDA;
  }
}

int stages_of(int scheme)
{
  switch (scheme) {
  case VFMM_EULER: return 1;
  case VFMM_RK2: return 2;
  case VFMM_RK3: return 3;
  case VFMM_RK4: return 4;
  }
  return 0;
}

void validate(const vfmm_config &c)
{
  if (c.p < PMIN || c.p > PMAX)
    throw Error(VFMM_ERR_UNSUPPORTED, "p must be in 2..16");
  if (c.ncrit < 1 || c.ncrit > NCRIT_MAX)
    throw Error(VFMM_ERR_UNSUPPORTED, "ncrit must be in 1..256");
  if (!(c.theta > 0) || !(c.theta < 10))
    throw Error(VFMM_ERR_INVALID, "theta must be positive");
  if (c.precision != VFMM_FP64 && c.precision != VFMM_MIXED)
    throw Error(VFMM_ERR_INVALID, "unknown precision");
  if (stages_of(c.integrator) == 0)
    throw Error(VFMM_ERR_INVALID, "unknown integrator");
  if (c.stretching != VFMM_TRANSPOSED && c.stretching != VFMM_CLASSIC)
    throw Error(VFMM_ERR_INVALID, "unknown stretching");
  if (c.formulation != VFMM_CVPM && c.formulation != VFMM_RVPM)
    throw Error(VFMM_ERR_INVALID, "unknown formulation");
  if (c.relax < 0 || c.relax > 1)
    throw Error(VFMM_ERR_INVALID, "relax must be in [0, 1]");
  if (c.m2l_batch != 0 && c.m2l_batch != 8 && c.m2l_batch != 16 && c.m2l_batch != 24 && c.m2l_batch != 30 && c.m2l_batch != 32)
    throw Error(VFMM_ERR_INVALID, "m2l_batch must be 0, 8, 16, 24, 30 or 32");
  if (c.m2l_batch != 0 && c.precision == VFMM_MIXED && !m2l_batch_fits(c.p, c.m2l_batch))
    throw Error(VFMM_ERR_INVALID, "m2l_batch: the batch's staging exceeds a block's shared memory at this p");
  if (c.p2p_chunk != 0 && c.p2p_chunk != 512 && c.p2p_chunk != 768)
    throw Error(VFMM_ERR_INVALID, "p2p_chunk must be 0, 512 or 768");
  if (c.m2l_kernel < 0 || c.m2l_kernel > 2)
    throw Error(VFMM_ERR_INVALID, "m2l_kernel must be 0 (by size), 1 (tensor cores) or 2 (CUDA cores)");
  if (c.viscous != VFMM_INVISCID && c.viscous != VFMM_PSE && c.viscous != VFMM_CSM)
    throw Error(VFMM_ERR_INVALID, "unknown viscous scheme");
  if (!(c.nu >= 0) || !(c.nu < 1e300))
    throw Error(VFMM_ERR_INVALID, "nu must be finite and >= 0");
}

void ensure_bodies(vfmm_handle h, size_t n)
{
  if (n == 0)
    throw Error(VFMM_ERR_INVALID, "no bodies");
  if (n > (size_t)0x7fffffff)
    throw Error(VFMM_ERR_INVALID, "too many bodies");
  if (n > h->cap) {
    size_t cap = n + n / 8 + 256;
    h->soa[0].release();
    h->soa[1].release();
    h->soa[0].reserve(cap * NFIELD);
    h->soa[1].reserve(cap * NFIELD);
    h->cap = cap;
  }
  h->aos.reserve(n * NFIELD);
  h->n = (int)n;
}

// The device address of `bytes` of host memory at p when all of it is pinned
// and mapped (vfmm_host_register), else null: both ends must resolve to one
// contiguous mapping.
void *mapped_host(const void *p, size_t bytes)
{
  cudaPointerAttributes a{}, z{};
  const char           *q = static_cast<const char *>(p);
  if (cudaPointerGetAttributes(&a, q) != cudaSuccess || cudaPointerGetAttributes(&z, q + bytes - 1) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || z.type != cudaMemoryTypeHost || !a.devicePointer || !z.devicePointer)
    return nullptr;
  if (static_cast<char *>(z.devicePointer) - static_cast<char *>(a.devicePointer) != (ptrdiff_t)(bytes - 1))
    return nullptr;
  return a.devicePointer;
}

// Bodies in: from pinned, mapped host memory the transposing kernel reads the
// records directly over the host link (one pass); otherwise a copy to the
// device staging buffer first.  `fields`: the fields the caller's computation
// reads (the others are set to NaN on the device).
void upload(vfmm_handle h, const vfmm_body *b, size_t n, uint64_t fields = ~0ull)
{
  ensure_bodies(h, n);
  if (const void *d = mapped_host(b, n * sizeof(vfmm_body)))
    aos_to_soa(h->stream, static_cast<const double *>(d), h->soa[h->cur].p, h->cap, (int)n, fields);
  else {
    VFMM_CUDA_TRY(cudaMemcpyAsync(h->aos.p, b, n * sizeof(vfmm_body), cudaMemcpyHostToDevice, h->stream));
    aos_to_soa(h->stream, h->aos.p, h->soa[h->cur].p, h->cap, (int)n, fields);
  }
}

// The fields of the caller's records that an advance reads.  The first
// stage's evaluation stores velocity, J, dadt and dr/dt of every body before
// anything reads them (both leaf kernels write all four for each body), and
// its stage update stores RK registers before reading them: all six with
// storeInitialState (RK2, RK4), the velocity, dadt and dr/dt registers for
// RK3, whose first stage assigns them.  The other registers pass through to
// the output unchanged, so they are read (Euler keeps all six).
uint64_t advance_input_fields(int scheme)
{
  uint64_t m    = (1ull << NFIELD) - 1;
  auto     drop = [&](int f0, int k) {
    for (int f = f0; f < f0 + k; f++)
      m &= ~(1ull << f);
  };
  drop(F_J, 9);
  drop(F_U, 3);
  drop(F_DADT, 3);
  drop(F_DRDT, 1);
  if (scheme == VFMM_RK2 || scheme == VFMM_RK4 || scheme == VFMM_RK3) {
    drop(F_VOLD, 3);
    drop(F_DOLD, 3);
    drop(F_DRDTOLD, 1);
  }
  if (scheme == VFMM_RK2 || scheme == VFMM_RK4) {
    drop(F_XOLD, 3);
    drop(F_AOLD, 3);
    drop(F_ROLD, 1);
  }
  return m;
}

void fetch_eval_err(vfmm_handle h);
void raise_eval_err(vfmm_handle h);

void download(vfmm_handle h, vfmm_body *b, size_t n)
{
  if ((int)n != h->n)
    throw Error(VFMM_ERR_INVALID, "body count differs from the bodies on the device");
  if (void *d = mapped_host(b, n * sizeof(vfmm_body)))
    soa_to_aos(h->stream, h->soa[h->cur].p, h->cap, static_cast<double *>(d), (int)n);
  else {
    soa_to_aos(h->stream, h->soa[h->cur].p, h->cap, h->aos.p, (int)n);
    VFMM_CUDA_TRY(cudaMemcpyAsync(b, h->aos.p, n * sizeof(vfmm_body), cudaMemcpyDeviceToHost, h->stream));
  }
  fetch_eval_err(h);
  VFMM_CUDA_TRY(cudaStreamSynchronize(h->stream));
  raise_eval_err(h);
}

void read_info(cudaStream_t s, DevInfo *info, DevInfo *hinfo)
{
  VFMM_CUDA_TRY(cudaMemcpyAsync(hinfo, info, sizeof(DevInfo), cudaMemcpyDeviceToHost, s));
  VFMM_CUDA_TRY(cudaStreamSynchronize(s));
}

void read_info(vfmm_handle h) { read_info(h->stream, h->info, h->hinfo); }

// Tree of the n bodies in soa[cur] (field-major, capacity cap).  The bodies
// are gathered into tree order in soa[cur ^ 1] and cur flips, as buildTree
// permutes its bodies (tree.hpp:101-113).  One host sync (node counts).
// `fields` selects the body fields carried into the new order (all by default).
void tree_enqueue(cudaStream_t s, DevBuf<double> *soa, int &cur, size_t cap, int n, int ncrit, DevInfo *info, DevInfo *hinfo, TreeScratch &ts,
                  Tree &t, uint64_t fields = (1ull << NFIELD) - 1)
{
  VFMM_CUDA_TRY(cudaMemsetAsync(info, 0, sizeof(DevInfo), s));
  check_finite(s, soa[cur].p, cap, n, info);
  tree_bounds(s, soa[cur].p + (size_t)F_X * cap, cap, n, info, ts);
  const int nncap = n + MAXL * (n / (ncrit + 1)) + 64;
  for (auto *b : {&t.nchild, &t.nbody, &t.child, &t.body, &t.level, &t.parent, &t.level_cells, &t.leaf_cells})
    b->reserve(nncap);
  for (auto *b : {&t.x, &t.y, &t.z, &t.R})
    b->reserve(nncap);
  t.level_start.reserve(MAXL + 2);
  // Keys only a few levels below the tree this Tree last held (at least 8
  // levels: 24 bits, three radix passes instead of eight); the full 21 levels
  // for a first build or when a cell at that depth holds more than ncrit
  // bodies.  Leaves, cells and body order do not depend on the key depth as
  // long as every leaf lies above it.
  int levels = t.ncells > 0 ? std::min(MAXL, std::max(8, t.maxLevel + 3)) : MAXL;
  for (;;) {
    tree_sort_bodies(s, soa[cur].p + (size_t)F_X * cap, cap, n, ncrit, levels, info, ts);
    gather_bodies(s, soa[cur].p, soa[cur ^ 1].p, cap, ts.perm.p, n, fields);
    if (tree_build_cells(s, n, ncrit, nncap, info, ts, t.view(), t.level_cells.p, t.level_start.p, t.leaf_cells.p))
      break;
    levels = MAXL; // soa[cur] still holds the incoming order
    VFMM_CUDA_TRY(cudaMemsetAsync(&info->deeper, 0, sizeof(int), s));
  }
  cur ^= 1;
  VFMM_CUDA_TRY(cudaMemcpyAsync(t.level_start_host, t.level_start.p, sizeof(int) * (MAXL + 2), cudaMemcpyDeviceToHost, s));
  VFMM_CUDA_TRY(cudaMemcpyAsync(hinfo, info, sizeof(DevInfo), cudaMemcpyDeviceToHost, s));
}

// Second half of a tree build: wait for the node counts, check them.
void tree_finish(cudaStream_t s, DevInfo *hinfo, Tree &t)
{
  VFMM_CUDA_TRY(cudaStreamSynchronize(s));
  if (hinfo->nonfinite)
    throw Error(VFMM_ERR_NONFINITE, "non-finite position, strength or radius");
  if (hinfo->err)
    throw Error(hinfo->err, "tree deeper than 21 levels: more than ncrit bodies (nearly) coincide");
  if (hinfo->overflow)
    throw Error(VFMM_ERR_CAPACITY, "tree node capacity exceeded");
  t.ncells   = hinfo->nnodes;
  t.nleaves  = hinfo->nleaves;
  t.maxLevel = hinfo->maxLevel;
  t.R0       = hinfo->R0;
}

void build_tree(cudaStream_t s, DevBuf<double> *soa, int &cur, size_t cap, int n, int ncrit, DevInfo *info, DevInfo *hinfo, TreeScratch &ts,
                Tree &t, uint64_t fields = (1ull << NFIELD) - 1)
{
  tree_enqueue(s, soa, cur, cap, n, ncrit, info, hinfo, ts, t, fields);
  tree_finish(s, hinfo, t);
}

// Lists of the traversal of targets tt against sources st (traverse.hpp:
// 32-85), growing the capacities until nothing overflows (one host sync per
// attempt), then sorted into CSR rows.  interactions (device counter, may be
// null) receives the body-body P2P count of a self traversal.
// First half of a traversal: enqueue it and the copy of its pair counts.
void lists_enqueue(cudaStream_t s, Tree &tt, Tree &st, double theta, DevInfo *info, DevInfo *hinfo, Lists &L)
{
  if (L.cap_front == 0) {
    const size_t nc = (size_t)std::max(tt.ncells, st.ncells), nl = (size_t)std::max(tt.nleaves, st.nleaves);
    L.cap_front     = std::max<size_t>(4096, nc * 16);
    L.cap_p2p       = std::max<size_t>(4096, nl * 48);
    L.cap_m2l       = std::max<size_t>(4096, nc * 240);
  }
  L.ls.front[0].reserve(L.cap_front);
  L.ls.front[1].reserve(L.cap_front);
  L.ls.p2p_raw.reserve(L.cap_p2p);
  L.ls.m2l_raw.reserve(L.cap_m2l);
  traverse(s, tt.view(), st.view(), tt.ncells, st.ncells, tt.maxLevel, st.maxLevel, theta, info, L.ls, L.ls.front[0].cap, L.ls.p2p_raw.cap,
           L.ls.m2l_raw.cap);
  VFMM_CUDA_TRY(cudaMemcpyAsync(hinfo, info, sizeof(DevInfo), cudaMemcpyDeviceToHost, s));
}

// Second half: wait for the pair counts.  On overflow the capacities grow and
// false is returned (enqueue again); else the CSR rows are enqueued.
bool lists_finish(cudaStream_t s, Tree &tt, DevInfo *info, DevInfo *hinfo, Lists &L, unsigned long long *interactions)
{
  VFMM_CUDA_TRY(cudaStreamSynchronize(s));
  if (hinfo->overflow) {
    L.cap_front = std::max(L.cap_front * 2, L.ls.front[0].cap * 2);
    L.cap_p2p   = std::max(L.cap_p2p * 2, L.ls.p2p_raw.cap * 2);
    L.cap_m2l   = std::max(L.cap_m2l * 2, L.ls.m2l_raw.cap * 2);
    VFMM_CUDA_TRY(cudaMemsetAsync(&info->overflow, 0, sizeof(int), s));
    return false;
  }
  L.n_p2p = hinfo->n_p2p;
  L.n_m2l = hinfo->n_m2l;
  L.p2p_start.reserve(tt.ncells + 1);
  L.m2l_start.reserve(tt.ncells + 1);
  L.p2p_src.reserve(L.n_p2p + 1);
  L.m2l_src.reserve(L.n_m2l + 1);
  if (interactions)
    VFMM_CUDA_TRY(cudaMemsetAsync(interactions, 0, sizeof(unsigned long long), s));
  lists_to_csr(s, L.ls, L.n_p2p, L.n_m2l, tt.ncells, 32, L.p2p_start.p, L.p2p_src.p, L.m2l_start.p, L.m2l_src.p,
               interactions ? tt.nbody.p : nullptr, interactions);
  return true;
}

void build_lists(cudaStream_t s, Tree &tt, Tree &st, double theta, DevInfo *info, DevInfo *hinfo, Lists &L, unsigned long long *interactions)
{
  for (int attempt = 0;; attempt++) {
    if (attempt > 9)
      throw Error(VFMM_ERR_CAPACITY, "interaction lists keep overflowing");
    lists_enqueue(s, tt, st, theta, info, hinfo, L);
    if (lists_finish(s, tt, info, hinfo, L, interactions))
      break;
  }
}

// Tree and lists of the bodies in soa[cur]; bodies are reordered into tree
// order.  for_evaluation: an evaluation follows that rewrites velocity, J and
// dadt of every body before anything reads them, so those fields are not
// carried into the new order.
void build_tree_and_lists(vfmm_handle h, bool for_evaluation = false)
{
  cudaStream_t s = h->stream;
  h->has_tree    = false;
  h->has_eval    = false;
  if (h->timing)
    VFMM_CUDA_TRY(cudaEventRecord(h->ph[0], s));
  uint64_t fields = (1ull << NFIELD) - 1;
  if (for_evaluation) {
    const int outputs[] = {F_J, F_J + 1, F_J + 2, F_J + 3, F_J + 4, F_J + 5, F_J + 6, F_J + 7, F_J + 8, F_U, F_U + 1, F_U + 2, F_DADT, F_DADT + 1, F_DADT + 2};
    for (int f : outputs)
      fields &= ~(1ull << f);
  }
  build_tree(s, h->soa, h->cur, h->cap, h->n, h->cfg.ncrit, h->info, h->hinfo, h->ts, h->tree, fields);
  build_lists(s, h->tree, h->tree, h->cfg.theta, h->info, h->hinfo, h->lists, &h->info->p2p_interactions);
  if (h->timing)
    VFMM_CUDA_TRY(cudaEventRecord(h->ph[1], s));
  h->has_tree = true;
  h->has_eval = false;
  h->moved    = false;
}

void ensure_items(vfmm_handle h)
{
  if (h->items_P == h->cfg.p && h->items_batch == h->cfg.m2l_batch)
    return;
  int  per = 0;
  auto tab = m2l_schedule(h->cfg.p, 32, 2, 4, &per);
  h->items.reserve(tab.size());
  VFMM_CUDA_TRY(cudaMemcpy(h->items.p, tab.data(), tab.size() * sizeof(int4), cudaMemcpyHostToDevice));
  int  per32 = 0;
  auto tab32 = m2l_schedule(h->cfg.p, 32, 4, 3, &per32);
  h->items32.reserve(tab32.size());
  VFMM_CUDA_TRY(cudaMemcpy(h->items32.p, tab32.data(), tab32.size() * sizeof(int4), cudaMemcpyHostToDevice));
  const char *sb = getenv("VFMM_M2L_BATCH");
  // sources per batch, measured best on GB300: 30 for p <= 10 (0.6-2.4% less
  // M2L time than 32 at p = 6-10), 24 for p = 11-12, else 16
  const int def  = h->cfg.p <= 10 ? 30 : (h->cfg.p <= 12 ? 24 : 16);
  const int env  = sb ? atoi(sb) : 0;
  h->m2l_batch   = (env == 8 || env == 16 || env == 24 || env == 30 || env == 32) && m2l_batch_fits(h->cfg.p, env) ? env : def;
  if (h->cfg.m2l_batch)
    h->m2l_batch = h->cfg.m2l_batch;
  auto lt32      = m2l_lane_table(h->cfg.p, m2l_half_width(h->cfg.p), h->m2l_batch); // half-tile width and batch of k_m2l32v2
  h->lanes32.reserve(lt32.size());
  VFMM_CUDA_TRY(cudaMemcpy(h->lanes32.p, lt32.data(), lt32.size() * sizeof(int4), cudaMemcpyHostToDevice));
  h->items_P        = h->cfg.p;
  h->items_batch    = h->cfg.m2l_batch;
  h->items_per_lane = per;
}

// Expansion arguments of the particle tree and its self lists.
ExpArgs particle_args(vfmm_handle h)
{
  ExpArgs e{};
  e.P                   = h->cfg.p;
  e.cells               = h->tree.view();
  e.ncells              = h->tree.ncells;
  e.level_cells         = h->tree.level_cells.p;
  e.level_start_host    = h->tree.level_start_host;
  e.maxLevel            = h->tree.maxLevel;
  e.leaf_cells          = h->tree.leaf_cells.p;
  e.nleaves             = h->tree.nleaves;
  e.soa                 = h->soa[h->cur].p;
  e.cap                 = h->cap;
  e.M                   = h->M.p;
  e.L                   = h->L.p;
  e.Mprep               = h->Mprep.p;
  e.m2l_start           = h->lists.m2l_start.p;
  e.m2l_src             = h->lists.m2l_src.p;
  e.p2p_start           = h->lists.p2p_start.p;
  e.p2p_src             = h->lists.p2p_src.p;
  e.m2l_items           = h->items.p;
  e.m2l_nitems_per_lane = h->items_per_lane;
  e.stretching          = h->cfg.stretching;
  e.formulation         = h->cfg.formulation;
  // the FP64 P2P's source weights (the particles; sensors use the FP64
  // kernels in both precision modes)
  h->srcw.reserve(h->n);
  e.srcw = h->srcw.p;
  e.nsrc = h->n;
  return e;
}

// Whether this evaluation's M2L runs on the tensor cores (mixed mode, p =
// 8..10): as vfmm_config.m2l_kernel says, by size when it is 0.
bool tensor_m2l(vfmm_handle h)
{
  if (h->cfg.precision != VFMM_MIXED || h->cfg.p < TC_PMIN || h->cfg.p > TC_PMAX || h->cfg.m2l_kernel == 2)
    return false;
  return h->cfg.m2l_kernel == 1 || h->lists.n_m2l >= VFMM_TC_MIN_PAIRS;
}

// Queue the copy of the evaluation error word on the handle's stream (before
// a synchronisation of that stream; only that stream is involved, so handles
// on other streams keep running).
void fetch_eval_err(vfmm_handle h)
{
  VFMM_CUDA_TRY(cudaMemcpyAsync(h->eval_err_host, h->eval_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
}

// After the synchronisation: raise the error an evaluation kernel recorded.
void raise_eval_err(vfmm_handle h)
{
  const int e = *h->eval_err_host;
  if (e) {
    *h->eval_err_host = 0;
    VFMM_CUDA_TRY(cudaMemsetAsync(h->eval_err, 0, sizeof(int), h->stream));
    throw Error(e, e == VFMM_ERR_TIMEOUT ? "a tensor-core M2L wait on the GPU gave up (time limit)" : "tensor-core M2L: more operator classes than its hash holds");
  }
}

void check_eval_err(vfmm_handle h)
{
  fetch_eval_err(h);
  VFMM_CUDA_TRY(cudaStreamSynchronize(h->stream));
  raise_eval_err(h);
}

void calculate(vfmm_handle h)
{
  if (!h->has_tree)
    throw Error(VFMM_ERR_STATE, "calculate needs a tree: call init first");
  cudaStream_t s  = h->stream;
  const int    K3 = 3 * h->cfg.p * (h->cfg.p + 1) / 2;
  ensure_items(h);
  h->M.reserve((size_t)h->tree.ncells * K3);
  h->L.reserve((size_t)h->tree.ncells * K3);
  h->Mprep.reserve((size_t)h->tree.ncells * 3 * h->cfg.p * h->cfg.p);
  VFMM_CUDA_TRY(cudaMemsetAsync(h->M.p, 0, sizeof(double2) * (size_t)h->tree.ncells * K3, s));
  const ExpArgs e = particle_args(h);
  if (h->cfg.precision == VFMM_MIXED) {
    h->Mp32.reserve((size_t)h->tree.ncells * 3 * h->cfg.p * h->cfg.p);
    h->pos32.reserve(h->n);
    h->alp32.reserve(h->n);
    MixedArgs m{};
    m.Mp32    = h->Mp32.p;
    m.pos32   = h->pos32.p;
    m.alp32   = h->alp32.p;
    m.items32 = h->items32.p;
    m.lanes32   = h->lanes32.p;
    m.m2l_batch = h->m2l_batch;
    m.p2p_chunk = h->cfg.p2p_chunk;
    if (tensor_m2l(h)) {
      const size_t rows = (size_t)h->tree.ncells * 3 * tc_kp(h->cfg.p);
      h->tcs.B.reserve(2 * rows);
      m.tc           = &h->tcs;
      m.Bhi          = h->tcs.B.p;
      m.Blo          = h->tcs.B.p + rows;
      m.m2l_keys     = h->lists.ls.m2l_sorted.p;
      m.m2l_key_bits = h->lists.ls.key_bits;
      m.n_m2l        = h->lists.n_m2l;
      m.eval_err     = h->eval_err;
    }
    // the FP32 kernels' scaling length: any positive value is exact; R0 = 0
    // (every body at one point, a single root leaf without far field) uses 1
    m.R0      = h->tree.R0 > 0 ? h->tree.R0 : 1.0;
    const bool split = m.tc && h->overlap > 0;
    h->split_ran     = split;
    if (m.tc) { // the tensor M2L's pre-pass needs only the tree and lists: beside P2M/M2M
      if (!h->side) {
        VFMM_CUDA_TRY(cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
        VFMM_CUDA_TRY(cudaEventCreateWithFlags(&h->side_go, cudaEventDisableTiming));
        VFMM_CUDA_TRY(cudaEventCreateWithFlags(&h->side_done, cudaEventDisableTiming));
        VFMM_CUDA_TRY(cudaEventCreateWithFlags(&h->near_go, cudaEventDisableTiming));
        VFMM_CUDA_TRY(cudaEventCreateWithFlags(&h->near_done, cudaEventDisableTiming));
      }
      if (split) {
        h->near32.reserve((size_t)h->n * 24);
        m.near32 = h->near32.p;
      }
      VFMM_CUDA_TRY(cudaEventRecord(h->side_go, s));
      VFMM_CUDA_TRY(cudaStreamWaitEvent(h->side, h->side_go, 0));
      m2l_tensor_prepare(h->side, e, m);
      VFMM_CUDA_TRY(cudaEventRecord(h->side_done, h->side));
    }
    p2m_mixed(s, e, m);
    m2m_mixed(s, e, m);
    if (h->timing)
      VFMM_CUDA_TRY(cudaEventRecord(h->ph[2], s));
    if (m.tc) {
      VFMM_CUDA_TRY(cudaStreamWaitEvent(s, h->side_done, 0));
      if (split)
        VFMM_CUDA_TRY(cudaEventRecord(h->near_go, s));
      m2l_tensor_run(s, e, m);
      if (split) { // the near field (no local expansion needed) beside the M2L kernel
        VFMM_CUDA_TRY(cudaStreamWaitEvent(h->side, h->near_go, 0));
        if (h->timing)
          VFMM_CUDA_TRY(cudaEventRecord(h->pn[0], h->side));
        l2p_p2p_mixed_split(h->side, e, m, h->soa[h->cur].p, 1);
        if (h->timing)
          VFMM_CUDA_TRY(cudaEventRecord(h->pn[1], h->side));
        VFMM_CUDA_TRY(cudaEventRecord(h->near_done, h->side));
      }
    } else
      m2l_mixed(s, e, m);
    if (h->timing)
      VFMM_CUDA_TRY(cudaEventRecord(h->ph[3], s));
    l2l_mixed(s, e, m);
    if (h->timing)
      VFMM_CUDA_TRY(cudaEventRecord(h->ph[4], s));
    if (split) {
      VFMM_CUDA_TRY(cudaStreamWaitEvent(s, h->near_done, 0));
      if (h->timing)
        VFMM_CUDA_TRY(cudaEventRecord(h->pn[2], s));
      l2p_p2p_mixed_split(s, e, m, h->soa[h->cur].p, 2);
    } else
      l2p_p2p_mixed(s, e, m, h->soa[h->cur].p);
    if (h->timing)
      VFMM_CUDA_TRY(cudaEventRecord(h->ph[5], s));
  } else {
    upward_pass(s, e);
    if (h->timing)
      VFMM_CUDA_TRY(cudaEventRecord(h->ph[2], s));
    m2l_pass(s, e);
    if (h->timing)
      VFMM_CUDA_TRY(cudaEventRecord(h->ph[3], s));
    downward_l2l(s, e);
    if (h->timing)
      VFMM_CUDA_TRY(cudaEventRecord(h->ph[4], s));
    l2p_p2p_pass(s, e, h->soa[h->cur].p);
    if (h->timing)
      VFMM_CUDA_TRY(cudaEventRecord(h->ph[5], s));
  }
  h->has_eval = true;
}

// getSensorData (fmmCalculator.hpp:726-731 with :117-161, :469-491): a tree
// of the sensors (buildTree permutes them), the traversal of the sensor tree
// as targets against the particle tree, M2L from the particles' multipoles
// of the last calculate, the velocity-only P2P against the particles as they
// are now, then L2L and L2P down the sensor tree.  The sensors come back in
// sensor-tree order.  FP64 in both precision modes.
// Point sets (sensors, re-interpolation points) in ssoa[scur].
void load_points(vfmm_handle h, const vfmm_body *pts, size_t n)
{
  if (n > (size_t)0x7fffffff)
    throw Error(VFMM_ERR_INVALID, "too many points");
  cudaStream_t s = h->stream;
  if (n > h->scap) {
    const size_t cap = n + n / 8 + 256;
    h->ssoa[0].release();
    h->ssoa[1].release();
    h->ssoa[0].reserve(cap * NFIELD);
    h->ssoa[1].reserve(cap * NFIELD);
    h->scap = cap;
  }
  h->aos.reserve(std::max(n, (size_t)h->n) * NFIELD);
  h->ns = (int)n;
  VFMM_CUDA_TRY(cudaMemcpyAsync(h->aos.p, pts, n * sizeof(vfmm_body), cudaMemcpyHostToDevice, s));
  aos_to_soa(s, h->aos.p, h->ssoa[h->scur].p, h->scap, (int)n);
}

void points_to_host(vfmm_handle h, vfmm_body *pts, size_t n)
{
  soa_to_aos(h->stream, h->ssoa[h->scur].p, h->scap, h->aos.p, (int)n);
  VFMM_CUDA_TRY(cudaMemcpyAsync(pts, h->aos.p, n * sizeof(vfmm_body), cudaMemcpyDeviceToHost, h->stream));
  VFMM_CUDA_TRY(cudaStreamSynchronize(h->stream));
}

void sensor_data(vfmm_handle h, vfmm_body *sens, size_t n)
{
  if (!h->has_eval)
    throw Error(VFMM_ERR_STATE, "sensor data needs the particles' multipoles: call calculate or advance first");
  if (n == 0)
    throw Error(VFMM_ERR_INVALID, "no sensors");
  if (n > (size_t)0x7fffffff)
    throw Error(VFMM_ERR_INVALID, "too many sensors");
  cudaStream_t s = h->stream;
  load_points(h, sens, n);
  build_tree(s, h->ssoa, h->scur, h->scap, (int)n, h->cfg.ncrit, h->sinfo, h->shinfo, h->ts, h->stree);
  build_lists(s, h->stree, h->tree, h->cfg.theta, h->sinfo, h->shinfo, h->slists, nullptr);

  const int K3 = 3 * h->cfg.p * (h->cfg.p + 1) / 2;
  h->sL.reserve((size_t)h->stree.ncells * K3);
  h->Mprep.reserve((size_t)h->tree.ncells * 3 * h->cfg.p * h->cfg.p);
  const ExpArgs pe = particle_args(h);
  mprep_pass(s, pe);
  ExpArgs se          = pe;
  se.cells            = h->stree.view();
  se.ncells           = h->stree.ncells;
  se.level_cells      = h->stree.level_cells.p;
  se.level_start_host = h->stree.level_start_host;
  se.maxLevel         = h->stree.maxLevel;
  se.leaf_cells       = h->stree.leaf_cells.p;
  se.nleaves          = h->stree.nleaves;
  se.soa              = h->ssoa[h->scur].p;
  se.cap              = h->scap;
  se.L                = h->sL.p;
  se.m2l_start        = h->slists.m2l_start.p;
  se.m2l_src          = h->slists.m2l_src.p;
  se.p2p_start        = h->slists.p2p_start.p;
  se.p2p_src          = h->slists.p2p_src.p;
  se.src_cells        = h->tree.view();
  se.src_soa          = h->soa[h->cur].p;
  se.src_cap          = h->cap;
  m2l_sensor_pass(s, se);
  downward_l2l(s, se);
  l2p_sensor_pass(s, se, h->ssoa[h->scur].p);
  points_to_host(h, sens, n);
}

// FMMCalculator::RBF (fmmCalculator.hpp:856-917), FP64: the particles' tree
// (init) and a tree of the points with their lists against the particles;
// the particles' vorticity at the points; points whose three components are
// all below 1e-6 are dropped (host side, as the reference does); a tree of the
// rest with point-to-point lists; strengths alpha = vorticity * volume as the
// start, then at most 100 iterations of three component-wise conjugate
// gradients (stop when every squared residual is below 1e-10).  Returns the
// kept points (their count in *m_out) in their tree order, alpha = solution.
void rbf(vfmm_handle h, vfmm_body *particles, size_t n, vfmm_body *points, size_t m, size_t *m_out, int *iterations)
{
  cudaStream_t s = h->stream;
  upload(h, particles, n);
  build_tree_and_lists(h);
  download(h, particles, n); // init permutes the particles (tree.hpp:101-113)
  load_points(h, points, m);
  build_tree(s, h->ssoa, h->scur, h->scap, (int)m, h->cfg.ncrit, h->sinfo, h->shinfo, h->ts, h->stree);
  build_lists(s, h->stree, h->tree, h->cfg.theta, h->sinfo, h->shinfo, h->slists, nullptr);
  rbf_vorticity(s, h->stree.view(), h->stree.leaf_cells.p, h->stree.nleaves, h->slists.p2p_start.p, h->slists.p2p_src.p, h->ssoa[h->scur].p,
                h->scap, h->tree.view(), h->soa[h->cur].p, h->cap, h->ssoa[h->scur].p, F_VOLD, 0);
  std::vector<vfmm_body> pts(m);
  points_to_host(h, pts.data(), m);
  std::vector<vfmm_body> kept;
  kept.reserve(m);
  for (const auto &p : pts)
    if (!(std::abs(p.velocity_old[0]) < 1e-6 && std::abs(p.velocity_old[1]) < 1e-6 && std::abs(p.velocity_old[2]) < 1e-6))
      kept.push_back(p);
  const size_t mk = kept.size();
  *m_out          = mk;
  if (iterations)
    *iterations = 0;
  if (mk == 0)
    return;
  load_points(h, kept.data(), mk);
  build_tree(s, h->ssoa, h->scur, h->scap, (int)mk, h->cfg.ncrit, h->sinfo, h->shinfo, h->ts, h->stree);
  build_lists(s, h->stree, h->stree, h->cfg.theta, h->sinfo, h->shinfo, h->slists, nullptr);
  h->dtmp.reserve(RBF_PARTIALS + 8);
  double *scratch = h->dtmp.p, *dsum = scratch + RBF_PARTIALS;
  double *soa     = h->ssoa[h->scur].p;
  auto    reduce  = [&](int op, const double *c, double out[3]) {
    rbf_op(s, op, soa, h->scap, (int)mk, c, scratch, dsum);
    VFMM_CUDA_TRY(cudaMemcpyAsync(h->shinfo->X0, dsum, 3 * sizeof(double), cudaMemcpyDeviceToHost, s)); // pinned staging
    VFMM_CUDA_TRY(cudaStreamSynchronize(s));
    for (int d = 0; d < 3; d++)
      out[d] = h->shinfo->X0[d];
  };
  auto apply = [&]() { // A p: the vorticity of the points' current strengths at the points
    rbf_vorticity(s, h->stree.view(), h->stree.leaf_cells.p, h->stree.nleaves, h->slists.p2p_start.p, h->slists.p2p_src.p, soa, h->scap,
                  h->stree.view(), soa, h->scap, soa, F_U, 1);
  };
  const double eps = 2.220446049250313080847263336181640625e-16, tol = 1e-10;
  rbf_op(s, RBF_INIT_ALPHA, soa, h->scap, (int)mk, nullptr, scratch, nullptr);
  apply();
  double res[3], resn[3], pAp[3], c[3];
  reduce(RBF_INIT_RESIDUAL, nullptr, res);
  int it = 0;
  for (; it < 100; it++) {
    apply();
    reduce(RBF_PAP, nullptr, pAp);
    for (int d = 0; d < 3; d++)
      c[d] = (res[d] > eps && std::abs(pAp[d]) > eps) ? res[d] / pAp[d] : 0.0;
    rbf_op(s, RBF_UPDATE, soa, h->scap, (int)mk, c, scratch, nullptr);
    reduce(RBF_RES_NORM, nullptr, resn);
    if (resn[0] < tol && resn[1] < tol && resn[2] < tol)
      break;
    for (int d = 0; d < 3; d++) {
      c[d]   = (resn[d] > eps && res[d] > eps) ? resn[d] / res[d] : 0.0;
      res[d] = resn[d];
    }
    rbf_op(s, RBF_UPDATE_P, soa, h->scap, (int)mk, c, scratch, nullptr);
  }
  if (iterations)
    *iterations = it;
  rbf_op(s, RBF_STORE, soa, h->scap, (int)mk, nullptr, scratch, nullptr);
  points_to_host(h, points, mk);
  h->has_eval = false; // the particle tree is current, its expansions are not
}

// relax = false leaves out the relaxation after the last stage (the caller
// applies it with relax_bodies: the same arithmetic on the same values).
void stage_update(vfmm_handle h, int stage, double dt, bool relax = true)
{
  StageArgs a{};
  a.scheme        = h->cfg.integrator;
  a.stage         = stage;
  a.stretching    = h->cfg.stretching;
  a.formulation   = h->cfg.formulation;
  a.rk4_fixed     = h->cfg.rk4_fixed;
  a.store_initial = (stage == 0 && (a.scheme == VFMM_RK2 || a.scheme == VFMM_RK4)) ? 1 : 0;
  a.do_update     = 1;
  h->moved        = true;
  a.dt            = dt;
  a.relax         = (relax && stage == stages_of(a.scheme) - 1) ? h->cfg.relax : 0.0;
  a.csm           = h->cfg.viscous == VFMM_CSM;
  a.nu            = h->cfg.nu;
  finish_and_update(h->stream, h->soa[h->cur].p, h->cap, h->n, a);
  if (h->timing)
    VFMM_CUDA_TRY(cudaEventRecord(h->ph[6], h->stream));
  h->ph_valid = h->timing;
}

// Evaluation, viscosity and the stage update of a stage whose tree and lists
// are built; all enqueued on the handle's stream.
void evaluate_and_update(vfmm_handle h, int stage, double dt)
{
  calculate(h);
  if (h->cfg.viscous == VFMM_PSE) // calculateViscosity after calculate (fmmCalculator.hpp:713-724)
    pse_pass(h->stream, particle_args(h), h->cfg.precision == VFMM_MIXED ? h->pos32.p : nullptr,
             h->cfg.precision == VFMM_MIXED ? h->alp32.p : nullptr, h->cfg.nu, h->soa[h->cur].p);
  stage_update(h, stage, dt);
}

void run_stage(vfmm_handle h, int stage, double dt)
{
  build_tree_and_lists(h, true);
  evaluate_and_update(h, stage, dt);
}

// advance for several independent systems, each on its own handle and
// stream.  The systems are shared out to a pool of host threads (the host's
// hardware threads, at most 16, or VFMM_BATCH_THREADS up to 64); each thread runs whole systems one after
// another through vfmm_advance's code path, so the kernel launches and the two
// host synchronisation points of every stage proceed for many systems at once
// and their kernels overlap on the GPU.  Each system's results are those of
// vfmm_advance on its own.
void advance_batch(vfmm_handle *hs, vfmm_body *const *bodies, const size_t *ns, int count, double dt)
{
  const unsigned hw  = std::thread::hardware_concurrency();
  const char    *env = getenv("VFMM_BATCH_THREADS");
  const int      cap = env && atoi(env) > 0 ? std::min(atoi(env), 64) : 16;
  const int      T   = std::max(1, std::min({count, hw ? (int)hw : 1, cap}));
  std::atomic<int>         next{0};
  std::vector<int>         codes(count, VFMM_OK);
  std::vector<std::string> msgs(count);
  auto                     work = [&]() {
    for (int b; (b = next.fetch_add(1)) < count;) {
      vfmm_handle h = hs[b];
      try {
        VFMM_CUDA_TRY(cudaSetDevice(h->device));
        g_launch_counter = &h->launches;
        h->timing        = false;
        upload(h, bodies[b], ns[b], advance_input_fields(h->cfg.integrator));
        const int S = stages_of(h->cfg.integrator);
        for (int st = 0; st < S; st++)
          run_stage(h, st, dt);
        download(h, bodies[b], ns[b]);
        h->timing = true;
      } catch (const Error &e) {
        h->timing = true;
        codes[b] = e.code;
        msgs[b]  = e.msg;
      } catch (const std::exception &e) {
        h->timing = true;
        codes[b]  = VFMM_ERR_CUDA;
        msgs[b]   = e.what();
      }
    }
    g_launch_counter = nullptr;
  };
  if (T == 1) {
    // on the caller's thread: leave its current device and launch counter as they were
    int                 dev0  = -1;
    unsigned long long *prev  = g_launch_counter;
    const bool          haved = cudaGetDevice(&dev0) == cudaSuccess;
    work();
    g_launch_counter = prev;
    if (haved)
      cudaSetDevice(dev0);
  } else {
    std::vector<std::thread> pool;
    for (int t = 0; t < T; t++)
      pool.emplace_back(work);
    for (auto &t : pool)
      t.join();
  }
  for (int b = 0; b < count; b++)
    if (codes[b] != VFMM_OK)
      throw Error(codes[b], msgs[b]);
}

} // namespace

extern "C" {

void vfmm_default_config(vfmm_config *c)
{
  if (!c)
    return;
  std::memset(c, 0, sizeof(*c));
  c->p           = 4;
  c->ncrit       = 128;
  c->theta       = 0.3;
  c->precision   = VFMM_FP64;
  c->integrator  = VFMM_RK3;
  c->stretching  = VFMM_TRANSPOSED;
  c->formulation = VFMM_CVPM;
  c->relax       = 0.0;
  c->rk4_fixed   = 0;
  c->device      = -1;
}

int vfmm_create(const vfmm_config *cfg, vfmm_handle *out)
{
  if (!cfg || !out)
    return VFMM_ERR_INVALID;
  *out = nullptr;
  auto *h = new vfmm_handle_s();
  h->cfg  = *cfg;
  try {
    validate(h->cfg);
    if (h->cfg.device >= 0)
      VFMM_CUDA_TRY(cudaSetDevice(h->cfg.device));
    VFMM_CUDA_TRY(cudaGetDevice(&h->device));
    if (const char *ov = getenv("VFMM_P2P_OVERLAP"))
      h->overlap = atoi(ov);
    VFMM_CUDA_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    for (auto &e : h->ev)
      VFMM_CUDA_TRY(cudaEventCreate(&e));
    for (auto &e : h->ph)
      VFMM_CUDA_TRY(cudaEventCreate(&e));
    for (auto &e : h->pn)
      VFMM_CUDA_TRY(cudaEventCreate(&e));
    VFMM_CUDA_TRY(cudaMalloc((void **)&h->info, sizeof(DevInfo)));
    VFMM_CUDA_TRY(cudaMalloc((void **)&h->eval_err, sizeof(int)));
    VFMM_CUDA_TRY(cudaMemset(h->eval_err, 0, sizeof(int)));
    VFMM_CUDA_TRY(cudaMallocHost((void **)&h->eval_err_host, sizeof(int)));
    *h->eval_err_host = 0;
    VFMM_CUDA_TRY(cudaMallocHost((void **)&h->hinfo, sizeof(DevInfo)));
    std::memset(h->hinfo, 0, sizeof(DevInfo));
    VFMM_CUDA_TRY(cudaMalloc((void **)&h->sinfo, sizeof(DevInfo)));
    VFMM_CUDA_TRY(cudaMallocHost((void **)&h->shinfo, sizeof(DevInfo)));
    std::memset(h->shinfo, 0, sizeof(DevInfo));
  } catch (const Error &e) {
    const int code = e.code;
    vfmm_destroy(h);
    return code;
  }
  *out = h;
  return VFMM_OK;
}

int vfmm_destroy(vfmm_handle h)
{
  if (!h)
    return VFMM_ERR_INVALID;
  cudaSetDevice(h->device);
  if (h->stream)
    cudaStreamSynchronize(h->stream);
  for (auto *b : {&h->soa[0], &h->soa[1], &h->aos, &h->dtmp, &h->ssoa[0], &h->ssoa[1]})
    b->release();
  h->tree.release();
  h->lists.release();
  h->stree.release();
  h->slists.release();
  h->sL.release();
  h->M.release();
  h->L.release();
  h->Mprep.release();
  h->srcw.release();
  h->items.release();
  h->items32.release();
  h->lanes32.release();
  h->Mp32.release();
  h->pos32.release();
  h->alp32.release();
  h->flushbuf.release();
  for (auto *b : {&h->ts.keys, &h->ts.skeys})
    b->release();
  for (auto *b : {&h->ts.idx, &h->ts.sidx, &h->ts.perm})
    b->release();
  for (auto *b : {&h->ts.lvl, &h->ts.lo, &h->ts.hi, &h->ts.cnt, &h->ts.off, &h->ts.nlevel, &h->ts.nstart, &h->ts.ncount, &h->ts.nparent,
                  &h->ts.nchild, &h->ts.nrank, &h->ts.nref, &h->ts.nbs, &h->ts.nsortidx, &h->ts.nsortlvl, &h->ts.nflag, &h->ts.noff})
    b->release();
  h->ts.bbox_part.release();
  h->ts.cub_tmp.release();
  h->tcs.B.release();
  for (auto *b : {&h->tcs.tkeys, &h->tcs.tkeys_sorted, &h->tcs.pkeys, &h->tcs.pkeys_sorted})
    b->release();
  for (auto *b : {&h->tcs.tile_of, &h->tcs.col_of, &h->tcs.tile_cells, &h->tcs.tile_level, &h->tcs.tile_start, &h->tcs.meta})
    b->release();
  for (auto *b : {&h->tcs.hkeys, &h->tcs.cls_of})
    b->release();
  h->tcs.hid.release();
  h->tcs.cidq.release();
  h->tcs.coords.release();
  h->tcs.table.release();
  if (h->tcs.ncls_host)
    cudaFreeHost(h->tcs.ncls_host);
  h->tcs.pvals.release();
  h->tcs.pvals_sorted.release();
  h->tcs.cub_tmp.release();
  if (h->eval_err)
    cudaFree(h->eval_err);
  if (h->eval_err_host)
    cudaFreeHost(h->eval_err_host);
  if (h->info)
    cudaFree(h->info);
  if (h->hinfo)
    cudaFreeHost(h->hinfo);
  if (h->sinfo)
    cudaFree(h->sinfo);
  if (h->shinfo)
    cudaFreeHost(h->shinfo);
  for (auto &e : h->ev)
    if (e)
      cudaEventDestroy(e);
  for (auto &e : h->ph)
    if (e)
      cudaEventDestroy(e);
  for (auto &e : h->pn)
    if (e)
      cudaEventDestroy(e);
  if (h->near_go)
    cudaEventDestroy(h->near_go);
  if (h->near_done)
    cudaEventDestroy(h->near_done);
  if (h->side_go)
    cudaEventDestroy(h->side_go);
  if (h->side_done)
    cudaEventDestroy(h->side_done);
  if (h->side)
    cudaStreamDestroy(h->side);
  if (h->stream)
    cudaStreamDestroy(h->stream);
  delete h;
  return VFMM_OK;
}

const char *vfmm_last_error(vfmm_handle h) { return h ? h->err.c_str() : "null handle"; }

int vfmm_get_config(vfmm_handle h, vfmm_config *cfg)
{
  if (!h || !cfg)
    return VFMM_ERR_INVALID;
  *cfg = h->cfg;
  return VFMM_OK;
}

int vfmm_init(vfmm_handle h, vfmm_body *bodies, size_t n)
{
  return guarded(h, [&] {
    if (!bodies)
      throw Error(VFMM_ERR_INVALID, "null bodies");
    upload(h, bodies, n);
    build_tree_and_lists(h);
    download(h, bodies, n); // buildTree permutes the caller's bodies (tree.hpp:101-113)
  });
}

int vfmm_calculate(vfmm_handle h)
{
  return guarded(h, [&] {
    calculate(h);
    VFMM_CUDA_TRY(cudaStreamSynchronize(h->stream));
  });
}

int vfmm_copy_bodies_to_host(vfmm_handle h, vfmm_body *bodies, size_t n)
{
  return guarded(h, [&] {
    if (!bodies)
      throw Error(VFMM_ERR_INVALID, "null bodies");
    download(h, bodies, n);
  });
}

int vfmm_advance(vfmm_handle h, vfmm_body *bodies, size_t n, double dt)
{
  return guarded(h, [&] {
    if (!bodies)
      throw Error(VFMM_ERR_INVALID, "null bodies");
    upload(h, bodies, n, advance_input_fields(h->cfg.integrator));
    const int ns = stages_of(h->cfg.integrator);
    for (int st = 0; st < ns; st++)
      run_stage(h, st, dt);
    download(h, bodies, n);
  });
}

int vfmm_get_sensor_data(vfmm_handle h, vfmm_body *sensors, size_t n)
{
  return guarded(h, [&] {
    if (!sensors)
      throw Error(VFMM_ERR_INVALID, "null sensors");
    sensor_data(h, sensors, n);
  });
}

int vfmm_advance_batch(vfmm_handle *handles, vfmm_body *const *bodies, const size_t *n, int count, double dt)
{
  if (!handles || !bodies || !n || count <= 0)
    return VFMM_ERR_INVALID;
  for (int b = 0; b < count; b++) {
    if (!handles[b] || !bodies[b])
      return VFMM_ERR_INVALID;
    for (int c = 0; c < b; c++)
      if (handles[c] == handles[b])
        return VFMM_ERR_INVALID;
  }
  unsigned long long *prev = g_launch_counter;
  int                 code = VFMM_OK;
  std::string         msg;
  try {
    advance_batch(handles, bodies, n, count, dt);
  } catch (const Error &e) {
    code = e.code;
    msg  = e.msg;
  } catch (const std::exception &e) {
    code = VFMM_ERR_CUDA;
    msg  = e.what();
  }
  g_launch_counter = prev;
  for (int b = 0; b < count; b++)
    handles[b]->err = msg;
  return code;
}

int vfmm_autotune(vfmm_handle h, const vfmm_body *bodies, size_t n, double dt, vfmm_tuning *out)
{
  return guarded(h, [&] {
    if (!bodies || !out)
      throw Error(VFMM_ERR_INVALID, "null argument");
    cudaStream_t s = h->stream;
    // one stage of `bodies` with the handle's current leaf size and batch: best of two after a warm-up
    auto time_stage = [&]() {
      float best = 1e30f;
      for (int r = 0; r < 3; r++) {
        upload(h, bodies, n);
        VFMM_CUDA_TRY(cudaEventRecord(h->ev[12], s));
        run_stage(h, 0, dt);
        VFMM_CUDA_TRY(cudaEventRecord(h->ev[13], s));
        VFMM_CUDA_TRY(cudaEventSynchronize(h->ev[13]));
        float ms = 0;
        VFMM_CUDA_TRY(cudaEventElapsedTime(&ms, h->ev[12], h->ev[13]));
        if (r > 0)
          best = std::min(best, ms);
      }
      return best;
    };
    const int  ncrit0 = h->cfg.ncrit, forced0 = h->cfg.m2l_batch, chunk0 = h->cfg.p2p_chunk;
    const bool mixed  = h->cfg.precision == VFMM_MIXED;
    std::memset(out, 0, sizeof(*out));
    out->default_ms_per_stage = time_stage();
    out->ncrit                = ncrit0;
    out->m2l_batch            = h->m2l_batch;
    out->p2p_chunk            = chunk0 ? chunk0 : 768;
    out->ms_per_stage         = out->default_ms_per_stage;
    const int leaf[] = {16, 24, 32, 48, 64, 96, 128, 192, 256};
    const int bat[]  = {16, 24, 30, 32};
    const int chk[]  = {768, 512};
    // the CUDA-core M2L's source batch matters only where the tensor-core M2L does not run
    const int nbat = mixed && !(h->cfg.m2l_kernel == 1 && h->cfg.p >= TC_PMIN && h->cfg.p <= TC_PMAX) ? 4 : 1;
    try {
      for (int nc : leaf)
        for (int b = 0; b < nbat; b++)
          for (int c = 0; c < (mixed ? 2 : 1); c++) {
            if (nbat > 1 && !m2l_batch_fits(h->cfg.p, bat[b]))
              continue;
            h->cfg.ncrit     = nc;
            h->cfg.m2l_batch = nbat > 1 ? bat[b] : forced0;
            h->cfg.p2p_chunk = mixed ? chk[c] : chunk0;
            const float ms   = time_stage();
            out->tried++;
            if (ms < out->ms_per_stage) {
              out->ms_per_stage = ms;
              out->ncrit        = nc;
              out->m2l_batch    = h->m2l_batch;
              out->p2p_chunk    = h->cfg.p2p_chunk ? h->cfg.p2p_chunk : 768;
            }
          }
    } catch (...) {
      h->cfg.ncrit     = ncrit0;
      h->cfg.m2l_batch = forced0;
      h->cfg.p2p_chunk = chunk0;
      throw;
    }
    h->cfg.ncrit     = out->ncrit;
    h->cfg.m2l_batch = nbat > 1 ? out->m2l_batch : forced0;
    h->cfg.p2p_chunk = mixed ? out->p2p_chunk : chunk0;
    h->has_tree = h->has_eval = false;
    VFMM_CUDA_TRY(cudaStreamSynchronize(s));
  });
}

// ---- reverse mode
namespace {

// Positions, strengths and radii (fields F_X..F_A+2 are contiguous) of the
// bodies in soa[cur], to or from 7 * cap doubles at p.
void save_state(vfmm_handle h, double *p)
{
  const double *q = h->soa[h->cur].p;
  VFMM_CUDA_TRY(cudaMemcpyAsync(p, q + (size_t)F_X * h->cap, 6 * h->cap * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  VFMM_CUDA_TRY(cudaMemcpyAsync(p + 6 * h->cap, q + (size_t)F_R * h->cap, h->cap * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
}
void load_state(vfmm_handle h, const double *p)
{
  double *q = h->soa[h->cur].p;
  VFMM_CUDA_TRY(cudaMemcpyAsync(q + (size_t)F_X * h->cap, p, 6 * h->cap * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  VFMM_CUDA_TRY(cudaMemcpyAsync(q + (size_t)F_R * h->cap, p + 6 * h->cap, h->cap * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
}

void adjoint(vfmm_handle h, const vfmm_body *bodies, size_t n, double dt, int steps, int every, const vfmm_objective *obj, double *value,
             double *gx, double *ga)
{
  const vfmm_config &c = h->cfg;
  if (c.viscous != VFMM_INVISCID)
    throw Error(VFMM_ERR_UNSUPPORTED, "the adjoint covers the inviscid path");
  if (!bodies || !obj || !value)
    throw Error(VFMM_ERR_INVALID, "null argument");
  if (steps < 0 || every < 1)
    throw Error(VFMM_ERR_INVALID, "steps must be >= 0 and checkpoint_every >= 1");
  cudaStream_t s    = h->stream;
  auto        &A    = h->adj;
  const int    S    = stages_of(c.integrator);
  const bool   grad = gx || ga;
  upload(h, bodies, n);
  const int    N   = h->n;
  const size_t cap = h->cap, slot = 7 * cap;
  A.orig[0].reserve(N);
  A.orig[1].reserve(N);
  int oc = 0;
  iota_int(s, A.orig[0].p, N);
  auto track = [&]() {
    orig_update(s, A.orig[oc].p, A.orig[oc ^ 1].p, h->ts.perm.p, N);
    oc ^= 1;
  };
  const double *dsx = nullptr, *dsa = nullptr;
  if (obj->seed_x) {
    A.seedx.reserve(3 * (size_t)N);
    VFMM_CUDA_TRY(cudaMemcpyAsync(A.seedx.p, obj->seed_x, 3 * (size_t)N * sizeof(double), cudaMemcpyHostToDevice, s));
    dsx = A.seedx.p;
  }
  if (obj->seed_alpha) {
    A.seeda.reserve(3 * (size_t)N);
    VFMM_CUDA_TRY(cudaMemcpyAsync(A.seeda.p, obj->seed_alpha, 3 * (size_t)N * sizeof(double), cudaMemcpyHostToDevice, s));
    dsa = A.seeda.p;
  }
  const int nck = grad ? (steps + every - 1) / every : 0;
  if (nck > 0)
    A.ckpt.reserve((size_t)nck * slot);
  // forward sweep, keeping the state at the start of every checkpoint_every-th step
  for (int st = 0; st < steps; st++) {
    if (grad && st % every == 0)
      save_state(h, A.ckpt.p + (size_t)(st / every) * slot);
    for (int k = 0; k < S; k++) {
      build_tree_and_lists(h, true);
      track();
      evaluate_and_update(h, k, dt);
    }
  }
  // the objective on the final state; evaluations of the reverse sweep run in
  // the handle's precision (mixed: FP32 P2P^T and M2L^T, the rest FP64)
  const bool mixed = c.precision == VFMM_MIXED;
  build_tree_and_lists(h, true);
  track();
  calculate(h);
  for (auto *b : {&A.g[0], &A.g[1]})
    b->reserve((size_t)NG * cap);
  A.w.reserve((size_t)NW * cap);
  A.part.reserve(ADJ_PARTIALS);
  A.value.reserve(1);
  int          gc    = 0;
  const double wI[3] = {obj->impulse[0], obj->impulse[1], obj->impulse[2]};
  adjoint_objective(s, h->soa[h->cur].p, cap, N, A.orig[oc].p, dsx, dsa, obj->energy, wI, A.g[gc].p, A.w.p, A.part.p, A.value.p);
  double v = 0;
  VFMM_CUDA_TRY(cudaMemcpyAsync(&v, A.value.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  VFMM_CUDA_TRY(cudaStreamSynchronize(s));
  *value = v;
  h->has_tree = h->has_eval = false;
  if (!grad)
    return;
  // vjp of the evaluation just made (tree, lists, FP64 expansions current;
  // seeds in A.w; adjoint state in tree order), then back to the order the
  // bodies had before this tree
  auto vjp = [&](const DevInfo *info) {
    const int    np = h->lists.n_p2p, nm = h->lists.n_m2l, nc = h->tree.ncells;
    const size_t K3 = 3 * (size_t)(c.p * (c.p + 1) / 2);
    A.p2pT_start.reserve(nc + 1);
    A.m2lT_start.reserve(nc + 1);
    A.p2pT_tgt.reserve(np + 1);
    A.m2lT_tgt.reserve(nm + 1);
    A.tkeys.reserve(std::max(np, nm) + 1);
    A.tsorted.reserve(std::max(np, nm) + 1);
    A.Mb.reserve(nc * K3);
    A.Lb.reserve(nc * K3);
    lists_transpose(s, h->lists.ls, np, nm, nc, A.tkeys.p, A.tsorted.p, A.p2pT_start.p, A.p2pT_tgt.p, A.m2lT_start.p, A.m2lT_tgt.p);
    AdjBufs b{};
    b.g          = A.g[gc].p;
    b.w          = A.w.p;
    b.n          = N;
    b.Mb         = A.Mb.p;
    b.Lb         = A.Lb.p;
    b.p2pT_start = A.p2pT_start.p;
    b.p2pT_tgt   = A.p2pT_tgt.p;
    b.m2lT_start = A.m2lT_start.p;
    b.m2lT_tgt   = A.m2lT_tgt.p;
    b.part       = A.part.p;
    if (mixed) {
      A.seeds32.reserve(4 * (size_t)N);
      A.Lhat32.reserve(nc * K3);
      b.Lhat32  = A.Lhat32.p;
      b.pos32   = h->pos32.p;
      b.alp32   = h->alp32.p;
      b.seeds32 = A.seeds32.p;
      b.R0      = h->tree.R0 > 0 ? h->tree.R0 : 1.0; // as calculate's scaling length
    }
    adjoint_eval(s, particle_args(h), b, info);
    adjoint_scatter(s, A.g[gc].p, A.g[gc ^ 1].p, cap, N, h->ts.perm.p);
    gc ^= 1;
  };
  vjp(h->info);
  // The evaluation context of a stage (everything the transposes read) is
  // exchanged between the handle and a segment slot: buffers swap owners,
  // the body fields and the bounding box are copied.
  using Ctx = std::remove_reference_t<decltype(A)>::Ctx;
  A.ctx.resize((size_t)every * S);
  auto exchange = [&](Ctx &x) {
    std::swap(h->tree, x.tree);
    std::swap(h->lists.p2p_start, x.p2p_start);
    std::swap(h->lists.p2p_src, x.p2p_src);
    std::swap(h->lists.m2l_start, x.m2l_start);
    std::swap(h->lists.m2l_src, x.m2l_src);
    std::swap(h->lists.ls.p2p_sorted, x.p2p_sorted);
    std::swap(h->lists.ls.m2l_sorted, x.m2l_sorted);
    std::swap(h->lists.n_p2p, x.n_p2p);
    std::swap(h->lists.n_m2l, x.n_m2l);
    std::swap(h->lists.ls.key_bits, x.key_bits);
    std::swap(h->L, x.L);
    std::swap(h->pos32, x.pos32);
    std::swap(h->alp32, x.alp32);
    std::swap(h->ts.perm, x.perm);
  };
  const size_t nbody_fields = (size_t)(F_A + 3) * cap; // J, X, alpha: fields 0 .. F_A+2
  // with relaxation, the last stage's context also keeps alpha after the
  // update and before the relaxation, which the transposed relaxation needs
  const bool   relax        = c.relax > 0;
  auto relaxed_stage = [&](int k) { return relax && k == S - 1; };
  // reverse sweep: per segment, recompute its steps from the checkpoint
  // keeping every stage's evaluation context, then run the stages backwards
  for (int seg = nck - 1; seg >= 0; seg--) {
    const int st0 = seg * every, st1 = std::min(steps, st0 + every);
    load_state(h, A.ckpt.p + (size_t)seg * slot);
    for (int st = st0; st < st1; st++)
      for (int k = 0; k < S; k++) {
        Ctx &x = A.ctx[(size_t)(st - st0) * S + k];
        build_tree_and_lists(h, true);
        calculate(h);
        x.body.reserve(nbody_fields + cap + (relaxed_stage(k) ? 3 * cap : 0));
        x.info.reserve(1);
        VFMM_CUDA_TRY(cudaMemcpyAsync(x.body.p, h->soa[h->cur].p, nbody_fields * sizeof(double), cudaMemcpyDeviceToDevice, s));
        VFMM_CUDA_TRY(cudaMemcpyAsync(x.body.p + nbody_fields, h->soa[h->cur].p + (size_t)F_R * cap, cap * sizeof(double),
                                      cudaMemcpyDeviceToDevice, s));
        VFMM_CUDA_TRY(cudaMemcpyAsync(x.info.p, h->info, sizeof(DevInfo), cudaMemcpyDeviceToDevice, s));
        exchange(x);
        if (relaxed_stage(k)) {
          stage_update(h, k, dt, false);
          VFMM_CUDA_TRY(cudaMemcpyAsync(x.body.p + nbody_fields + cap, h->soa[h->cur].p + (size_t)F_A * cap, 3 * cap * sizeof(double),
                                        cudaMemcpyDeviceToDevice, s));
          relax_bodies(s, h->soa[h->cur].p, cap, N, c.relax);
        } else
          stage_update(h, k, dt);
      }
    for (int st = st1 - 1; st >= st0; st--)
      for (int k = S - 1; k >= 0; k--) {
        Ctx &x = A.ctx[(size_t)(st - st0) * S + k];
        exchange(x);
        VFMM_CUDA_TRY(cudaMemcpyAsync(h->soa[h->cur].p, x.body.p, nbody_fields * sizeof(double), cudaMemcpyDeviceToDevice, s));
        VFMM_CUDA_TRY(cudaMemcpyAsync(h->soa[h->cur].p + (size_t)F_R * cap, x.body.p + nbody_fields, cap * sizeof(double),
                                      cudaMemcpyDeviceToDevice, s));
        if (relaxed_stage(k))
          adjoint_relax(s, A.g[gc].p, A.w.p, h->soa[h->cur].p, x.body.p + nbody_fields + cap, cap, N, c.relax);
        adjoint_stage_pre(s, A.g[gc].p, A.w.p, cap, N, c.integrator, k, dt, c.rk4_fixed);
        adjoint_seeds(s, h->soa[h->cur].p, A.w.p, cap, N, c.stretching, relaxed_stage(k), c.formulation);
        vjp(x.info.p);
      }
  }
  A.rows.reserve(3 * (size_t)N);
  if (gx) {
    adjoint_rows(s, A.g[gc].p, cap, N, G_XB, A.rows.p);
    VFMM_CUDA_TRY(cudaMemcpyAsync(gx, A.rows.p, 3 * (size_t)N * sizeof(double), cudaMemcpyDeviceToHost, s));
    VFMM_CUDA_TRY(cudaStreamSynchronize(s));
  }
  if (ga) {
    adjoint_rows(s, A.g[gc].p, cap, N, G_AB, A.rows.p);
    VFMM_CUDA_TRY(cudaMemcpyAsync(ga, A.rows.p, 3 * (size_t)N * sizeof(double), cudaMemcpyDeviceToHost, s));
    VFMM_CUDA_TRY(cudaStreamSynchronize(s));
  }
  h->has_tree = h->has_eval = false;
}

} // namespace

int vfmm_adjoint(vfmm_handle h, const vfmm_body *bodies, size_t n, double dt, int steps, int checkpoint_every, const vfmm_objective *objective,
                 double *value, double *grad_x, double *grad_alpha)
{
  return guarded(h, [&] { adjoint(h, bodies, n, dt, steps, checkpoint_every, objective, value, grad_x, grad_alpha); });
}

int vfmm_rbf(vfmm_handle h, vfmm_body *particles, size_t n, vfmm_body *points, size_t m, size_t *m_out, int *iterations)
{
  return guarded(h, [&] {
    if (!particles || !points || !m_out)
      throw Error(VFMM_ERR_INVALID, "null argument");
    if (m == 0)
      throw Error(VFMM_ERR_INVALID, "no points");
    rbf(h, particles, n, points, m, m_out, iterations);
  });
}

int vfmm_diagnostics(vfmm_handle h, double *out)
{
  return guarded(h, [&] {
    if (!out)
      throw Error(VFMM_ERR_INVALID, "null output");
    if (h->n == 0)
      throw Error(VFMM_ERR_STATE, "no bodies on the device");
    h->dtmp.reserve(DIAG_SCRATCH + 16);
    diagnostics(h->stream, h->soa[h->cur].p, h->cap, h->n, h->dtmp.p, h->dtmp.p + DIAG_SCRATCH);
    VFMM_CUDA_TRY(cudaMemcpyAsync(out, h->dtmp.p + DIAG_SCRATCH, 9 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    VFMM_CUDA_TRY(cudaStreamSynchronize(h->stream));
  });
}

int vfmm_relax(vfmm_handle h, double f)
{
  return guarded(h, [&] {
    if (!h->has_eval)
      throw Error(VFMM_ERR_STATE, "relaxation needs J from a calculate");
    if (f < 0 || f > 1)
      throw Error(VFMM_ERR_INVALID, "relaxation factor must be in [0, 1]");
    relax_bodies(h->stream, h->soa[h->cur].p, h->cap, h->n, f);
    VFMM_CUDA_TRY(cudaStreamSynchronize(h->stream));
  });
}

int vfmm_get_tree(vfmm_handle h, vfmm_cell *cells, size_t cap, size_t *ncells)
{
  return guarded(h, [&] {
    if (!h->has_tree)
      throw Error(VFMM_ERR_STATE, "no tree: call init first");
    if (ncells)
      *ncells = (size_t)h->tree.ncells;
    if (!cells || cap < (size_t)h->tree.ncells)
      return;
    const int        nc = h->tree.ncells;
    std::vector<int> ni(nc), nb(nc), ch(nc), bo(nc), lv(nc);
    std::vector<double> x(nc), y(nc), z(nc), R(nc);
    VFMM_CUDA_TRY(cudaMemcpy(ni.data(), h->tree.nchild.p, nc * sizeof(int), cudaMemcpyDeviceToHost));
    VFMM_CUDA_TRY(cudaMemcpy(nb.data(), h->tree.nbody.p, nc * sizeof(int), cudaMemcpyDeviceToHost));
    VFMM_CUDA_TRY(cudaMemcpy(ch.data(), h->tree.child.p, nc * sizeof(int), cudaMemcpyDeviceToHost));
    VFMM_CUDA_TRY(cudaMemcpy(bo.data(), h->tree.body.p, nc * sizeof(int), cudaMemcpyDeviceToHost));
    VFMM_CUDA_TRY(cudaMemcpy(lv.data(), h->tree.level.p, nc * sizeof(int), cudaMemcpyDeviceToHost));
    VFMM_CUDA_TRY(cudaMemcpy(x.data(), h->tree.x.p, nc * sizeof(double), cudaMemcpyDeviceToHost));
    VFMM_CUDA_TRY(cudaMemcpy(y.data(), h->tree.y.p, nc * sizeof(double), cudaMemcpyDeviceToHost));
    VFMM_CUDA_TRY(cudaMemcpy(z.data(), h->tree.z.p, nc * sizeof(double), cudaMemcpyDeviceToHost));
    VFMM_CUDA_TRY(cudaMemcpy(R.data(), h->tree.R.p, nc * sizeof(double), cudaMemcpyDeviceToHost));
    for (int i = 0; i < nc; i++) {
      cells[i].NCHILD      = (uint64_t)ni[i];
      cells[i].NBODY       = (uint64_t)nb[i];
      cells[i].ChildOffset = (uint64_t)ch[i];
      cells[i].BodyOffset  = (uint64_t)bo[i];
      cells[i].X[0]        = x[i];
      cells[i].X[1]        = y[i];
      cells[i].X[2]        = z[i];
      cells[i].R           = R[i];
      cells[i].level       = (uint64_t)lv[i];
    }
  });
}

int vfmm_get_lists(vfmm_handle h, uint64_t *p2p, size_t cap_p2p, size_t *n_p2p, uint64_t *m2l, size_t cap_m2l, size_t *n_m2l)
{
  return guarded(h, [&] {
    if (!h->has_tree)
      throw Error(VFMM_ERR_STATE, "no lists: call init first");
    if (n_p2p)
      *n_p2p = (size_t)h->lists.n_p2p;
    if (n_m2l)
      *n_m2l = (size_t)h->lists.n_m2l;
    const int kb   = h->lists.ls.key_bits;
    auto      fetch = [&](const unsigned long long *src, int cnt, uint64_t *dst, size_t cap) {
      if (!dst || cap < (size_t)cnt || cnt == 0)
        return;
      std::vector<unsigned long long> k(cnt);
      VFMM_CUDA_TRY(cudaMemcpy(k.data(), src, cnt * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
      for (int i = 0; i < cnt; i++) {
        dst[2 * i]     = k[i] >> kb;
        dst[2 * i + 1] = k[i] & ((1ull << kb) - 1);
      }
    };
    VFMM_CUDA_TRY(cudaStreamSynchronize(h->stream));
    fetch(h->lists.ls.p2p_sorted.p, h->lists.n_p2p, p2p, cap_p2p);
    fetch(h->lists.ls.m2l_sorted.p, h->lists.n_m2l, m2l, cap_m2l);
  });
}

int vfmm_get_expansions(vfmm_handle h, double *M, double *L, size_t cap_cells)
{
  return guarded(h, [&] {
    if (!h->has_eval)
      throw Error(VFMM_ERR_STATE, "no expansions: call calculate first");
    if (cap_cells < (size_t)h->tree.ncells)
      throw Error(VFMM_ERR_INVALID, "capacity below the cell count");
    const size_t cnt = (size_t)h->tree.ncells * 3 * h->cfg.p * (h->cfg.p + 1) / 2;
    VFMM_CUDA_TRY(cudaStreamSynchronize(h->stream));
    if (M)
      VFMM_CUDA_TRY(cudaMemcpy(M, h->M.p, cnt * sizeof(double2), cudaMemcpyDeviceToHost));
    if (L)
      VFMM_CUDA_TRY(cudaMemcpy(L, h->L.p, cnt * sizeof(double2), cudaMemcpyDeviceToHost));
  });
}

int vfmm_load(vfmm_handle h, const vfmm_body *bodies, size_t n)
{
  return guarded(h, [&] {
    if (!bodies)
      throw Error(VFMM_ERR_INVALID, "null bodies");
    upload(h, bodies, n);
    VFMM_CUDA_TRY(cudaStreamSynchronize(h->stream));
    h->has_tree = false;
    h->has_eval = false;
  });
}

int vfmm_stage(vfmm_handle h, int stage, double dt)
{
  return guarded(h, [&] {
    if (h->n == 0)
      throw Error(VFMM_ERR_STATE, "no bodies: call load first");
    if (stage < 0 || stage >= stages_of(h->cfg.integrator))
      throw Error(VFMM_ERR_INVALID, "stage index out of range");
    run_stage(h, stage, dt);
  });
}

int vfmm_num_stages(vfmm_handle h) { return h ? stages_of(h->cfg.integrator) : 0; }

int vfmm_direct(vfmm_handle h, vfmm_body *targets, size_t nt, const vfmm_body *sources, size_t ns)
{
  return guarded(h, [&] {
    if (!targets || !sources || nt == 0 || ns == 0)
      throw Error(VFMM_ERR_INVALID, "empty direct sum");
    cudaStream_t s = h->stream;
    // sources through the handle's body buffers, targets through scratch
    upload(h, sources, ns);
    h->has_tree = false;
    h->has_eval = false;
    h->dtmp.reserve(nt * (3 + 12));
    double *tx = h->dtmp.p, *out = tx + 3 * nt;
    std::vector<double> hx(3 * nt);
    for (size_t i = 0; i < nt; i++)
      for (int d = 0; d < 3; d++)
        hx[d * nt + i] = targets[i].X[d];
    VFMM_CUDA_TRY(cudaMemcpyAsync(tx, hx.data(), 3 * nt * sizeof(double), cudaMemcpyHostToDevice, s));
    direct_sum(s, tx, tx + nt, tx + 2 * nt, (int)nt, h->soa[h->cur].p, h->cap, (int)ns, out);
    std::vector<double> ho(12 * nt);
    VFMM_CUDA_TRY(cudaMemcpyAsync(ho.data(), out, 12 * nt * sizeof(double), cudaMemcpyDeviceToHost, s));
    VFMM_CUDA_TRY(cudaStreamSynchronize(s));
    for (size_t i = 0; i < nt; i++) {
      for (int d = 0; d < 3; d++)
        targets[i].velocity[d] = ho[d * nt + i];
      for (int k = 0; k < 9; k++)
        targets[i].J[k / 3][k % 3] = ho[(3 + k) * nt + i];
    }
  });
}

namespace {
// The model-consistent direct sum at tree-order bodies `targets` (host) into
// out (host, nt x 12), on the handle's current tree and lists.
void direct_model_host(vfmm_handle h, const uint32_t *targets, size_t nt, double *out)
{
  cudaStream_t s       = h->stream;
  const int    nchunks = std::max(1, std::min(64, h->n / 4096));
  h->dtmp.reserve((size_t)nt * 12 * (nchunks + 2) + nt / 2 + 1);
  double   *scratch = h->dtmp.p, *dout = scratch + (size_t)nt * 12 * (nchunks + 1);
  uint32_t *dtgt    = reinterpret_cast<uint32_t *>(dout + (size_t)nt * 12);
  VFMM_CUDA_TRY(cudaMemcpyAsync(dtgt, targets, nt * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
  direct_model_sum(s, h->soa[h->cur].p, h->cap, h->n, h->tree.view(), h->tree.leaf_cells.p, h->tree.nleaves, h->lists.p2p_start.p,
                   h->lists.p2p_src.p, dtgt, (int)nt, scratch, nchunks, dout);
  VFMM_CUDA_TRY(cudaMemcpyAsync(out, dout, nt * 12 * sizeof(double), cudaMemcpyDeviceToHost, s));
  VFMM_CUDA_TRY(cudaStreamSynchronize(s));
}
} // namespace

int vfmm_direct_model(vfmm_handle h, const uint32_t *targets, size_t nt, double *out)
{
  return guarded(h, [&] {
    if (!targets || !out || nt == 0)
      throw Error(VFMM_ERR_INVALID, "empty target set");
    if (!h->has_tree || h->moved)
      throw Error(VFMM_ERR_STATE, "the model direct sum needs the tree of the current positions: call init first");
    if (nt > (size_t)INT_MAX / 16)
      throw Error(VFMM_ERR_INVALID, "too many targets");
    for (size_t i = 0; i < nt; i++)
      if (targets[i] >= (uint32_t)h->n)
        throw Error(VFMM_ERR_INVALID, "target index out of range");
    direct_model_host(h, targets, nt, out);
  });
}

int vfmm_choose_order(vfmm_handle h, const vfmm_body *bodies, size_t n, double tol, int pmin, int pmax, int targets, int *p_out,
                      double *err_out)
{
  return guarded(h, [&] {
    if (!bodies || !p_out || n == 0 || targets < 1 || !(tol > 0) || pmin < PMIN || pmax > PMAX || pmin > pmax)
      throw Error(VFMM_ERR_INVALID, "choose_order: bad argument (orders 2..16, tol > 0, targets >= 1)");
    upload(h, bodies, n);
    build_tree_and_lists(h);
    const size_t          nt = std::min<size_t>((size_t)targets, n);
    std::vector<uint32_t> tgt(nt);
    for (size_t i = 0; i < nt; i++)
      tgt[i] = (uint32_t)(i * n / nt);
    std::vector<double> ref(nt * 12), u(3 * (size_t)n);
    direct_model_host(h, tgt.data(), nt, ref.data());
    double nref = 0;
    for (size_t i = 0; i < nt; i++)
      for (int d = 0; d < 3; d++)
        nref += ref[12 * i + d] * ref[12 * i + d];
    const int p0     = h->cfg.p;
    int       chosen = pmax;
    double    err    = 0;
    try {
      for (int p = pmin; p <= pmax; p++) {
        h->cfg.p = p;
        calculate(h);
        VFMM_CUDA_TRY(cudaMemcpyAsync(u.data(), h->soa[h->cur].p + (size_t)F_U * h->cap, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
        VFMM_CUDA_TRY(cudaMemcpyAsync(u.data() + n, h->soa[h->cur].p + (size_t)(F_U + 1) * h->cap, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                      h->stream));
        VFMM_CUDA_TRY(cudaMemcpyAsync(u.data() + 2 * n, h->soa[h->cur].p + (size_t)(F_U + 2) * h->cap, sizeof(double) * n,
                                      cudaMemcpyDeviceToHost, h->stream));
        check_eval_err(h);
        double e2 = 0;
        for (size_t i = 0; i < nt; i++)
          for (int d = 0; d < 3; d++) {
            const double diff = u[(size_t)d * n + tgt[i]] - ref[12 * i + d];
            e2 += diff * diff;
          }
        err = nref > 0 ? std::sqrt(e2 / nref) : 0.0;
        if (err <= tol || p == pmax) {
          chosen = p;
          break;
        }
      }
    } catch (...) {
      h->cfg.p = p0;
      throw;
    }
    h->cfg.p = chosen;
    *p_out   = chosen;
    if (err_out)
      *err_out = err;
  });
}

int vfmm_event_record(vfmm_handle h, int slot)
{
  return guarded(h, [&] {
    if (slot < 0 || slot >= 16)
      throw Error(VFMM_ERR_INVALID, "event slot out of range");
    VFMM_CUDA_TRY(cudaEventRecord(h->ev[slot], h->stream));
  });
}

int vfmm_event_elapsed(vfmm_handle h, int a, int b, float *ms)
{
  return guarded(h, [&] {
    if (a < 0 || a >= 16 || b < 0 || b >= 16 || !ms)
      throw Error(VFMM_ERR_INVALID, "event slot out of range");
    VFMM_CUDA_TRY(cudaEventSynchronize(h->ev[b]));
    VFMM_CUDA_TRY(cudaEventElapsedTime(ms, h->ev[a], h->ev[b]));
  });
}

int vfmm_synchronize(vfmm_handle h)
{
  return guarded(h, [&] { check_eval_err(h); });
}

uint64_t vfmm_launch_count(vfmm_handle h) { return h ? h->launches : 0; }

int vfmm_phase_times(vfmm_handle h, float *ms, int n)
{
  return guarded(h, [&] {
    if (!h->ph_valid)
      throw Error(VFMM_ERR_STATE, "no timed stage yet");
    VFMM_CUDA_TRY(cudaEventSynchronize(h->ph[6]));
    for (int i = 0; i < n && i < 6; i++)
      VFMM_CUDA_TRY(cudaEventElapsedTime(&ms[i], h->ph[i], h->ph[i + 1]));
    // the split leaf kernel's own passes: near field (beside M2L), far field
    if (n > 6)
      ms[6] = 0.f;
    if (n > 7)
      ms[7] = 0.f;
    if (h->split_ran && n > 6)
      VFMM_CUDA_TRY(cudaEventElapsedTime(&ms[6], h->pn[0], h->pn[1]));
    if (h->split_ran && n > 7)
      VFMM_CUDA_TRY(cudaEventElapsedTime(&ms[7], h->pn[2], h->ph[5]));
  });
}

int vfmm_tree_stats(vfmm_handle h, uint64_t *st, int n)
{
  return guarded(h, [&] {
    if (!h->has_tree)
      throw Error(VFMM_ERR_STATE, "no tree");
    read_info(h);
    const uint64_t v[7] = {(uint64_t)h->tree.ncells, (uint64_t)h->tree.nleaves, (uint64_t)h->lists.n_p2p, (uint64_t)h->lists.n_m2l, h->hinfo->p2p_interactions,
                           (uint64_t)h->tree.maxLevel, (uint64_t)tensor_m2l(h)};
    for (int i = 0; i < n && i < 7; i++)
      st[i] = v[i];
  });
}

int vfmm_host_register(void *ptr, size_t bytes)
{
  const cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterMapped | cudaHostRegisterPortable);
  return e == cudaSuccess ? VFMM_OK : VFMM_ERR_CUDA;
}

int vfmm_host_unregister(void *ptr)
{
  const cudaError_t e = cudaHostUnregister(ptr);
  return e == cudaSuccess ? VFMM_OK : VFMM_ERR_CUDA;
}

int vfmm_flush_l2(vfmm_handle h)
{
  return guarded(h, [&] {
    const size_t bytes = (size_t)256 << 20;
    h->flushbuf.reserve(bytes);
    fill_bytes(h->stream, h->flushbuf.p, bytes, 0x5a5a5a5a);
  });
}

int vfmm_measure_fma_peak(vfmm_handle h, int precision, double *tflops)
{
  return guarded(h, [&] {
    if (!tflops)
      throw Error(VFMM_ERR_INVALID, "null output");
    h->dtmp.reserve(16);
    const bool fp64 = precision == VFMM_FP64;
    const int  iters = fp64 ? 4000 : 40000;
    float      ms = 0;
    fma_probe(h->stream, fp64, h->dtmp.p, iters / 10, &ms, h->ev[14], h->ev[15]); // warm-up
    double best = 0;
    for (int r = 0; r < 3; r++) {
      const double flops = fma_probe(h->stream, fp64, h->dtmp.p, iters, &ms, h->ev[14], h->ev[15]);
      best               = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    *tflops = best;
  });
}

} // extern "C"
