// The C ABI (include/vfmm.h): handle, device memory, and the per-stage
// pipeline of the reference's FMMCalculator (src/fmmCalculator.hpp):
//   init      = tree build + lists            (createTree, :71-115)
//   calculate = upward, M2L, downward, L2P+P2P, stretching   (:420-467)
//   advance   = stages of init + calculate + stage update    (:919-1005)
// All work runs on the handle's stream; the host synchronises twice per
// tree build (node counts, pair counts) and at the end of each API call.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <exception>
#include "vfmm_internal.cuh"

namespace vfmm {
thread_local unsigned long long *g_launch_counter = nullptr;
}

using namespace vfmm;

static_assert(sizeof(vfmm_config) == 72, "vfmm_config layout");
static_assert(sizeof(vfmm_body) == 296, "vfmm_body must match exafmm::Body");
static_assert(sizeof(vfmm_cell) == 72, "vfmm_cell layout");

struct vfmm_handle_s {
  vfmm_config  cfg;
  int          device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t  ev[16]{};
  cudaEvent_t  ph[8]{};
  bool         ph_valid = false;
  std::string  err;
  unsigned long long launches = 0;

  // bodies, field-major SoA, double-buffered for reordering
  size_t         cap = 0;
  int            n   = 0;
  DevBuf<double> soa[2];
  int            cur = 0;
  DevBuf<double> aos; // device staging for 296-byte records

  // tree
  DevInfo       *info  = nullptr; // device
  DevInfo       *hinfo = nullptr; // pinned host
  TreeScratch    ts;
  ListScratch    ls;
  DevBuf<int>    c_nchild, c_nbody, c_child, c_body, c_level, c_parent;
  DevBuf<double> c_x, c_y, c_z, c_R;
  DevBuf<int>    level_cells, level_start, leaf_cells;
  int            level_start_host[MAXL + 2]{};
  int            ncells = 0, nleaves = 0, maxLevel = 0;

  // lists
  DevBuf<int>        p2p_start, p2p_src, m2l_start, m2l_src;
  int                n_p2p = 0, n_m2l = 0;
  unsigned long long interactions = 0;
  size_t             cap_front = 0, cap_p2p = 0, cap_m2l = 0;

  // expansions
  DevBuf<double2> M, L, Mprep;
  DevBuf<int4>    items, items32, lanes32;
  int             m2l_batch = 16; // sources per mixed-M2L batch; VFMM_M2L_BATCH = 8, 16 or 32 overrides
  int             items_P = 0, items_per_lane = 0;
  DevBuf<float2>  Mp32;
  DevBuf<float4>  pos32, alp32;

  DevBuf<unsigned char> flushbuf;
  DevBuf<double>        dtmp;
  bool                  has_tree = false, has_eval = false;

  CellsView cells()
  {
    return CellsView{c_nchild.p, c_nbody.p, c_child.p, c_body.p, c_level.p, c_parent.p, c_x.p, c_y.p, c_z.p, c_R.p};
  }
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

void upload(vfmm_handle h, const vfmm_body *b, size_t n)
{
  ensure_bodies(h, n);
  VFMM_CUDA_TRY(cudaMemcpyAsync(h->aos.p, b, n * sizeof(vfmm_body), cudaMemcpyHostToDevice, h->stream));
  aos_to_soa(h->stream, h->aos.p, h->soa[h->cur].p, h->cap, (int)n);
}

void download(vfmm_handle h, vfmm_body *b, size_t n)
{
  if ((int)n != h->n)
    throw Error(VFMM_ERR_INVALID, "body count differs from the bodies on the device");
  soa_to_aos(h->stream, h->soa[h->cur].p, h->cap, h->aos.p, (int)n);
  VFMM_CUDA_TRY(cudaMemcpyAsync(b, h->aos.p, n * sizeof(vfmm_body), cudaMemcpyDeviceToHost, h->stream));
  VFMM_CUDA_TRY(cudaStreamSynchronize(h->stream));
}

void read_info(vfmm_handle h)
{
  VFMM_CUDA_TRY(cudaMemcpyAsync(h->hinfo, h->info, sizeof(DevInfo), cudaMemcpyDeviceToHost, h->stream));
  VFMM_CUDA_TRY(cudaStreamSynchronize(h->stream));
}

// Tree and lists of the bodies in soa[cur]; bodies are reordered into tree order.
void build_tree_and_lists(vfmm_handle h)
{
  cudaStream_t s = h->stream;
  const int    n = h->n;
  const auto  &c = h->cfg;
  h->has_tree    = false;
  h->has_eval    = false;
  VFMM_CUDA_TRY(cudaEventRecord(h->ph[0], s));
  VFMM_CUDA_TRY(cudaMemsetAsync(h->info, 0, sizeof(DevInfo), s));
  check_finite(s, h->soa[h->cur].p, h->cap, n, h->info);
  tree_bounds(s, h->soa[h->cur].p + (size_t)F_X * h->cap, h->cap, n, h->info, h->ts);
  tree_sort_bodies(s, h->soa[h->cur].p + (size_t)F_X * h->cap, h->cap, n, c.ncrit, h->info, h->ts);
  gather_bodies(s, h->soa[h->cur].p, h->soa[h->cur ^ 1].p, h->cap, h->ts.perm.p, n, (1ull << NFIELD) - 1);
  h->cur ^= 1;
  const int nncap = n + MAXL * (n / (c.ncrit + 1)) + 64;
  h->c_nchild.reserve(nncap);
  h->c_nbody.reserve(nncap);
  h->c_child.reserve(nncap);
  h->c_body.reserve(nncap);
  h->c_level.reserve(nncap);
  h->c_parent.reserve(nncap);
  h->c_x.reserve(nncap);
  h->c_y.reserve(nncap);
  h->c_z.reserve(nncap);
  h->c_R.reserve(nncap);
  h->level_cells.reserve(nncap);
  h->leaf_cells.reserve(nncap);
  h->level_start.reserve(MAXL + 2);
  tree_build_cells(s, n, c.ncrit, nncap, h->info, h->ts, h->cells(), h->level_cells.p, h->level_start.p, h->leaf_cells.p);
  VFMM_CUDA_TRY(cudaMemcpyAsync(h->level_start_host, h->level_start.p, sizeof(int) * (MAXL + 2), cudaMemcpyDeviceToHost, s));
  read_info(h);
  if (h->hinfo->nonfinite)
    throw Error(VFMM_ERR_NONFINITE, "non-finite position, strength or radius");
  if (h->hinfo->err)
    throw Error(h->hinfo->err, "tree deeper than 21 levels: more than ncrit bodies (nearly) coincide");
  if (h->hinfo->overflow)
    throw Error(VFMM_ERR_CAPACITY, "tree node capacity exceeded");
  h->ncells   = h->hinfo->nnodes;
  h->nleaves  = h->hinfo->nleaves;
  h->maxLevel = h->hinfo->maxLevel;

  // traversal, growing the list capacities until nothing overflows
  if (h->cap_front == 0) {
    h->cap_front = std::max<size_t>(4096, (size_t)h->ncells * 16);
    h->cap_p2p   = std::max<size_t>(4096, (size_t)h->nleaves * 48);
    h->cap_m2l   = std::max<size_t>(4096, (size_t)h->ncells * 240);
  }
  for (int attempt = 0;; attempt++) {
    h->ls.front[0].reserve(h->cap_front);
    h->ls.front[1].reserve(h->cap_front);
    h->ls.p2p_raw.reserve(h->cap_p2p);
    h->ls.m2l_raw.reserve(h->cap_m2l);
    traverse(s, h->cells(), h->cells(), h->ncells, h->maxLevel, h->maxLevel, c.theta, h->info, h->ls, h->ls.front[0].cap, h->ls.p2p_raw.cap,
             h->ls.m2l_raw.cap);
    read_info(h);
    if (!h->hinfo->overflow)
      break;
    if (attempt > 8)
      throw Error(VFMM_ERR_CAPACITY, "interaction lists keep overflowing");
    h->cap_front = std::max(h->cap_front * 2, h->ls.front[0].cap * 2);
    h->cap_p2p   = std::max(h->cap_p2p * 2, h->ls.p2p_raw.cap * 2);
    h->cap_m2l   = std::max(h->cap_m2l * 2, h->ls.m2l_raw.cap * 2);
    VFMM_CUDA_TRY(cudaMemsetAsync(&h->info->overflow, 0, sizeof(int), s));
  }
  h->n_p2p = h->hinfo->n_p2p;
  h->n_m2l = h->hinfo->n_m2l;
  h->p2p_start.reserve(h->ncells + 1);
  h->m2l_start.reserve(h->ncells + 1);
  h->p2p_src.reserve(h->n_p2p + 1);
  h->m2l_src.reserve(h->n_m2l + 1);
  VFMM_CUDA_TRY(cudaMemsetAsync(&h->info->p2p_interactions, 0, sizeof(unsigned long long), s));
  lists_to_csr(s, h->ls, h->n_p2p, h->n_m2l, h->ncells, 32, h->p2p_start.p, h->p2p_src.p, h->m2l_start.p, h->m2l_src.p, h->c_nbody.p,
               &h->info->p2p_interactions);
  VFMM_CUDA_TRY(cudaEventRecord(h->ph[1], s));
  h->has_tree = true;
  h->has_eval = false;
}

void ensure_items(vfmm_handle h)
{
  if (h->items_P == h->cfg.p)
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
  h->m2l_batch   = sb && (atoi(sb) == 8 || atoi(sb) == 32) ? atoi(sb) : 16;
  auto lt32      = m2l_lane_table(h->cfg.p, h->cfg.p >= 15 ? 8 : 4, h->m2l_batch); // tile width and batch of k_m2l32v2
  h->lanes32.reserve(lt32.size());
  VFMM_CUDA_TRY(cudaMemcpy(h->lanes32.p, lt32.data(), lt32.size() * sizeof(int4), cudaMemcpyHostToDevice));
  h->items_P        = h->cfg.p;
  h->items_per_lane = per;
}

void calculate(vfmm_handle h)
{
  if (!h->has_tree)
    throw Error(VFMM_ERR_STATE, "calculate needs a tree: call init first");
  cudaStream_t s  = h->stream;
  const int    K3 = 3 * h->cfg.p * (h->cfg.p + 1) / 2;
  ensure_items(h);
  h->M.reserve((size_t)h->ncells * K3);
  h->L.reserve((size_t)h->ncells * K3);
  h->Mprep.reserve((size_t)h->ncells * 3 * h->cfg.p * h->cfg.p);
  VFMM_CUDA_TRY(cudaMemsetAsync(h->M.p, 0, sizeof(double2) * (size_t)h->ncells * K3, s));
  ExpArgs e{};
  e.P                   = h->cfg.p;
  e.cells               = h->cells();
  e.ncells              = h->ncells;
  e.level_cells         = h->level_cells.p;
  e.level_start_host    = h->level_start_host;
  e.maxLevel            = h->maxLevel;
  e.leaf_cells          = h->leaf_cells.p;
  e.nleaves             = h->nleaves;
  e.soa                 = h->soa[h->cur].p;
  e.cap                 = h->cap;
  e.M                   = h->M.p;
  e.L                   = h->L.p;
  e.Mprep               = h->Mprep.p;
  e.m2l_start           = h->m2l_start.p;
  e.m2l_src             = h->m2l_src.p;
  e.p2p_start           = h->p2p_start.p;
  e.p2p_src             = h->p2p_src.p;
  e.m2l_items           = h->items.p;
  e.m2l_nitems_per_lane = h->items_per_lane;
  e.stretching          = h->cfg.stretching;
  e.formulation         = h->cfg.formulation;
  if (h->cfg.precision == VFMM_MIXED) {
    h->Mp32.reserve((size_t)h->ncells * 3 * h->cfg.p * h->cfg.p);
    h->pos32.reserve(h->n);
    h->alp32.reserve(h->n);
    MixedArgs m{};
    m.Mp32    = h->Mp32.p;
    m.pos32   = h->pos32.p;
    m.alp32   = h->alp32.p;
    m.items32 = h->items32.p;
    m.lanes32   = h->lanes32.p;
    m.m2l_batch = h->m2l_batch;
    m.R0      = h->hinfo->R0;
    p2m_mixed(s, e, m);
    m2m_pass(s, e);
    VFMM_CUDA_TRY(cudaEventRecord(h->ph[2], s));
    m2l_mixed(s, e, m);
    VFMM_CUDA_TRY(cudaEventRecord(h->ph[3], s));
    downward_l2l(s, e);
    VFMM_CUDA_TRY(cudaEventRecord(h->ph[4], s));
    l2p_p2p_mixed(s, e, m, h->soa[h->cur].p);
    VFMM_CUDA_TRY(cudaEventRecord(h->ph[5], s));
  } else {
    upward_pass(s, e);
    VFMM_CUDA_TRY(cudaEventRecord(h->ph[2], s));
    m2l_pass(s, e);
    VFMM_CUDA_TRY(cudaEventRecord(h->ph[3], s));
    downward_l2l(s, e);
    VFMM_CUDA_TRY(cudaEventRecord(h->ph[4], s));
    l2p_p2p_pass(s, e, h->soa[h->cur].p);
    VFMM_CUDA_TRY(cudaEventRecord(h->ph[5], s));
  }
  h->has_eval = true;
}

void stage_update(vfmm_handle h, int stage, double dt)
{
  StageArgs a{};
  a.scheme        = h->cfg.integrator;
  a.stage         = stage;
  a.stretching    = h->cfg.stretching;
  a.formulation   = h->cfg.formulation;
  a.rk4_fixed     = h->cfg.rk4_fixed;
  a.store_initial = (stage == 0 && (a.scheme == VFMM_RK2 || a.scheme == VFMM_RK4)) ? 1 : 0;
  a.do_update     = 1;
  a.dt            = dt;
  a.relax         = (stage == stages_of(a.scheme) - 1) ? h->cfg.relax : 0.0;
  finish_and_update(h->stream, h->soa[h->cur].p, h->cap, h->n, a);
  VFMM_CUDA_TRY(cudaEventRecord(h->ph[6], h->stream));
  h->ph_valid = true;
}

void run_stage(vfmm_handle h, int stage, double dt)
{
  build_tree_and_lists(h);
  calculate(h);
  stage_update(h, stage, dt);
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
    VFMM_CUDA_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    for (auto &e : h->ev)
      VFMM_CUDA_TRY(cudaEventCreate(&e));
    for (auto &e : h->ph)
      VFMM_CUDA_TRY(cudaEventCreate(&e));
    VFMM_CUDA_TRY(cudaMalloc((void **)&h->info, sizeof(DevInfo)));
    VFMM_CUDA_TRY(cudaMallocHost((void **)&h->hinfo, sizeof(DevInfo)));
    std::memset(h->hinfo, 0, sizeof(DevInfo));
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
  for (auto *b : {&h->soa[0], &h->soa[1], &h->aos, &h->c_x, &h->c_y, &h->c_z, &h->c_R, &h->dtmp})
    b->release();
  for (auto *b : {&h->c_nchild, &h->c_nbody, &h->c_child, &h->c_body, &h->c_level, &h->c_parent, &h->level_cells, &h->level_start, &h->leaf_cells,
                  &h->p2p_start, &h->p2p_src, &h->m2l_start, &h->m2l_src})
    b->release();
  h->M.release();
  h->L.release();
  h->Mprep.release();
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
  h->ls.front[0].release();
  h->ls.front[1].release();
  for (auto *b : {&h->ls.p2p_raw, &h->ls.m2l_raw, &h->ls.p2p_sorted, &h->ls.m2l_sorted})
    b->release();
  h->ls.cub_tmp.release();
  if (h->info)
    cudaFree(h->info);
  if (h->hinfo)
    cudaFreeHost(h->hinfo);
  for (auto &e : h->ev)
    if (e)
      cudaEventDestroy(e);
  for (auto &e : h->ph)
    if (e)
      cudaEventDestroy(e);
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
    upload(h, bodies, n);
    const int ns = stages_of(h->cfg.integrator);
    for (int st = 0; st < ns; st++)
      run_stage(h, st, dt);
    download(h, bodies, n);
  });
}

int vfmm_get_sensor_data(vfmm_handle h, vfmm_body *sensors, size_t n)
{
  return guarded(h, [&] {
    (void)sensors;
    (void)n;
    throw Error(VFMM_ERR_UNSUPPORTED, "sensor evaluation is not implemented yet");
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
      *ncells = (size_t)h->ncells;
    if (!cells || cap < (size_t)h->ncells)
      return;
    const int        nc = h->ncells;
    std::vector<int> ni(nc), nb(nc), ch(nc), bo(nc), lv(nc);
    std::vector<double> x(nc), y(nc), z(nc), R(nc);
    VFMM_CUDA_TRY(cudaMemcpy(ni.data(), h->c_nchild.p, nc * sizeof(int), cudaMemcpyDeviceToHost));
    VFMM_CUDA_TRY(cudaMemcpy(nb.data(), h->c_nbody.p, nc * sizeof(int), cudaMemcpyDeviceToHost));
    VFMM_CUDA_TRY(cudaMemcpy(ch.data(), h->c_child.p, nc * sizeof(int), cudaMemcpyDeviceToHost));
    VFMM_CUDA_TRY(cudaMemcpy(bo.data(), h->c_body.p, nc * sizeof(int), cudaMemcpyDeviceToHost));
    VFMM_CUDA_TRY(cudaMemcpy(lv.data(), h->c_level.p, nc * sizeof(int), cudaMemcpyDeviceToHost));
    VFMM_CUDA_TRY(cudaMemcpy(x.data(), h->c_x.p, nc * sizeof(double), cudaMemcpyDeviceToHost));
    VFMM_CUDA_TRY(cudaMemcpy(y.data(), h->c_y.p, nc * sizeof(double), cudaMemcpyDeviceToHost));
    VFMM_CUDA_TRY(cudaMemcpy(z.data(), h->c_z.p, nc * sizeof(double), cudaMemcpyDeviceToHost));
    VFMM_CUDA_TRY(cudaMemcpy(R.data(), h->c_R.p, nc * sizeof(double), cudaMemcpyDeviceToHost));
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
      *n_p2p = (size_t)h->n_p2p;
    if (n_m2l)
      *n_m2l = (size_t)h->n_m2l;
    auto fetch = [&](const unsigned long long *src, int cnt, uint64_t *dst, size_t cap) {
      if (!dst || cap < (size_t)cnt || cnt == 0)
        return;
      std::vector<unsigned long long> k(cnt);
      VFMM_CUDA_TRY(cudaMemcpy(k.data(), src, cnt * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
      for (int i = 0; i < cnt; i++) {
        dst[2 * i]     = k[i] >> 32;
        dst[2 * i + 1] = k[i] & 0xffffffffull;
      }
    };
    VFMM_CUDA_TRY(cudaStreamSynchronize(h->stream));
    fetch(h->ls.p2p_sorted.p, h->n_p2p, p2p, cap_p2p);
    fetch(h->ls.m2l_sorted.p, h->n_m2l, m2l, cap_m2l);
  });
}

int vfmm_get_expansions(vfmm_handle h, double *M, double *L, size_t cap_cells)
{
  return guarded(h, [&] {
    if (!h->has_eval)
      throw Error(VFMM_ERR_STATE, "no expansions: call calculate first");
    if (cap_cells < (size_t)h->ncells)
      throw Error(VFMM_ERR_INVALID, "capacity below the cell count");
    const size_t cnt = (size_t)h->ncells * 3 * h->cfg.p * (h->cfg.p + 1) / 2;
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
  return guarded(h, [&] { VFMM_CUDA_TRY(cudaStreamSynchronize(h->stream)); });
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
  });
}

int vfmm_tree_stats(vfmm_handle h, uint64_t *st, int n)
{
  return guarded(h, [&] {
    if (!h->has_tree)
      throw Error(VFMM_ERR_STATE, "no tree");
    read_info(h);
    const uint64_t v[6] = {(uint64_t)h->ncells, (uint64_t)h->nleaves, (uint64_t)h->n_p2p, (uint64_t)h->n_m2l, h->hinfo->p2p_interactions,
                           (uint64_t)h->maxLevel};
    for (int i = 0; i < n && i < 6; i++)
      st[i] = v[i];
  });
}

int vfmm_host_register(void *ptr, size_t bytes)
{
  const cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
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
