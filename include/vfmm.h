/* vfmm — GB300-native vortex-particle FMM: the C ABI.
 *
 * Drop-in for the particle velocity-and-stretching evaluation of
 * kursatyurt/UVLM, whose call surface is the header-only class template
 * Vortex::FMMCalculator<Host, Device, Integration, Viscous, Formulation,
 * Stretching> (src/fmmCalculator.hpp:25-26) and the free functions
 * exafmm::buildTree (src/tree.hpp:101) and exafmm::getList
 * (src/traverse.hpp:32).  The reference has no FFI of its own; each entry
 * point below names the reference function it replaces.  include/vfmm.hpp
 * wraps these calls in a class with the reference's method names.
 *
 * Conventions
 *  - Every function returns a vfmm_status; VFMM_OK is 0.  After an error,
 *    vfmm_last_error(h) describes it.  A handle owns one CUDA stream and all
 *    of its device memory; calls on one handle must not overlap.
 *  - Bodies cross the boundary as arrays of vfmm_body, byte-compatible with
 *    the reference's exafmm::Body (37 doubles, 296 bytes).
 *  - Compile-time constants of the reference (P, ncrit, MAC_theta,
 *    exafmmTypes.hpp:12-15) and its template policy tags
 *    (fmmCalculator.hpp:9-23) are fields of vfmm_config.
 */
#ifndef VFMM_H
#define VFMM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  VFMM_OK               = 0,
  VFMM_ERR_INVALID      = 1, /* bad argument or configuration */
  VFMM_ERR_NONFINITE    = 2, /* NaN/Inf in positions, strengths or radii */
  VFMM_ERR_DEPTH        = 3, /* more than ncrit bodies closer than the deepest level can split */
  VFMM_ERR_CAPACITY     = 4, /* an internal list outgrew its capacity (handled internally; reported only if growth fails) */
  VFMM_ERR_CUDA         = 5, /* a CUDA call failed */
  VFMM_ERR_TIMEOUT      = 6, /* a bounded device-side wait gave up */
  VFMM_ERR_UNSUPPORTED  = 7, /* configuration not implemented (e.g. an expansion order outside 2..16) */
  VFMM_ERR_STATE        = 8  /* call order violated (e.g. calculate before init) */
} vfmm_status;

/* Integration scheme: Vortex::Euler / RK2 / RK3 / RK4 (fmmCalculator.hpp:14-17). */
enum { VFMM_EULER = 0, VFMM_RK2 = 1, VFMM_RK3 = 2, VFMM_RK4 = 3 };
/* Stretching formulation: Vortex::Transposed / Classic (fmmCalculator.hpp:22-23). */
enum { VFMM_TRANSPOSED = 0, VFMM_CLASSIC = 1 };
/* VPM formulation: Vortex::cVPM / rVPM (fmmCalculator.hpp:19-20). */
enum { VFMM_CVPM = 0, VFMM_RVPM = 1 };
/* Viscous scheme: Vortex::Inviscid / PSE / CSM (fmmCalculator.hpp:11-12, 713-724). */
enum { VFMM_INVISCID = 0, VFMM_PSE = 1, VFMM_CSM = 2 };
/* Arithmetic of the evaluation: FP64 throughout (the drop-in), or mixed
 * (FP32 P2P with compensated sums, FP32 P2M/M2M/M2L/L2L/L2P with per-cell
 * scaling, FP64 tree and FP64 expansion arrays between the kernels). */
enum { VFMM_FP64 = 0, VFMM_MIXED = 1 };

typedef struct {
  int    p;           /* expansion terms n = 0..p-1; reference P (exafmmTypes.hpp:12); 2..16 */
  int    ncrit;       /* bodies per leaf; reference ncrit (exafmmTypes.hpp:14); 1..256 */
  double theta;       /* multipole acceptance criterion; reference MAC_theta (exafmmTypes.hpp:15) */
  int    precision;   /* VFMM_FP64 or VFMM_MIXED */
  int    integrator;  /* VFMM_EULER .. VFMM_RK4 */
  int    stretching;  /* VFMM_TRANSPOSED or VFMM_CLASSIC */
  int    formulation; /* VFMM_CVPM or VFMM_RVPM */
  double relax;       /* relaxation factor f in [0,1]; 0 = off (relaxation.hpp:8-19) */
  int    rk4_fixed;   /* 1: RK4 stage 3 uses dt; 0: 0.5*dt as the reference (fmmCalculator.hpp:683-689) */
  int    device;      /* CUDA device ordinal; -1 = the caller's current device */
  int    viscous;     /* VFMM_INVISCID, VFMM_PSE or VFMM_CSM, applied after every evaluation of a stage */
  int    m2l_batch;   /* mixed mode: M2L sources per batch, 8, 16, 24, 30 or 32 (at most 227 KB of staging: 32 to p = 14, 30 to p = 15); 0 = by p (30 up to 10, 24 to 12, else 16) */
  double nu;          /* kinematic viscosity for PSE/CSM (the reference leaves its _nu unset, fmmCalculator.hpp:56) */
  int    p2p_chunk; /* mixed mode: near-field source bodies the leaf kernel stages per chunk (its P2P tile), 512 or 768; 0 = 768 */
  int    m2l_kernel; /* mixed mode, p = 8..10: 0 = by size (tensor cores from VFMM_TC_MIN_PAIRS M2L pairs up), 1 = tensor cores, 2 = CUDA cores */
} vfmm_config;

/* Below this many M2L pairs an evaluation with m2l_kernel = 0 uses the CUDA-core
 * M2L: the tensor-core M2L's per-evaluation offset-class table pays only when
 * a level's many targets share their offset classes (dense sets). */
#define VFMM_TC_MIN_PAIRS 1500000

/* exafmm::Body (exafmmTypes.hpp:18-32), 296 bytes. J[a][b] = du_a/dx_b. */
typedef struct {
  double J[3][3];
  double X[3];
  double alpha[3];
  double velocity[3];
  double dadt[3];
  double velocity_old[3];
  double dadt_old[3];
  double X_old[3];
  double alpha_old[3];
  double radius;
  double drdt;
  double radius_old;
  double drdt_old;
} vfmm_body;

/* exafmm::Cell without its pointers (exafmmTypes.hpp:36-46), 72 bytes. */
typedef struct {
  uint64_t NCHILD;
  uint64_t NBODY;
  uint64_t ChildOffset;
  uint64_t BodyOffset;
  double   X[3];
  double   R;
  uint64_t level;
} vfmm_cell;

typedef struct vfmm_handle_s *vfmm_handle;

/* Defaults of the reference: p=4, ncrit=128, theta=0.3, RK3, Transposed,
 * cVPM, FP64, no relaxation (exafmmTypes.hpp:12-15, main.cpp:119), current device. */
void vfmm_default_config(vfmm_config *cfg);

/* Create / destroy a calculator on the current CUDA device (the reference
 * constructs Vortex::FMMCalculator by value, fmmCalculator.hpp:25-26). */
int vfmm_create(const vfmm_config *cfg, vfmm_handle *out);
int vfmm_destroy(vfmm_handle h);
const char *vfmm_last_error(vfmm_handle h);
int vfmm_get_config(vfmm_handle h, vfmm_config *cfg);

/* FMMCalculator::init (fmmCalculator.hpp:282-288): copy the bodies to the
 * device, build the octree (exafmm::buildTree, tree.hpp:101-113) and the
 * interaction lists (exafmm::getList, traverse.hpp:32-85).  As in the
 * reference, `bodies` is permuted in place into tree order. */
int vfmm_init(vfmm_handle h, vfmm_body *bodies, size_t n);

/* FMMCalculator::calculate (fmmCalculator.hpp:420-467): velocity, J and
 * dadt (stretching, plus rVPM terms when configured) of the bodies given to
 * the last vfmm_init, left on the device. */
int vfmm_calculate(vfmm_handle h);

/* FMMCalculator::copyBodies2Host (fmmCalculator.hpp:235-243): the device
 * bodies, in tree order, into `bodies` (n must match the last init). */
int vfmm_copy_bodies_to_host(vfmm_handle h, vfmm_body *bodies, size_t n);

/* FMMCalculator::advance (fmmCalculator.hpp:919-1005): one time step of the
 * configured scheme; each stage rebuilds the tree from the current
 * positions.  `bodies` is read, then overwritten with the bodies after the
 * step in the last stage's tree order (velocity, J, dadt from the last stage's
 * evaluation).  With relax > 0, relaxation follows the step (using that J).
 * Only the fields the step reads are loaded: X, alpha and the radius (Euler
 * and RK3 also the RK registers they carry through); velocity, J, dadt, drdt
 * and the other registers are written before they are read. */
int vfmm_advance(vfmm_handle h, vfmm_body *bodies, size_t n, double dt);

/* advance (fmmCalculator.hpp:919-1005) for `count` independent systems at
 * once: system b is bodies[b][0 .. n[b]) on handles[b] (distinct handles, each
 * with its own configuration and stream).  Every system's stages run as in
 * vfmm_advance and give the same results; the work of all systems is
 * interleaved on the GPU.  On an error every handle's vfmm_last_error holds
 * the message and the systems' states are unspecified.  No counterpart in the
 * reference, which advances one system per calculator. */
int vfmm_advance_batch(vfmm_handle *handles, vfmm_body *const *bodies, const size_t *n, int count, double dt);

/* Result of vfmm_autotune. */
typedef struct {
  int    ncrit;                /* chosen leaf size */
  int    m2l_batch;            /* chosen M2L source batch (mixed mode) */
  double ms_per_stage;         /* its measured stage time */
  double default_ms_per_stage; /* the stage time with the configuration before tuning */
  int    tried;                /* configurations timed */
  int    p2p_chunk;            /* chosen P2P tile: near-field sources staged per chunk (mixed mode) */
  int    reserved[2];
} vfmm_tuning;

/* Opt-in autotuner: times one stage (best of two after a warm-up) of `bodies`
 * for leaf sizes 16..256 and, in mixed mode, the leaf kernel's P2P tile (512
 * or 768 staged sources) and, where M2L runs on the CUDA cores, its source
 * batches 16/24/30/32 (those whose staging fits in shared memory at this p);
 * keeps the fastest in the handle (vfmm_get_config shows ncrit, m2l_batch
 * and p2p_chunk).  A
 * leaf size other than the reference's compile-time ncrit (exafmmTypes.hpp:14)
 * builds a different tree and lists, so results are no longer those of the
 * reference at its ncrit.  The bodies on the device afterwards are a copy of
 * `bodies` after one stage; call vfmm_init / vfmm_advance as usual.  No
 * counterpart in the reference. */
int vfmm_autotune(vfmm_handle h, const vfmm_body *bodies, size_t n, double dt, vfmm_tuning *out);

/* Opt-in order choice (no counterpart in the reference, whose P is a
 * compile-time constant, exafmmTypes.hpp:12): the lowest expansion order p in
 * pmin..pmax whose velocity error, relative L2 over `targets` bodies spread
 * over the set, against the model-consistent FP64 direct sum
 * (vfmm_direct_model) is at most tol, in the handle's precision, leaf size and
 * theta.  The handle keeps that order; *p_out receives it (pmax when none
 * meets tol) and *err_out (may be NULL) its error.  The truncation error of
 * the reference's FMM at theta = 0.5 falls roughly 2.3x per two orders (about
 * 2e-3 at p = 10 on a uniform cloud), so tol must suit theta.  Leaves the
 * bodies on the device in tree order after one evaluation. */
int vfmm_choose_order(vfmm_handle h, const vfmm_body *bodies, size_t n, double tol, int pmin, int pmax, int targets, int *p_out,
                      double *err_out);

/* Objective of vfmm_adjoint, evaluated on the state after the last step:
 *   energy * E + impulse . I + sum_i seed_x_i . x_i + seed_alpha_i . alpha_i,
 * E = sum_i u_i . (x_i cross alpha_i) (the kinetic energy of an unbounded
 * flow, u from an FP64 evaluation of that state) and I = 1/2 sum_i x_i cross
 * alpha_i.  The seed arrays hold n x 3 doubles indexed like the `bodies`
 * passed in (bodies move in memory as the trees reorder them; the adjoint
 * tracks that), or are NULL. */
typedef struct vfmm_objective {
  double        energy;
  double        impulse[3];
  const double *seed_x;
  const double *seed_alpha;
} vfmm_objective;

/* Reverse-mode gradient of the objective after `steps` steps of advance
 * from `bodies` (not modified) with respect to their initial positions and
 * strengths: grad_x and grad_alpha receive n x 3 doubles in the order of
 * `bodies`.  The reverse sweep is the transpose of the evaluation (P2P
 * pairs, transposed L2P, L2L, M2L, M2M, P2M, the bounding-box dependence of
 * the cell centres) and of the stage updates, at the states of the forward
 * trajectory, all in the handle's precision: FP64 (the exact derivative of
 * the FP64 step) or mixed (the forward kernels and the transposes in FP32
 * with per-cell scaling).  States are kept every `checkpoint_every` steps;
 * each segment between them is recomputed once, keeping every stage's
 * evaluation (tree, lists, local expansions, body fields: roughly 450 bytes
 * per body at p = 8), and then run backwards, so device memory holds
 * ceil(steps / checkpoint_every) body states plus stages x checkpoint_every
 * stage evaluations.  With grad_x and grad_alpha both NULL only
 * *value is computed.  Covers Euler, RK2, RK3 and RK4 (either third stage,
 * cfg.rk4_fixed), with or without relaxation (cfg.relax; its stage contexts
 * then also keep alpha before each relaxation), for the cVPM and rVPM
 * formulations (rVPM evolves the radii: the gradient runs through them)
 * without viscosity (VFMM_ERR_UNSUPPORTED for PSE/CSM).  The
 * reference has no adjoint; its L2P takes one derivative by complex step
 * (multipoleKernels.hpp:630-742, complexify.hpp). */
int vfmm_adjoint(vfmm_handle h, const vfmm_body *bodies, size_t n, double dt, int steps, int checkpoint_every, const vfmm_objective *objective,
                 double *value, double *grad_x, double *grad_alpha);

/* FMMCalculator::getSensorData (fmmCalculator.hpp:726-731): velocity at probe
 * points from the particles (multipoles of the last calculate, near field
 * from the particles as they are now); velocity and dadt are overwritten, the
 * far-field J is added to the sensors' J.  `sensors` is permuted into its own
 * tree order, as the reference's buildTree does.  Evaluated in FP64.
 * VFMM_ERR_STATE before the first calculate/advance. */
int vfmm_get_sensor_data(vfmm_handle h, vfmm_body *sensors, size_t n);

/* FMMCalculator::RBF (fmmCalculator.hpp:856-917): re-interpolates the
 * particles' vorticity onto new points.  The particles are permuted into their
 * tree order (as init does); points whose vorticity is below 1e-6 in all three
 * components are dropped; the first *m_out entries of `points` then hold the
 * kept points in their tree order with alpha = the strengths that reproduce the
 * vorticity (conjugate gradients, at most 100 iterations, squared residual
 * 1e-10; *iterations, if not null, gets the count).  FP64.  Leaves the handle
 * with the particles' tree and no evaluation. */
int vfmm_rbf(vfmm_handle h, vfmm_body *particles, size_t n, vfmm_body *points, size_t m, size_t *m_out, int *iterations);

/* Global invariants of the bodies on the device, FP64, reproducible:
 * out[0..2] circulation sum alpha, out[3..5] linear impulse 1/2 sum x cross
 * alpha, out[6..8] angular impulse 1/3 sum x cross (x cross alpha).  No
 * counterpart in the reference. */
int vfmm_diagnostics(vfmm_handle h, double *out);

/* Relaxation (relaxation.hpp:8-19, written 0-based) of the device bodies with
 * factor f, using the J of the last evaluation. */
int vfmm_relax(vfmm_handle h, double f);

/* The tree of the last init (exafmm::buildTree output, tree.hpp:101): cells in
 * the reference's order.  *ncells receives the count; at most `cap` are written. */
int vfmm_get_tree(vfmm_handle h, vfmm_cell *cells, size_t cap, size_t *ncells);

/* The interaction lists of the last init (exafmm::getList, traverse.hpp:32):
 * (target, source) cell pairs, sorted by target then source.  Counts are
 * always written; pairs are written when the capacities suffice. */
int vfmm_get_lists(vfmm_handle h, uint64_t *p2p, size_t cap_p2p, size_t *n_p2p, uint64_t *m2l, size_t cap_m2l, size_t *n_m2l);

/* Multipole and local expansions of the last calculate, as
 * ncells * 3*p(p+1)/2 complex doubles (interleaved re, im) in the reference's
 * layout [cell][3*(n(n+1)/2+m) + d] (multipoleKernels.hpp:468-471). */
int vfmm_get_expansions(vfmm_handle h, double *M, double *L, size_t cap_cells);

/* ---- device-resident stepping (inputs already in HBM) ------------------- */

/* Upload bodies once (no tree yet); later stages work on the device copy. */
int vfmm_load(vfmm_handle h, const vfmm_body *bodies, size_t n);
/* One stage of the configured scheme on the device copy: tree, lists,
 * evaluation, stretching and the stage update (stage = 0 .. stages-1). */
int vfmm_stage(vfmm_handle h, int stage, double dt);
/* Number of stages per step of the configured scheme (1, 2, 3 or 4). */
int vfmm_num_stages(vfmm_handle h);

/* ---- direct sum ---------------------------------------------------------- */

/* FP64 all-pairs sum with the reference's regularised kernel
 * (multipoleKernels.hpp:239-283): velocity and J at `nt` targets from `ns`
 * sources, all arrays on the host; the targets' velocity and J are
 * overwritten.  The reference's exafmm::direct (traverse.hpp:88) computes
 * the same velocity. */
int vfmm_direct(vfmm_handle h, vfmm_body *targets, size_t nt, const vfmm_body *sources, size_t ns);

/* No counterpart in the reference (an accuracy yardstick for its FMM).  FP64
 * direct sum with the FMM's own kernel split, on the handle's current tree:
 * pairs whose leaves are on the P2P list use the regularised kernel
 * (multipoleKernels.hpp:239-283), all other pairs the singular Biot-Savart
 * kernel that the multipole and local expansions represent
 * (multipoleKernels.hpp:519-552, :631-742).  Its difference from the FMM is
 * the expansions' truncation error alone.  targets[i] are body indices in
 * tree order (the order vfmm_init leaves the caller's bodies in); out
 * receives nt records of 12 doubles: velocity[3], J[3][3] row-major.  Needs
 * the tree of the current positions (after vfmm_init or vfmm_calculate, not
 * after a stage update): VFMM_ERR_STATE otherwise. */
int vfmm_direct_model(vfmm_handle h, const uint32_t *targets, size_t nt, double *out);

/* ---- instrumentation ----------------------------------------------------- */

/* Record event `slot` (0..15) on the handle's stream; elapsed ms between two
 * recorded slots (waits for the later one). */
int vfmm_event_record(vfmm_handle h, int slot);
int vfmm_event_elapsed(vfmm_handle h, int slot_a, int slot_b, float *ms);
int vfmm_synchronize(vfmm_handle h);
/* Kernel launches issued by this handle since creation. */
uint64_t vfmm_launch_count(vfmm_handle h);
/* Per-phase device time of the last calculate/stage, ms: [0] tree+lists,
 * [1] upward, [2] M2L, [3] downward L2L, [4] L2P+P2P, [5] update.  When the
 * leaf kernel ran split (mixed mode with the tensor-core M2L: the near field
 * on a second stream beside M2L, the far field after L2L), [6] is the near
 * pass from its start to its end and [7] the far pass; both 0 otherwise, and
 * [3] and [4] then include waits for the near pass. */
int vfmm_phase_times(vfmm_handle h, float *ms, int n);
/* Sizes of the last tree: cells, leaves, P2P pairs, M2L pairs, P2P body-body
 * interactions (self pairs excluded), max level; [6] is 1 when M2L of an
 * evaluation on these lists runs on the tensor cores (vfmm_config.m2l_kernel). */
int vfmm_tree_stats(vfmm_handle h, uint64_t *stats, int n);
/* Page-lock and map a host range (cudaHostRegister, mapped).  Calls given
 * bodies that lie wholly in such a range read and write them directly from
 * the transposing kernels over the host link, with no staging copy. */
int vfmm_host_register(void *ptr, size_t bytes);
int vfmm_host_unregister(void *ptr);
/* Fill a device scratch buffer larger than L2 to evict cached data. */
int vfmm_flush_l2(vfmm_handle h);
/* Measured CUDA-core throughput of independent FMA chains on this GPU, in
 * TFLOP/s (2 flops per FMA): precision VFMM_FP64 or VFMM_MIXED (FP32).  The
 * roofline denominator for the compute-bound FMM kernels, which run on the
 * FP64/FP32 pipes rather than on tensor cores. */
int vfmm_measure_fma_peak(vfmm_handle h, int precision, double *tflops);

/* No counterpart in the reference.  Self-test of the tensor-core operand
 * layouts the mixed-precision M2L relies on (sm_100-family GPUs): one
 * tcgen05 kind::tf32 MMA D[128 x 16] = A[128 x 8] x B[8 x 16] with A in tensor
 * memory and B in shared memory (K-major, no swizzle; core matrices adjacent
 * in K 256 bytes apart, adjacent in N 128 bytes apart, or the reverse when
 * mode bit 0 is set), on small integers, A[m][k] = (3m + 5k) mod 11 - 5 and
 * B[k][n] = (7k + 3n) mod 13 - 6.  Mode bit 1: the MMA is M = 64 with
 * A[m][0] = m + 1 and A[m][k > 0] = 0 on a zeroed D, so D[lane][n] =
 * (a + 1) B[0][n] names the TMEM lane a whose A row lane `lane` received (0:
 * untouched).  Writes the 128 TMEM lanes x 16 columns of D row-major to the
 * host array out.  VFMM_ERR_UNSUPPORTED on other GPUs. */
int vfmm_tcgen05_selftest(int device, int mode, float *out);

/* ---- output --------------------------------------------------------------- */

/* Writes n bodies to `path` as legacy-VTK polydata, the file of the
 * reference driver's writeTovtk (src/main.cpp:127-164): POINTS X, one
 * VERTICES cell per body, POINT_DATA with VECTORS alpha and velocity and
 * SCALARS radius.  binary = 0: ASCII, byte-identical to the reference's file
 * (numbers as printf "%g"); binary = 1: the same dataset as legacy-VTK
 * BINARY data (big-endian FP64 values, 32-bit vertex indices, n < 2^31).
 * Host only; needs no handle and no GPU.  VFMM_ERR_INVALID on a null
 * argument or when the file cannot be written. */
int vfmm_write_vtk(const vfmm_body *bodies, size_t n, const char *path, int binary);

/* ---- no allocation -------------------------------------------------------- */

/* No counterpart in the reference.  Root cell of the octree -- centre out[0..2]
 * and half-width out[3], the values exafmm::getBounds produces -- for n
 * bodies whose coordinates x, y, z are already in device memory; out is a
 * device pointer to 4 doubles; the work is queued on `stream` (a
 * cudaStream_t; NULL = the default stream).  Allocates nothing, for callers
 * that cannot call cudaMalloc (work issued under CUDA-graph stream capture,
 * hosts whose device memory belongs to their own pool, plugins that must not
 * touch the allocator): its scratch is a fixed 29,184-byte array in the
 * library, present on every GPU that loads it.  n must be 1 .. 2^31-1.  The
 * first call on a device looks up the array's address and should come before
 * any stream capture; the address is kept for the life of the process, so do
 * not call this after cudaDeviceReset on that device.  Calls that overlap on the GPU share the array and race:
 * serialise them. */
int vfmm_bounds_noalloc(const double *x, const double *y, const double *z, size_t n, double *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif
