/*
 * femflow_mpm.h — C ABI of the GB300 (sm_103a) MLS-MPM substep.
 *
 * Drop-in boundary for FEMFlow's numba solver path (femflow/solvers/mpm).  Every entry point
 * takes plain device pointers, sizes, a POD parameter block and a CUDA stream (passed as void*,
 * i.e. a cudaStream_t), launches its kernels on that stream and returns an FFMPM_* code for
 * host-side problems (bad arguments, launch failures).  Problems that only the kernels can see
 * (a particle outside the grid — the reference raises RuntimeError there, utils.py:138-150 and
 * three_d/p2g.py:51-52) are OR-ed into a status word inside the workspace; read it with
 * ffmpm_status_read after the stream has run.
 *
 * No entry point allocates device memory.  Functions that need scratch take a caller-allocated
 * workspace of ffmpm_workspace_size() bytes that ffmpm_workspace_init() has prepared once.
 * A workspace is bound to one (params, n) shape and one stream at a time.
 *
 * Array layouts (row-major, element type float or double per params.real_bytes):
 *   x, v        [n][dim]              (reference: particle.pos / x, v)
 *   F, C        [n][dim][dim]         (reference: F, C)
 *   Jp          [n]                   (reference: Jp[n][1])
 *   mass, mu_0, lambda_0  [n] or NULL (reference Particle fields, particle.py:10-27; NULL = scalar
 *                                      params.mass / mu_0 / lambda_0, as two_d/p2g.py:11-29)
 *   grid velocity [(res+1)^dim][dim], grid mass [(res+1)^dim]  (reference grid_velocity /
 *                                      grid_mass, first index = x node)
 */
#ifndef FEMFLOW_MPM_H
#define FEMFLOW_MPM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* return codes */
#define FFMPM_OK 0
#define FFMPM_ERR_BADARG 3
#define FFMPM_ERR_WORKSPACE 4
#define FFMPM_ERR_CUDA 5
#define FFMPM_ERR_UNSUPPORTED 7

/* status-word bits (device side, see ffmpm_status_read) */
#define FFMPM_STATUS_OOB 1       /* particle stencil outside the grid, or non-finite position */
#define FFMPM_STATUS_NONFINITE 2 /* non-finite value produced in the particle state */
#define FFMPM_STATUS_TIMEOUT 4   /* a bounded device wait expired (never expected); the results of
                                  * the call are not valid, and kernels that would index particles
                                  * through an unfinished sort skip their work until the word is
                                  * cleared */

/* Fault injection for tests of the bounded waits (ffmpm_params.inject, ffmpm_batch2d_set_waits).
 * Each makes one wait impossible to satisfy, so that it can only end by running out; 0 in
 * production. */
#define FFMPM_INJECT_LOOKBACK_STALL 1 /* radix sort: the first tile of every pass never publishes
                                       * its digit counts */
#define FFMPM_INJECT_BARRIER_ABSENT 2 /* batched 2D: CTA 0 leaves before the first grid barrier */

/* material models: reference strings of three_d/p2g.py:57-61 */
#define FFMPM_MODEL_NEO_HOOKEAN 0 /* "neo_hookean": fixed-corotated stress, constant hardening */
#define FFMPM_MODEL_SNOW 1        /* "snow": exp hardening in P2G + singular-value clamp in G2P */
/* "fixed_corotated": the textbook fixed-corotated stress PF = 2mu(F-R)F^T + lam(J-1)J I (the volume term
 * on the diagonal only), constant hardening.  Not a reference model: the reference's "neo_hookean"
 * adds lam(J-1)J to all nine entries of PF (utils.py:129), a stress that derives from no energy and
 * makes long elastic runs grow. */
#define FFMPM_MODEL_FIXED_COROTATED 2

/* boundary rules of the grid update */
#define FFMPM_WALLS_REFERENCE 0 /* 3D: three_d/grid_op.py:38-47;  2D: two_d/grid_op.py:13-24 */
#define FFMPM_WALLS_STICKY3 1   /* all velocity zeroed within 3 cells of every face */

#define FFMPM_MAX_PLANES 8
#define FFMPM_PLANES_STICKY 0
#define FFMPM_PLANES_REFERENCE_LITERAL 1

typedef struct ffmpm_params {
  int32_t dim;          /* 2 or 3 */
  int32_t res;          /* grid resolution; nodes per axis = res + 1 */
  int32_t real_bytes;   /* 4 = float32 arrays and arithmetic, 8 = float64 */
  int32_t model;        /* FFMPM_MODEL_* */
  int32_t wall_mode;    /* FFMPM_WALLS_* */
  int32_t deterministic;/* 1: P2G sums in a fixed order (bit-identical across runs) */
  int32_t block_size;   /* nodes per block side for work assignment, a power of two in 2..16; 0 =
                         * default (3D 8, 2D 16; deterministic 3D 4, 2D 8).  Sides whose P2G tile
                         * does not fit in shared memory (3D float64 with 16) answer
                         * FFMPM_ERR_UNSUPPORTED */
  int32_t variant;      /* kernel variant flags; 0 = default.  Bit 0: P2G scatters straight to the
                         * grid; bit 1: P2G with one shared-memory atomic per (particle, node) (both
                         * with a re-sort every substep); bit 2: ffmpm_substeps_sorted launches G2P
                         * and P2G separately instead of the fused kernel; bits 8..15: substeps
                         * between re-sorts of ffmpm_substeps_sorted (0 or 1: every substep) */
  double dx, inv_dx, dt;
  double gravity;       /* added to the axis-1 (y) grid velocity, as the reference */
  double volume;        /* particle volume (reference argument `volume`) */
  double hardening;     /* reference argument `hardening` */
  double mass, mu_0, lambda_0; /* scalar material used when the per-particle pointers are NULL */
  /* Planar colliders applied by the grid update after the walls (three_d/grid_op.py:50-67
   * check_collision_points, which the reference defines but never calls): a node I with
   * (I dx - point) . normal' < 0 has its velocity set to zero (sticky).  plane_rule picks normal':
   * FFMPM_PLANES_STICKY = the given normal (the reference's evident intent: normalising does not
   * change the sign), FFMPM_PLANES_REFERENCE_LITERAL = normal + 1/|normal| as the reference's line
   * :60 writes it.  planes[i] = {point x, y, z, normal x, y, z} (z ignored in 2D). */
  int32_t n_planes;     /* 0..FFMPM_MAX_PLANES */
  int32_t plane_rule;   /* FFMPM_PLANES_* */
  double planes[FFMPM_MAX_PLANES][6];
  /* Iterations of the radix sort's look-back wait (a tile waiting for its predecessors' digit
   * counts) before it gives up and raises FFMPM_STATUS_TIMEOUT; 0 = the default, 2^22 (about a
   * second).  Lowered only by tests that make the wait run out. */
  uint32_t wait_limit;
  uint32_t inject;      /* FFMPM_INJECT_* bits; 0 in production */
} ffmpm_params;

typedef struct ffmpm_particles {
  int64_t n;
  void *x, *v, *F, *C, *Jp;
  const void *mass, *mu_0, *lambda_0;
  /* 0: the row-major layouts above.  > 0 (>= n): component-major — component c of particle p at
   * [c * stride + p] (x, v: dim components; F, C: dim*dim, row-major within the matrix).  Lets a
   * resident solver keep coalesced per-component arrays; the reference-facing calls use 0. */
  int64_t stride;
} ffmpm_particles;

typedef struct ffmpm_grid {
  void *velocity; /* [(res+1)^dim][dim] */
  void *mass;     /* [(res+1)^dim] */
} ffmpm_grid;

/* three_d.check_collision_points (three_d/grid_op.py:50-67) on the caller's dense grid velocity
 * [(res+1)^dim][dim] (real type p->real_bytes): for each of the n planes (points[i], normals[i],
 * host arrays of dim doubles each) and every node I, zero the node's velocity where
 * (I dx - point) . normal' < 0, normal' as p->plane_rule says (the planes in p are not used).
 * Asynchronous on `stream`; no workspace. */
int ffmpm_check_collision_points(const ffmpm_params *p, const double *points, const double *normals, int32_t n,
                                 void *grid_velocity, void *stream);

/* Bytes of workspace needed for `n` particles with these params (n < 2^30 for every call that
 * takes a workspace; larger n answers FFMPM_ERR_BADARG). */
int ffmpm_workspace_size(const ffmpm_params *p, int64_t n, size_t *bytes);

/* Prepare a freshly allocated workspace (zeroes its grids and counters).  Call once. */
int ffmpm_workspace_init(const ffmpm_params *p, int64_t n, void *ws, size_t ws_bytes, void *stream);

/* Synchronise `stream`, then copy out the status word (FFMPM_STATUS_* bits) and the number of
 * particles whose polar decomposition was redone in float64. */
int ffmpm_status_read(void *ws, int32_t *status, uint32_t *polar_fallbacks, void *stream);
int ffmpm_status_clear(void *ws, void *stream);

/* three_d.p2g / two_d.p2g (three_d/p2g.py:14-80, two_d/p2g.py:11-76): scatter the particles'
 * momentum and mass, ADDING into the caller's grid. */
int ffmpm_p2g(const ffmpm_params *p, const ffmpm_particles *P, ffmpm_grid *grid, void *ws, size_t ws_bytes,
              void *stream);

/* three_d.grid_op / two_d.grid_op (three_d/grid_op.py:5-47, two_d/grid_op.py:5-24), in place. */
int ffmpm_grid_op(const ffmpm_params *p, ffmpm_grid *grid, void *stream);

/* three_d.g2p / two_d.g2p (three_d/g2p.py:9-59, two_d/g2p.py:5-47): gather from the caller's
 * grid and update x, v, C, F (and Jp) in place. */
int ffmpm_g2p(const ffmpm_params *p, const ffmpm_grid *grid, ffmpm_particles *P, void *ws, size_t ws_bytes,
              void *stream);

/* solve_mls_mpm_3d (mls_mpm.py:40-79) and its 2D analogue: one full substep on the caller's
 * arrays, in place, particle order preserved.  The grid lives in the workspace. */
int ffmpm_substep(const ffmpm_params *p, ffmpm_particles *P, void *ws, size_t ws_bytes, void *stream);

/* solve_mls_mpm_3d (mls_mpm.py:40-79) and its 2D analogue on particle arrays in HOST memory
 * (`host`: the row-major layouts above, stride 0; pinned memory lets the copies run while the
 * kernels do).  The arrays go to the caller's device arrays `dev` (same shapes; mass / mu_0 /
 * lambda_0 only where the host gives them), the substep runs there, and x, v, F, C, Jp come back
 * into the host arrays.  Uploads and the scatter, and the gather and the downloads, are pipelined
 * over chunks of particles: each chunk is scattered in the caller's order as soon as it has landed
 * (one vector atomic per node, no block sort), the grid update covers every node, and each chunk
 * is gathered and sent back while the next one is gathered.  Same arithmetic per particle as
 * ffmpm_substep; the node sums run in another order.  The deterministic mode uploads everything,
 * runs ffmpm_substep and downloads.  The copies use two streams and a few events of the library's
 * own, created by the first call on a device and kept until exit: make that first call before any
 * stream capture.  Everything is ordered after the work already queued on `stream`, and the host
 * arrays hold the result once `stream` has run. */
int ffmpm_substep_host(const ffmpm_params *p, const ffmpm_particles *host, ffmpm_particles *dev, void *ws,
                       size_t ws_bytes, void *stream);

/* `nsteps` substeps that keep the particles physically sorted by grid block: step k reads
 * buffer (k even ? a : b) and writes the other one in sorted order, carrying the particle ids
 * (ids_a/ids_b) along.  After the call the state is in `a` when nsteps is even, else in `b`.
 * Same arithmetic as ffmpm_substep (MPMSimulation._simulate_offline, simulation.py:122-142). */
int ffmpm_substeps_sorted(const ffmpm_params *p, ffmpm_particles *a, ffmpm_particles *b, int32_t *ids_a,
                          int32_t *ids_b, int32_t nsteps, void *ws, size_t ws_bytes, void *stream);

/* ffmpm_substeps_sorted that also keeps every substep's positions, for a caller that hands each
 * substep's positions out while the run goes on (MPMSimulation._simulate_offline appends them
 * after every substep, simulation.py:140-142).  a and b must be component-major (stride >= n)
 * and carry ids.  After substep k the positions of the buffer the substep wrote (dim components of
 * n reals, in its block-sorted order) are copied to snap_x + k * dim * n and its ids to
 * snap_ids + k * n (device arrays, real type of p): particle snap_ids[k][i] sits at column i. */
int ffmpm_substeps_sorted_snapshots(const ffmpm_params *p, ffmpm_particles *a, ffmpm_particles *b, int32_t *ids_a,
                                    int32_t *ids_b, int32_t nsteps, void *snap_x, int32_t *snap_ids, void *ws,
                                    size_t ws_bytes, void *stream);

/* Stable radix sort of the particles by grid-block key (the block of each particle's base node,
 * then its cell inside the block): keys_out[i] is the i-th smallest key, perm_out[i] the index of
 * that particle.  Particles outside the grid get key 0xFFFFFFFF and sort last.  No reference
 * counterpart: it replaces the reference's unordered particle loop (three_d/p2g.py:49). */
int ffmpm_sort_by_block(const ffmpm_params *p, const void *x, int64_t n, uint32_t *keys_out, uint32_t *perm_out,
                        void *ws, size_t ws_bytes, void *stream);

/* Float64 diagnostics of a particle state, written to device memory `out` (8 doubles):
 * [kinetic energy, elastic (fixed-corotated) energy, gravitational energy (-g*y*m),
 *  momentum x, y, z, total mass, min det F].  No reference counterpart. */
int ffmpm_diagnostics_fp64(const ffmpm_params *p, const ffmpm_particles *P, double *out, void *stream);

/* Same as ffmpm_substeps_sorted, with CUDA events recorded around each phase on `stream`; the
 * call synchronises the stream and ADDS the per-phase milliseconds and launch counts into
 * phase_ms[FFMPM_NPHASES] / phase_launches[FFMPM_NPHASES] (host arrays).  Phases: 0 keys,
 * 1 sort, 2 plan, 3 P2G, 4 grid update, 5 G2P, 6 fused G2P + next substep's P2G.  No reference
 * counterpart (measurement only). */
#define FFMPM_NPHASES 7
int ffmpm_profile_substeps(const ffmpm_params *p, ffmpm_particles *a, ffmpm_particles *b, int32_t *ids_a,
                           int32_t *ids_b, int32_t nsteps, void *ws, size_t ws_bytes, void *stream,
                           double *phase_ms, int64_t *phase_launches);

/* Host-only description of the work decomposition for (params, n): info[0] block side, [1] blocks
 * per axis, [2] blocks, [3] key bits, [4] radix passes, [5] kernels per substep of a sorted run
 * with separate G2P and P2G launches, [6] tile side, [7] max work chunks.  No reference
 * counterpart. */
int ffmpm_plan_info(const ffmpm_params *p, int64_t n, int64_t *info);

/* Number of kernels one ffmpm_substeps_sorted call of `nsteps` substeps on n particles launches
 * (the kernels that return early on a substep without a re-sort included).  No reference
 * counterpart (measurement only). */
int ffmpm_kernels_per_call(const ffmpm_params *p, int64_t n, int32_t nsteps, int64_t *count);

/* Largest n accepted by ffmpm_sort_by_block_static, and its error when n is larger. */
#define FFMPM_STATIC_SORT_MAX_N 262144
#define FFMPM_ERR_CAPACITY 8

/* The block sort of ffmpm_sort_by_block (same keys, same stable permutation) without a workspace
 * and without any device allocation.  It is meant for callers that cannot allocate device memory:
 * a host application that owns every GPU allocation and hands its plugins device pointers only,
 * or a real-time loop that forbids allocation once it has started.  The scratch (about 5.5 MB:
 * five n-sized key/index arrays plus the digit histograms) is one static array in this library,
 * which every GPU that loads the library keeps until the process exits.
 *   - n must be <= FFMPM_STATIC_SORT_MAX_N, otherwise FFMPM_ERR_CAPACITY and nothing runs.
 *   - The first call in a CUDA context looks up the array's device address with that context's
 *     device current (cudaGetSymbolAddress); make that first call before any stream capture.  A
 *     new context on the device (cudaDeviceReset) makes the next call look the address up again.
 *   - Every call uses the same array, which keeps the previous call's contents: two calls whose
 *     work overlaps on the GPU (different streams or host threads) race and corrupt each other's
 *     results, so serialise them.
 *   - status_out (device memory, or NULL): receives the call's FFMPM_STATUS_* bits, copied on
 *     `stream` after the sort — FFMPM_STATUS_OOB when some particle lies outside the grid (it is
 *     sorted last with key 0xFFFFFFFF; the reference raises RuntimeError for such a particle),
 *     FFMPM_STATUS_TIMEOUT when a bounded wait of the sort gave up (keys_out and perm_out are then
 *     not valid).  0 for a clean sort.  The word in the shared array is overwritten by the next
 *     call, so this copy is the only way to see it.
 * No counterpart in the reference. */
int ffmpm_sort_by_block_static(const ffmpm_params *p, const void *x, int64_t n, uint32_t *keys_out,
                               uint32_t *perm_out, int32_t *status_out, void *stream);

/* ---- scene sampling ---- */

/* The reference's triply periodic surfaces (femflow/simulation/mpm/primitives.py:9-38). */
#define FFMPM_TPMS_GYROID 0
#define FFMPM_TPMS_DIAMOND 1
#define FFMPM_TPMS_PRIMITIVE 2
#define FFMPM_IMPLICIT_MAX_RES 1024

/* Workspace bytes of ffmpm_implicit_points for a res^3 lattice (16-byte aligned workspace). */
int ffmpm_implicit_points_workspace_size(int32_t res, size_t *bytes);

/* generate_implicit_points(kind, k, t, res) (primitives.py:46-61): the points of the res^3 lattice
 * in [0, 1]^3 (numerics/geometry.py:100-116, first axis fastest, coordinate i / (res - 1)) whose
 * implicit value (which has t subtracted already) is larger than t, in lattice order, written to
 * points[count][3] (device, float64).  *count (device int64) receives the number of such points
 * even when it exceeds `capacity`; points beyond capacity are not written (call with capacity 0
 * to size the output).  float64 arithmetic with each product and sum rounded on its own, in the
 * reference's order.  1 <= res <= FFMPM_IMPLICIT_MAX_RES, k finite and nonzero. */
int ffmpm_implicit_points(int32_t kind, double k, double t, int32_t res, double *points, int64_t capacity,
                          int64_t *count, void *ws, size_t ws_bytes, void *stream);

/* ---- batched 2D scenes: one persistent launch per substep for many independent scenes ---- */
#define FFMPM_BATCH2D_MAX_SCENES 256

/* One scene of a batch: its particles are [offset, offset + count) of the batch's concatenated
 * arrays (scenes in order, back to back), with the two_d.p2g scalar material and its own grid. */
typedef struct ffmpm_scene2d {
  int64_t offset, count;
  int32_t res, model, wall_mode, pad;
  double dx, inv_dx, dt, gravity, volume, hardening, mass, mu_0, lambda_0;
} ffmpm_scene2d;

/* Workspace bytes for a batch (scene table + every scene's two grids). */
int ffmpm_batch2d_workspace_size(const ffmpm_scene2d *scenes, int32_t nscenes, int32_t real_bytes, size_t *bytes);

/* Copy the scene table into the workspace (with each scene's parameters converted to the compute
 * type `real_bytes`, which every later call on this workspace must pass too), empty the scenes'
 * node boxes and zero the grids (synchronises `stream`). */
int ffmpm_batch2d_init(const ffmpm_scene2d *scenes, int32_t nscenes, int32_t real_bytes, void *ws, size_t ws_bytes,
                       void *stream);

/* `nsteps` substeps of every scene in one cooperative launch: P2G, then per substep the grid update
 * and G2P of all scenes (two_d/p2g.py, grid_op.py, g2p.py per scene), separated by grid-wide
 * barriers; between substeps each particle's G2P is followed in the same pass by its next P2G.
 * The grid update visits only the nodes inside each scene's box of touched nodes.  P2G sums the
 * contributions of neighbouring particles with the same base cell before its atomics, which pays
 * when each scene's particles are ordered by base cell (Batch2D orders them).  `threads`
 * (128/256/512) and `ctas_per_sm` (0 = as many as fit) set the launch shape; the autotuner
 * chooses them.  Particles are updated in place.  No reference counterpart (the reference steps
 * one scene at a time). */
int ffmpm_batch2d_substeps(int32_t nscenes, int32_t real_bytes, ffmpm_particles *P, int32_t nsteps, int32_t threads,
                           int32_t ctas_per_sm, void *ws, size_t ws_bytes, void *stream);

/* Status word of a batch workspace (FFMPM_STATUS_* bits); synchronises `stream`. */
int ffmpm_batch2d_status(void *ws, int32_t *status, void *stream);

/* Bound of the grid-barrier waits of a batch (iterations before a CTA gives up, raises
 * FFMPM_STATUS_TIMEOUT and leaves the launch; 0 = the default, 2^24) and FFMPM_INJECT_* bits
 * (FFMPM_INJECT_BARRIER_ABSENT), stored in the workspace for the following calls.  Tests lower
 * the bound to make a barrier run out; a batch whose status shows FFMPM_STATUS_TIMEOUT holds
 * partial results.  No reference counterpart. */
int ffmpm_batch2d_set_waits(void *ws, uint32_t wait_limit, uint32_t inject, void *stream);

/* ---- adjoint of one 3D or 2D substep (reverse mode, for differentiable rollouts) ---- */

/* Adjoints of a particle state, laid out exactly like the ffmpm_particles they belong to (same
 * real type, same `stride`).  On entry x, v, F, C hold dL/d(state after the substep); on return
 * they hold dL/d(state before it).  mu_0 / lambda_0 (nullable, always double, one per particle)
 * are ADDED TO: dL/dmu_0 and dL/dlambda_0 of this substep's stress, per particle (sum them for a
 * uniform material). */
typedef struct ffmpm_adjoint {
  void *x, *v, *F, *C;
  double *mu_0, *lambda_0;
} ffmpm_adjoint;

/* Workspace bytes of ffmpm_substep_adjoint (status header + three dense (res+1)^dim grids of
 * 32-byte nodes, for either real type).  dim other than 2 or 3: FFMPM_ERR_UNSUPPORTED. */
int ffmpm_adjoint_workspace_size(const ffmpm_params *p, int64_t n, size_t *bytes);

/* Reverse of one ffmpm_substep (3D or 2D, model FFMPM_MODEL_NEO_HOOKEAN or
 * FFMPM_MODEL_FIXED_COROTATED, either wall mode) at the state P (the state BEFORE the substep; P is
 * only read).  The substep's grid is recomputed from P, then G2P is reversed as a scatter of
 * node-velocity adjoints, the grid update as a per-node rule (the division by mass, the clamp and
 * the walls pass no gradient where they clip; in 2D the y < 0.05 band passes v_y's adjoint only
 * where v_y > 0), and P2G as a gather that also differentiates the stress, including the polar
 * factor (3D) or the closed-form rotation (2D).  Jp is not differentiated (it does not feed back
 * for these models).  The workspace's status header reads with ffmpm_status_read.  Other
 * dims/models (snow): FFMPM_ERR_UNSUPPORTED.  The reference has no derivative; this is the exact
 * derivative of solve_mls_mpm_3d (mls_mpm.py:40-79) and of the 2D substep (two_d/p2g.py,
 * grid_op.py, g2p.py). */
int ffmpm_substep_adjoint(const ffmpm_params *p, const ffmpm_particles *P, ffmpm_adjoint *A, void *ws,
                          size_t ws_bytes, void *stream);

/* ---- BF16 tensor-core (tcgen05) kernels of the learned corrector ---- */

/* D[M][N] (float32, row-major) = A[M][K] . B[N][K]^T, with A and B bf16 row-major (raw 16-bit
 * words) and float32 accumulation in tensor memory.  M % 128 == 0, N % 16 == 0 and N <= 256,
 * K % 64 == 0, A and B 16-byte aligned.  split_k > 1 splits K over up to that many CTAs, which then
 * ADD into D (zero D first); split_k = 1 overwrites D.  `status` (device int32, nullable) gets
 * FFMPM_STATUS_TIMEOUT if a bounded wait on the tensor core expired.  No reference counterpart. */
int ffmpm_tc_gemm_bf16(const uint16_t *A, const uint16_t *B, float *D, int32_t M, int32_t N, int32_t K,
                       int32_t split_k, int32_t *status, void *stream);

/* The corrector network: FFMPM_MLP_FEATURES features (padded to FFMPM_MLP_IN) -> 64 -> 64 -> 64 -> 12 outputs,
 * GELU between layers.  Weights bf16 row-major [out][in] (W4 padded to 16 rows, zero beyond 12),
 * biases and scales float32: features are multiplied by in_scale[FFMPM_MLP_IN] before the first
 * layer, outputs by out_scale[16] after the last. */
#define FFMPM_MLP_IN 128
#define FFMPM_MLP_FEATURES 113 /* features in use; the rest of the FFMPM_MLP_IN inputs are zero */
#define FFMPM_MLP_HIDDEN 64
#define FFMPM_MLP_OUT 12
typedef struct ffmpm_mlp {
  const uint16_t *W1, *W2, *W3, *W4; /* [64][128], [64][64], [64][64], [16][64] */
  const float *b1, *b2, *b3, *b4;    /* [64], [64], [64], [16] */
  const float *in_scale, *out_scale; /* [128] (nullable: 1), [16] */
} ffmpm_mlp;

/* G2P of a coarse 3D substep (float32, dense caller grid after ffmpm_grid_op) fused with the
 * learned corrector: every particle gathers its 27 nodes, forms v', C', F', x' as three_d.g2p
 * (g2p.py:9-59), builds its features [F' - I, C' dt, (v' - u) dt/dx, (v_i - u) dt/dx for the 27
 * nodes, mu k, lam k, PF k with k = dt^2 / (rho dx^2); u = the stencil's centre node velocity, PF
 * the stress of the pre-step F], and, when `net` is given, runs the network on the
 * tensor cores and applies F' += y[0:9], v' += y[9:12] dx/dt, x' += dt y[9:12] dx/dt.  The particle
 * state is updated in place.  features_out (nullable, bf16 [n][FFMPM_MLP_IN], 16-byte aligned)
 * receives the scaled features.  det_range (nullable, device int32[2], initialise to
 * {0x7FFFFFFF, 0x80000000}) receives the min / max of det F' as order-preserving keys (k >= 0 ? k :
 * k ^ 0x7FFFFFFF are the float bits).  status: device int32 (OOB, TIMEOUT bits).  The reference has
 * no counterpart. */
int ffmpm_corrector_g2p(const ffmpm_params *p, const ffmpm_grid *grid, ffmpm_particles *P, const ffmpm_mlp *net,
                        uint16_t *features_out, int32_t *det_range, int32_t *status, void *stream);

/* Training of the corrector network on the tensor cores.  Master parameters, gradients and Adam
 * moments are float32 in one flat layout of FFMPM_MLP_PARAMS floats:
 *   W1 at 0 (rows of 128, 64 used), W2 at 16384, W3 at 24576, W4 at 32768 (rows of 64; W2, W3: 64
 *   rows used; W4: 12), b1 at 40960, b2 at 41024, b3 at 41088, b4 at 41152 (16).
 * Activation buffers are sized for max_batch rows (a multiple of 128); transposed buffers are
 * strided by the batch of the call and their padding rows (Xt rows 113.., dYt rows 12.., dZt rows
 * 64..) are zeroed by the calls themselves.  All buffers are caller allocated. */
#define FFMPM_MLP_PARAMS 41168
#define FFMPM_MLP_OFF_W1 0
#define FFMPM_MLP_OFF_W2 16384
#define FFMPM_MLP_OFF_W3 24576
#define FFMPM_MLP_OFF_W4 32768
#define FFMPM_MLP_OFF_B1 40960
#define FFMPM_MLP_OFF_B2 41024
#define FFMPM_MLP_OFF_B3 41088
#define FFMPM_MLP_OFF_B4 41152
typedef struct ffmpm_mlp_trainer {
  int32_t max_batch;
  float *params, *grads, *adam_m, *adam_v;
  uint16_t *W1, *W2, *W3, *W4;       /* packed bf16 weights, as ffmpm_mlp */
  uint16_t *W2t, *W3t, *W4t;         /* [64][64]: W2^T, W3^T, W4^T (zero beyond W4's 12 rows) */
  float *Z1, *Z2, *Z3;               /* [B][64] pre-activations */
  float *Y;                          /* [B][16] */
  float *dH;                         /* [B][64] */
  uint16_t *H1, *H2, *H3;            /* [B][64] */
  uint16_t *H1t, *H2t, *H3t;         /* [64][B] */
  uint16_t *Xt;                      /* [128][B] */
  uint16_t *dY, *dZ;                 /* [B][64] */
  uint16_t *dYt, *dZt;               /* [128][B] */
  int32_t *status;                   /* device int32 (TIMEOUT bit from the tensor-core waits) */
} ffmpm_mlp_trainer;

/* Forward pass of `batch` rows of bf16 features X [batch][FFMPM_MLP_IN] (16-byte aligned) with the
 * packed weights and the biases in params: keeps Z1..Z3, H1..H3 (and their transposes, and Xt) and
 * leaves the network output (before out_scale) in Y. */
int ffmpm_mlp_train_forward(const ffmpm_mlp_trainer *t, const uint16_t *X, int32_t batch, void *stream);

/* Loss sum_b sum_j w[j] (Y[b][j] - T[b][j])^2 / batch over the 12 outputs (T: float32 [batch][12],
 * w: float32 [12]), ADDED to *loss (device double), and its gradient with respect to every
 * parameter written to grads (overwritten).  Needs the preceding ffmpm_mlp_train_forward. */
int ffmpm_mlp_train_backward(const ffmpm_mlp_trainer *t, const float *T, const float *w, int32_t batch,
                             double *loss, void *stream);

/* One Adam step (learning rate lr, betas b1 b2, eps; `step` counts from 1) on params, then repack
 * the bf16 weights W1..W4 and their transposes. */
int ffmpm_mlp_train_update(const ffmpm_mlp_trainer *t, float lr, float beta1, float beta2, float eps, int32_t step,
                           void *stream);

/* Library version string. */
const char *ffmpm_version(void);

#ifdef __cplusplus
}
#endif

#endif /* FEMFLOW_MPM_H */
