/*
 * bssn_gb300.h -- C ABI of the GB300 (sm_103a) BSSN evolution kernels.
 *
 * Every entry point takes plain device pointers, sizes and a cudaStream_t
 * (passed as void*), launches asynchronously on that stream, never allocates
 * on the hot path (work buffers are caller-provided; sizes come from
 * bssn_workspace_bytes), and returns an int status: 0 on success, a positive
 * BSSN_ERR_* code otherwise.  bssn_last_error() returns a message for the
 * calling thread's most recent failure.
 *
 * Field layout at the boundary is the reference's: seven C-ordered float64
 * arrays with the spatial axes last and z fastest (JAX_BSSN/bssn/variables.py:8-16,
 * docs/bssn.rst:11-49):
 *   conformal_metric (3,3,nx,ny,nz)  conformal_factor W (nx,ny,nz)
 *   traceless_K      (3,3,nx,ny,nz)  trace_K (nx,ny,nz)
 *   conformal_connection (3,nx,ny,nz) lapse (nx,ny,nz)  shift (3,nx,ny,nz)
 * Symmetric tensors are read from their upper triangle and written to both
 * halves.
 *
 * Resident state ("patch" layout) is the GB300-side working format: 21
 * independent float64 components, each a contiguous padded block of
 * (nx+2G)(ny+2G)(nz+2G) samples, z fastest, owned samples at [G, G+n).
 * Component order: gt_xx gt_xy gt_xz gt_yy gt_yz gt_zz, W,
 * At_xx At_xy At_xz At_yy At_yz At_zz, K, Gt_x Gt_y Gt_z, alpha, beta_x beta_y beta_z.
 */
#ifndef BSSN_GB300_H
#define BSSN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BSSN_ABI_VERSION 2

/* status codes */
#define BSSN_OK 0
#define BSSN_ERR_INVALID 1      /* argument validation failed (host side) */
#define BSSN_ERR_WORKSPACE 2    /* workspace pointer null or too small */
#define BSSN_ERR_CUDA 3         /* a CUDA launch or runtime call failed */
#define BSSN_ERR_NONFINITE 4    /* non-finite value detected in the state */
/* 5 is unused: no entry point waits on the device */
#define BSSN_ERR_NOT_CONVERGED 6 /* an iterative solve ran out of iterations */

#define BSSN_NCOMP 21           /* independent evolved components */
#define BSSN_NLEAF_VALUES 27    /* stored values per point in the reference layout */

/* Mirrors BSSNParameters (JAX_BSSN/bssn/variables.py:19-46).  Face codes:
 * 0 periodic, 1 Sommerfeld, in xl xr yl yr zl zr order. */
typedef struct BssnParams {
    double eta, kappa, nu, g, dx, dt;
    int32_t zero_shift;      /* 1 holds the shift fixed */
    int32_t gauge;           /* 0 harmonic, 1 1+log */
    int32_t bc[6];
    double xmin[3];          /* coordinate of array index 0 on each axis */
    double mad_q;            /* D4 weight of the MAD D4/D6 blend */
    int32_t guard_cells;     /* lower padding before the first owned sample */
    int32_t owned_shape[3];  /* owned samples per axis; -1: the whole array */
    int32_t owned_faces[6];  /* 1 when this array owns the global face */
    int32_t reduced_axes[3]; /* 1 reduced, 0 not, -1 infer (owned count == 1 when owned_shape given) */
    int32_t precision;       /* BSSN_PRECISION_F64 (default), BSSN_PRECISION_F32 or BSSN_PRECISION_F32_PAIRED;
                                no reference counterpart */
} BssnParams;

/* Arithmetic of the RHS kernels.  F64: plain float64 throughout, matching the
 * reference to roundoff.  F32: the RHS stencils and algebra in float on
 * perturbations about the flat background, W, alpha and 1/W from the float64
 * state, the RHS written in float64; the state, the RK4 combination, the
 * projection and the constraints stay float64. */
#define BSSN_PRECISION_F64 0
#define BSSN_PRECISION_F32 1
/* BSSN_PRECISION_F32 with the fields whose second derivatives are taken (gt,
 * W, alpha, beta) held as float pairs hi + lo: their 1/dx^2-amplified
 * rounding falls from float's to about FP64's, for ~20% more FP32 time. */
#define BSSN_PRECISION_F32_PAIRED 2

/* The seven reference leaves as device pointers (float64). */
typedef struct BssnFields {
    double* conformal_metric;
    double* conformal_factor;
    double* traceless_K;
    double* trace_K;
    double* conformal_connection;
    double* lapse;
    double* shift;
} BssnFields;

/* Optional matter sources in the reference layout: rho (n), S_i (3,n), S_ij (3,3,n).
 * All three null selects the vacuum equations. */
typedef struct BssnMatter {
    const double* energy_density;
    const double* momentum_density;
    const double* spatial_stress;
} BssnMatter;

/* Operation selector for bssn_workspace_bytes. */
#define BSSN_OP_RHS 1
#define BSSN_OP_RK4 2
#define BSSN_OP_CONSTRAINTS 3
#define BSSN_OP_RHS_MATTER 4   /* bssn_rhs with matter sources */

const char* bssn_last_error(void);
int bssn_abi_version(void);

/* Bytes of device workspace an operation needs on an (nx,ny,nz) array. */
size_t bssn_workspace_bytes(int op, const int32_t shape[3], const BssnParams* params);

/* compute_bssn_rhs(vars, params) -> rhs (JAX_BSSN/evolution/time_evolve.py:41-57),
 * and compute_bssn_rhs_with_matter (time_evolve.py:60-91) when matter holds the
 * three source arrays (workspace: bssn_workspace_bytes(BSSN_OP_RHS_MATTER); S_ij is
 * read from its upper triangle, a symmetric stress).  Like the reference, the RHS is
 * evaluated at every sample of the array, with periodic wrap across the array
 * extent and face closures/Sommerfeld replacement on the owned range given by
 * guard_cells/owned_shape. */
int bssn_rhs(const BssnFields* in, BssnFields* out, const int32_t shape[3],
             const BssnParams* params, const BssnMatter* matter,
             void* workspace, size_t workspace_bytes, void* stream);

/* No counterpart in the reference.  bssn_rhs for callers that cannot allocate
 * device memory (a host framework that owns all device memory, a solver with a
 * memory budget fixed at start-up, a loop that must avoid the synchronisation
 * of cudaMalloc/cudaFree): same inputs, outputs and results as bssn_rhs, but
 * the work buffer is an array built into the library (26.9 MB of device
 * memory, held on every GPU that loads the library until the process exits).
 * Limit: (nx+8)*(ny+8)*(nz+8) <= 21952 samples (e.g. 20x20x20); larger arrays
 * return BSSN_ERR_INVALID.  The first call on each device looks up the
 * array's device address with that device current; make that first call
 * before any stream capture.  The looked-up address is kept per device index
 * and belongs to the device's primary context (the CUDA runtime's): it does
 * not survive cudaDeviceReset, and a caller's own driver context must not be
 * current.  All calls share the one array, so calls that overlap on the GPU
 * (different streams or threads) race; serialise them. */
int bssn_rhs_noalloc(const BssnFields* in, BssnFields* out, const int32_t shape[3],
                     const BssnParams* params, void* stream);

/* enforce_algebraic_constraints(vars) (time_evolve.py:134-141): det(gt)=1 then
 * trace-free At.  In place on all samples of the array. */
int bssn_project(BssnFields* state, const int32_t shape[3], void* stream);

/* rk4_step(vars, params) (time_evolve.py:144-217), repeated `steps` times, in place.
 * In the FP64 form with a Sommerfeld face, the lower triangles of At and gt
 * are carried as the reference evolves them: their differences from the upper
 * triangles, which the reference's two orderings of the mixed derivatives
 * create on the rows next to the faces, are read from the input there,
 * evolved to first order and written back (work buffer: 24 more blocks). */
int bssn_rk4_step(BssnFields* state, const int32_t shape[3], const BssnParams* params,
                  int32_t steps, void* workspace, size_t workspace_bytes, void* stream);

/* compute_all_constraints(vars, params) (JAX_BSSN/bssn/constraints.py:387-412):
 * writes H (n), M (3,n), det-1 (n), trace A (n), Gamma constraint (3,n). */
int bssn_constraints(const BssnFields* in, const int32_t shape[3], const BssnParams* params,
                     double* hamiltonian, double* momentum, double* det_gamma,
                     double* trace_A, double* gamma_condition,
                     void* workspace, size_t workspace_bytes, void* stream);

/* ---------------- resident patch layout (fast path) ---------------- */

typedef struct BssnPatch {
    int32_t n[3];     /* owned samples per axis */
    int32_t ghost;    /* padding G on every face */
} BssnPatch;

size_t bssn_patch_values(const BssnPatch* patch);            /* 21 * prod(n+2G) */
size_t bssn_patch_workspace_bytes(const BssnPatch* patch, const BssnParams* params);

/* Reference layout (nx,ny,nz) -> patch owned samples (ghosts left untouched). */
int bssn_patch_import(const BssnFields* in, double* patch_state, const BssnPatch* patch, void* stream);
/* Patch owned samples -> reference layout. */
int bssn_patch_export(const double* patch_state, BssnFields* out, const BssnPatch* patch, void* stream);
/* Fill the ghost shell by periodic wrap of owned samples (parallel/communication.py:45-52). */
int bssn_patch_fill_periodic(double* patch_state, const BssnPatch* patch, void* stream);
/* `steps` RK4 steps of a periodic/Sommerfeld patch, in place (time_evolve.py:144-217). */
int bssn_patch_rk4(double* patch_state, const BssnPatch* patch, const BssnParams* params,
                   int32_t steps, void* workspace, size_t workspace_bytes, void* stream);
/* Count of non-finite owned values into *flag (device int32), for step monitors. */
int bssn_patch_check_finite(const double* patch_state, const BssnPatch* patch,
                            int32_t* device_flag, void* stream);

/* ---------------- instance batches ----------------
 * No reference counterpart: the reference evolves one state per call (a vmap
 * over rk4_step would batch it).  ninst independent instances of the same
 * patch and parameters advance in the same launches.  Layout [component]
 * [instance][padded block]: component c of instance i starts at
 * (c * ninst + i) * prod(n + 2G) doubles.  Results are bit-identical to
 * ninst separate single-patch calls.  The bssn_patch_* calls above are the
 * one-instance batch. */
size_t bssn_batch_values(const BssnPatch* patch, int32_t ninst);
size_t bssn_batch_workspace_bytes(const BssnPatch* patch, int32_t ninst, const BssnParams* params);
/* Reference layout -> owned samples of instance `instance` (ghosts untouched). */
int bssn_batch_import(const BssnFields* in, double* states, const BssnPatch* patch, int32_t ninst, int32_t instance,
                      void* stream);
/* Owned samples of instance `instance` -> reference layout. */
int bssn_batch_export(const double* states, BssnFields* out, const BssnPatch* patch, int32_t ninst,
                      int32_t instance, void* stream);
int bssn_batch_fill_periodic(double* states, const BssnPatch* patch, int32_t ninst, void* stream);
/* `steps` RK4 steps of every instance, in place (time_evolve.py:144-217 per instance). */
int bssn_batch_rk4(double* states, const BssnPatch* patch, int32_t ninst, const BssnParams* params, int32_t steps,
                   void* workspace, size_t workspace_bytes, void* stream);
int bssn_batch_check_finite(const double* states, const BssnPatch* patch, int32_t ninst, int32_t* device_flag,
                            void* stream);
/* bssn_batch_rk4 with a failure monitor (no reference counterpart: the
 * reference lets NaN propagate).  Before the first step and after every
 * `check_every` steps (and the last) it counts the non-finite owned values of
 * all instances into *device_counter (one caller-provided device int32) and
 * reads the count back, synchronising `stream`.  A nonzero count stops the
 * run: BSSN_ERR_NONFINITE, with the count and the step in bssn_last_error();
 * *steps_done (host) receives the steps completed before the check that
 * failed, or `steps`. */
int bssn_batch_rk4_monitored(double* states, const BssnPatch* patch, int32_t ninst, const BssnParams* params,
                             int32_t steps, int32_t check_every, int32_t* device_counter, int32_t* steps_done,
                             void* workspace, size_t workspace_bytes, void* stream);

/* ---------------- adjoint (reverse mode) ----------------
 * Gradients of evolutions.  The reference has no hand-written adjoint:
 * differentiating its rk4_step (JAX_BSSN/evolution/time_evolve.py:144-217)
 * means jax.grad / jax.vjp through XLA.  These entry points are the
 * vector-Jacobian products of the same forward path, on instance batches
 * (layout of bssn_batch_*).  Scope: both faces of each axis periodic (bc 0)
 * or both Sommerfeld (bc 1: the one-sided closure rows and the radial face
 * condition are transposed too), kappa = 0, no matter sources,
 * BSSN_PRECISION_F64, at least 8 samples per axis; anything else returns
 * BSSN_ERR_INVALID.  Adjoint arrays have the
 * batch layout; only their owned samples carry values (ghosts are scratch).
 * Gradients are with respect to the 21 independent components. */

/* Bytes of workspace bssn_rhs_vjp needs (111 + 33 padded blocks per instance). */
size_t bssn_rhs_vjp_workspace_bytes(const BssnPatch* patch, int32_t ninst);
/* state_adjoint = (d RHS / d state)^T rhs_adjoint at `states`
 * (compute_bssn_rhs, time_evolve.py:41-57).  Fills the ghosts of `states`
 * and `rhs_adjoint` (periodic wrap, on periodic grids) in place. */
int bssn_rhs_vjp(double* states, double* rhs_adjoint, double* state_adjoint, const BssnPatch* patch, int32_t ninst,
                 const BssnParams* params, void* workspace, size_t workspace_bytes, void* stream);

/* Checkpointed evolution for reverse mode.  `segment` <= 0 selects
 * ceil(sqrt(steps)) steps between checkpoints.  While the backward pass re-runs
 * a segment it keeps, by store_stages: 0 the step-start states only (each
 * step's stages are then recomputed: two forward re-runs in total); 1 also
 * every step's four stage RHS values (one re-run; 4 more states per segment
 * step); 2 also the four stage states (8 more).  With 1 or 2 the forward pass
 * records the last segment itself.  The workspace holds ceil(steps / segment)
 * checkpoints, the segment's states and about 20 working states. */
size_t bssn_adjoint_workspace_bytes(const BssnPatch* patch, int32_t ninst, const BssnParams* params, int32_t steps,
                                    int32_t segment, int32_t store_stages);
/* `steps` RK4 steps of every instance in place (bit-identical to
 * bssn_batch_rk4), recording the checkpoints in the workspace. */
int bssn_adjoint_forward(double* states, const BssnPatch* patch, int32_t ninst, const BssnParams* params,
                         int32_t steps, int32_t segment, int32_t store_stages, void* workspace, size_t workspace_bytes,
                         void* stream);
/* After bssn_adjoint_forward with the same arguments and workspace: on entry
 * `adjoint` holds d loss / d (final state), on exit d loss / d (initial state).
 * One backward pass per forward pass: with store_stages the forward pass
 * records the last segment's stages, which the backward pass then overwrites. */
int bssn_adjoint_backward(double* adjoint, const BssnPatch* patch, int32_t ninst, const BssnParams* params,
                          int32_t steps, int32_t segment, int32_t store_stages, void* workspace, size_t workspace_bytes,
                          void* stream);

/* No reference counterpart: launch-shape autotuning.  Times five RHS
 * evaluations of this batch's state (ghosts refilled, owned values untouched)
 * for each candidate block size (32, 64, 128 threads) of each RHS launch slot
 * -- kernel class x interior/shell -- one slot at a time, and keeps the
 * fastest when its time is below `margin` (> 0) x the time with the shapes in
 * force (0.98: only a 2% gain changes a shape; 1 or more: always the fastest).
 * Later launches of that slot at that launch size on this device in
 * this arithmetic form use it (also single patches, FMR patches of the same
 * padded extent, and CUDA-graph captures made afterwards); results are
 * identical bit for bit.  Synchronises `stream`; refuses a stream that is being
 * captured.  `report` (host, optional) receives a one-line summary. */
int bssn_tune_patch(double* states, const BssnPatch* patch, int32_t ninst, const BssnParams* params, float margin,
                    void* workspace, size_t workspace_bytes, char* report, size_t report_bytes, void* stream);

/* No reference counterpart: the float forms' TMA-staged kernels.  On the box
 * interior, and where every closed axis has Sommerfeld faces at both ends also
 * on the rows next to them, where the geometry allows it -- a z pitch
 * (nz + 2 ghost) that is a multiple of four, no MAD axis, kappa = 0 for all
 * but the gauge RHS, vacuum for the curvature RHS -- the gauge RHS (dt gt, W,
 * alpha, beta; BSSN_TMA_GAUGE), the first derivatives (BSSN_TMA_DERIVS), dt At
 * (BSSN_TMA_AT) and dt K with dt Gt (BSSN_TMA_KGT) can run from TMA-staged
 * shared-memory tiles instead of the generic kernels.  `kernels` is the mask
 * of those to use (default BSSN_TMA_ALL; 0: the generic kernels everywhere);
 * results agree to float rounding.  Process-wide; affects later launches and
 * captures. */
#define BSSN_TMA_GAUGE 1
#define BSSN_TMA_DERIVS 2
#define BSSN_TMA_AT 4
#define BSSN_TMA_KGT 8
#define BSSN_TMA_ALL 15
int bssn_set_tma(int32_t kernels);

/* TMA kernel status: *timeouts receives the number of tile waits on the
 * current device that gave up since the last call (each leaves its tile's RHS
 * unwritten and should never happen; the count is reset), *launches the TMA
 * kernel launches of the process so far (optional).  Synchronises the device. */
int bssn_tma_status(int32_t* timeouts, int64_t* launches);

/* Whole-array conversion between the reference layout (seven leaves) and the
 * 21-component layout, over all samples of an array of the given extent
 * (e.g. a padded FMR patch, whose guards are part of the array). */
int bssn_fields_to_components(const BssnFields* in, double* state, const int32_t extent[3], void* stream);
int bssn_components_to_fields(const double* state, BssnFields* out, const int32_t extent[3], void* stream);

/* ---------------- fixed mesh refinement (single-tile patches) ---------------- */

/* One patch of a vertex-centred 2:1 hierarchy (JAX_BSSN/fmr/refinement.py:15-75).
 * States are in the resident layout with ghost 4: 21 x (n+8)^3 doubles. */
typedef struct BssnFmrPatch {
    int32_t n[3];          /* active (owned) samples per axis; children: 2*(hi-lo)+1 */
    int32_t parent;        /* parent patch index (< own index), -1 for the root */
    int32_t coarse_lo[3];  /* inclusive bounds in the parent's active indices */
    int32_t coarse_hi[3];
} BssnFmrPatch;

/* Workspace for bssn_fmr_rk4_step / bssn_fmr_stage_rhs on this hierarchy. */
size_t bssn_fmr_workspace_bytes(const BssnFmrPatch* patches, const BssnParams* params, int32_t npatch);
/* refresh_bssn_halos of one single-tile patch: periodic self-wrap, linear
 * exterior on Sommerfeld faces (refresh_bssn_halos, JAX_BSSN/parallel/evolution.py:74-92;
 * the single-tile sweep of JAX_BSSN/parallel/communication.py:36-106). */
int bssn_fmr_refresh(double* state, const int32_t n[3], const int32_t codes[6], void* stream);
/* fill_tiled_fine_ghosts (JAX_BSSN/fmr/transfer.py:237-244): six-node Lagrange
 * prolongation of the prepared parent into the child's exterior shell. */
int bssn_fmr_prolong(const double* parent, const int32_t parent_n[3], double* child,
                     const int32_t child_n[3], const int32_t coarse_lo[3], void* stream);
/* restrict_tiled_to_coarse (JAX_BSSN/fmr/transfer.py:247-252): injection of
 * coincident owned fine vertices into the parent. */
int bssn_fmr_inject(double* parent, const int32_t parent_n[3], const double* child,
                    const int32_t child_n[3], const int32_t coarse_lo[3], void* stream);
/* prepare_fmr_states (JAX_BSSN/fmr/tiled.py:146-166): project owned samples
 * (when project != 0), refresh halos and prolong child shells, parent first. */
int bssn_fmr_prepare(double* const* states, const BssnFmrPatch* patches, const BssnParams* params,
                     int32_t npatch, int32_t project, void* stream);
/* fmr_stage (JAX_BSSN/fmr/tiled.py:169-179): prepare in place, then the RHS of
 * every patch on its owned samples into rhs[p] (resident layout). */
int bssn_fmr_stage_rhs(double* const* states, double* const* rhs, const BssnFmrPatch* patches,
                       const BssnParams* params, int32_t npatch, void* workspace,
                       size_t workspace_bytes, void* stream);
/* fmr_rk4_step (JAX_BSSN/fmr/tiled.py:182-209), `steps` times, in place.
 * params[p] are the per-patch evolution parameters (MAD weight, child faces periodic). */
int bssn_fmr_rk4_step(double* const* states, const BssnFmrPatch* patches, const BssnParams* params,
                      int32_t npatch, int32_t steps, void* workspace, size_t workspace_bytes, void* stream);
/* fmr_constraint_norms statistics (JAX_BSSN/fmr/tiled.py:212-246): prepares the
 * states (no projection) and accumulates, over owned samples not covered by a
 * child, the sum of squares and max |.| of H, M, det-1, tr A, Gamma into
 * stats[10] (device, pairs per constraint).  Workspace: see the implementation. */
int bssn_fmr_constraint_stats(double* const* states, const BssnFmrPatch* patches, const BssnParams* params,
                              int32_t npatch, double* stats, void* workspace, size_t workspace_bytes,
                              void* stream);

/* ---------------- Cartoon reductions ---------------- */

/* Compact Cartoon states in the 21-component layout (bssn_fields_to_components
 * over the compact extent): axisymmetric (axisymmetric != 0) shape
 * (Nrho+4, 1, Nz), spherical (Nr+4, 1, 1); x index 0..3 are parity ghosts.
 * params must satisfy validate_axisymmetric_grid
 * (JAX_BSSN/cartoon/axisymmetry/reconstruction.py:65-112) or
 * validate_cartoon_grid (JAX_BSSN/cartoon/spherical_symmetry/reconstruction.py:61-111),
 * with no guard description. */
size_t bssn_cartoon_workspace_bytes(int32_t axisymmetric, const int32_t shape[3], const BssnParams* params);
/* Axisymmetric: fill_axisymmetric_ghosts (axisymmetry/reconstruction.py:131-143).
 * Spherical: enforce_spherical_symmetry (spherical_symmetry/reconstruction.py:174-189).
 * In place. */
int bssn_cartoon_fill_ghosts(int32_t axisymmetric, double* compact, const int32_t shape[3], void* stream);
/* reconstruct_axisymmetric_support (axisymmetry/reconstruction.py:251-289) into a
 * 21 x (Nrho+4) x 9 x Nz support, or reconstruct_cartoon_support
 * (spherical_symmetry/reconstruction.py:336-385) into 21 x (Nr+4) x 9 x 9. */
int bssn_cartoon_reconstruct(int32_t axisymmetric, const double* compact, double* support, const int32_t shape[3],
                             const BssnParams* params, void* stream);
/* compute_axisymmetric_rhs (axisymmetry/evolution.py:18-26) / compute_cartoon_rhs
 * (spherical_symmetry/evolution.py:17-25): the compact RHS with parity ghosts. */
int bssn_cartoon_rhs(int32_t axisymmetric, const double* compact, double* rhs, const int32_t shape[3],
                     const BssnParams* params, void* workspace, size_t workspace_bytes, void* stream);
/* axisymmetric_rk4_step (axisymmetry/evolution.py:40-65) / cartoon_rk4_step
 * (spherical_symmetry/evolution.py:44-72), `steps` times, in place. */
int bssn_cartoon_rk4_step(int32_t axisymmetric, double* compact, const int32_t shape[3], const BssnParams* params,
                          int32_t steps, void* workspace, size_t workspace_bytes, void* stream);
/* compute_axisymmetric_constraints (axisymmetry/diagnostics.py:22-37) /
 * compute_cartoon_constraints (spherical_symmetry/diagnostics.py:21-37): nine
 * compact blocks of the compact extent -- H, M_x, M_y, M_z, det-1, tr A,
 * G_x, G_y, G_z -- with parity ghosts. */
int bssn_cartoon_constraints(int32_t axisymmetric, const double* compact, const int32_t shape[3],
                             const BssnParams* params, double* out, void* workspace, size_t workspace_bytes,
                             void* stream);

/* ---------------- wave diagnostics ---------------- */

/* h_plus (JAX_BSSN/diagnostics/waves.py:11-20): 0.5 (gt_yy - gt_zz) / W^2 on
 * the reference layout of `shape`, bit-identical to the float64 reference.
 * Asynchronous on `stream`. */
int bssn_h_plus(const BssnFields* state, const int32_t shape[3], double* h_plus, void* stream);

/* Scratch needed by bssn_wave_norm_sums. */
size_t bssn_wave_norm_workspace_bytes(void);

/* One level of composite_wave_diagnostics (waves.py:43-91): over the vertices of
 * the C-ordered `shape` arrays not inside any of the `ncovered` (<= 8) boxes
 * `covered` (6 int32 each: lo[3], hi[3], inclusive), writes to the 5 device
 * doubles `sums`: sum of (h_plus - amplitude sin(2 pi (x - time)/wavelength))^2
 * with x = `coordinates`, max |that error|, sum of H^2, sum over vertices of
 * |M|^2 (`momentum` = three blocks), and the vertex count.  Deterministic
 * block partials in `workspace`.  Asynchronous on `stream`. */
int bssn_wave_norm_sums(const double* h_plus, const double* coordinates, const double* hamiltonian,
                        const double* momentum, const int32_t shape[3], const int32_t* covered,
                        int32_t ncovered, double time, double amplitude, double wavelength, double* sums,
                        void* workspace, size_t workspace_bytes, void* stream);

/* ---------------- instrumentation ---------------- */

/* Output staging (diagnostics/openpmd.py:51-71 _strip_ghost_cells,
 * :254-285 tiled_output_fields): copies the box [lo, lo + extent) of each
 * C-ordered float64 device array src (extents `shape`) into dst, box after
 * box, each box C-ordered, so a writer gathers every owned sample of a level
 * with one launch and one device-to-host copy.  At most
 * BSSN_MAX_GATHER_BOXES boxes per call. */
#define BSSN_MAX_GATHER_BOXES 32
typedef struct BssnBox {
    const double* src;
    int32_t shape[3];
    int32_t lo[3];
    int32_t extent[3];
} BssnBox;
int bssn_gather_boxes(int32_t count, const BssnBox* boxes, double* dst, void* stream);

/* ---------------------------------------------------------------------------
 * Bowen-York puncture initial data (JAX_BSSN/utilities/bowen_york_solver.py).
 * Grids are the reference's cell-centred grids: Cartesian (n0, n1, n2), or the
 * meridional (Nrho, 1, Nz) grid with axisymmetric = 1.  Arrays are C-ordered
 * float64 on the device.
 * ------------------------------------------------------------------------- */
#define BSSN_MAX_PUNCTURES 16

/* brill_lindquist_conformal_factor (:52-63), bowen_york_extrinsic_curvature
 * (:66-91) and contract_conformal_curvature (:93-101) at npoints coordinates
 * grid[npoints][3].  masses[np], positions[np][3], momenta[np][3] are HOST
 * arrays.  Any of psi_bl[npoints], curvature[npoints][3][3] and
 * curvature_squared[npoints] may be NULL. */
int bssn_puncture_fields(const double* grid, int64_t npoints, const double* masses, const double* positions,
                         const double* momenta, int32_t npunctures, double* psi_bl, double* curvature,
                         double* curvature_squared, void* stream);

/* Operators of bowen_york_solver.py, in the reference's operation order:
 *   CONTRACT              out = K_ij K_ij of a = K[n][3][3]; shape = (n, 1, 1)      (:93-101)
 *   SOURCE                out = 1/8 b psi^-7, a = psi, b = A^2 (pointwise, shape = any) (:151-155)
 *   LINEARIZED_SOURCE     out = -7/8 c b^-8 a, a = delta, b = psi, c = A^2 (pointwise)  (:158-162)
 *   LAPLACIAN             seven-point / axisymmetric Laplacian of the interior-shaped a (:104-148)
 *   LINEARIZED_OPERATOR   Laplacian(a) + LINEARIZED_SOURCE(a, b, c), all interior-shaped (:165-198)
 *   RESIDUAL              Laplacian(u) + SOURCE(psi_bl + u, A^2) at the interior, with
 *                         full-grid a = u, b = psi_bl, c = A^2; out interior-shaped (:201-230)
 * For the last three, shape is the FULL grid's; the interior of a Cartesian
 * grid is (n0-2, n1-2, n2-2), of a meridional grid (Nrho-1, Nz-2).  LAPLACIAN
 * and LINEARIZED_OPERATOR need a workspace of one full-grid array. */
#define BSSN_PUNCTURE_CONTRACT 0
#define BSSN_PUNCTURE_SOURCE 1
#define BSSN_PUNCTURE_LINEARIZED_SOURCE 2
#define BSSN_PUNCTURE_LAPLACIAN 3
#define BSSN_PUNCTURE_LINEARIZED_OPERATOR 4
#define BSSN_PUNCTURE_RESIDUAL 5
int bssn_puncture_operator(int32_t op, const double* a, const double* b, const double* c, const int32_t shape[3],
                           double dx, int32_t axisymmetric, double* out, void* workspace, size_t workspace_bytes,
                           void* stream);

/* Bytes of device workspace bssn_puncture_solve needs on a grid (0 if the
 * grid is invalid). */
size_t bssn_puncture_workspace_bytes(const int32_t shape[3], int32_t axisymmetric);

/* solve_conformal_factor (:283-366; conjugate gradients) or, with
 * axisymmetric = 1, solve_axisymmetric_conformal_factor (:369-479; BiCGSTAB):
 * Newton iterations on the regular correction u, fixed to zero on the outer
 * cells, each correction from a matrix-free Krylov solve of the negative
 * linearised operator.  Inputs psi_bl and curvature_squared and outputs u and
 * psi = psi_bl + u span the full grid.  residual_history (HOST, room for
 * max_newton_iterations + 1 values) receives the interior RMS residual before
 * each correction and after the last; *history_length its count;
 * linear_iterations (HOST, optional, max_newton_iterations entries) the Krylov
 * iterations of each correction.  Synchronises `stream` once per Newton step
 * and once per 16 Krylov iterations.  Returns BSSN_ERR_NOT_CONVERGED when the
 * Newton iterations run out, and (axisymmetric) BSSN_ERR_NONFINITE for a
 * nonfinite residual or correction or a nonpositive psi, each with the
 * reference's message in bssn_last_error(). */
int bssn_puncture_solve(const double* psi_bl, const double* curvature_squared, const int32_t shape[3], double dx,
                        int32_t axisymmetric, double newton_tolerance, int32_t max_newton_iterations,
                        double linear_tolerance, int32_t max_linear_iterations, double* u, double* psi,
                        double* residual_history, int32_t* history_length, int32_t* linear_iterations,
                        void* workspace, size_t workspace_bytes, void* stream);

/* ---------------------------------------------------------------------------
 * Apparent-horizon finder (JAX_BSSN/utilities/apparent_horizon.py,
 * hermite_interpolation.py).  The geometry is the physical metric and extrinsic
 * curvature, each (3, 3, *grid) C-ordered float64 on the device, on a radial
 * line (dims 1, axis r), a signed x-z plane (dims 2, axes x and z) or a
 * Cartesian volume (dims 3): build_geometry (:22-98).  Surfaces are radii
 * h[n_theta][n_phi] on the cell-centred polar and periodic azimuthal grid of
 * angular_grid (:101-117), n_theta, n_phi >= 6, n_phi even.
 * ------------------------------------------------------------------------- */
typedef struct BssnHorizonGeometry {
    const double* gamma;
    const double* curvature;
    int32_t dims;
    int32_t size[3];     /* points per axis (entries past dims ignored) */
    double origin[3];    /* first coordinate of each axis */
    double spacing[3];
    int32_t margin;      /* resolved region: [margin, size - 1 - margin] */
} BssnHorizonGeometry;

/* sample (:91-98) at points[n][3]: gamma[n][3][3], d_gamma[n][3][3][3]
 * (derivative index first), curvature[n][3][3] and valid[n] (int32); any
 * output may be NULL.  Reads the upper triangle of each tensor. */
int bssn_horizon_sample(const BssnHorizonGeometry* geometry, const double* points, int64_t npoints,
                        double* gamma, double* d_gamma, double* curvature, int32_t* valid, void* stream);

/* angular_derivatives (:125-144): out[5][n_theta][n_phi] = h_theta,
 * h_thetatheta, h_phi, h_phiphi, h_thetaphi. */
int bssn_horizon_angular_derivatives(const double* radius, int32_t n_theta, int32_t n_phi, double* out,
                                     void* stream);

/* Bytes of device workspace for the surface, Jacobian and Newton-direction
 * calls on an (n_theta, n_phi) surface (0 if the surface is invalid). */
size_t bssn_horizon_workspace_bytes(int32_t n_theta, int32_t n_phi);

/* surface (:160-236) of h = radius, or (direction not NULL) of the trial
 * surface h = radius + step * direction, which is written to trial.
 * expansion[n] and density[n] (may be NULL) per node; summary[4] (device) =
 * sum of h, max |expansion|, count of unusable nodes (outside the resolved
 * region, non-positive-definite metric, nonfinite expansion or density, or
 * h <= 0) and the area sum_theta weights[theta] sum_phi density * 2 pi / n_phi
 * (0 when area_weights is NULL).  center is a HOST triple. */
int bssn_horizon_surface(const BssnHorizonGeometry* geometry, const double center[3], const double* radius,
                         const double* direction, double step, int32_t n_theta, int32_t n_phi,
                         const double* area_weights, double* trial, double* expansion, double* density,
                         double* summary, void* workspace, size_t workspace_bytes, void* stream);

/* The Jacobian d expansion / d radius (N x N, N = n_theta n_phi, row-major)
 * that dense_jacobian (:239-250) forms with jax.linearize; here from central
 * differences of relative step fd_step in each node's radius and angular
 * derivatives, assembled in band storage and expanded. */
int bssn_horizon_jacobian(const BssnHorizonGeometry* geometry, const double center[3], const double* radius,
                          int32_t n_theta, int32_t n_phi, double fd_step, double* dense, void* workspace,
                          size_t workspace_bytes, void* stream);

/* Newton direction delta = -J^-1 expansion of find_apparent_horizon (:296-299):
 * the band Jacobian as above, factorised by band LU with partial pivoting.
 * summary[2] (device) = max |delta| over finite entries and the count of
 * nonfinite entries. */
int bssn_horizon_newton_direction(const BssnHorizonGeometry* geometry, const double center[3],
                                  const double* radius, const double* expansion, int32_t n_theta, int32_t n_phi,
                                  double fd_step, double* delta, double* summary, void* workspace,
                                  size_t workspace_bytes, void* stream);

/* interpolate_angular (:147-157): out[n_theta_out][n_phi_out] at polar angles
 * theta[n_theta_out] and azimuths phi[n_phi_out] (device arrays). */
int bssn_horizon_regrid(const double* radius, int32_t n_theta, int32_t n_phi, const double* theta,
                        int32_t n_theta_out, const double* phi, int32_t n_phi_out, double* out, void* stream);

/* No reference counterpart.  FMA throughput of this GPU in GFLOP/s (FMA = 2
 * flops) for BSSN_PRECISION_F64 or BSSN_PRECISION_F32: sixteen independent FMA
 * chains per thread, 8 x 256 threads per SM, one timed launch after a warm-up
 * (synchronous; the denominator of the RHS kernels' compute roofline). */
int bssn_probe_fma_peak(int32_t precision, double* gflops);

/* No reference counterpart.  Self-check of the final RK4 division: for the n
 * device doubles a, fast[i] = the three-operation correctly rounded a[i]/6 the
 * RK4 stage kernel uses and hw[i] = the hardware-rounded division a[i]/6.0.
 * Asynchronous on `stream`. */
int bssn_check_div6(const double* a, double* fast, double* hw, int64_t n, void* stream);

/* Kernel launches issued by this library since load (all threads). */
long long bssn_launch_count(void);
/* Per-kernel-class device-time accounting with CUDA events on each launch's
 * stream; off by default.  Classes: fill, first derivatives, gauge RHS, K/Gt
 * RHS, At RHS, momentum derived fields, momentum damping, Sommerfeld, RK4
 * stage, projection, import, export, constraints, FMR transfer, Cartoon,
 * FP32 conversion, other, K/Gt/At RHS in one pass (FP64 form), puncture
 * Newton-level kernels, puncture Krylov operator kernels, puncture Krylov
 * vector updates, horizon surface kernels, horizon band solve, adjoint point
 * kernel, adjoint stencil transposes, adjoint stage and projection kernels.  bssn_profile_read synchronises the recorded events, accumulates and
 * returns the number of classes. */
void bssn_profile_enable(int on);
void bssn_profile_reset(void);
int bssn_profile_read(double* ms, long long* counts, int n);

#ifdef __cplusplus
}
#endif

#endif /* BSSN_GB300_H */
