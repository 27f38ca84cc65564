/*
 * ffv.h -- C ABI of the GB300-native explicit finite-volume step of ForestFV.
 *
 * This header is the drop-in boundary for the reference's per-RK-stage path, which in
 * the reference is a set of C calls on a malloc'd leaf linked list:
 *
 *   advancetimeexplicit(run)         advancetimeexplicit.c:3-28   -> ffv_step
 *   RK(irk, run) / m5_RK(irk, run)    RK.c:3-53, m5_RK.c:3-127     -> ffv_stage
 *   grad_scheme(run)                  grad_scheme.c:3-41           -> (fused into ffv_stage)
 *   RHS(run)                          RHS.c:3-72                   -> (fused into ffv_stage)
 *   leaf S[NEQ] arrays (LEAF.S)       strdata.h:233-254            -> ffv_upload_state /
 *                                                                      ffv_download_state
 *   neigtr/neigfc/lfc_neigs, CELL     strdata.h:265-332, elconn.c  -> ffv_mesh_build +
 *     geometry (meshproperties.c)                                      ffv_set_mesh
 *   global DT (inputset.c:69)         strdata.h:67                 -> dt argument
 *   globals MODEL, ORDER, RK_STEPS,   strdata.h:45-217             -> ffv_params
 *     MATERGAMA/MATERPINF ...
 *
 * Conventions
 *   - Cells ("leaves") are numbered in the reference's leaf-list order: trees in the
 *     order given, then depth-first by child index (rebuildlist.c:30-91).  For a
 *     Cartesian forest whose trees are listed in Morton order this is a global Morton
 *     order; ffv_mesh_build returns that order.
 *   - Conserved state is structure-of-arrays: S[v * ncells + c], v < neq.
 *   - Every function returns FFV_OK (0) or an FFV_ERR_* code; ffv_error_string names it.
 *   - A context owns its device memory and one CUDA stream.  It is not thread-safe.
 *   - No function falls back to the CPU: without a usable CUDA device, ffv_create fails.
 */
#ifndef FFV_H
#define FFV_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FFV_OK 0
#define FFV_ERR_ARG 1          /* bad argument (NULL pointer, size mismatch, bad enum)   */
#define FFV_ERR_CUDA 2         /* a CUDA runtime call failed                             */
#define FFV_ERR_TABLE 3        /* mesh description rejected (overlap, hole, range)       */
#define FFV_ERR_BALANCE 4      /* face neighbours differ by more than one level          */
#define FFV_ERR_NAN 5          /* non-finite residual or state found on the device       */
#define FFV_ERR_NEG_DENSITY 6  /* non-positive density found on the device               */
#define FFV_ERR_TIMEOUT 7      /* a bounded device wait ran out                          */
#define FFV_ERR_UNSUPPORTED 8  /* option outside what this library implements            */
#define FFV_ERR_NOMEM 9        /* host or device allocation failed                       */
#define FFV_ERR_STATE 10       /* call out of order (e.g. step before mesh/state upload) */
#define FFV_ERR_TOO_LARGE 11   /* mesh larger than the fixed scratch of ffv_step_noalloc */
#define FFV_ERR_IO 12          /* file cannot be opened, read or written, or is corrupt  */

#define FFV_MAX_MATERIALS 8
#define FFV_MAX_NEQ 32
#define FFV_MAX_LEVEL 15

/* arithmetic of the flux path */
#define FFV_FP64 0        /* everything in FP64, bit-identical to the reference's C code */
#define FFV_FP32_FLUX 1   /* reconstruction, wave speeds, HLLC in FP32; FP64 residuals,  */
                          /* RK state and stiffened-gas pressure recovery                 */

/* Model 5's flux, as the reference writes it or made consistent (ffv_params.flux_form).
 * FFV_FLUX_REFERENCE is the reference's m5 flux to the last bit.  Three of its expressions
 * disagree with the rest of its own HLLC solver:
 *   - the star-state energy (m5_star_region.c:59),
 *       (rho E)* = (rho E_K (u_K - S_K) + s11_K u_K - s12_K v_K - s13_K w_K + sigma* . u*)
 *                  / (u* + S_K),
 *     gives (rho E)* = -rho E at u* = 0: every face at rest carries a spurious energy flux of
 *     about 2 c rho E, which boundary faces and material interfaces feed into the solution;
 *   - m5_flux.c:20-34 takes the momentum flux as rho u u + sigma, while m5_flux_gfm.c:20-34,
 *     the contact speed (m5_wave_speeds.c) and model 0 (m0_flux.c: rho u u + p) all have
 *     rho u u - sigma with the Cauchy stress sigma = -p I + deviator: the fluid is pushed by
 *     the negated pressure;
 *   - m5_flux.c:53-56 advects the deformation tensor of the left and right states negated
 *     (-A) where m5_flux_gfm.c and the star states take +A.
 * On these the reference's model-5 scheme stops with a NaN wave speed after one step of
 * Sod's problem, and amplifies rounding-level differences by ~1e9 within 20 steps of the
 * bubble configurations.  FFV_FLUX_CONSISTENT (a deliberate deviation, off by default)
 * takes the Rankine-Hugoniot energy jump across the S_K wave with the normal energy flux
 * rho E u - sigma_n . u,
 *       (rho E)* = (rho E_K (u_K - S_K) - sigma_K . u_K + sigma* . u*) / (u* - S_K),
 * and m5_flux_gfm.c's signs in m5_flux.c (rho u u - sigma, +A); with it model 5 reproduces
 * model 0's solution of Sod's problem. */
#define FFV_FLUX_REFERENCE 0
#define FFV_FLUX_CONSISTENT 1

/* boundary codes, as the reference's fc[].bc (m0_bc.c:3-31, m5_bc.c:3-31); every code is
 * accepted by both models.  Model 5's symmetry face takes the central flux of the cell state
 * and its mirror image (m5_hllc.c:56-85); its inlet, like the reference's, has no state of its
 * own (m5_bc.c:35-48: a transmissive face). */
#define FFV_BC_SYMMETRY 1
#define FFV_BC_OUTLET 2     /* transmissive */
#define FFV_BC_INLET 3
#define FFV_BC_REFLECTIVE 4
#define FFV_BC_WALL 5

/* Solver parameters: the reference's input globals for this path. */
typedef struct ffv_params {
  int32_t model;        /* MODEL: 0 (Euler, stiffened gas, m0_*) or 5 (m5_*: multi-material,
                           hyperelastic solids, ghost-fluid coupling, pressure relaxation) */
  int32_t nmaterials;   /* NMATERIALS (1 for model 0; 2 or 3 for model 5) */
  int32_t order;        /* ORDER: 1 (first order) or 2 (MUSCL, GRAD_SCHEME 1) */
  int32_t rk_steps;     /* RK_STEPS: 1..4; stage k uses the combination of RK.c case k */
  int32_t precision;    /* FFV_FP64 or FFV_FP32_FLUX */
  int32_t prelax;       /* model 5: PRELAX 1 (two materials, closed form) or 3 (iterative) */
  double gamma[FFV_MAX_MATERIALS]; /* MATERGAMA */
  double pinf[FFV_MAX_MATERIALS];  /* MATERPINF */
  double mu[FFV_MAX_MATERIALS];    /* model 5: MATERMUSH, shear modulus (0 for fluids) */
  double amin;          /* model 5: AMIN, volume-fraction floor */
  double avf_lim;       /* model 5: AVF_LIM, solid-fraction level of the ghost-fluid interface */
  int32_t zerou[3];     /* model 5: ZEROU0..2 (freeze a velocity component, m5_RK.c:93-122) */
  int32_t flux_form;    /* model 5: FFV_FLUX_REFERENCE (0, default) or FFV_FLUX_CONSISTENT */
  double yield[FFV_MAX_MATERIALS]; /* model 5: von Mises yield stress of each solid material,
                           0 = none (hyperelastic, as the reference).  A solid with a yield
                           stress gets a J2 radial return of its deformation tensor after every
                           cell relaxation (no counterpart in the reference: its plastic step
                           is only prototyped, strdata.h:809, and the call commented out,
                           m5_relaxation_solid.c:14) */
} ffv_params;

/* A Cartesian forest: ntrees[0] x ntrees[1] x ntrees[2] cubic hex trees of edge
 * tree_edge with corner at the origin, each refined as an octree.  Trees are level 1,
 * their children level 2, ... (spawntopo.c:136, split.c:25), up to FFV_MAX_LEVEL.
 * bc[side] gives the boundary code of the domain sides -x,+x,-y,+y,-z,+z.
 * tree_edge * 2^k must be exact for every level: a power of two times an integer. */
typedef struct ffv_forest_desc {
  int32_t ntrees[3];
  int32_t bc[6];
  double tree_edge;
} ffv_forest_desc;

typedef struct ffv_mesh ffv_mesh; /* host-side face tables */
typedef struct ffv_ctx ffv_ctx;   /* device context */

/* Build the owner-sorted face tables of a 2:1-balanced forest from its leaves.
 * Leaf i lies in tree (tree_ijk[3i..3i+2]) at `level[i]` with integer coordinates
 * cell_ijk[3i..3i+2] inside the tree (0 <= c < 2^(level-1)).  Leaves may come in any
 * order; `order_out` (nleaves entries, may be NULL) receives, for each cell of the
 * built mesh, the index of the input leaf it holds.  Replaces the reference's
 * neighbour search (elconn.c:3-145, elconnfin.c) and geometry
 * (meshproperties.c:3-126, distance.c:120-167) for Cartesian forests. */
int ffv_mesh_build(const ffv_forest_desc *desc, int64_t nleaves, const int32_t *tree_ijk,
                   const int32_t *level, const int32_t *cell_ijk, ffv_mesh **out,
                   int64_t *order_out);
/* ffv_mesh_build for a part of a forest -- one rank's cells and their halo under a Morton-range
 * partition (replaces the proxy layer the reference builds per rank, rebuildprox.c:3-246,
 * restructtopo.c:3-14): a face whose neighbour, or any of whose four finer neighbours, is not
 * among the leaves becomes a transmissive boundary face (FFV_BC_OUTLET) instead of an error.
 * The halo cells next to such faces compute with a stand-in neighbour; a halo deep enough for
 * the cells a rank owns keeps those exact (forestfv_public_gb300/partition.py). */
int ffv_mesh_build_part(const ffv_forest_desc *desc, int64_t nleaves, const int32_t *tree_ijk,
                        const int32_t *level, const int32_t *cell_ijk, ffv_mesh **out,
                        int64_t *order_out);
int64_t ffv_mesh_ncells(const ffv_mesh *m);
void ffv_mesh_free(ffv_mesh *m);

/* Expand the tables into the reference's per-leaf geometry, for validation against
 * the reference (one row per cell-face, 6 per cell, in cell order):
 *   bc, lfc_neigs (0 boundary, 1, 4), neigfc, nb[4] (cell ids, -1 unused),
 *   area[4], nrm[9] (n, t1, t2 as in normalvector.c / tagvector.c),
 *   dist_cf, dist_cc (distance.c:120-167); per cell: vol (meshproperties.c:76-124),
 *   centroid[3] (meshproperties.c:27-38).  Any output pointer may be NULL. */
int ffv_mesh_export(const ffv_mesh *m, int32_t *bc, int32_t *lfc_neigs, int32_t *neigfc,
                    int32_t *nb, double *area, double *nrm, double *dist_cf,
                    double *dist_cc, double *vol, double *centroid);

/* Device context on CUDA device `device`. */
int ffv_create(ffv_ctx **ctx, const ffv_params *p, int device);
int ffv_destroy(ffv_ctx *ctx);
/* Upload the face tables (after every regrid).  Invalidates the state. */
int ffv_set_mesh(ffv_ctx *ctx, const ffv_mesh *m);
/* Conserved state, SoA [neq][ncells], host memory, FP64. */
int ffv_upload_state(ffv_ctx *ctx, const double *S_soa, int64_t ncells, int32_t neq);
int ffv_download_state(ffv_ctx *ctx, double *S_soa, int64_t ncells, int32_t neq);
/* One RK stage, the counterpart of RK(irk) / m5_RK(irk) preceded for irk >= 1 by
 * grad_scheme and RHS (advancetimeexplicit.c:9-19): irk 0 copies S to SN; irk >= 1
 * reconstructs face states, accumulates face fluxes and applies stage irk.  Queued
 * on the context's stream; errors seen on the device are reported by ffv_sync. */
int ffv_stage(ffv_ctx *ctx, int32_t irk, double dt);
/* nsteps full time steps of rk_steps stages each (advancetimeexplicit x nsteps),
 * launched as one CUDA graph per step; synchronises and checks the device status. */
int ffv_step(ffv_ctx *ctx, double dt, int32_t nsteps);
/* As ffv_step, but only queues the graph launches on the context's stream. */
int ffv_step_async(ffv_ctx *ctx, double dt, int32_t nsteps);
/* Wait for queued work and return the first error the device recorded. */
int ffv_sync(ffv_ctx *ctx);
/* Largest stable dt for the given CFL number: cfl * min over cells of
 * h / max(|u_a| + c) (new: the reference uses a fixed DT, inputset.c:69). */
int ffv_cfl_dt(ffv_ctx *ctx, double cfl, double *dt_out);
/* Device pointer of the conserved state (SoA), valid until the next ffv_set_mesh. */
int ffv_state_device_ptr(ffv_ctx *ctx, double **d_S);
/* The context's CUDA stream (a cudaStream_t), for callers that order their own work or
 * timing events against the solver's. */
int ffv_stream(ffv_ctx *ctx, void **stream);
/* Diagnostic timing: run stage irk (>= 1) with a CUDA event around each kernel it
 * launches; ms[i] receives kernel i's duration, *nkernels their count. */
int ffv_profile_stage(ffv_ctx *ctx, int32_t irk, double dt, float *ms, int32_t max_kernels,
                      int32_t *nkernels);
const char *ffv_stage_kernel_name(const ffv_ctx *ctx, int32_t i);
/* Number of kernel launches one time step issues (for launch accounting). */
int ffv_launches_per_step(const ffv_ctx *ctx, int32_t *n);

/* Refinement criteria, the reference's input globals for its tagging (strdata.h:78-106;
 * inputset.c:78-104, m5_input.c:39-57): a leaf's target level is the largest of the
 * uniform level, the gradient criterion's level and the interface layers' levels. */
typedef struct ffv_tag_params {
  int32_t uniform, lvl_uniform;            /* CRT_UNIFORM, CRT_LVL_UNIFORM                */
  int32_t grad_prs, lvl_prs; double thr_prs; /* CRT_GRAD_PRS (relative pressure jump)     */
  int32_t grad_rho, lvl_rho; double thr_rho; /* CRT_GRAD_RHO (relative density jump)      */
  int32_t grad_vel, lvl_vel; double thr_vel; /* CRT_GRAD_VEL (the reference evaluates it on
                                              the density jump, criterionsplt.c:120; it
                                              needs grad_rho)                             */
  int32_t inter0, lvl_inter0, lrs_inter0;  /* CRT_ADAPT_INTER_0: SI layers 1..lrs0-1       */
  int32_t inter1, lvl_inter1, lrs_inter1;  /* CRT_ADAPT_INTER_1: SI layers lrs0..lrs0+lrs1-1,
                                              as the input file gives lrs1 (m5_input.c:50) */
} ffv_tag_params;

/* Refinement tags of the current device state, the counterpart of interface_location +
 * criterionsplt (interface_location.c:7-86, criterionsplt.c:3-140; on the device) followed
 * by criterionsmth (criterionsmth.c:3-58; on the host, in leaf order).  `m` is the mesh
 * set on the context.  split[n] receives the smoothed target level per leaf; split_raw[n]
 * (nullable) the level before smoothing; si[2 n] (nullable) the interface layer numbers
 * SI[0], SI[1] as [2][n].  Model 5 as the reference; for model 0 (extension: the
 * reference's gradient criterion has no model-0 branch, criterionsplt.c:64-70) the same
 * relative jumps of the cell states, and no interface layers. */
int ffv_tags(ffv_ctx *ctx, const ffv_mesh *m, const ffv_tag_params *p, int32_t *split,
             int32_t *split_raw, int32_t *si);
/* ffv_tags without the smoothing: the raw target level per leaf (and optionally SI), for
 * callers that combine it with other targets before ffv_tags_smooth. */
int ffv_tags_raw(ffv_ctx *ctx, const ffv_mesh *m, const ffv_tag_params *p, int32_t *split_raw,
                 int32_t *si);
/* The plain criterion as a judge (no counterpart in the reference): the device part of
 * ffv_tags (SI layers and the raw target levels) and, on the device, the number of leaves
 * whose raw target level is above their level -- the leaves a regrid would refine.  No
 * host smoothing, one 8-byte copy back. */
int ffv_tags_missed(ffv_ctx *ctx, const ffv_mesh *m, const ffv_tag_params *p, int64_t *missed);
/* criterionsmth alone, in place on split[n] (host): level_max is the reference's LEVEL,
 * the largest level any criterion names. */
int ffv_tags_smooth(const ffv_mesh *m, int32_t level_max, int32_t *split);
/* One refineh pass (refineh.c:3-57, merge.c, split.c): with split[n] the target levels of
 * the leaves of `m` (the mesh set on the context), eight sibling leaves that all want a
 * coarser level merge (state: the mean of the eight, then for model 5 the reference's
 * pressure relaxation), a leaf that wants a finer level splits into eight children with
 * its state, the rest stay.  *out receives the new mesh (ffv_mesh_free); the context holds
 * its tables and the carried-over state.  The reference's meshadaptation is LEVEL + 1 rounds
 * of ffv_tags + ffv_adapt. */
int ffv_adapt(ffv_ctx *ctx, const ffv_mesh *m, const int32_t *split, ffv_mesh **out);
/* ffv_adapt, and src[n_new] (nullable) receives the source of every new leaf: the old
 * leaf it copies or splits from (>= 0), or -1 - j for a parent merged from the old leaves
 * j..j+7.  n_new = n + 7 (nsplit - nmerge) with the counts of ffv_adapt_changes. */
int ffv_adapt_map(ffv_ctx *ctx, const ffv_mesh *m, const int32_t *split, ffv_mesh **out,
                  int64_t *src);
/* The host half of ffv_adapt (no GPU): the leaves of one refineh pass with targets split[n]
 * and their face tables -- equal to ffv_mesh_build's for those leaves, rebuilt only around
 * the leaves that split or merge (the other rows are the old ones, renumbered).  src[n_new]
 * (nullable) as ffv_adapt_map's. */
int ffv_mesh_adapt(const ffv_mesh *m, const int32_t *split, ffv_mesh **out, int64_t *src);
/* What one refineh pass with targets split[n] would do (host, no GPU): the number of
 * leaves that split and of sibling groups that merge.  Both 0: the pass changes nothing. */
int ffv_adapt_changes(const ffv_mesh *m, const int32_t *split, int64_t *nsplit, int64_t *nmerge);
/* The leaves of a mesh in its cell order (tree_ijk[3n], level[n], cell_ijk[3n]); an output
 * may be null (not all three). */
int ffv_mesh_leaves(const ffv_mesh *m, int32_t *tree_ijk, int32_t *level, int32_t *cell_ijk);

/* Global conservation sums in FP64: sums[v] = sum over leaves of |V| S[v] for every conserved
 * variable (mass of each material, momentum, total energy, ...), a reproducible device
 * reduction (fixed cell-to-thread assignment and reduction order). */
int ffv_conservation_sums(ffv_ctx *ctx, double *sums);

/* Checkpoint/restart and field export (host side, no GPU).
 *
 * Binary checkpoint (no counterpart in the reference): the leaves Morton-keyed (tree rank,
 * level, child-index path) and the SoA FP64 state [neq][n] in the mesh's cell order, with an
 * FNV-1a hash; bit-exact.  Read it back with ffv_checkpoint_info (sizes, forest) and
 * ffv_checkpoint_read (mesh and state; S may be NULL).  A corrupt or truncated file gives
 * FFV_ERR_IO. */
int ffv_checkpoint_write(const char *path, const ffv_mesh *m, const double *S, int32_t neq,
                         int64_t istep, double time);
int ffv_checkpoint_info(const char *path, ffv_forest_desc *desc, int64_t *n, int32_t *neq,
                        int64_t *istep, double *time);
int ffv_checkpoint_read(const char *path, ffv_mesh **out, double *S);
/* The reference's text restart file (restart_save.c:13-50 writes it, restart_load.c:13-45
 * reads it): header "istep time nleaves ntrees neq", one line per leaf "root tag S..." with
 * "%15.10e" values.  The write is byte-identical to the reference's for the same leaves and
 * state (levels up to 10: tags are 32-bit base-10 numbers); the read takes the forest's
 * tree counts and boundary codes from desc (the file has only the total tree count). */
int ffv_restart_text_write(const char *path, const ffv_mesh *m, const double *S, int32_t neq,
                           int64_t istep, double time);
int ffv_restart_text_info(const char *path, int64_t *n, int32_t *neq, int64_t *istep, double *time,
                          int32_t *ntrees_total);
int ffv_restart_text_read(const char *path, const ffv_forest_desc *desc, ffv_mesh **out,
                          double *S);
/* Tecplot ASCII export of per-leaf fields (headless; the reference's m5_exportfield_linked.c
 * writes node-averaged fields of the same kind): one FEBRICK zone whose nodes are shared
 * between leaves on the finest level's lattice, F [nfields][n] cell-centred in BLOCK form. */
int ffv_tecplot_write(const char *path, const ffv_mesh *m, int32_t nfields, const char *const *names,
                      const double *F, double time);
/* Per-leaf fields of the context's state into F_dev (device, FP64 [nf][n]; *nf receives nf):
 * model 5: density, velocity u v w (physical: the state holds the negated momentum in this
 * forest's node layout), mixture pressure sum_k alpha_k p_k, the N volume
 * fractions, the N material pressures and the von Mises equivalent of the mixture stress
 * (nf = 5 + 2 N + 1); model 0: density, u, v, w, pressure (nf = 5).  F_dev NULL: only nf. */
int ffv_export_fields(ffv_ctx *ctx, double *F_dev, int32_t *nf);

/* Learned refinement indicator (no counterpart in the reference): a 135-64-64-1
 * perceptron with GELU hidden layers and a sigmoid output over the 27-cell stencil of five
 * per-cell fields (log rho, log p, alpha_0, |u|, von Mises stress), BF16 operands and FP32
 * accumulation on the tensor cores, trained on the GPU with AdamW.  Parameters are one
 * FP32 vector: W1 [64][135], b1 [64], W2 [64][64], b2 [64], w3 [64], b3. */
#define FFV_MLP_NPARAM 12929
#define FFV_MLP_INPUT_STRIDE 144 /* BF16 values per feature row (135 + zero padding) */
typedef struct ffv_mlp ffv_mlp;
int ffv_mlp_create(ffv_mlp **mlp, int device, uint64_t seed);
int ffv_mlp_destroy(ffv_mlp *mlp);
int ffv_mlp_get_params(ffv_mlp *mlp, float *params);
int ffv_mlp_set_params(ffv_mlp *mlp, const float *params); /* also resets AdamW state */
/* per-field normalisation of the features (mean, standard deviation; 5 each) */
int ffv_mlp_set_norm(ffv_mlp *mlp, const float *mean, const float *stdev);
/* the five per-cell fields of the context's state into F_dev (device, FP32 [5][n]); for
 * model 0 the volume fraction is 1 and the stress 0 */
int ffv_mlp_fields(ffv_ctx *ctx, float *F_dev);
/* feature rows of the context's state into X_dev (device, BF16 [n][144]) */
int ffv_mlp_features(ffv_ctx *ctx, ffv_mlp *mlp, void *X_dev);
/* probabilities of n feature rows (device pointers).  Inference runs on the fifth-generation
 * tensor cores (tcgen05.mma, accumulators in tensor memory) with bounded waits: a wait that
 * runs out is returned as FFV_ERR_TIMEOUT (by ffv_mlp_forward and ffv_mlp_predict, which
 * wait for the device; by the next ffv_mlp_mark, which does not). */
int ffv_mlp_forward(ffv_mlp *mlp, const void *X_dev, int64_t n, float *prob_dev);
/* features + forward of the context's state, probabilities to the host (n) */
int ffv_mlp_predict(ffv_ctx *ctx, ffv_mlp *mlp, float *prob_host);
/* The network on the context's state, on the context's stream with no copy back:
 * marks_dev[c] (device, uint8 [n]) becomes 1 where the probability exceeds threshold, OR-ed
 * into its previous value when accumulate is nonzero. */
int ffv_mlp_mark(ffv_ctx *ctx, ffv_mlp *mlp, float threshold, uint8_t *marks_dev,
                 int32_t accumulate);
/* gradient (host, FFV_MLP_NPARAM) and loss of the mean binary cross-entropy over the first
 * B rows of X_dev / labels y_dev (device, FP32 0 or 1) */
int ffv_mlp_grad(ffv_mlp *mlp, const void *X_dev, const float *y_dev, int64_t B,
                 float *grad_host, float *loss_host);
/* steps AdamW steps (beta 0.9, 0.999, eps 1e-8, decoupled weight decay wd on the weights)
 * on batches of `batch` rows drawn from the N rows of X_dev / y_dev with a seeded hash
 * (seed != 0); loss_host (nullable) receives each step's mean loss */
int ffv_mlp_train(ffv_mlp *mlp, const void *X_dev, const float *y_dev, int64_t N, int32_t batch,
                  int32_t steps, float lr, float wd, uint64_t seed, float *loss_host);

const char *ffv_error_string(int code);

/* No-allocation model-0 step -- no counterpart in the reference.
 * For callers that cannot allocate device memory: a plugin or library that is handed
 * device buffers by a host application or framework which owns all allocation (its own
 * arena or caching allocator, a fixed memory budget), or a loop that must not call
 * cudaMalloc/cudaFree because they synchronise the device.  Advances the model-0 FP64
 * state d_S (device memory of the current device, SoA [5][ncells], updated in place) by
 * nsteps time steps of p->rk_steps stages on `stream` (a cudaStream_t; NULL = the legacy
 * default stream), with the same kernels and results as ffv_step, then waits for the
 * stream and returns the first error the device recorded.  It allocates nothing, on the
 * device or the host: the face tables of `m`, the RK copy and the face states live in one
 * fixed device array of FFV_NOALLOC_SCRATCH_BYTES inside this library, which every GPU
 * that loads the library holds until the process exits.  Meshes of more than
 * FFV_NOALLOC_MAX_CELLS cells are rejected with FFV_ERR_TOO_LARGE; models other than 0
 * and precisions other than FFV_FP64 with FFV_ERR_UNSUPPORTED.  All calls on a device
 * share the array and it keeps the last call's contents (each call rewrites what it
 * reads and clears its status word first); calls whose work overlaps on the GPU race on
 * it.  The first call on a device looks up the array's address (cudaGetSymbolAddress) and
 * should come before any stream capture on that device; the address is cached per device
 * together with the id of the CUDA context it belongs to, and looked up again in a new
 * context (after cudaDeviceReset).  With lazy module loading (CUDA_MODULE_LOADING=LAZY, the
 * default) that first lookup also loads the library's module and reserves the array, so it
 * can fail for lack of device memory (FFV_ERR_CUDA): a caller with a fixed budget makes its
 * first call, or sets CUDA_MODULE_LOADING=EAGER, before it takes the rest of the memory. */
#define FFV_NOALLOC_MAX_CELLS 65536
#define FFV_NOALLOC_SCRATCH_BYTES 21758464
int ffv_step_noalloc(const ffv_mesh *m, const ffv_params *p, double *d_S, double dt,
                     int32_t nsteps, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FFV_H */
