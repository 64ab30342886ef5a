/*
 * fvs2d.h — C-ABI of the GB300 residual-and-update library for fvs2d.
 *
 * The reference has no FFI: its hot path is a pair of Fortran module
 * procedures over module-global state,
 *   compute_residual(time)            src/residual.f90:23
 *   time_integration(t1, ntimes_sub)  src/runge_kutta.f90:94
 * reading the mesh of src/data_grid.f90:23-68, the solution arrays of
 * src/data_solution.f90:16-28 and the scheme flags of src/input.f90:9-56.
 * The entry points below replace those procedures one-for-one.  A Fortran
 * host binds them through an ISO_C_BINDING interface block that declares
 * each prototype below with bind(C) and value/reference arguments to match.
 *
 * Conventions
 *  - All arrays are caller-owned host memory unless a name says "device".
 *    The library copies in and out; no pointer is kept after a call returns.
 *  - Cell, node and edge numbers crossing the ABI are 1-based, in the
 *    reference's numbering (cells: triangles first, then quads, as read
 *    from the .grid file, src/grid_procs.f90:95-108).
 *  - Per-cell 4-vectors are laid out [ncells][4] (row-major C), which is the
 *    Fortran column-major cvar(4,ncells) of src/data_solution.f90:18.
 *  - Every call returns an FVS_* status; nothing calls exit/stop/abort
 *    (the reference stops the program, e.g. src/residual.f90:208,220).
 *  - One handle is not re-entrant; separate handles may be used from
 *    separate host threads.  Each handle owns one CUDA stream.
 */
#ifndef FVS2D_H
#define FVS2D_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define FVS_OK            0
#define FVS_ERR_INVALID   1  /* bad argument or unsupported option combination */
#define FVS_ERR_MESH      2  /* mesh fails a reference consistency check        */
#define FVS_ERR_CUDA      3  /* CUDA runtime error (message via fvs_last_error)  */
#define FVS_ERR_NONFINITE 4  /* a residual norm became NaN/Inf                   */
#define FVS_ERR_DIVERGED  5  /* residual norm grew past options.diverge_factor   */
#define FVS_ERR_TIMEOUT   6  /* a bounded device-side wait expired               */
#define FVS_ERR_NOMEM     7  /* device or host allocation failed                 */
#define FVS_ERR_BOUNDS    8  /* index-checking kernels met an out-of-range index */

/* ---- boundary types (src/residual.f90:194-221; .bc strings) ------------ */
#define FVS_BC_FREESTREAM 1  /* 'freestream'  */
#define FVS_BC_SLIP_WALL  2  /* 'slip_wall'   */
#define FVS_BC_SOLID_WALL 3  /* 'solid_wall'  (the reference stops: rejected) */
#define FVS_BC_DIRICHLET  4  /* 'dirichlet'   (exact vortex or MMS)           */

/* ---- gradient / limiter / reconstruction codes (src/input.f90:190-263) -- */
#define FVS_GRAD_GGCB 1
#define FVS_GRAD_GGNB 2
#define FVS_GRAD_LSQ  3
#define FVS_LSQ_FN 0          /* face-neighbour stencil, kd-tree padding  */
#define FVS_LSQ_NN 1          /* node-neighbour stencil                    */
#define FVS_LIM_NONE   0
#define FVS_LIM_VENK   1
#define FVS_LIM_BARTH  2
#define FVS_LIM_ALBADA 3
#define FVS_RECON_UPWIND1 1
#define FVS_RECON_UPWIND2 2
#define FVS_RECON_UMUSCL  3

/* ---- arithmetic of the device path ---------------------------------------
 * FP64_STRICT: every operation of the reference in source order, no FMA
 *              contraction; bit-identical to the CPU oracle built with
 *              -ffp-contract=off wherever no transcendental is involved.
 * FP64:        same operations, FMA contraction allowed, reciprocals and
 *              square roots from the hardware approximations refined by a
 *              Newton-Raphson step (fast FP64 drop-in).
 * MIXED:       gradients, limiter, reconstruction and flux in FP32; the
 *              residual accumulated exactly (TwoSum), the RK increment in
 *              FP32 added to the FP64 state, which is stored in FP64; norms
 *              summed as pairs of FP32 numbers (~48 significant bits).  The
 *              LSQ weight matrices are built in FP64 and rounded once to FP32
 *              for the gradient: that rounding moves the gradient by at most
 *              8.8e-8 of max|grad| (1,048,576-cell vortex), against 1.3e-5
 *              from the FP32 primitives the weights multiply.
 * FP64_DF:     gradients, limiter, reconstruction, flux, the residual gather
 *              and the RK stage in double-float (pairs of FP32, 48-bit
 *              significand: FP64-class accuracy on the FP32 pipe); the state
 *              is stored in FP64 (exactly its double-float value), the local
 *              time step is FP64, the norms are summed as FP32 pairs.       */
#define FVS_PREC_FP64_STRICT 0
#define FVS_PREC_FP64        1
#define FVS_PREC_MIXED       2
#define FVS_PREC_FP64_DF     3

/* ---- mesh: what grid_read / grid_bc_read load (src/grid_procs.f90:65-164) */
typedef struct fvs_mesh {
  int32_t nnodes;
  int32_t ncells_tri;
  int32_t ncells_quad;
  const double*  node_xy;      /* [nnodes][2]                                   */
  const int32_t* tri_nodes;    /* [ncells_tri][3], 1-based node ids             */
  const int32_t* quad_nodes;   /* [ncells_quad][4], 1-based (may be NULL if 0)  */
  int32_t nbndries;
  const int32_t* bndry_ncells; /* [nbndries]                                    */
  const int32_t* bndry_type;   /* [nbndries] FVS_BC_*                           */
  const int32_t* bndry_cells;  /* concatenated per boundary, 1-based cell ids   */
  /* Extension, not in the reference: doubly periodic meshes.  When > 0 the
   * node ids of cells wrap across x (resp. y) with this period and every
   * geometric difference is taken as the minimum image.                    */
  double period_x;
  double period_y;
} fvs_mesh;

/* ---- options: the scheme flags of src/input.f90:9-56 ------------------- */
typedef struct fvs_options {
  double  gamma;        /* gamma (cp/cv)                                      */
  double  mach_inf;     /* free-stream Mach (src/data_solution.f90:55-58)     */
  double  aoa_inf_deg;  /* free-stream angle of attack, degrees               */
  double  dt;           /* time step (unsteady); initial dt_local (steady)    */
  double  cfl;          /* cfl_user (steady local time step)                  */
  int32_t steady;       /* lsteady: local time stepping                       */
  int32_t vortex;       /* lvortex: Dirichlet BC = exact isentropic vortex    */
  int32_t ntstart;      /* 0 -> manufactured solution (MMS) start and BC      */
  int32_t grad_method;  /* FVS_GRAD_*                                         */
  int32_t lsq_stencil;  /* FVS_LSQ_FN / FVS_LSQ_NN                            */
  double  lsq_pow;      /* LSQ weight 1/d^p                                   */
  int32_t limiter;      /* FVS_LIM_*                                          */
  int32_t reconst;      /* FVS_RECON_*                                        */
  double  umuscl;       /* kappa (forced 0 for methods 1-2)                   */
  int32_t flux;         /* 1 = Roe (the only scheme)                          */
  int32_t rk_nstages;   /* 4 (reference); 3 with ssprk = SSP-RK3 (extension)  */
  int32_t rk_order;     /* 1..4                                               */
  int32_t ssprk;        /* lSSPRK                                             */
  /* fvs2d.vortex (src/mms.f90:55-62) */
  double  vortex_x, vortex_y, vortex_kappa;
  double  vortex_inf[4];  /* rho, u, v, p */
  /* extensions, not in the reference */
  int32_t dt_from_cfl;  /* unsteady: dt = min_cells cfl*vol/(0.5*ws) of the  */
                        /* first residual evaluation, kept for the whole run  */
  int32_t precision;    /* FVS_PREC_*                                         */
  double  diverge_factor; /* >0: FVS_ERR_DIVERGED when rho-norm > factor*first */
} fvs_options;

typedef struct fvs_handle fvs_handle;

/* Fills the defaults of the reference's example inputs (LSQ-fn, p=0, no
 * limiter, 2nd-order upwind, Roe, classic RK4, gamma 1.4). */
int fvs_options_default(fvs_options* opt);

/* Builds connectivity bit-exactly as grid_data (src/grid_procs.f90:170-794),
 * the gradient operator (src/gradient.f90:18-38 and the grad_*_init
 * routines), verifies LSQ linear exactness (src/gradient_lsq.f90:490-529),
 * sets the free-stream state (src/data_solution.f90:41-66) and the RK
 * coefficients (src/runge_kutta.f90:25-88), renumbers cells for the device
 * and uploads everything.  On failure *out is NULL and the message is
 * available from fvs_last_error(NULL). */
int fvs_create(const fvs_mesh* mesh, const fvs_options* opt, fvs_handle** out);
/* Host-only handle: runs the mesh preprocessing and the gradient setup of
 * fvs_create without touching a GPU (for hosts that only need the
 * reference-numbered connectivity, or machines without a device).  Only
 * fvs_get_sizes, fvs_export*, fvs_mms_source and fvs_destroy accept it. */
int fvs_create_host(const fvs_mesh* mesh, const fvs_options* opt, fvs_handle** out);
void fvs_destroy(fvs_handle* h);
/* Last error message of h, or of the calling thread's last failed create
 * when h is NULL.  The string lives until the next call on that handle. */
const char* fvs_last_error(const fvs_handle* h);

typedef struct fvs_sizes {
  int32_t nnodes, ncells, ncells_tri, ncells_quad;
  int32_t nedges, nedges_intr, nedges_bndr;
  int32_t ncells_intr, ncells_bndr;
  int32_t nbndries;
  int32_t stencil_len;   /* total entries of the gradient stencil CSR       */
  int32_t nstages;       /* RK stages per step                              */
  double  heff1, heff2;  /* src/grid_procs.f90:233-243                      */
  double  vol_sum, vol_green; /* grid_data_verify src/grid_procs.f90:824-840 */
  double  dt;            /* current global dt                               */
} fvs_sizes;
int fvs_get_sizes(const fvs_handle* h, fvs_sizes* s);

/* Named host-side setup arrays in reference order (connectivity, geometry,
 * stencils), for bit-level comparison: see fvs_export for the names. */
int fvs_export_size(const fvs_handle* h, const char* name, int64_t* nbytes);
int fvs_export(const fvs_handle* h, const char* name, void* dst, int64_t nbytes);

/* initialize_solution (src/initialize.f90:19-90) for ntstart <= 1:
 * free stream, exact vortex at t=(ntstart-1)*dt, or MMS.  ntstart > 1 (a
 * restart from the cont.cd / cont.s8 files, src/initialize.f90:56-77) returns
 * FVS_ERR_INVALID: the host reads the files and calls fvs_set_state. */
int fvs_init_state(fvs_handle* h);
int fvs_set_state(fvs_handle* h, const double* cvar);   /* [ncells][4] */
int fvs_get_state(fvs_handle* h, double* cvar);         /* [ncells][4] */

/* compute_residual (src/residual.f90:23-177): resid = dU/dt = -R/vol and
 * ws_nrml = sum of 0.5(|un|+a)*A.  Either output may be NULL. */
int fvs_residual(fvs_handle* h, double time, double* resid, double* ws_nrml);
/* Gradient grad(4,ncells,2) as [2][ncells][4] and phi_lim[ncells] of the
 * last residual evaluation (src/data_solution.f90:19-21). */
int fvs_get_gradient(fvs_handle* h, double* grad, double* phi);

/* time_integration (src/runge_kutta.f90:94-114): nsteps RK steps from t1.
 * resnorm (may be NULL) receives [nsteps][4] RMS(|U-U0|) per component,
 * the log_res.plt columns (src/runge_kutta.f90:395-410). */
int fvs_time_integration(fvs_handle* h, double t1, int32_t nsteps, double* resnorm);

/* Extension: steps until RMS(dU_rho)(n) <= drop * RMS(dU_rho)(1) or
 * max_steps.  The norm is checked on the host every check_every steps
 * (steps run as captured CUDA graphs in between). */
int fvs_run_to_drop(fvs_handle* h, double t1, int32_t max_steps, double drop,
                    int32_t check_every, int32_t* steps_done, double* resnorm);

/* Wall pressure and loads of slip-wall boundary ib (1-based), the numbers
 * write_inst_cp_un writes (src/io.f90:340-446).  Face values use the
 * configured cell-centre gradient of the current state without limiter
 * (gradient_cellcntr_1var, src/gradient.f90:75-96), also for first-order
 * runs.  edge_out [nedges][4] = (x_face, cp_wall, cp_cell, un) in the
 * boundary's edge order, or NULL; loads[11] = cl, cd, cl1, cd1, |Vn|max,
 * |Vn|_2, |Vn|_1, cn, ca, cn1, ca1 (the "1" values use the cell pressure). */
int fvs_wall_loads(fvs_handle* h, int32_t ib, double* edge_out, double* loads);

/* error_isentropic_vortex (src/mms.f90:271-365): the 13 numbers of one
 * log_vortex_err.plt row after the time column. */
int fvs_vortex_error(fvs_handle* h, double time, double* err13);

/* MMS source term at cell centres (src/mms.f90:105-114), [ncells][4]. */
int fvs_mms_source(fvs_handle* h, double* src);

/* ---- device-resident path (benchmarks, batched drivers) --------------- */
/* Runs nsteps steps on the device state without host copies; if ms is not
 * NULL it receives the CUDA-event time of the call on the handle's stream. */
int fvs_steps_device(fvs_handle* h, int32_t nsteps, float* ms);
/* Per-kernel timing of one step (CUDA events on the handle's stream):
 * names[i] / ms[i] for up to cap kernels; returns the count in *n. */
int fvs_profile_step(fvs_handle* h, int32_t cap, int32_t* n, char* names /*[cap][32]*/, float* ms);
/* Number of kernel launches one step issues. */
int fvs_launches_per_step(const fvs_handle* h, int32_t* n);
/* Device pointer of the conservative state (RCM order) and the permutation
 * old->new (host copy, 0-based) for callers that keep data on the device. */
int fvs_device_state(fvs_handle* h, void** dptr);
/* Index-checking kernels (no counterpart in the reference, which has no
 * sanitizer either).  With the environment variable FVS2D_BOUNDS=1 at
 * fvs_create, an FVS_PREC_FP64 handle runs kernels built with every
 * indirect index (stencil cells, edge cells, gather slots) checked against
 * its array's extent.  A kernel that meets a violation records the first one
 * in a device word, substitutes index 0 and carries on (no trap, no fault);
 * fvs_time_integration, fvs_steps_device and fvs_residual then return
 * FVS_ERR_BOUNDS with the site, index and extent in fvs_last_error.  The
 * arithmetic is the FP64 handle's, so results are bit-identical to it.
 * fvs_debug_set_gather writes one entry of a cell's gather list (cell
 * 1-based, entry 0..3, value: signed 1-based edge slot or 0) and is refused
 * except on such a handle: it exists to show that the checks fire. */
int fvs_debug_set_gather(fvs_handle* h, int32_t cell, int32_t entry, int32_t value);
/* Host-only check of the fused stage's tile plan (no counterpart in the
 * reference; no GPU needed): builds the plan a mixed or double-float handle
 * would use for this mesh and checks every index its kernel derives from it.
 * info[8] = (tiles, largest local cell count, largest gradient cell count,
 * largest face count, 1 if every check holds, halo entries, shared memory of
 * a block of the bulk-copy form in bytes (mixed), 1 if every alignment and
 * extent of its copies holds).  Returns FVS_ERR_MESH (message in
 * fvs_last_error(NULL)) on the first violation. */
int fvs_tile_plan_info(const fvs_mesh* mesh, const fvs_options* opt, int32_t* info);
/* Check of the FP64 kernels' reciprocal and square root (no counterpart in
 * the reference): for n host values x (positive normal numbers), out
 * [n][5] = (the kernels' 1/x, IEEE 1/x, the kernels' 1/sqrt(x), the
 * kernels' sqrt(x), IEEE sqrt(x)), all evaluated on the current device. */
int fvs_check_fp64_math(const double* x, int32_t n, double* out);

/* ---- batched independent cases ------------------------------------------
 * No counterpart in the reference, which runs one case per process: many
 * cases (e.g. an airfoil sweep over Mach and angle of attack) advanced
 * together.  All cases share the scheme flags of fvs_options (LSQ gradients,
 * any precision, fixed dt or steady); only mach_inf / aoa_inf_deg differ.
 * The meshes are preprocessed on host_threads threads (<= 0: all cores),
 * packed as one disjoint union on the device, and advanced by one
 * cooperative persistent kernel per chunk of steps (captured in a CUDA
 * graph).  Every grid-barrier wait of that kernel is bounded; a wait that
 * runs out returns FVS_ERR_TIMEOUT instead of hanging. */
typedef struct fvs_batch fvs_batch;
int fvs_batch_create(const fvs_mesh* meshes, const fvs_options* opts, int32_t ncases, int32_t host_threads,
                     fvs_batch** out);
void fvs_batch_destroy(fvs_batch* b);
const char* fvs_batch_last_error(const fvs_batch* b);
/* total cells and edge slots; launch4 = {block, tile, blocks per SM, flags}
 * with flags bit 0 = persistent launches graph-captured, bit 1 = tiled mode,
 * bit 2 = fused first-order stages in use */
int fvs_batch_info(const fvs_batch* b, int32_t* ncells, int32_t* nedges, int32_t* launch4);
int fvs_batch_init_state(fvs_batch* b);                                  /* free stream per case */
int fvs_batch_set_state(fvs_batch* b, int32_t icase, const double* cvar); /* [ncells_case][4] */
int fvs_batch_get_state(fvs_batch* b, int32_t icase, double* cvar);
/* times the launch-shape candidates on the batch (state restored after) */
int fvs_batch_autotune(fvs_batch* b, int32_t trial_steps, float* best_ms_per_step);
int fvs_batch_set_launch(fvs_batch* b, int32_t block, int32_t tile, int32_t blocks_per_sm);
/* mode 0: one cooperative persistent launch per chunk of steps (grid
 * barriers between phases); FVS_BATCH_TILED: each step a CUDA graph of tile
 * launches, one block per tile and phase (fvs_batch_autotune times both).
 * First-order mixed-precision stages with an even number of stages are
 * fused: each cell evaluates the flux of its own faces (every interior face
 * twice, once from each side, in the edge's orientation) and applies the
 * stage, one phase per stage; FVS_BATCH_UNFUSED keeps the separate edge-flux
 * and update phases (the autotuner times both).  FVS_BATCH_DC_FUSED fuses the
 * defect-correction stages the same way (off by default: slower than the
 * separate phases on the measured sweeps).  The run-to-target calls choose
 * the launch shape again on line as cases converge: once the active cells
 * fall to half of those at the last choice (and at the start of a
 * defect-correction run), the next chunks run a few candidate shapes for 20
 * steps each, timed on the device, and keep the fastest for the rest of the
 * call; FVS_BATCH_FIXED_SHAPE keeps the set shape throughout. */
#define FVS_BATCH_TILED 1
#define FVS_BATCH_UNFUSED 2
#define FVS_BATCH_DC_FUSED 4
#define FVS_BATCH_FIXED_SHAPE 8
int fvs_batch_set_mode(fvs_batch* b, int32_t mode);
/* switches the arithmetic of all cases (FVS_PREC_*), keeping the FP64
 * state: e.g. MIXED until the FP32 flux floor, then FP64 to a 1e-10 drop */
int fvs_batch_set_precision(fvs_batch* b, int32_t precision);
/* budget of one grid-barrier wait, seconds (default 4) */
int fvs_batch_set_barrier_budget(fvs_batch* b, double seconds);
/* nsteps (<= 1024) steps of every case; norms [ncases][nsteps][4] or NULL */
int fvs_batch_steps(fvs_batch* b, int32_t nsteps, double* norms, float* ms);
/* Groups of cases that stop together: when a case meets its target in a run
 * below, the other active cases with the same group id stop at that step
 * (several starts of one problem raced; the first to converge wins).
 * group [ncases], or NULL: every case alone (the default). */
int fvs_batch_set_groups(fvs_batch* b, const int32_t* group);
/* steps until each case's RMS(dU) <= drop x its first value in all four
 * components; converged cases leave the work lists.  steps_done [ncases];
 * first, last [ncases][4] */
int fvs_batch_run_to_drop(fvs_batch* b, int32_t max_steps, double drop, int32_t chunk, int32_t* steps_done,
                          double* first, double* last, float* ms);
/* the same with absolute targets: RMS(dU_k) <= levels[c][k] for k = 0..3
 * (a warm start judged on the thresholds of a free-stream start) */
int fvs_batch_run_to_level(fvs_batch* b, int32_t max_steps, const double* levels, int32_t chunk, int32_t* steps_done,
                           double* first, double* last, float* ms);
/* Defect correction for first-order steady batches (no counterpart in the
 * reference): per chunk of `chunk` steps the FP64 residual R0 of the current
 * state is evaluated once, then the RK stages iterate a correction dU with
 * the linearised residual R0 + J dU (J dU by forward-mode differentiation of
 * the Roe flux in FP32) and the correction is added to the FP64 state.  The
 * fixed point is the FP64 residual's.  Norms are the RMS of the correction
 * increments per step; stops like fvs_batch_run_to_level.  The batch is in
 * FP64 afterwards (confirm the levels with fvs_batch_run_to_level). */
int fvs_batch_run_to_level_dc(fvs_batch* b, int32_t max_steps, const double* levels, int32_t chunk,
                              int32_t* steps_done, double* first, double* last, float* ms);

/* ---- learned warm start: a small MLP on the GPU ---------------------------
 * No counterpart in the reference.  n_in -> width (GELU) x depth -> n_out,
 * FP32 master weights, BF16 tensor-core GEMMs with FP32 accumulation, Adam
 * on the mean squared error, all on the GPU.  Parameters in the unpadded
 * layout: for each layer W[out][in] then b[out]. */
typedef struct fvs_mlp fvs_mlp;
int fvs_mlp_create(int32_t n_in, int32_t width, int32_t depth, int32_t n_out, uint64_t seed, fvs_mlp** out);
void fvs_mlp_destroy(fvs_mlp* m);
const char* fvs_mlp_last_error(const fvs_mlp* m);
/* GEMM engine: 0 = tcgen05 tensor-core MMA with the accumulator in tensor
 * memory (default), 1 = warp-level mma.sync (the comparison engine) */
int fvs_mlp_set_engine(fvs_mlp* m, int32_t engine);
int fvs_mlp_num_params(const fvs_mlp* m, int64_t* n);
int fvs_mlp_get_params(fvs_mlp* m, float* dst, int64_t n);
int fvs_mlp_set_params(fvs_mlp* m, const float* src, int64_t n);
/* loss and gradients of one batch x[n][n_in], y[n][n_out], no update */
int fvs_mlp_loss_grad(fvs_mlp* m, const float* x, const float* y, int32_t n, float* loss, float* grads);
int fvs_mlp_train(fvs_mlp* m, const float* x, const float* y, int64_t n, int32_t batch, int32_t epochs, float lr,
                  uint64_t seed, float* loss_per_epoch);
int fvs_mlp_predict(fvs_mlp* m, const float* x, int64_t n, float* y);

/* ---- allocation-free residual norm ---------------------------------------
 * No counterpart in the reference: an addition for callers that cannot
 * allocate device memory where they need the norm (hosts whose device memory
 * is reserved up front by another allocator, loops that must not pay
 * cudaMalloc's implicit synchronisation).  Computes what fvs_time_integration
 * logs per step, RMS over cells of |U - U0| per component, from two device
 * arrays [ncells][4] into dev_norm4[4], on `stream` (a cudaStream_t; NULL =
 * the legacy default stream).  Allocates nothing: its block partial sums live
 * in a fixed device array of FVS_NOALLOC_MAX_BLOCKS x 4 doubles (256 KB per
 * GPU that loads the library, held until exit), so ncells is limited to
 * FVS_NOALLOC_MAX_CELLS; larger inputs return FVS_ERR_INVALID.  Every call on
 * a device shares that array: calls that overlap on the GPU race.  The first
 * call on a device (with that device current) looks up the array's address
 * and keeps it for the life of the process; make it before any stream
 * capture.  A cudaDeviceReset after that first call is not supported: the
 * kept address would then point into the destroyed context.  The call is
 * asynchronous on `stream`. */
#define FVS_NOALLOC_MAX_BLOCKS 8192
#define FVS_NOALLOC_MAX_CELLS (FVS_NOALLOC_MAX_BLOCKS * 256)
int fvs_rms_delta_noalloc(const double* dev_u, const double* dev_u0, int32_t ncells, double* dev_norm4, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FVS2D_H */
