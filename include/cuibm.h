/*
 * cuibm.h - C ABI of the GB300-native fractional-step solver (libcuibm_gb300.so).
 *
 * This is the drop-in boundary for cuIBM's solver classes.  A case folder holds
 * the same four files the reference reads (simParams.yaml, flow.yaml,
 * domain.yaml, bodies.yaml) and the same command-line overrides apply.  One
 * context = one simulation on one GPU and one CUDA stream; a context is not
 * thread-safe, several contexts may coexist.  No entry point exits or aborts:
 * each returns a cuibm_status and cuibm_last_error() gives the message.
 *
 * Reference interfaces replaced (paths inside the cuIBM source tree):
 *   cuibm_create      src/io/io.cu:108-138 readInputs (+ defaults io.cu:145-197,
 *                     command line io.cu:207-299) and the solver switch src/cuIBM.cu:42-60
 *   cuibm_initialise  NavierStokesSolver::initialise (NavierStokesSolver.cu:34-40),
 *                     luo_base::initialise (luo_base.cu:28-107), luoIBM::initialise (luoIBM.cu:27-52)
 *   cuibm_step        NavierStokesSolver::stepTime (NavierStokesSolver.cu:163-188),
 *                     luo_base::stepTime (luo_base.cu:208-233)
 *   cuibm_finished    NavierStokesSolver::finished (NavierStokesSolver.cu:195-199)
 *   cuibm_write_data  NavierStokesSolver::writeData/writeCommon (NavierStokesSolver.cu:339-363),
 *                     luoIBM::writeData (luoIBM.cu:69-80), luo_base::writeCommon (luo_base.cu:180-206)
 *   cuibm_shutdown    NavierStokesSolver::shutDown (NavierStokesSolver.cu:368-372)
 *   cuibm_get_field   the protected members u, uhat, pressure, ... (NavierStokesSolver.h:28-123,
 *                     luo_base.h tag and interpolation arrays)
 *   cuibm_get_forces  bodies::forceX/forceY after luo_base::calculateForce (calculateForce.cu:21-74)
 *   cuibm_run         one phase or kernel group of the step (the reference's
 *                     generateRHS1/solveIntermediateVelocity/generateRHS2/... methods)
 */
#ifndef CUIBM_H
#define CUIBM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cuibm_ctx cuibm_ctx;

typedef enum {
    CUIBM_OK = 0,
    CUIBM_ERR_BAD_INPUT = 1,     /* malformed case file, bad argument or size */
    CUIBM_ERR_IO = 2,            /* a case or output file could not be opened */
    CUIBM_ERR_CUDA = 3,          /* a CUDA runtime call failed */
    CUIBM_ERR_NOT_CONVERGED = 4, /* a linear solve hit maxIterations (reference: std::exit(-1)) */
    CUIBM_ERR_NAN = 5,           /* a non-finite residual appeared in a solve */
    CUIBM_ERR_STATE = 6,         /* call out of order (e.g. step before initialise) */
    CUIBM_ERR_UNSUPPORTED = 7    /* a configuration the library does not implement */
} cuibm_status;

/* solver types, same order and names as the reference's src/types.h */
enum { CUIBM_NAVIER_STOKES = 0, CUIBM_FADLUN = 1, CUIBM_OSC_CYLINDER = 2, CUIBM_FSI = 3, CUIBM_LUO = 4 };

typedef struct {
    int nx, ny, numU, numV, numUV, numP;
    int solver_type;
    int time_step, nt, nsave;
    double dt, nu;
    int total_points;                 /* body points (0 without a body) */
    int bb_start_i, bb_start_j, bb_ncx, bb_ncy; /* scaled bounding box of body 0 */
    int nnz_lhs1, nnz_lhs2;           /* entries of the reference's COO matrices */
    int velocity_precond, poisson_precond;   /* 0 NONE 1 DIAGONAL 2 SMOOTHED_AGGREGATION 3 AINV */
    int velocity_krylov, poisson_krylov;     /* 0 BiCGSTAB, 1 CG */
    int amg_levels;                   /* levels of the Poisson SA hierarchy (0 if none) */
    int velocity_precision, poisson_precision; /* 0 FP64, 1 MIXED (simParams.yaml `precision`) */
    int sa_rebuilds;                  /* SA hierarchies rebuilt for a moving embedded body so far */
    int sa_structured;                /* 1: the Poisson SA hierarchy is the structured one (3 x 3
                                         aggregates of the pressure grid, 9-point coarse operators,
                                         set up on the device; -saStructured 0 turns it off) */
} cuibm_info;

/* Fields readable/writable through cuibm_get_field / cuibm_set_field.
 * D = double, I = int32.  Sizes: UV = numUV, P = numP. */
enum {
    CUIBM_F_U = 0,        /* D UV  velocity u^{n+1} (u block then v block) */
    CUIBM_F_UHAT,         /* D UV  intermediate velocity */
    CUIBM_F_UOLD,         /* D UV  previous velocity */
    CUIBM_F_P,            /* D P   pressure */
    CUIBM_F_P_OLD,        /* D P   previous pressure */
    CUIBM_F_N,            /* D UV  convection term of the current step */
    CUIBM_F_NOLD,         /* D UV  convection term of the previous step */
    CUIBM_F_L,            /* D UV  explicit diffusion term (written by CUIBM_OP_RHS1_TERMS) */
    CUIBM_F_BC1,          /* D UV  implicit-diffusion boundary term (CUIBM_OP_RHS1_TERMS) */
    CUIBM_F_RHS1,         /* D UV  */
    CUIBM_F_RHS2,         /* D P   */
    CUIBM_F_BC_XMINUS,    /* D 2ny-1 */
    CUIBM_F_BC_XPLUS,     /* D 2ny-1 */
    CUIBM_F_BC_YMINUS,    /* D 2nx-1 */
    CUIBM_F_BC_YPLUS,     /* D 2nx-1 */
    CUIBM_F_X, CUIBM_F_DX, CUIBM_F_XU, CUIBM_F_XV,   /* D nx, nx, nx-1, nx */
    CUIBM_F_Y, CUIBM_F_DY, CUIBM_F_YU, CUIBM_F_YV,   /* D ny, ny, ny, ny-1 */
    CUIBM_F_BODY_X, CUIBM_F_BODY_Y,                  /* D total_points */
    CUIBM_F_BODY_UB, CUIBM_F_BODY_VB,                /* D total_points */
    CUIBM_F_GHOST_TAGS_UV,  /* I UV */
    CUIBM_F_HYBRID_TAGS_UV, /* I UV */
    CUIBM_F_HYBRID_TAGS_UV2,/* I UV */
    CUIBM_F_GHOST_TAGS_P,   /* I P  */
    CUIBM_F_HYBRID_TAGS_P,  /* I P  */
    CUIBM_F_BI_X, CUIBM_F_BI_Y, CUIBM_F_IP_X, CUIBM_F_IP_Y,      /* D UV body intercept / image point */
    CUIBM_F_BIP_X, CUIBM_F_BIP_Y, CUIBM_F_IPP_X, CUIBM_F_IPP_Y,  /* D P  same for pressure nodes */
    CUIBM_F_DIST_NODE, CUIBM_F_DIST_BETWEEN, CUIBM_F_UV_BODY,    /* D UV Fadlun distances, body velocity */
    CUIBM_F_USTAR,          /* D UV hybrid-node interpolated velocity */
    CUIBM_F_PSTAR,          /* D P  hybrid-node interpolated pressure */
    CUIBM_F_DPDN,           /* D P  ghost-node pressure normal-derivative term */
    CUIBM_F_BI_P,           /* D P  pressure at the body intercept (ghost nodes) */
    /* interpolation stencils: 4 corner indices (I, 4 per node) and 4 weights (D, 4 per node),
     * stored per node class; index = node index, entries [4*node .. 4*node+3] */
    CUIBM_F_GHOST_UV_INDEX,  CUIBM_F_GHOST_UV_COEF,   /* size 4*UV */
    CUIBM_F_HYBRID_UV_INDEX, CUIBM_F_HYBRID_UV_COEF,  /* size 4*UV */
    CUIBM_F_GHOST_P_INDEX,   CUIBM_F_GHOST_P_COEF,    /* size 4*P  */
    CUIBM_F_HYBRID_P_INDEX,  CUIBM_F_HYBRID_P_COEF,   /* size 4*P  */
    CUIBM_F_IMAGE_VALUE_UV,  /* D UV value interpolated at the image point */
    CUIBM_F_CFL,             /* D P  */
    CUIBM_F_WORK_X,          /* D max(UV,P) operator test input  */
    CUIBM_F_WORK_Y,          /* D max(UV,P) operator test output */
    CUIBM_F_SOLVE_TRACE,     /* uint64 2*4096: per-barrier timestamps (ns) of the last persistent
                                velocity (first 4096) and Poisson solve: [count, start, ...], each
                                entry the timer's low 48 bits with the barrier's source line of
                                fused_kernels.cuh in the top 16; written only while the option
                                "trace_solve" is 1 */
    CUIBM_F_BODY_MOTION,     /* D 12: body centre x, y and centre velocity u, v; the same at the
                                start of the step; the coupling tolerance and the sub-iterations
                                of the last strongly coupled step (VIV: 2); 4 spare */
    CUIBM_F_SURFACE_FORCE,   /* D 3*total_points+2: pressure, du/dn, dv/dn per body point, then Fx, Fy
                                (written by CUIBM_OP_SURFACE_FORCE*, or each step with the option
                                "force_method" 1 or 2) */
    CUIBM_F_FORCES,          /* D 2: Fx, Fy of the last step (what cuibm_get_forces reads) */
    CUIBM_F_BODY_VELOCITY_OFFSET, /* D 2*total_points: per-point offsets of the prescribed body velocity
                                (u of each point, then v), zero by default; writing them (after
                                cuibm_initialise) sets uB = unew + offset_u and vB = offset_v at once
                                and at every later motion update (prescribed motion only).  No
                                counterpart in the reference, whose motion sets every point's velocity
                                alike (luo_base/move.cu:11-36); it is the perturbation behind the
                                per-point gradients of cuibm_adjoint */
    CUIBM_F_COUNT
};

/* Phases and kernel groups for cuibm_run (state in, state out). */
enum {
    CUIBM_OP_RHS1_TERMS = 0,   /* N, L, bc1, rhs1 from u and Nold (writes all four) */
    CUIBM_OP_GENERATE_RHS1,    /* the method's full generateRHS1 (IB interpolation included) */
    CUIBM_OP_SOLVE_VELOCITY,   /* LHS1 uhat = rhs1 */
    CUIBM_OP_WEIGHT_UHAT,      /* external method: blend uhat with ustar at hybrid nodes */
    CUIBM_OP_GENERATE_RHS2,    /* the method's full generateRHS2 */
    CUIBM_OP_RHS2,             /* rhs2 = -D uhat only */
    CUIBM_OP_SOLVE_POISSON,    /* LHS2 p = rhs2 */
    CUIBM_OP_WEIGHT_PRESSURE,  /* external method: hybrid/ghost pressure interpolation and blend */
    CUIBM_OP_PROJECT,          /* u = uhat - dt G p, uold = u (plain projection only) */
    CUIBM_OP_PROJECT_VELOCITY, /* the method's full projection phase */
    CUIBM_OP_UPDATE_BODY,      /* force, motion, bounding box, tagging, CFL */
    CUIBM_OP_APPLY_LHS1,       /* WORK_Y = LHS1 WORK_X */
    CUIBM_OP_APPLY_LHS2,       /* WORK_Y = LHS2 WORK_X */
    CUIBM_OP_TAG_POINTS,       /* tagging of u, v, p nodes */
    CUIBM_OP_GHOST_VELOCITY_U, /* interpolate u to ghost nodes and set them (set=true) */
    CUIBM_OP_GHOST_VELOCITY_UHAT, /* same on uhat */
    CUIBM_OP_HYBRID_VELOCITY,  /* ustar at hybrid nodes from u */
    CUIBM_OP_HYBRID_PRESSURE,  /* pstar at hybrid pressure nodes */
    CUIBM_OP_GHOST_PRESSURE,   /* ghost pressure values (set=true) */
    CUIBM_OP_SET_INSIDE,       /* u inside the body := body velocity */
    CUIBM_OP_ROBIN_BOUNDARY,   /* convective outflow update of the x+ boundary */
    CUIBM_OP_FORCE,            /* control-volume force on body 0 */
    CUIBM_OP_CFL,              /* CFL field */
    CUIBM_OP_SURFACE_FORCE,    /* surface-integral force on body 0 (luo_base::luoForce, unused by the
                                  reference's step) into CUIBM_F_SURFACE_FORCE, as the reference wrote it */
    CUIBM_OP_SURFACE_FORCE_CORRECTED, /* the same with its two index slips corrected */
    CUIBM_OP_APPLY_LHS1_T,     /* WORK_Y = LHS1^T WORK_X (embedded method: the adjoint's operator) */
    CUIBM_OP_APPLY_LHS2_T,     /* WORK_Y = LHS2^T WORK_X */
    CUIBM_OP_PRECONDITION_POISSON, /* WORK_Y = M WORK_X: one V-cycle of the Poisson system's
                                      smoothed-aggregation preconditioner (stepwise kernels) */
    CUIBM_OP_COUNT
};

int cuibm_create(const char *case_folder, int argc, const char **argv, cuibm_ctx **out);
int cuibm_initialise(cuibm_ctx *ctx);
int cuibm_step(cuibm_ctx *ctx, int nsteps);
int cuibm_finished(const cuibm_ctx *ctx);
int cuibm_write_data(cuibm_ctx *ctx);
int cuibm_shutdown(cuibm_ctx *ctx);
void cuibm_destroy(cuibm_ctx *ctx);
const char *cuibm_last_error(const cuibm_ctx *ctx);

int cuibm_get_info(const cuibm_ctx *ctx, cuibm_info *info);
/* copy a field; bytes must equal the field size.  Flags (*_on_device): bit 0 set
 * means the caller's pointer is device memory of the context's GPU; bit 1 set
 * (CUIBM_COPY_ASYNC) enqueues the copy on the context's stream after the work
 * already there and returns without waiting (host memory should then be pinned and
 * must stay valid until the stream has passed the copy) */
#define CUIBM_COPY_ASYNC 2
int cuibm_get_field(cuibm_ctx *ctx, int field, void *dst, size_t bytes, int dst_on_device);
int cuibm_set_field(cuibm_ctx *ctx, int field, const void *src, size_t bytes, int src_on_device);
int cuibm_get_forces(cuibm_ctx *ctx, double *fx, double *fy);
int cuibm_get_iterations(cuibm_ctx *ctx, int *velocity_iterations, int *poisson_iterations);
/* The reference's COO matrix for system 1 (LHS1) or 2 (LHS2), entries in the
 * reference's order; arrays of length info.nnz_lhs1 / nnz_lhs2. */
int cuibm_get_matrix(cuibm_ctx *ctx, int system, int *row, int *col, double *val, size_t nnz);
int cuibm_run(cuibm_ctx *ctx, int op);
/* the context's cudaStream_t, for callers that order their own work after it */
int cuibm_get_stream(cuibm_ctx *ctx, void **stream);
/* accumulated device time (ms) and count of a named phase; names as the
 * reference Logger: "Intermediate Velocity Setup", "Intermediate Velocity Solve",
 * "Poisson Setup", "Poisson Solve", "Velocity Projection", "Update Solver", ... */
int cuibm_get_timer(cuibm_ctx *ctx, const char *name, double *ms, int *count);
/* Options (no counterpart in the reference): "use_graph" (1: a step is one CUDA
 * graph launch), "fused_solve" (1: each linear solve is one persistent
 * cooperative launch; 0: a launch per Krylov/multigrid phase), "profile_phases"
 * (1: time each phase with events, steps run without the graph), "step_sync"
 * (1: cuibm_step waits and checks the solves' status; 0: it only enqueues the
 * steps on the context's stream and a later cuibm_step(ctx, 0) checks),
 * "trace_solve" (1: record per-barrier timestamps in CUIBM_F_SOLVE_TRACE),
 * "write_output" (0: no files), "sa_rebuild_interval" (a moving body with the
 * embedded method: the SA hierarchy is rebuilt from the current rows when the set of
 * patched rows changed and at least this many steps passed since the last rebuild;
 * default 1, as the reference rebuilds every step; <= 0 never), "solver_blocks"
 * (blocks of the persistent solves,
 * 0: one per SM; as -solverBlocks, changeable after cuibm_initialise),
 * "force_method" (the step's body force, which the
 * forces file, cuibm_get_forces and the flow-induced motion use: 0 the control
 * volume of luo_base::calculateForce, as the reference; 1 the surface integral of
 * luo_base::luoForce as the reference wrote it; 2 that integral corrected). */
int cuibm_set_option(cuibm_ctx *ctx, const char *key, double value);

/* Time one kernel of the step on the context's stream with CUDA events: reps
 * back-to-back launches on the current state; *avg_ms is the mean launch time
 * and *bytes the kernel's algorithmic DRAM bytes per launch (unique inputs read
 * plus outputs written).  Names: "rhs1", "rhs2", "project", "apply_lhs1",
 * "apply_lhs2", "poisson_vcycle", "poisson_solve", "velocity_solve", and "fp64_fma" (a
 * throughput probe of the GPU's FP64 fused multiply-add issue: *bytes then gets the
 * FLOPs of one launch). */
int cuibm_profile_kernel(cuibm_ctx *ctx, const char *kernel, int reps, double *avg_ms, double *bytes);

/* Kernels of this library launched by the last time step: the kernel nodes of
 * the step graph plus those of each solver's iteration body times the number
 * of iterations it ran. */
int cuibm_launch_count(cuibm_ctx *ctx, long long *per_step);

/* Control-volume force on the body (drag, lift) from caller-owned device arrays,
 * for callers that must not allocate GPU memory: a coupling code or host
 * framework whose own pool has reserved the device memory (a cudaMalloc there
 * fails or fragments the pool), and a time-stepping loop that cannot take the
 * device-wide synchronisation that cudaMalloc/cudaFree imply.  This entry
 * point calls no cudaMalloc, cudaFree or allocating library routine: the
 * kernel's scratch (its per-block partial sums and arrival counter) is a fixed
 * array compiled into the library, which every GPU that loads the library
 * holds until the process exits.  It has no counterpart in the reference.
 *
 * Inputs (device pointers of the current device): u and uold (numUV doubles,
 * velocity at the new and previous step), p (numP), ghost_tags_uv (numUV ints,
 * -1 marks fluid nodes), dx (nx), dy (ny); the box (bb_i, bb_j, bb_ncx, bb_ncy)
 * in cell indices, which must be the box of the current step (a moving body's
 * box moves every step; a stale box gives a wrong force, not an error); nu and
 * dt.  Output: force_out[0..1] = (Fx, Fy), device memory.  Limits:
 * (bb_ncx+1)*(bb_ncy+1) <= 262144 box nodes (a 511 x 511 box), bb_i, bb_j >= 1,
 * bb_i + bb_ncx <= nx - 2 and bb_j + bb_ncy <= ny - 2 (the box's east and north
 * edges read one more u column and v row); other boxes are rejected with
 * CUIBM_ERR_BAD_INPUT.  The first call on a
 * device looks up the scratch address with cudaGetSymbolAddress; make it
 * before any stream capture.  Every call shares the one scratch array, so
 * calls that overlap on the GPU (different streams, or different host
 * threads) race: order them on one stream.  Error text: cuibm_case_error(),
 * which returns the calling host thread's last message. */
int cuibm_cv_force_noalloc(const double *u, const double *uold, const double *p, const int *ghost_tags_uv,
                           const double *dx, const double *dy, int nx, int ny, int bb_i, int bb_j, int bb_ncx,
                           int bb_ncy, double nu, double dt, double *force_out, void *stream);

/* ---- discrete adjoint ---------------------------------------------------------
 * Gradients of J = sum_{n=1..nsteps} wx[n-1] Fx^n + wy[n-1] Fy^n, the control-volume
 * force of each step (period-averaged drag coefficient: wx = 2 / nsteps, wy = 0), for the
 * embedded method (SolverType OSC_CYLINDER) with a prescribed body motion (VIV: 0) and
 * the control-volume force (force_method 0).  No counterpart in the reference, whose
 * step (luo_base::stepTime, luo_base.cu:208-233 with luo_iter's phases) it differentiates.
 * Runs steps 1..nsteps from the initial condition (call it right after cuibm_initialise)
 * and the reverse sweep: transposed stencils, transposed ghost-node interpolation with
 * the tags of the forward step, transposed solves (the Poisson one preconditioned by the
 * transposed cycle of the forward smoothed-aggregation hierarchy), binomial
 * checkpointing over `snapshots` stored states (each holds u, uhat, N, p, the x+ boundary
 * and the body state).  On return the context is back at its initial state.  grad
 * (ngrad = 2 + 2 * total_points):
 *   grad[0]                     dJ / d nu
 *   grad[1]                     dJ / d uCoefficient (the prescribed velocity amplitude of
 *                               bodies.yaml; the prescribed path xCoefficient held fixed)
 *   grad[2 + k], grad[2 + np + k]  dJ / d (u, v offset of point k's velocity,
 *                               CUIBM_F_BODY_VELOCITY_OFFSET); zero for k > 0 because the
 *                               reference's kernels read point 0's velocity only
 * *J (may be null) gets J.  The transposed solves stop at the relative residual of the
 * option "adjoint_tolerance" (default 1e-10).  stats (may be null): device time of the
 * whole call, forward steps recomputed from snapshots, steps taped, the transposed
 * solves' iterations, and the taped steps whose two solves were taken from a snapshot of
 * the step's end (with snapshots to spare, a taped step solves nothing).  The transposed stencils accumulate with atomic adds: results
 * agree from run to run to rounding, not bit for bit. */
typedef struct {
    double ms;
    long long forward_steps, tape_steps, velocity_iterations, poisson_iterations, solves_reused;
} cuibm_adjoint_stats;
int cuibm_adjoint(cuibm_ctx *ctx, int nsteps, int snapshots, const double *wx, const double *wy, double *J,
                  double *grad, size_t ngrad, cuibm_adjoint_stats *stats);

/* ---- batched instances ------------------------------------------------------
 * Many independent cases advanced together on one GPU.  No counterpart in the
 * reference, which runs one case per process (src/cuIBM.cu:61-74).  Each instance
 * is a full context (cuibm_batch_instance gives its handle for fields, forces and
 * output) with its own stream; its persistent solves use solver_blocks blocks
 * (<= 0: a quarter of the SMs; the solves are built for two blocks per SM,
 * -solverPack 2), so that several instances' solves run at once
 * while each instance's step stays one graph.  argc/argv are the command-line
 * overrides every instance gets (cuibm_create).  cuibm_batch_step enqueues nsteps
 * steps of every instance, interleaved step by step, then waits for all and
 * checks their solves; the first failure is reported with its instance index.
 * Error text: cuibm_batch_error(). */
typedef struct cuibm_batch cuibm_batch;
int cuibm_batch_create(int n, const char *const *case_folders, int argc, const char **argv, int solver_blocks,
                       cuibm_batch **out);
int cuibm_batch_initialise(cuibm_batch *b);
int cuibm_batch_step(cuibm_batch *b, int nsteps);
/* Autotuner of the batch's persistent-solve grid: times `steps` batch steps with each
 * candidate - one block count for every instance (a quarter, sixth or eighth of the
 * SMs) or a count per instance from its pressure unknowns at 6, 8, 12, 16 or 24 rows a
 * thread (at least 2 blocks, at most half the SMs) - in two passes of opposite order,
 * and keeps the fastest (option "solver_blocks" of every instance).  The timed steps
 * are steps of the simulation (each instance advances 16 x steps).
 * *blocks_out (may be null) gets the choice: the block count, or minus the rows a
 * thread of a per-instance choice. */
int cuibm_batch_autotune(cuibm_batch *b, int steps, int *blocks_out);
int cuibm_batch_size(const cuibm_batch *b);
cuibm_ctx *cuibm_batch_instance(cuibm_batch *b, int k);
const char *cuibm_batch_error(const cuibm_batch *b);
void cuibm_batch_destroy(cuibm_batch *b);

/* Host-only (no GPU needed): parse a case folder and build its grid and body
 * exactly as cuibm_create does.  cuibm_case_array copies CUIBM_F_X..CUIBM_F_YV
 * or CUIBM_F_BODY_X/Y into dst (count doubles).  Replaces the reference's
 * io::readInputs + io::parseDomainFile/parseBodiesFile (src/io/io.cu:108-138). */
int cuibm_case_info(const char *case_folder, int argc, const char **argv, cuibm_info *info);
int cuibm_case_array(const char *case_folder, int argc, const char **argv, int field, double *dst, size_t count);
/* the calling host thread's last error of a context-free entry point */
const char *cuibm_case_error(void);

#ifdef __cplusplus
}
#endif
#endif /* CUIBM_H */
