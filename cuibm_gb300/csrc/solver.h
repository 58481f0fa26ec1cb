// Device context of one simulation and the declarations shared by the
// translation units of libcuibm_gb300.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "config.h"
#include "geometry.h"

namespace cuibm {

#define CUIBM_TRY(expr)                                                                         \
    do {                                                                                        \
        cudaError_t e_ = (expr);                                                                \
        if (e_ != cudaSuccess) throw CudaError(std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

struct CudaError {
    std::string msg;
    explicit CudaError(const std::string &m) : msg(m) {}
};
struct InputError {
    std::string msg;
    explicit InputError(const std::string &m) : msg(m) {}
};

constexpr int kBlock = 256;
constexpr int kTraceLen = 4096;  // timestamps kept per persistent solve (diagnostic trace)
inline int blocks_for(long n, int bs = kBlock) { return (int)((n + bs - 1) / bs); }

// ---- structured operators --------------------------------------------------
// 1-D coefficient tables of the separable 5-point operators.  Index ranges are
// noted per array; every value is computed on the host with the reference's
// formula and operation order.
// Rows that replace the structured stencil (the modified Fadlun method's rows at
// tagged nodes): row i with pid[i] = k >= 0 is pdiag[k] x_i + sum_m pval[5k+m] x_pcol[5k+m]
// over the entries with pcol >= 0.  pid is null for the other methods.
struct RowPatch {
    const int *pid, *pcol;
    const double *pval, *pdiag;
};
struct Lhs1Coef {
    // u rows: E/W depend on I (0..nx-2), N/S on J (0..ny-1, boundary spacing folded in)
    const double *uE, *uW, *uN, *uS;
    // v rows: E/W on I (0..nx-1), N/S on J (0..ny-2)
    const double *vE, *vW, *vN, *vS;
    RowPatch patch;
    // embedded method: rows without a patch are scaled by rscale[i] (1 / diagonal on the
    // interior rows, 1 on the boundary rows); null for the other methods
    const double *rscale;
};
// The patched rows holding each column (discrete adjoint): column i appears in
// min(cnt[i], tmax) entries ent[i * tmax + t] of the RowPatch arrays (entry e is slot
// e / 5, position e % 5), slot k being the row prow[k].  cnt is null where no row is
// patched.
struct TransposeList {
    const int *cnt, *ent, *prow;
    int tmax;
};
struct Lhs2Coef {
    const double *E, *W;  // on I (0..nx-1), zero where the neighbour is missing
    const double *N, *S;  // on J (0..ny-1)
    int pin0, pinc;       // doubled diagonals: cell 0 and (if >= 0) the centre cell
    RowPatch patch;
};
struct Grid {
    int nx, ny, nU, nV, nUV, nP;
};

// explicit-term metric tables for the fused RHS kernel (convection/diffusion)
struct RhsCoef {
    // u nodes, per I (0..nx-2)
    const double *uxE, *uxW, *uxC, *uxA;   // convection x-part, v-bar weight a/(a+b)
    const double *ulE, *ulW;               // diffusion 1/(dx[I+1](dx[I+1]+dx[I])/2), 1/(dx[I](..)/2)
    // u nodes, per J (0..ny-1), boundary spacing folded in
    const double *uyN, *uyS, *uyC;
    const double *ulN, *ulS;               // diffusion (2/dy^2 at the top/bottom walls)
    // v nodes, per I (0..nx-1)
    const double *vxE, *vxW, *vxC;
    const double *vlE, *vlW;
    // v nodes, per J (0..ny-2)
    const double *vyN, *vyS, *vyC, *vyA;   // v-bar weight c/(c+d) for u at v nodes
    const double *vlN, *vlS;
    const double *dx, *dy;
    // folded forms for fewer FP64 operations (the kernel is FP64-issue bound):
    // v-bar = uhA (vne + vse) + uhB (vn + vs) with uhA = a/2, uhB = (1 - a)/2 (u nodes, per I);
    // u-bar likewise with vhA, vhB (v nodes, per J); 1/dx, 1/dy for the divergence
    const double *uhA, *uhB;
    const double *vhA, *vhB;
    const double *rdx, *rdy;
};

// ---- Krylov state living in device memory -------------------------------------
// the step's error word: solver * 16 + KStatus, or this (a moving body left its tagging box)
constexpr int kErrBodyOutsideTagBox = 0x100;
// ... or this (the strongly coupled sub-iterations of a step reached kCouplingMaxIterations)
constexpr int kErrCouplingNotConverged = 0x200;
constexpr int kCouplingMaxIterations = 50;
constexpr int kMotionLen = 12;  // doubles of IbArrays::motion
enum KStatus { KS_RUNNING = 0, KS_CONVERGED = 1, KS_MAXIT = 2, KS_NAN = 3, KS_TIMEOUT = 4,
               KS_STALLED = 5 };  // KS_STALLED: an FP32 inner solve stopped at a breakdown (refinement goes on)
struct KrylovScalars {
    double rho, alpha, omega, beta;
    double bnorm, tol, rnorm, snorm;
    double rtol, inner_rtol;  // inner_rtol: mixed precision, the FP32 solves' relative tolerance floor
    int it, maxit, status, s_done;
    int body_runs, inner_maxit;  // executions of the iteration body in the last solve; mixed
                                 // precision: iterations of one FP32 solve at most
    unsigned int arrive;  // last-block-done counter of the fused reductions
    int pad;
};

// grid-barrier state of the persistent solver (fused_solve.cu), zeroed before each launch
struct FusedSyncState {
    unsigned long long arrivals;
    int abort;  // set by a block whose barrier wait timed out
    int pad;
};

struct SaLevel;  // amg.cu

struct LinearSystem {
    int which = 1;  // 1 = LHS1 (velocity), 2 = LHS2 (Poisson)
    int n = 0;
    int krylov = 0, precond = 0;
    double rtol = 1e-5;
    int maxit = 1000;
    // workspaces
    double *r = nullptr, *rs = nullptr, *p = nullptr, *Mp = nullptr, *AMp = nullptr, *s = nullptr, *Ms = nullptr,
           *AMs = nullptr, *z = nullptr, *q = nullptr;
    double *dinv = nullptr;      // Jacobi of the (possibly symmetrised) operator
    double *w = nullptr;         // CG symmetrisation weights (row scaling), n
    double *partials = nullptr;  // per-block partial sums, 4 per block
    KrylovScalars *ks = nullptr; // device
    std::vector<SaLevel *> amg;  // SA hierarchy (Poisson)
    int last_iterations = 0;
    int body_kernels = 0;  // kernel nodes in one captured iteration body
    // persistent solver (fused_solve.cu); fused_fn is null where it does not apply
    void *fused_fn = nullptr;
    int fused_grid = 0, fused_threads = 512;
    int fused_grid_default = 0, fused_grid_max = 0;  // one block per SM; every block the SMs hold
    double *p2 = nullptr, *AMp2 = nullptr, *fpartials = nullptr;
    double *diag = nullptr, *winv = nullptr;  // operator diagonal, 1 / w (CG)
    int precision = PRECISION_FP64;
    double strength = 0.0;  // smoothed aggregation's strength threshold
    // the SA hierarchy built from the operator without the body's patched rows (a moving
    // embedded body's option "sa_body_free"): it never needs rebuilding as the body moves
    bool sa_body_free = false;
    // the hierarchy is the structured one (3 x 3 aggregates of the pressure grid, 9-point
    // coarse operators, set up on the device; structured.cuh)
    bool sa_structured = false;
    // the SA hierarchy in its own allocations (so that it can be rebuilt) and the
    // checksum of the patched-row pattern it was built from
    bool sa_dynamic = false;
    std::vector<void *> sa_blocks;
    unsigned long long sa_key = 0;
    void *mixed = nullptr;  // mixed precision: the float tables (fused_solve.cu)
    double *aedef = nullptr;                // A e (the operator's row sums), with wdef
    double *ym = nullptr, *wdef = nullptr;  // constant-mode correction of the SA cycle (Poisson):
    double Edef = 0;                        // cycle output, A^T e, e^T A e
    FusedSyncState *fsync = nullptr;
    void *fargs = nullptr;  // device copy of the solver arguments
};

struct Timer {
    double ms = 0;
    int count = 0;
};

struct IbArrays {
    int *ghostUV, *hybridUV, *hybrid2UV, *ghostP, *hybridP;
    double *biX, *biY, *ipX, *ipY;        // numUV
    double *bipX, *bipY, *ippX, *ippY;    // numP
    double *distNode, *distBetween, *distU, *distV, *uvBody;  // Fadlun distances (numUV / numP)
    double *ustar, *pstar, *dpdn, *biP, *imageValue;
    int *gIdx, *hIdx, *gpIdx, *hpIdx;     // 4 per node
    double *gCoef, *hCoef, *gpCoef, *hpCoef;
    double *gnValue;                      // staging of ghost values (snapshot semantics)
    // tagging work records
    void *tagRec;
    // body (device)
    double *bx, *by, *uB, *vB, *uBk, *vBk, *bdx, *bdy;
    // force partial sums
    double *forcePart;
    double *forceOut;  // [fx, fy]
    double *surf;      // surface force: pressure, du/dn, dv/dn per body point, then Fx, Fy
    double *velOff;    // 2 * total: per-point offsets of the prescribed body velocity (u, then v)
    double *motion;    // kMotionLen: [midX, midY, centerVelocityU, centerVelocityV, midX0, midY0,
                       //  U0, V0, SCtol, sub-iterations done, continue flag, spare]
};

struct Context {
    Params P;
    Axis gx, gy;
    BodyState body;
    BoundingBox bb;      // control-volume box of the initial body (the force's box until the body moves)
    BoundingBox bb_tag;  // the box the tagging and interpolation scan: bb, or for a moving body a box
                         // holding every position of its prescribed motion
    Grid g{};
    int device = 0;
    cudaStream_t stream = nullptr, side_stream = nullptr;
    cudaStream_t coupling_stream = nullptr;  // captures the body of a strongly coupled step's loop
    int *err_word = nullptr;          // device: first failing solve, system*16 + status
    int *step_counter_dev = nullptr;  // device copy of timeStep (read by the body motion)
    std::vector<double> htab;         // host copy of the metric tables (see upload_ns_tables)
    std::map<std::string, size_t> hoff;
    std::string err;
    bool created = false, initialised = false;
    int timeStep = 0;

    // device memory: one arena carved into 256-byte aligned slices
    char *arena = nullptr;
    size_t arena_bytes = 0, arena_used = 0;

    double *u, *uhat, *uold, *N, *Nold, *L, *bc1, *rhs1;
    double *p, *p_old, *rhs2, *cfl, *work_x, *work_y;
    double *bc[4];
    double *x, *dx, *xu, *xv, *y, *dy, *yu, *yv;
    RhsCoef rc{};
    Lhs1Coef l1{};
    Lhs2Coef l2{};
    double *gradU, *gradV;  // projection: dt / (0.5 dx[I+1] + 0.5 dx[I]), dt / (0.5 dy[J+1] + 0.5 dy[J])
    LinearSystem sys1, sys2;
    IbArrays ib{};
    bool has_body = false;
    bool ib_dirty = false;
    int ib_slot = -1;                   // host-side IB bookkeeping of this context
    double ib_midX = 0, ib_midY = 0;    // body centre used by the tagging
    int force_method = 0;  // the step's force: 0 control volume, 1/2 surface integral (mode)
    // moving body with the embedded method and an SA preconditioner: the hierarchy is
    // rebuilt when the pattern of the patched rows changes (checksum below, per tagging)
    bool sa_rebuild = false;
    unsigned long long *rows_key_dev = nullptr;
    int sa_rebuilds = 0;
    int sa_rebuild_interval = 1;   // option "sa_rebuild_interval": fewest steps between rebuilds
    int sa_last_rebuild = 0;       // time step of the last one
    double cfl_max = 0;
    double forceX = 0, forceY = 0;

    // host mirrors read back once per step
    double *h_scalars = nullptr;  // pinned: [it1, it2, fx, fy, status1, status2]
    std::map<std::string, Timer> timers;
    bool profile_phases = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;

    // CUDA graph of one step
    bool use_graph = true;
    bool step_sync = true;    // cuibm_step waits for the steps and checks the solves' status;
                              // when false it only enqueues them (cuibm_step(ctx, 0) then checks)
    bool fused_solve = true;  // persistent one-launch solves where available
    bool trace_solve = false; // persistent solves record per-barrier timestamps
    unsigned long long *solve_trace = nullptr;  // device, 2 x kTraceLen
    cudaGraphExec_t step_exec = nullptr;
    cudaGraph_t step_graph = nullptr;
    int static_kernels = 0;  // kernel nodes of the step graph outside the solver loops

    // modified Fadlun: host copies of the patched rows (for the host matrices)
    struct FadlunRows {
        std::vector<int> pid1, pcol1, pid2, pcol2;
        std::vector<double> pval1, pdiag1, pval2, pdiag2;
        int nnz1 = 0, nnz2 = 0;  // entries of the matrices cuibm_get_matrix returns
    } fadlun;

    // embedded method (OSC_CYLINDER): the patched rows of the tagged nodes, rebuilt at
    // every tagging.  Velocity slots: ghost nodes [0, cap1), hybrid nodes [cap1, 2 cap1);
    // pressure slots: ghost [0, cap2), hybrid [cap2, 2 cap2)
    struct EmbeddedRows {
        int cap1 = 0, cap2 = 0;
        int *pid1 = nullptr, *pcol1 = nullptr, *pid2 = nullptr, *pcol2 = nullptr;
        double *pval1 = nullptr, *pdiag1 = nullptr, *pval2 = nullptr, *pdiag2 = nullptr;
        double *pns1 = nullptr, *pint1 = nullptr;  // rhs1 = rhs1 pns + pint (hybrid slots)
        int *gin = nullptr;                        // ghost slots: corners that are ghost nodes
        double *pns2 = nullptr, *pAu2 = nullptr, *pAv2 = nullptr;  // rhs2 = rhs2 pns + dudt pAu + dvdt pAv
        double *rscale1 = nullptr;                 // numUV
    } emb;

    // discrete adjoint (adjoint.cu): its buffers and snapshots, allocated by the first
    // cuibm_adjoint call; the relative tolerance of its transposed solves
    void *adj = nullptr;
    double adjoint_rtol = 1e-10;

    // output files
    FILE *iterationsFile = nullptr, *forceFile = nullptr, *midPositionFile = nullptr;

    template <class T>
    T *carve(size_t count)
    {
        size_t bytes = ((count * sizeof(T)) + 255) & ~size_t(255);
        if (arena_used + bytes > arena_bytes) throw CudaError("device arena exhausted");
        T *p_ = reinterpret_cast<T *>(arena + arena_used);
        arena_used += bytes;
        return p_;
    }
};

// ---- entry points between translation units ----------------------------------
// context.cu: the phases of a step's pass (record_pass runs them in this order), one
// whole step as cuibm_step runs it, and the step error word
void phase_generate_rhs1(Context &c, bool first);
void phase_solve_velocity(Context &c, bool in_graph);
void phase_generate_rhs2(Context &c);
void phase_solve_poisson(Context &c, bool in_graph);
void step_once(Context &c);
int read_step_error(Context &c);

// ns_kernels.cu
void upload_ns_tables(Context &c);
// body_free: every row as if no body patched it (the SA hierarchy of a moving body)
void host_matrix_coo(Context &c, int which, std::vector<int> &row, std::vector<int> &col, std::vector<double> &val,
                     bool body_free = false);
void host_operator_csr(Context &c, int which, const double *w, std::vector<int> &ptr, std::vector<int> &col,
                       std::vector<double> &val, bool body_free = false);
void launch_rhs1(Context &c, bool debug_terms, bool shift = true);  // shift: Nold = N first
void launch_rhs2(Context &c, const double *uh);
void launch_project(Context &c);
void launch_initial_velocity(Context &c);
void launch_apply(Context &c, int which, const double *xin, double *yout);
void launch_cfl(Context &c);
void launch_copy(Context &c, double *dst, const double *src, int n);
double launch_fp64_fma(Context &c, int blocks, double *out);  // FP64 issue peak probe; returns FLOPs

// krylov.cu
void setup_system(Context &c, LinearSystem &S);
void launch_solve(Context &c, LinearSystem &S, const double *b, double *x, bool in_graph);
int read_solve_status(Context &c, LinearSystem &S, int *iterations);
int read_body_runs(Context &c, LinearSystem &S);
int count_kernel_nodes(cudaGraph_t g);
void refresh_system_diagonals(Context &c, LinearSystem &S);  // after the operator's rows changed

// krylov.cu: the transposed systems of the discrete adjoint (adjoint.cu)
void setup_transposed_system(Context &c, const LinearSystem &F, LinearSystem &S, std::vector<void *> &allocs);
int launch_solve_transposed(Context &c, LinearSystem &S, LinearSystem &F, const TransposeList &T, const double *b,
                            double *x, int *iterations);
void launch_apply_transposed(Context &c, int which, const TransposeList &T, const double *x, double *y);

// fused_solve.cu
void setup_fused(Context &c, LinearSystem &S);
void launch_fused_solve(Context &c, LinearSystem &S, const double *b, double *x);
void set_fused_trace(Context &c, LinearSystem &S, bool on);
double solve_bytes(const LinearSystem &S, int iterations);        // algorithmic bytes
double solve_dense_bytes(const LinearSystem &S, int iterations);  // the coarsest dense inverse's
void refresh_fused_diag(Context &c, LinearSystem &S);
void refresh_fused_level0(Context &c, LinearSystem &S);
void free_fused(LinearSystem &S);

// fadlun.cu
void setup_fadlun(Context &c);
void launch_fadlun_rhs1(Context &c);
void launch_fadlun_rhs2(Context &c);
void launch_fadlun_project(Context &c);

// embedded.cu
void setup_embedded(Context &c);
void launch_embedded_rows(Context &c);  // after each tagging: the patched rows of the new tags
int embedded_hybrid_count(Context &c, int system);

// amg.cu
void build_sa_hierarchy(Context &c, LinearSystem &S);
void launch_vcycle(Context &c, LinearSystem &S, const double *r, double *z);
void free_sa_hierarchy(LinearSystem &S);
double sa_vcycle_bytes(const LinearSystem &S);
// the transposed cycle of the discrete adjoint (its level matrices made on first use)
void ensure_transposed_levels(Context &c, LinearSystem &S);
void launch_vcycle_transposed(Context &c, LinearSystem &S, const TransposeList &T, const double *r, double *z);
int sa_coarsest_size(const LinearSystem &S);

// ib_kernels.cu
void setup_ib(Context &c);
void launch_tag_points(Context &c);
void launch_ghost_velocity(Context &c, double *field, bool set);
void launch_hybrid_velocity(Context &c, const double *field);
void launch_set_inside(Context &c, double *field);
void launch_weight_uhat(Context &c);
void launch_hybrid_pressure(Context &c);
void launch_ghost_pressure(Context &c, bool set);
void launch_weight_pressure(Context &c);
void launch_robin(Context &c);
void launch_ib_rhs1(Context &c);             // Robin, ghost u, inside, hybrid u
void launch_ib_after_velocity(Context &c);   // weight uhat, ghost uhat
void launch_ib_after_poisson(Context &c);    // hybrid p, weight p, ghost p
void launch_ib_after_projection(Context &c); // ghost u, inside
void launch_ib_robin_inside(Context &c);     // Robin, inside (embedded rhs1)
void launch_force(Context &c);
// the surface-integral force (luo_base::luoForce); mode 1 as the reference wrote it,
// mode 2 with its two index corrections; to_step: also the step's force (forceOut)
void launch_surface_force(Context &c, int mode, bool to_step);
void launch_body_motion(Context &c, double t);
void launch_body_pre_step(Context &c);
void apply_velocity_offsets(Context &c);  // after CUIBM_F_BODY_VELOCITY_OFFSET was written
const int *force_box_dev(Context &c);     // the control-volume box [i0, j0, ncx, ncy] (device)
bool body_moves(Context &c);
void launch_body_box(Context &c);
void launch_step_counter(Context &c);
void launch_coupling_next(Context &c, cudaGraphConditionalHandle h, int use_cond);  // VIV: 2 loop test
// fused_solve.cu: the persistent solves' grid (blocks <= 0: the default); the step graph
// must be rebuilt after
void set_fused_grid(LinearSystem &S, int blocks);
void refresh_fused_hierarchy(Context &c, LinearSystem &S);  // after the SA hierarchy was rebuilt
// embedded.cu: the checksum of the Poisson patched-row pattern (written at every tagging)
unsigned long long read_rows_key(Context &c);
void initialise_body(Context &c);

// adjoint.cu: the discrete adjoint of the embedded method's steps (cuibm_adjoint)
struct AdjointStats {
    double ms;
    long long forward_steps, tape_steps, velocity_iterations, poisson_iterations, solves_reused;
};
void run_adjoint(Context &c, int nsteps, int snapshots, const double *wx, const double *wy, double *J, double *grad,
                 size_t ngrad, double adjoint_rtol, AdjointStats *stats);
void free_adjoint(Context &c);
void apply_transposed(Context &c, int which, const double *x, double *y);

// io.cpp / fields.cu
void write_grid_file(Context &c);
void write_info_file(Context &c);  // run.info
void write_step_output(Context &c);
void read_restart_state(Context &c);  // restart: the state written at step startStep
void *field_pointer(Context &c, int field, size_t *bytes);
void field_changed(Context &c, int field);

}  // namespace cuibm
