// Context life cycle, step orchestration and the extern "C" entry points.
//
// The time step follows the reference's phase order exactly:
//   NAVIER_STOKES  NavierStokesSolver::stepTime (NavierStokesSolver.cu:163-188)
//   LUO (external) luo_base::stepTime (luo_base.cu:208-233) with luoIBM's phases
//                  (luoIBM.cu:91-102, luoIBM/intermediateVelocity.cu:128-167,
//                  luoIBM/intermediatePressure.cu:280-342, luo_base/projectVelocity.cu:237-279,
//                  luo_base.cu:255-264 update body)
// and is recorded once into a CUDA graph whose linear solves are WHILE
// conditional nodes: one graph launch per step, no host synchronisation inside a
// step.  cuibm_step checks the solver status once at the end of the call.
#include <chrono>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <functional>
#include <sys/stat.h>

#include "../../include/cuibm.h"
#include "solver.h"
#include "batch_member.h"

namespace cuibm {

static int *g_err_word_of(Context &c) { return c.err_word; }

static void alloc_fields(Context &c)
{
    const Grid &g = c.g;
    const size_t nUV = g.nUV, nP = g.nP, nx = g.nx, ny = g.ny;
    size_t est = (nUV + nP) * 1800 + ((size_t)96 << 20);
    if (c.has_body) est += (nUV + nP) * 400;
    CUIBM_TRY(cudaMalloc(&c.arena, est));
    c.arena_bytes = est;
    // device arrays start at zero, as the reference's value-initialised cusp arrays do
    CUIBM_TRY(cudaMemset(c.arena, 0, est));
    c.arena_used = 0;
    CUIBM_TRY(cudaMemsetAsync(c.arena, 0, est, c.stream));
    c.u = c.carve<double>(nUV);
    c.uhat = c.carve<double>(nUV);
    c.uold = c.carve<double>(nUV);
    c.N = c.carve<double>(nUV);
    c.Nold = c.carve<double>(nUV);
    c.L = c.carve<double>(nUV);
    c.bc1 = c.carve<double>(nUV);
    c.rhs1 = c.carve<double>(nUV);
    c.p = c.carve<double>(nP);
    c.p_old = c.carve<double>(nP);
    c.rhs2 = c.carve<double>(nP);
    c.cfl = c.carve<double>(nP);
    c.work_x = c.carve<double>(nUV > nP ? nUV : nP);
    c.work_y = c.carve<double>(nUV > nP ? nUV : nP);
    c.solve_trace = c.carve<unsigned long long>(2 * kTraceLen);
    CUIBM_TRY(cudaMemset(c.solve_trace, 0, 2 * kTraceLen * sizeof(unsigned long long)));
    c.bc[XMINUS] = c.carve<double>(2 * ny - 1);
    c.bc[XPLUS] = c.carve<double>(2 * ny - 1);
    c.bc[YMINUS] = c.carve<double>(2 * nx - 1);
    c.bc[YPLUS] = c.carve<double>(2 * nx - 1);
    c.x = c.carve<double>(nx);
    c.dx = c.carve<double>(nx);
    c.xu = c.carve<double>(nx - 1);
    c.xv = c.carve<double>(nx);
    c.y = c.carve<double>(ny);
    c.dy = c.carve<double>(ny);
    c.yu = c.carve<double>(ny);
    c.yv = c.carve<double>(ny - 1);
    c.err_word = c.carve<int>(4);
    c.step_counter_dev = c.carve<int>(4);
    auto up = [&](double *d, const std::vector<double> &h) {
        CUIBM_TRY(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    };
    up(c.x, c.gx.centre);
    up(c.dx, c.gx.width);
    up(c.xu, c.gx.face);
    up(c.xv, c.gx.centre);
    up(c.y, c.gy.centre);
    up(c.dy, c.gy.width);
    up(c.yu, c.gy.centre);
    up(c.yv, c.gy.face);
}

// boundary arrays from the flow BCs (NavierStokesSolver.cu:104-128)
static void init_boundary_arrays(Context &c)
{
    const int nx = c.g.nx, ny = c.g.ny;
    std::vector<double> xm(2 * ny - 1), xp(2 * ny - 1), ym(2 * nx - 1), yp(2 * nx - 1);
    const BC(*b)[2] = c.P.bc;
    for (int i = 0; i < nx - 1; ++i) {
        ym[i] = b[YMINUS][0].value;
        yp[i] = b[YPLUS][0].value;
        ym[i + nx - 1] = b[YMINUS][1].value;
        yp[i + nx - 1] = b[YPLUS][1].value;
    }
    ym[2 * nx - 2] = b[YMINUS][1].value;
    yp[2 * nx - 2] = b[YPLUS][1].value;
    for (int i = 0; i < ny - 1; ++i) {
        xm[i] = b[XMINUS][0].value;
        xp[i] = b[XPLUS][0].value;
        xm[i + ny] = b[XMINUS][1].value;
        xp[i + ny] = b[XPLUS][1].value;
    }
    xm[ny - 1] = b[XMINUS][0].value;
    xp[ny - 1] = b[XPLUS][0].value;
    auto up = [&](double *d, const std::vector<double> &h) {
        CUIBM_TRY(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    };
    up(c.bc[XMINUS], xm);
    up(c.bc[XPLUS], xp);
    up(c.bc[YMINUS], ym);
    up(c.bc[YPLUS], yp);
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
}

struct PhaseTimer {
    Context &c;
    const char *name;
    bool on;
    PhaseTimer(Context &c_, const char *n) : c(c_), name(n), on(c_.profile_phases)
    {
        if (on) CUIBM_TRY(cudaEventRecord(c.ev0, c.stream));
    }
    ~PhaseTimer()
    {
        if (!on) return;
        cudaEventRecord(c.ev1, c.stream);
        cudaEventSynchronize(c.ev1);
        float ms = 0;
        cudaEventElapsedTime(&ms, c.ev0, c.ev1);
        Timer &t = c.timers[name];
        t.ms += ms;
        t.count++;
    }
};

// ---- phases ---------------------------------------------------------------------
static bool is_luo(const Context &c) { return c.P.solverType == ST_LUO && c.has_body; }
static bool is_fadlun(const Context &c) { return c.P.solverType == ST_FADLUN && c.has_body; }
static bool is_embedded(const Context &c) { return c.P.solverType == ST_OSC && c.has_body; }
static bool is_ib(const Context &c) { return is_luo(c) || is_fadlun(c) || is_embedded(c); }

static bool strong_coupling(const Context &c) { return is_ib(c) && c.P.VIV == 2; }

// first: the step's first pass, which moves N to Nold; the later passes of a strongly
// coupled step keep Nold and restart from u = uold (luoIBM/intermediateVelocity.cu:33,
// luo_iter/intermediateVelocity.cu:29; the Fadlun method has no such reset)
void phase_generate_rhs1(Context &c, bool first)
{
    PhaseTimer t(c, "Intermediate Velocity Setup");
    if (!first && (is_luo(c) || is_embedded(c))) launch_copy(c, c.u, c.uold, c.g.nUV);
    // updateRobinBoundary, rhs1GNInterpolation, zeroVelocity, rhs1HNInterpolation
    if (is_luo(c)) launch_ib_rhs1(c);
    if (is_fadlun(c)) launch_robin(c);
    if (is_embedded(c)) launch_ib_robin_inside(c);  // updateRobinBoundary, setInsideVelocity
    launch_rhs1(c, false, first);  // with the embedded method's update_rhs1_x/y
    if (is_fadlun(c)) launch_fadlun_rhs1(c);  // updateRHS1forIBX/Y
}

void phase_solve_velocity(Context &c, bool in_graph)
{
    PhaseTimer t(c, "Intermediate Velocity Solve");
    launch_solve(c, c.sys1, c.rhs1, c.uhat, in_graph);
}

void phase_generate_rhs2(Context &c)
{
    PhaseTimer t(c, "Poisson Setup");
    if (is_fadlun(c))
        launch_fadlun_rhs2(c);
    else
        launch_rhs2(c, c.uhat);
}

void phase_solve_poisson(Context &c, bool in_graph)
{
    PhaseTimer t(c, "Poisson Solve");
    launch_solve(c, c.sys2, c.rhs2, c.p, in_graph);
}

static void phase_project(Context &c)
{
    PhaseTimer t(c, "Velocity Projection");
    if (is_fadlun(c)) {
        launch_fadlun_project(c);
        return;
    }
    launch_project(c);
    if (is_luo(c) || is_embedded(c)) launch_ib_after_projection(c);  // ghost u, inside velocity
}

static void phase_update_body(Context &c)
{
    if (!is_ib(c)) return;
    {
        PhaseTimer t(c, "Calculate Force");
        launch_force(c);
    }
    {
        PhaseTimer t(c, "Move Body");
        launch_body_motion(c, -1.0);  // time taken from the device step counter
    }
    if (body_moves(c)) {
        // updateSolver: the box of the moved body, then its tags (and the interpolation
        // plan); a static body keeps its tags: re-tagging it reproduces them exactly
        PhaseTimer t(c, "Update Solver");
        launch_body_box(c);
        launch_tag_points(c);
    }
}

// One pass of the step's phases, from the explicit terms to the body update.
static void record_pass(Context &c, bool in_graph, bool first)
{
    phase_generate_rhs1(c, first);
    phase_solve_velocity(c, in_graph);
    if (is_luo(c)) {
        PhaseTimer t(c, "Intermediate Velocity Weight");
        launch_ib_after_velocity(c);  // weightUhat, preRHS2Interpolation
    }
    phase_generate_rhs2(c);
    phase_solve_poisson(c, in_graph);
    if (is_luo(c)) {
        PhaseTimer t(c, "Poisson Weight");
        launch_ib_after_poisson(c);  // hybrid pressure, weightPressure, ghost pressure
    }
    phase_project(c);
    phase_update_body(c);  // motion reads the step counter before it advances
}

// The strongly coupled step's further passes (luo_base.cu:211-223), after its first:
// while |SCtol| > 0.001 or fewer than two passes ran.  In a graph the passes are the
// body of a WHILE conditional node (default value 1: the second pass always runs)
// whose condition k_coupling_next sets; otherwise the host reads the answer after
// each pass.
static void record_coupling_loop(Context &c, bool in_graph)
{
    if (!in_graph) {
        for (int k = 1; k <= kCouplingMaxIterations; ++k) {
            record_pass(c, false, false);
            launch_coupling_next(c, 0, 0);
            double more = 0;
            CUIBM_TRY(cudaMemcpyAsync(&more, c.ib.motion + 10, sizeof more, cudaMemcpyDeviceToHost, c.stream));
            CUIBM_TRY(cudaStreamSynchronize(c.stream));
            if (more == 0) break;
        }
        return;
    }
    cudaStreamCaptureStatus st;
    cudaGraph_t graph;
    const cudaGraphNode_t *deps = nullptr;
    size_t ndeps = 0;
    CUIBM_TRY(cudaStreamGetCaptureInfo(c.stream, &st, nullptr, &graph, &deps, nullptr, &ndeps));
    cudaGraphConditionalHandle h;
    CUIBM_TRY(cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    CUIBM_TRY(cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &cp));
    cudaGraph_t bodyg = cp.conditional.phGraph_out[0];
    cudaStream_t main = c.stream;
    CUIBM_TRY(cudaStreamBeginCaptureToGraph(c.coupling_stream, bodyg, nullptr, nullptr, 0,
                                            cudaStreamCaptureModeRelaxed));
    c.stream = c.coupling_stream;
    try {
        record_pass(c, true, false);
        launch_coupling_next(c, h, 1);
    } catch (...) {
        c.stream = main;
        cudaGraph_t dummy;
        cudaStreamEndCapture(c.coupling_stream, &dummy);
        throw;
    }
    c.stream = main;
    cudaGraph_t got;
    CUIBM_TRY(cudaStreamEndCapture(c.coupling_stream, &got));
    CUIBM_TRY(cudaStreamUpdateCaptureDependencies(c.stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
}

static void record_step(Context &c, bool in_graph)
{
    if (is_ib(c)) {
        launch_copy(c, c.p_old, c.p, c.g.nP);    // _pre_step: pressure_old = pressure
        launch_copy(c, c.uold, c.u, c.g.nUV);    //            uold = u
        launch_body_pre_step(c);                 //            uB0 = uB, ..., SCtol, SC_count
    }
    record_pass(c, in_graph, true);
    if (strong_coupling(c)) record_coupling_loop(c, in_graph);
    launch_step_counter(c);  // _post_step: timeStep++
    {
        PhaseTimer t(c, "CFL");
        launch_cfl(c);
    }
}

static void build_step_graph(Context &c)
{
    if (c.step_exec) {
        cudaGraphExecDestroy(c.step_exec);
        cudaGraphDestroy(c.step_graph);
        c.step_exec = nullptr;
    }
    CUIBM_TRY(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeRelaxed));
    try {
        record_step(c, true);
    } catch (...) {
        cudaGraph_t g;
        cudaStreamEndCapture(c.stream, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    CUIBM_TRY(cudaStreamEndCapture(c.stream, &c.step_graph));
    CUIBM_TRY(cudaGraphInstantiate(&c.step_exec, c.step_graph, 0));
    c.static_kernels = count_kernel_nodes(c.step_graph);
}

}  // namespace cuibm

using namespace cuibm;

struct cuibm_ctx {
    Context c;
};

static int fail(cuibm_ctx *h, int code, const std::string &msg)
{
    if (h) h->c.err = msg;
    return code;
}

#define CUIBM_GUARD(h, ...)                                                       \
    try {                                                                         \
        __VA_ARGS__;                                                              \
    } catch (const CudaError &e) {                                                \
        return fail(h, CUIBM_ERR_CUDA, e.msg);                                    \
    } catch (const InputError &e) {                                               \
        return fail(h, CUIBM_ERR_BAD_INPUT, e.msg);                               \
    } catch (const std::exception &e) {                                           \
        return fail(h, CUIBM_ERR_BAD_INPUT, e.what());                            \
    }

// error text of the context-free entry points, one per host thread: cuibm_case_error
// returns the calling thread's last message, so a failure on one thread cannot free or
// overwrite the text another thread is reading
static thread_local std::string g_create_error;

// error text of the context-free entry points (read back through cuibm_case_error)
std::string cuibm_noalloc_error_sink(const std::string &msg)
{
    g_create_error = msg;
    return msg;
}

extern "C" {

int cuibm_create(const char *case_folder, int argc, const char **argv, cuibm_ctx **out)
{
    if (!out) return CUIBM_ERR_BAD_INPUT;
    *out = nullptr;
    cuibm_ctx *h = new cuibm_ctx();
    Context &c = h->c;
    std::string err = load_case(case_folder ? case_folder : ".", argc, argv, c.P);
    if (!err.empty()) {
        g_create_error = err;
        delete h;
        return err.rfind("cannot open", 0) == 0 ? CUIBM_ERR_IO : CUIBM_ERR_BAD_INPUT;
    }
    if (c.P.solverType == ST_FSI) {
        g_create_error = "SolverType FSI is not implemented by the reference either";
        delete h;
        return CUIBM_ERR_UNSUPPORTED;
    }
    try {
        if (!(err = build_axis(c.P.axis[0], c.gx)).empty()) throw InputError(err);
        if (!(err = build_axis(c.P.axis[1], c.gy)).empty()) throw InputError(err);
        if (!(err = build_bodies(c.P.bodies, c.body)).empty()) throw InputError(err);
        Grid &g = c.g;
        g.nx = c.gx.n;
        g.ny = c.gy.n;
        g.nU = (g.nx - 1) * g.ny;
        g.nV = g.nx * (g.ny - 1);
        g.nUV = g.nU + g.nV;
        g.nP = g.nx * g.ny;
        c.has_body = c.body.total > 0 && c.P.solverType != ST_NAVIERSTOKES;
        if ((c.P.solverType == ST_FADLUN || c.P.solverType == ST_OSC) &&
            (c.P.krylovVelocity == KRYLOV_CG || c.P.krylovPoisson == KRYLOV_CG))
            throw InputError("the Fadlun and embedded operators are not symmetric: use BICGSTAB (krylov: CG is for "
                             "the other methods)");
        if (c.has_body && c.P.VIV != 0 && c.P.VIV != 1 && c.P.VIV != 2)
            throw InputError("simulation VIV must be 0 (prescribed motion), 1 (loosely coupled) or 2 (strongly "
                             "coupled)");
        if (c.has_body && c.P.VIV != 0 && c.P.Ured <= 0) throw InputError("simulation Ured must be positive");
        if (c.has_body && c.P.VIV == 2 && c.P.solverType == ST_FADLUN)
            throw InputError("simulation VIV: 2 needs the LUO or OSC_CYLINDER method: the Fadlun method's "
                             "generateRHS1 does not restart a sub-iteration from uold, so each one advances the "
                             "flow by another time step and the coupling test does not settle");
        if (c.P.solverType != ST_NAVIERSTOKES && c.body.total == 0)
            throw InputError("an immersed-boundary SolverType needs a body in bodies.yaml");
        if (c.has_body) {
            c.bb = bounding_box(c.body.x.data(), c.body.y.data(), c.body.total, c.gx, c.gy, c.P.scaleCV);
            c.bb_tag = c.bb;
            if (c.body.xCoeff != 0 || c.body.uCoeff != 0) {
                // a prescribed motion x = xnew + (x0 - midX), |xnew| <= |xCoefficient|: tag
                // over the box of the body at both ends of its travel (tags near the body
                // do not depend on how far the scanned box reaches)
                const int n = c.body.total;
                const double a = std::fabs(c.body.xCoeff);
                std::vector<double> xs(2 * n), ys(2 * n);
                for (int k = 0; k < n; ++k) {
                    xs[k] = -a + c.body.dxp[k];
                    xs[n + k] = a + c.body.dxp[k];
                    ys[k] = ys[n + k] = c.body.y[k];
                }
                c.bb_tag = bounding_box(xs.data(), ys.data(), 2 * n, c.gx, c.gy, c.P.scaleCV);
            }
            if (c.P.VIV == 1 || c.P.VIV == 2) {
                // flow-induced motion in y of unknown amplitude: tag over the box of the body
                // displaced by up to half a body height either way (vortex-induced
                // amplitudes of a free cylinder stay below that; a step whose body leaves the
                // box reports an error)
                const int n = c.body.total;
                double ymin = c.body.y[0], ymax = c.body.y[0];
                for (double v : c.body.y) ymin = std::min(ymin, v), ymax = std::max(ymax, v);
                const double a = 0.5 * (ymax - ymin);
                std::vector<double> xs(2 * n), ys(2 * n);
                for (int k = 0; k < n; ++k) {
                    xs[k] = xs[n + k] = c.body.dxp[k];
                    ys[k] = c.body.y[k] - a;
                    ys[n + k] = c.body.y[k] + a;
                }
                c.bb_tag = bounding_box(xs.data(), ys.data(), 2 * n, c.gx, c.gy, c.P.scaleCV);
            }
            for (const BoundingBox &b : {c.bb, c.bb_tag})
                if (b.i0 < 6 || b.j0 < 6 || b.i0 + b.ncx > g.nx - 7 || b.j0 + b.ncy > g.ny - 7)
                    throw InputError("the body's scaled bounding box reaches the domain boundary");
        }
        CUIBM_TRY(cudaSetDevice(c.P.deviceNumber));
        c.device = c.P.deviceNumber;
        CUIBM_TRY(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
        CUIBM_TRY(cudaStreamCreateWithFlags(&c.side_stream, cudaStreamNonBlocking));
        CUIBM_TRY(cudaStreamCreateWithFlags(&c.coupling_stream, cudaStreamNonBlocking));
        CUIBM_TRY(cudaEventCreate(&c.ev0));
        CUIBM_TRY(cudaEventCreate(&c.ev1));
        CUIBM_TRY(cudaHostAlloc(&c.h_scalars, 64 * sizeof(double), cudaHostAllocDefault));
        alloc_fields(c);
        upload_ns_tables(c);
        c.sys1.which = 1;
        c.sys2.which = 2;
        if (c.has_body) setup_ib(c);
        if (c.P.solverType == ST_FADLUN && c.has_body) {
            // the Fadlun operators are assembled from the tags of the initial body
            // position (fadlunModified::initialise), before the solvers are set up
            c.timeStep = c.P.startStep;
            initialise_body(c);
            launch_tag_points(c);
            setup_fadlun(c);
        }
        if (c.P.solverType == ST_OSC && c.has_body) {
            // the embedded operators' rows of the initial tags, before the solvers (and the
            // SA hierarchy, built from these rows) are set up
            setup_embedded(c);
            c.timeStep = c.P.startStep;
            initialise_body(c);
            launch_tag_points(c);
        }
        // a moving embedded body changes the operator's rows at every tagging: an SA
        // hierarchy is rebuilt whenever the set of patched rows changes (the reference
        // rebuilds its preconditioner every step, luo_iter/poisson.cu:38-45)
        if (c.P.solverType == ST_OSC && c.has_body && body_moves(c)) {
            for (LinearSystem *S : {&c.sys1, &c.sys2}) {
                const LinearSolve &L = S->which == 1 ? c.P.velocity : c.P.poisson;
                if (L.precond == PC_SMOOTHED_AGGREGATION && L.precision != PRECISION_MIXED) {
                    S->sa_dynamic = true;
                    S->sa_body_free = true;  // option "sa_body_free" 0: rebuild from the current rows
                    c.sa_rebuild = true;
                }
            }
        }
        setup_system(c, c.sys1);
        setup_system(c, c.sys2);
        // a hierarchy without the body's rows smooths level 0 with the current rows
        for (LinearSystem *S : {&c.sys1, &c.sys2})
            if (S->sa_body_free) refresh_system_diagonals(c, *S);
        if (c.sa_rebuild) c.sys1.sa_key = c.sys2.sa_key = read_rows_key(c);
        CUIBM_TRY(cudaStreamSynchronize(c.stream));
        const char *ev = getenv("CUIBM_GRAPH");
        c.use_graph = !(ev && ev[0] == '0');
        const char *fv = getenv("CUIBM_FUSED");
        c.fused_solve = !(fv && fv[0] == '0');
        c.created = true;
    } catch (const CudaError &e) {
        g_create_error = e.msg;
        cuibm_destroy(h);
        return CUIBM_ERR_CUDA;
    } catch (const InputError &e) {
        g_create_error = e.msg;
        cuibm_destroy(h);
        return CUIBM_ERR_BAD_INPUT;
    }
    *out = h;
    return CUIBM_OK;
}

const char *cuibm_last_error(const cuibm_ctx *h) { return h ? h->c.err.c_str() : g_create_error.c_str(); }

int cuibm_initialise(cuibm_ctx *h)
{
    if (!h || !h->c.created) return CUIBM_ERR_STATE;
    Context &c = h->c;
    CUIBM_GUARD(h, {
        CUIBM_TRY(cudaSetDevice(c.device));
        c.timeStep = c.P.startStep;
        // initialiseNoBody: rhs2 = uhat = Nold = N = 0, initial velocity, uhat = u, boundary arrays
        CUIBM_TRY(cudaMemsetAsync(c.rhs2, 0, c.g.nP * sizeof(double), c.stream));
        CUIBM_TRY(cudaMemsetAsync(c.N, 0, c.g.nUV * sizeof(double), c.stream));
        CUIBM_TRY(cudaMemsetAsync(c.Nold, 0, c.g.nUV * sizeof(double), c.stream));
        CUIBM_TRY(cudaMemsetAsync(c.p, 0, c.g.nP * sizeof(double), c.stream));
        launch_initial_velocity(c);
        launch_copy(c, c.uhat, c.u, c.g.nUV);
        init_boundary_arrays(c);
        int zero[2] = {0, 0};
        CUIBM_TRY(cudaMemcpyAsync(c.step_counter_dev, &c.timeStep, sizeof(int), cudaMemcpyHostToDevice, c.stream));
        CUIBM_TRY(cudaMemcpyAsync(g_err_word_of(c), zero, sizeof(int), cudaMemcpyHostToDevice, c.stream));
        // restart: the state the run wrote at startStep (fields, boundary arrays, body)
        const bool restart = c.P.restart && c.P.startStep > 0;
        if (c.has_body) initialise_body(c);  // luo_base::initialise movement at t = dt*timeStep
        if (restart) read_restart_state(c);
        if (c.has_body) {
            launch_tag_points(c);     // tagPoints()
            if (c.P.solverType == ST_LUO) launch_set_inside(c, c.u);  // luoIBM::zeroVelocity
        }
        CUIBM_TRY(cudaStreamSynchronize(c.stream));
        c.cfl_max = 0;
        if (c.P.writeOutput) {
            mkdir(c.P.caseFolder.c_str(), 0755);
            std::string f = c.P.caseFolder + "/iterations";
            const char *mode = restart ? "a" : "w";  // a restarted run appends to the histories
            c.iterationsFile = fopen(f.c_str(), mode);
            if (c.has_body) {
                c.forceFile = fopen((c.P.caseFolder + "/forces").c_str(), mode);
                c.midPositionFile = fopen((c.P.caseFolder + "/midPosition").c_str(), mode);
            }
            write_grid_file(c);
            write_info_file(c);
        }
        if (c.use_graph) build_step_graph(c);
        c.initialised = true;
    });
    return CUIBM_OK;
}

// Between steps: a moving embedded body whose patched rows changed gets new SA
// hierarchies, built from the current rows (and the step graph follows them).
static void rebuild_hierarchies(Context &c)
{
    if (c.sa_rebuild_interval <= 0 || c.timeStep - c.sa_last_rebuild < c.sa_rebuild_interval) return;
    bool any = false;  // hierarchies without the body's rows never need rebuilding
    for (LinearSystem *S : {&c.sys1, &c.sys2}) any = any || (S->sa_dynamic && !S->sa_body_free);
    if (!any) return;
    const unsigned long long key = read_rows_key(c);
    bool rebuilt = false;
    for (LinearSystem *S : {&c.sys1, &c.sys2}) {
        if (!S->sa_dynamic || S->sa_body_free || S->sa_key == key) continue;
        const auto t0 = std::chrono::steady_clock::now();
        free_sa_hierarchy(*S);
        build_sa_hierarchy(c, *S);
        refresh_fused_hierarchy(c, *S);
        S->sa_key = key;
        c.sa_rebuilds++;
        c.sa_last_rebuild = c.timeStep;
        Timer &tm = c.timers["SA rebuild"];  // host time, read with cuibm_get_timer
        tm.ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        tm.count++;
        rebuilt = true;
    }
    if (rebuilt && c.use_graph) build_step_graph(c);
}

}  // extern "C"

namespace cuibm {

// one time step as cuibm_step runs it: the step graph (or the phases one by one), the
// host's step count, and a rebuilt SA hierarchy when the embedded rows' pattern changed
void step_once(Context &c)
{
    if (c.use_graph && !c.profile_phases && c.step_exec)
        CUIBM_TRY(cudaGraphLaunch(c.step_exec, c.stream));
    else
        record_step(c, false);
    c.timeStep++;
    if (c.sa_rebuild) ::rebuild_hierarchies(c);
}

// the step error word of the steps enqueued so far (0: every solve converged)
int read_step_error(Context &c)
{
    int errw = 0;
    CUIBM_TRY(cudaMemcpyAsync(&errw, c.err_word, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
    return errw;
}

}  // namespace cuibm

extern "C" {

int cuibm_step(cuibm_ctx *h, int nsteps)
{
    if (!h || !h->c.initialised) return CUIBM_ERR_STATE;
    if (nsteps < 0) return fail(h, CUIBM_ERR_BAD_INPUT, "nsteps < 0");
    Context &c = h->c;
    CUIBM_GUARD(h, {
        for (int s = 0; s < nsteps; ++s) step_once(c);
        if (!c.step_sync && nsteps > 0) return CUIBM_OK;  // enqueued only; checked by a later synchronising call
        int errw = 0;
        CUIBM_TRY(cudaMemcpyAsync(&errw, g_err_word_of(c), sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        CUIBM_TRY(cudaStreamSynchronize(c.stream));
        if (errw == kErrCouplingNotConverged) {
            c.err = "ERROR: the strongly coupled sub-iterations (VIV: 2) of a step did not converge in " +
                    std::to_string(kCouplingMaxIterations) + " passes by time step " + std::to_string(c.timeStep);
            return CUIBM_ERR_NOT_CONVERGED;
        }
        if (errw == kErrBodyOutsideTagBox) {
            c.err = "ERROR: the body left the region it is tagged over by time step " + std::to_string(c.timeStep) +
                    " (flow-induced motion beyond half a body height)";
            return CUIBM_ERR_UNSUPPORTED;
        }
        if (errw) {
            int sys = errw / 16, st = errw % 16;
            char msg[256];
            snprintf(msg, sizeof msg, "ERROR: Solve for %s failed (%s) by time step %d",
                     sys == 1 ? "uhat" : "pressure",
                     st == KS_NAN       ? "non-finite residual"
                     : st == KS_TIMEOUT ? "a grid barrier of the persistent solver timed out"
                                        : "maxIterations reached",
                     c.timeStep);
            c.err = msg;
            if (st == KS_TIMEOUT) return CUIBM_ERR_CUDA;
            return st == KS_NAN ? CUIBM_ERR_NAN : CUIBM_ERR_NOT_CONVERGED;
        }
    });
    return CUIBM_OK;
}

// the batch's view of an instance (batch_member.h)
cudaGraph_t cuibm_batch_member_graph(cuibm_ctx *h)
{
    if (!h) return nullptr;
    const Context &c = h->c;
    if (!c.initialised || !c.use_graph || c.profile_phases || c.sa_rebuild || !c.step_exec) return nullptr;
    return c.step_graph;
}

cudaStream_t cuibm_batch_member_stream(cuibm_ctx *h) { return h ? h->c.stream : nullptr; }

void cuibm_batch_member_advance(cuibm_ctx *h, int n)
{
    if (h) h->c.timeStep += n;
}

int cuibm_finished(const cuibm_ctx *h)
{
    if (!h) return 1;
    return h->c.timeStep < h->c.P.nt ? 0 : 1;
}

int cuibm_get_info(const cuibm_ctx *h, cuibm_info *info)
{
    if (!h || !info || !h->c.created) return CUIBM_ERR_STATE;
    const Context &c = h->c;
    std::memset(info, 0, sizeof *info);
    info->nx = c.g.nx;
    info->ny = c.g.ny;
    info->numU = c.g.nU;
    info->numV = c.g.nV;
    info->numUV = c.g.nUV;
    info->numP = c.g.nP;
    info->solver_type = c.P.solverType;
    info->time_step = c.timeStep;
    info->nt = c.P.nt;
    info->nsave = c.P.nsave;
    info->dt = c.P.dt;
    info->nu = c.P.nu;
    info->total_points = c.body.total;
    info->bb_start_i = c.bb.i0;
    info->bb_start_j = c.bb.j0;
    info->bb_ncx = c.bb.ncx;
    info->bb_ncy = c.bb.ncy;
    const int nx = c.g.nx, ny = c.g.ny;
    info->nnz_lhs1 = (nx - 1) * ny * 5 - 2 * ny - 2 * (nx - 1) + (ny - 1) * nx * 5 - 2 * (ny - 1) - 2 * nx;
    info->nnz_lhs2 = 5 * nx * ny - 2 * ny - 2 * nx;
    if (is_fadlun(c)) {
        info->nnz_lhs1 = c.fadlun.nnz1;
        info->nnz_lhs2 = c.fadlun.nnz2;
    }
    if (is_embedded(c)) {  // size_LHS1 / size_LHS2: one extra slot per hybrid node
        // the plan's node counts live on the device: read them on the context's stream
        Context &cm = const_cast<Context &>(c);
        try {
            info->nnz_lhs1 += embedded_hybrid_count(cm, 1);
            info->nnz_lhs2 += embedded_hybrid_count(cm, 2);
        } catch (const CudaError &e) {
            cm.err = e.msg;
            return CUIBM_ERR_CUDA;
        }
    }
    info->velocity_precond = c.P.velocity.precond;
    info->poisson_precond = c.P.poisson.precond;
    info->velocity_krylov = c.P.krylovVelocity;
    info->poisson_krylov = c.P.krylovPoisson;
    info->velocity_precision = c.P.velocity.precision;
    info->poisson_precision = c.P.poisson.precision;
    info->sa_rebuilds = c.sa_rebuilds;
    info->sa_structured = c.sys2.sa_structured ? 1 : 0;
    info->amg_levels = (int)c.sys2.amg.size();
    return CUIBM_OK;
}

int cuibm_get_field(cuibm_ctx *h, int field, void *dst, size_t bytes, int dst_on_device)
{
    if (!h || !h->c.created) return CUIBM_ERR_STATE;
    Context &c = h->c;
    CUIBM_GUARD(h, {
        size_t need = 0;
        void *src = field_pointer(c, field, &need);
        if (!src) return fail(h, CUIBM_ERR_BAD_INPUT, "unknown or unavailable field " + std::to_string(field));
        if (bytes != need)
            return fail(h, CUIBM_ERR_BAD_INPUT, "field " + std::to_string(field) + " needs " + std::to_string(need) +
                                                    " bytes, got " + std::to_string(bytes));
        CUIBM_TRY(cudaMemcpyAsync(dst, src, bytes,
                                  (dst_on_device & 1) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c.stream));
        if (!(dst_on_device & CUIBM_COPY_ASYNC)) CUIBM_TRY(cudaStreamSynchronize(c.stream));
    });
    return CUIBM_OK;
}

int cuibm_set_field(cuibm_ctx *h, int field, const void *src, size_t bytes, int src_on_device)
{
    if (!h || !h->c.created) return CUIBM_ERR_STATE;
    Context &c = h->c;
    CUIBM_GUARD(h, {
        size_t need = 0;
        void *dst = field_pointer(c, field, &need);
        if (!dst) return fail(h, CUIBM_ERR_BAD_INPUT, "unknown or unavailable field " + std::to_string(field));
        if (bytes != need) return fail(h, CUIBM_ERR_BAD_INPUT, "wrong byte count for field " + std::to_string(field));
        CUIBM_TRY(cudaMemcpyAsync(dst, src, bytes,
                                  (src_on_device & 1) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c.stream));
        if (!(src_on_device & CUIBM_COPY_ASYNC)) CUIBM_TRY(cudaStreamSynchronize(c.stream));
        field_changed(c, field);
    });
    return CUIBM_OK;
}

int cuibm_get_forces(cuibm_ctx *h, double *fx, double *fy)
{
    if (!h || !h->c.created) return CUIBM_ERR_STATE;
    Context &c = h->c;
    CUIBM_GUARD(h, {
        double f[2] = {0, 0};
        if (c.has_body) {
            CUIBM_TRY(cudaMemcpyAsync(f, c.ib.forceOut, 2 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            CUIBM_TRY(cudaStreamSynchronize(c.stream));
        }
        if (fx) *fx = f[0];
        if (fy) *fy = f[1];
    });
    return CUIBM_OK;
}

int cuibm_get_iterations(cuibm_ctx *h, int *it1, int *it2)
{
    if (!h || !h->c.created) return CUIBM_ERR_STATE;
    Context &c = h->c;
    CUIBM_GUARD(h, {
        int a = 0, b = 0;
        read_solve_status(c, c.sys1, &a);
        read_solve_status(c, c.sys2, &b);
        if (it1) *it1 = a;
        if (it2) *it2 = b;
    });
    return CUIBM_OK;
}

int cuibm_get_matrix(cuibm_ctx *h, int system, int *row, int *col, double *val, size_t nnz)
{
    if (!h || !h->c.created) return CUIBM_ERR_STATE;
    Context &c = h->c;
    CUIBM_GUARD(h, {
        std::vector<int> r, cc;
        std::vector<double> v;
        if (system != 1 && system != 2) return fail(h, CUIBM_ERR_BAD_INPUT, "system must be 1 or 2");
        host_matrix_coo(c, system, r, cc, v);
        if (nnz != r.size()) return fail(h, CUIBM_ERR_BAD_INPUT, "nnz mismatch: need " + std::to_string(r.size()));
        std::memcpy(row, r.data(), r.size() * sizeof(int));
        std::memcpy(col, cc.data(), cc.size() * sizeof(int));
        std::memcpy(val, v.data(), v.size() * sizeof(double));
    });
    return CUIBM_OK;
}

int cuibm_run(cuibm_ctx *h, int op)
{
    if (!h || !h->c.created) return CUIBM_ERR_STATE;
    Context &c = h->c;
    CUIBM_GUARD(h, {
        bool ib = c.has_body;
        auto need_ib = [&]() {
            if (!ib) throw InputError("operation needs an immersed body");
        };
        switch (op) {
        case CUIBM_OP_RHS1_TERMS: launch_rhs1(c, true); break;
        case CUIBM_OP_GENERATE_RHS1: phase_generate_rhs1(c, true); break;
        case CUIBM_OP_SOLVE_VELOCITY: phase_solve_velocity(c, false); break;
        case CUIBM_OP_WEIGHT_UHAT: need_ib(); launch_weight_uhat(c); break;
        case CUIBM_OP_GENERATE_RHS2:  // preRHS2Interpolation, then the right-hand side
            if (is_luo(c)) launch_ghost_velocity(c, c.uhat, true);
            phase_generate_rhs2(c);
            break;
        case CUIBM_OP_RHS2:
            if (is_fadlun(c)) launch_fadlun_rhs2(c); else launch_rhs2(c, c.uhat);
            break;
        case CUIBM_OP_SOLVE_POISSON: phase_solve_poisson(c, false); break;
        case CUIBM_OP_WEIGHT_PRESSURE:
            need_ib();
            launch_ib_after_poisson(c);
            break;
        case CUIBM_OP_PROJECT:
            if (is_fadlun(c)) launch_fadlun_project(c); else launch_project(c);
            break;
        case CUIBM_OP_PROJECT_VELOCITY: phase_project(c); break;
        case CUIBM_OP_UPDATE_BODY: need_ib(); phase_update_body(c); break;
        case CUIBM_OP_APPLY_LHS1: launch_apply(c, 1, c.work_x, c.work_y); break;
        case CUIBM_OP_APPLY_LHS2: launch_apply(c, 2, c.work_x, c.work_y); break;
        case CUIBM_OP_TAG_POINTS: need_ib(); launch_tag_points(c); break;
        case CUIBM_OP_GHOST_VELOCITY_U: need_ib(); launch_ghost_velocity(c, c.u, true); break;
        case CUIBM_OP_GHOST_VELOCITY_UHAT: need_ib(); launch_ghost_velocity(c, c.uhat, true); break;
        case CUIBM_OP_HYBRID_VELOCITY: need_ib(); launch_hybrid_velocity(c, c.u); break;
        case CUIBM_OP_HYBRID_PRESSURE: need_ib(); launch_hybrid_pressure(c); break;
        case CUIBM_OP_GHOST_PRESSURE: need_ib(); launch_ghost_pressure(c, true); break;
        case CUIBM_OP_SET_INSIDE: need_ib(); launch_set_inside(c, c.u); break;
        case CUIBM_OP_ROBIN_BOUNDARY: launch_robin(c); break;
        case CUIBM_OP_FORCE: need_ib(); launch_force(c); break;
        case CUIBM_OP_CFL: launch_cfl(c); break;
        case CUIBM_OP_SURFACE_FORCE: need_ib(); launch_surface_force(c, 1, false); break;
        case CUIBM_OP_SURFACE_FORCE_CORRECTED: need_ib(); launch_surface_force(c, 2, false); break;
        case CUIBM_OP_APPLY_LHS1_T: apply_transposed(c, 1, c.work_x, c.work_y); break;
        case CUIBM_OP_APPLY_LHS2_T: apply_transposed(c, 2, c.work_x, c.work_y); break;
        case CUIBM_OP_PRECONDITION_POISSON: {
            LinearSystem &S = c.sys2;
            if (S.amg.empty()) throw InputError("the Poisson system has no smoothed-aggregation preconditioner");
            // the cycle's kernels run while the system's status word says a solve runs
            int saved = 0, running = KS_RUNNING;
            CUIBM_TRY(cudaMemcpyAsync(&saved, &S.ks->status, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
            CUIBM_TRY(cudaStreamSynchronize(c.stream));
            CUIBM_TRY(cudaMemcpyAsync(&S.ks->status, &running, sizeof(int), cudaMemcpyHostToDevice, c.stream));
            launch_vcycle(c, S, c.work_x, c.work_y);
            CUIBM_TRY(cudaMemcpyAsync(&S.ks->status, &saved, sizeof(int), cudaMemcpyHostToDevice, c.stream));
            break;
        }
        default: return fail(h, CUIBM_ERR_BAD_INPUT, "unknown operation " + std::to_string(op));
        }
        CUIBM_TRY(cudaStreamSynchronize(c.stream));
        CUIBM_TRY(cudaGetLastError());
        if (op == CUIBM_OP_SOLVE_VELOCITY || op == CUIBM_OP_SOLVE_POISSON) {
            int it = 0;
            int st = read_solve_status(c, op == CUIBM_OP_SOLVE_VELOCITY ? c.sys1 : c.sys2, &it);
            if (st == KS_MAXIT) return fail(h, CUIBM_ERR_NOT_CONVERGED, "linear solve reached maxIterations");
            if (st == KS_NAN) return fail(h, CUIBM_ERR_NAN, "linear solve produced a non-finite residual");
            if (st == KS_TIMEOUT) return fail(h, CUIBM_ERR_CUDA, "a grid barrier of the persistent solver timed out");
        }
    });
    return CUIBM_OK;
}

int cuibm_get_stream(cuibm_ctx *h, void **stream)
{
    if (!h || !stream) return CUIBM_ERR_BAD_INPUT;
    *stream = (void *)h->c.stream;
    return CUIBM_OK;
}

int cuibm_get_timer(cuibm_ctx *h, const char *name, double *ms, int *count)
{
    if (!h || !name) return CUIBM_ERR_BAD_INPUT;
    auto it = h->c.timers.find(name);
    if (it == h->c.timers.end()) {
        if (ms) *ms = 0;
        if (count) *count = 0;
        return CUIBM_OK;
    }
    if (ms) *ms = it->second.ms;
    if (count) *count = it->second.count;
    return CUIBM_OK;
}

int cuibm_set_option(cuibm_ctx *h, const char *key, double value)
{
    if (!h || !key) return CUIBM_ERR_BAD_INPUT;
    Context &c = h->c;
    std::string k(key);
    if (k == "profile_phases") c.profile_phases = value != 0;
    else if (k == "use_graph") {
        bool want = value != 0;
        if (want != c.use_graph && c.initialised) {
            CUIBM_GUARD(h, {
                c.use_graph = want;
                if (want) build_step_graph(c);
            });
        }
        c.use_graph = want;
    } else if (k == "fused_solve") {
        bool want = value != 0;
        if (want != c.fused_solve) {
            c.fused_solve = want;
            if (c.initialised && c.use_graph) CUIBM_GUARD(h, { build_step_graph(c); });
        }
    } else if (k == "trace_solve") {
        c.trace_solve = value != 0;
        CUIBM_GUARD(h, {
            set_fused_trace(c, c.sys1, c.trace_solve);
            set_fused_trace(c, c.sys2, c.trace_solve);
        });
    } else if (k == "step_sync") {
        c.step_sync = value != 0;
    } else if (k == "write_output") c.P.writeOutput = value != 0;
    else if (k == "sa_rebuild_interval") {
        if (value != (int)value) return fail(h, CUIBM_ERR_BAD_INPUT, "sa_rebuild_interval must be a whole number");
        c.sa_rebuild_interval = (int)value;
    } else if (k == "solver_blocks") {
        const int nb = (int)value;
        if (nb != value || nb < 0) return fail(h, CUIBM_ERR_BAD_INPUT, "solver_blocks must be a count >= 0");
        c.P.solverBlocks = nb;
        set_fused_grid(c.sys1, nb);
        set_fused_grid(c.sys2, nb);
        if (c.initialised && c.use_graph) CUIBM_GUARD(h, { build_step_graph(c); });
    } else if (k == "force_method") {
        const int m = (int)value;
        if (m < 0 || m > 2 || m != value) return fail(h, CUIBM_ERR_BAD_INPUT, "force_method must be 0, 1 or 2");
        if (m && c.has_body && c.body.total < 2)
            return fail(h, CUIBM_ERR_BAD_INPUT, "the surface force needs at least two body points");
        if (m != c.force_method) {
            c.force_method = m;
            if (c.initialised && c.use_graph) CUIBM_GUARD(h, { build_step_graph(c); });
        }
    } else if (k == "sa_body_free") {
        // a moving embedded body's SA hierarchies from the operator without the body's rows
        // (the level-0 smoother and residual keep the current rows): built once, never
        // rebuilt as the body moves (the default); 0: rebuilt from the current rows whenever
        // the set of patched rows changes
        const bool want = value != 0;
        CUIBM_GUARD(h, {
            if (!c.initialised) return fail(h, CUIBM_ERR_STATE, "sa_body_free is set after cuibm_initialise");
            for (LinearSystem *S : {&c.sys1, &c.sys2}) {
                if (!S->sa_dynamic || S->sa_body_free == want) continue;
                S->sa_body_free = want;
                free_sa_hierarchy(*S);
                build_sa_hierarchy(c, *S);
                refresh_fused_hierarchy(c, *S);
                refresh_system_diagonals(c, *S);  // level 0 smooths with the current rows
                S->sa_key = read_rows_key(c);
            }
            if (c.use_graph) build_step_graph(c);
        });
    } else if (k == "adjoint_tolerance") {
        if (!(value > 0 && value < 1)) return fail(h, CUIBM_ERR_BAD_INPUT, "adjoint_tolerance must lie in (0, 1)");
        c.adjoint_rtol = value;
    } else return fail(h, CUIBM_ERR_BAD_INPUT, "unknown option " + k);
    return CUIBM_OK;
}

int cuibm_profile_kernel(cuibm_ctx *h, const char *kernel, int reps, double *avg_ms, double *bytes)
{
    if (!h || !h->c.initialised || !kernel || reps <= 0) return CUIBM_ERR_STATE;
    Context &c = h->c;
    CUIBM_GUARD(h, {
        std::string k(kernel);
        const double UV = c.g.nUV, P = c.g.nP, D = sizeof(double);
        std::function<void()> launch;
        double b = 0;
        if (k == "rhs1") {
            // production form: u, N in; N, Nold, rhs1 out.  Algorithmic: u, Nold in; N, rhs1 out
            launch = [&] { launch_rhs1(c, false); };
            b = 4 * UV * D;
        } else if (k == "rhs2") {
            launch = [&] { launch_rhs2(c, c.uhat); };
            b = UV * D + P * D;
        } else if (k == "project") {
            launch = [&] { launch_project(c); };
            b = 3 * UV * D + P * D;  // uhat, u, p in; u, uold out (u read+write counted once each)
            b += UV * D;
        } else if (k == "apply_lhs1") {
            launch = [&] { launch_apply(c, 1, c.work_x, c.work_y); };
            b = 2 * UV * D;
        } else if (k == "apply_lhs2") {
            launch = [&] { launch_apply(c, 2, c.work_x, c.work_y); };
            b = 2 * P * D;
        } else if (k == "poisson_solve" || k == "velocity_solve") {
            // the last step's solve again (same right-hand side, same starting guess: the
            // field before the step), each repetition timed alone
            LinearSystem &S = k == "poisson_solve" ? c.sys2 : c.sys1;
            const double *rhs = S.which == 1 ? c.rhs1 : c.rhs2;
            const double *x0 = S.which == 1 ? c.uold : c.p_old;
            double total = 0;
            for (int r = 0; r <= reps; ++r) {
                launch_copy(c, c.work_x, x0, S.n);
                CUIBM_TRY(cudaEventRecord(c.ev0, c.stream));
                launch_solve(c, S, rhs, c.work_x, false);
                CUIBM_TRY(cudaEventRecord(c.ev1, c.stream));
                CUIBM_TRY(cudaEventSynchronize(c.ev1));
                float ms = 0;
                CUIBM_TRY(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
                if (r > 0) total += ms;
            }
            int it = 0;
            if (read_solve_status(c, S, &it) != KS_CONVERGED)
                return fail(h, CUIBM_ERR_NOT_CONVERGED, "profiled solve did not converge");
            if (avg_ms) *avg_ms = total / reps;
            if (bytes) *bytes = solve_bytes(S, it);
            return CUIBM_OK;
        } else if (k == "fp64_fma") {
            // the GPU's FP64 issue rate: *bytes gets the FLOPs of one launch (not bytes)
            int sms = 0;
            CUIBM_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device));
            const int blocks = 8 * sms;  // 8 blocks of 256 threads per SM
            launch = [&, blocks] { b = launch_fp64_fma(c, blocks, c.work_y); };
        } else if (k == "poisson_vcycle") {
            if (c.sys2.amg.empty()) return fail(h, CUIBM_ERR_BAD_INPUT, "the Poisson system has no SA hierarchy");
            launch = [&] { launch_vcycle(c, c.sys2, c.work_x, c.work_y); };
            b = sa_vcycle_bytes(c.sys2);
        } else {
            return fail(h, CUIBM_ERR_BAD_INPUT, "unknown kernel " + k);
        }
        launch();  // warm
        CUIBM_TRY(cudaEventRecord(c.ev0, c.stream));
        for (int r = 0; r < reps; ++r) launch();
        CUIBM_TRY(cudaEventRecord(c.ev1, c.stream));
        CUIBM_TRY(cudaEventSynchronize(c.ev1));
        float ms = 0;
        CUIBM_TRY(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
        if (avg_ms) *avg_ms = ms / reps;
        if (bytes) *bytes = b;
    });
    return CUIBM_OK;
}

int cuibm_launch_count(cuibm_ctx *h, long long *per_step)
{
    if (!h || !h->c.initialised || !per_step) return CUIBM_ERR_STATE;
    Context &c = h->c;
    CUIBM_GUARD(h, {
        if (!c.step_exec) return fail(h, CUIBM_ERR_STATE, "launch counts need the step graph");
        if (strong_coupling(c))
            return fail(h, CUIBM_ERR_STATE, "a strongly coupled step's launches vary with its sub-iterations");
        *per_step = c.static_kernels + (long long)c.sys1.body_kernels * read_body_runs(c, c.sys1) +
                    (long long)c.sys2.body_kernels * read_body_runs(c, c.sys2);
    });
    return CUIBM_OK;
}

int cuibm_write_data(cuibm_ctx *h)
{
    if (!h || !h->c.initialised) return CUIBM_ERR_STATE;
    Context &c = h->c;
    CUIBM_GUARD(h, { write_step_output(c); });
    return CUIBM_OK;
}

int cuibm_shutdown(cuibm_ctx *h)
{
    if (!h) return CUIBM_ERR_STATE;
    Context &c = h->c;
    if (c.iterationsFile) fclose(c.iterationsFile);
    if (c.forceFile) fclose(c.forceFile);
    if (c.midPositionFile) fclose(c.midPositionFile);
    c.iterationsFile = c.forceFile = c.midPositionFile = nullptr;
    return CUIBM_OK;
}

struct HostCase {
    Params P;
    Axis gx, gy;
    BodyState body;
    BoundingBox bb;
};

static int host_case(const char *folder, int argc, const char **argv, HostCase &hc)
{
    std::string err = load_case(folder ? folder : ".", argc, argv, hc.P);
    if (err.empty()) err = build_axis(hc.P.axis[0], hc.gx);
    if (err.empty()) err = build_axis(hc.P.axis[1], hc.gy);
    if (err.empty()) err = build_bodies(hc.P.bodies, hc.body);
    if (!err.empty()) {
        g_create_error = err;
        return err.rfind("cannot open", 0) == 0 ? CUIBM_ERR_IO : CUIBM_ERR_BAD_INPUT;
    }
    if (hc.body.total > 0)
        hc.bb = bounding_box(hc.body.x.data(), hc.body.y.data(), hc.body.total, hc.gx, hc.gy, hc.P.scaleCV);
    return CUIBM_OK;
}

int cuibm_case_info(const char *folder, int argc, const char **argv, cuibm_info *info)
{
    if (!info) return CUIBM_ERR_BAD_INPUT;
    HostCase hc;
    int st = host_case(folder, argc, argv, hc);
    if (st != CUIBM_OK) return st;
    std::memset(info, 0, sizeof *info);
    const int nx = hc.gx.n, ny = hc.gy.n;
    info->nx = nx;
    info->ny = ny;
    info->numU = (nx - 1) * ny;
    info->numV = nx * (ny - 1);
    info->numUV = info->numU + info->numV;
    info->numP = nx * ny;
    info->solver_type = hc.P.solverType;
    info->time_step = hc.P.startStep;
    info->nt = hc.P.nt;
    info->nsave = hc.P.nsave;
    info->dt = hc.P.dt;
    info->nu = hc.P.nu;
    info->total_points = hc.body.total;
    info->bb_start_i = hc.bb.i0;
    info->bb_start_j = hc.bb.j0;
    info->bb_ncx = hc.bb.ncx;
    info->bb_ncy = hc.bb.ncy;
    info->nnz_lhs1 = (nx - 1) * ny * 5 - 2 * ny - 2 * (nx - 1) + (ny - 1) * nx * 5 - 2 * (ny - 1) - 2 * nx;
    info->nnz_lhs2 = 5 * nx * ny - 2 * ny - 2 * nx;
    info->velocity_precond = hc.P.velocity.precond;
    info->poisson_precond = hc.P.poisson.precond;
    info->velocity_krylov = hc.P.krylovVelocity;
    info->poisson_krylov = hc.P.krylovPoisson;
    info->velocity_precision = hc.P.velocity.precision;
    info->poisson_precision = hc.P.poisson.precision;
    return CUIBM_OK;
}

int cuibm_case_array(const char *folder, int argc, const char **argv, int field, double *dst, size_t count)
{
    HostCase hc;
    int st = host_case(folder, argc, argv, hc);
    if (st != CUIBM_OK) return st;
    const std::vector<double> *v = nullptr;
    switch (field) {
    case CUIBM_F_X: case CUIBM_F_XV: v = &hc.gx.centre; break;
    case CUIBM_F_DX: v = &hc.gx.width; break;
    case CUIBM_F_XU: v = &hc.gx.face; break;
    case CUIBM_F_Y: case CUIBM_F_YU: v = &hc.gy.centre; break;
    case CUIBM_F_DY: v = &hc.gy.width; break;
    case CUIBM_F_YV: v = &hc.gy.face; break;
    case CUIBM_F_BODY_X: v = &hc.body.x; break;
    case CUIBM_F_BODY_Y: v = &hc.body.y; break;
    default: g_create_error = "field not available from a case description"; return CUIBM_ERR_BAD_INPUT;
    }
    if (!dst || count != v->size()) {
        g_create_error = "count must be " + std::to_string(v->size());
        return CUIBM_ERR_BAD_INPUT;
    }
    std::memcpy(dst, v->data(), count * sizeof(double));
    return CUIBM_OK;
}

const char *cuibm_case_error(void) { return g_create_error.c_str(); }

int cuibm_adjoint(cuibm_ctx *h, int nsteps, int snapshots, const double *wx, const double *wy, double *J,
                  double *grad, size_t ngrad, cuibm_adjoint_stats *stats)
{
    if (!h || !h->c.initialised) return CUIBM_ERR_STATE;
    if (!wx || !wy || !grad) return fail(h, CUIBM_ERR_BAD_INPUT, "null weights or gradient array");
    Context &c = h->c;
    CUIBM_GUARD(h, {
        if (!(c.P.solverType == ST_OSC && c.has_body))
            return fail(h, CUIBM_ERR_UNSUPPORTED,
                        "the adjoint covers the embedded method (SolverType OSC_CYLINDER) with a body");
        AdjointStats st{};
        run_adjoint(c, nsteps, snapshots, wx, wy, J, grad, ngrad, c.adjoint_rtol, &st);
        if (stats) {
            stats->ms = st.ms;
            stats->forward_steps = st.forward_steps;
            stats->tape_steps = st.tape_steps;
            stats->velocity_iterations = st.velocity_iterations;
            stats->poisson_iterations = st.poisson_iterations;
            stats->solves_reused = st.solves_reused;
        }
    });
    return CUIBM_OK;
}

void cuibm_destroy(cuibm_ctx *h)
{
    if (!h) return;
    Context &c = h->c;
    cuibm_shutdown(h);
    if (c.stream) cudaStreamSynchronize(c.stream);
    if (c.step_exec) cudaGraphExecDestroy(c.step_exec);
    if (c.step_graph) cudaGraphDestroy(c.step_graph);
    free_sa_hierarchy(c.sys1);
    free_sa_hierarchy(c.sys2);
    free_fused(c.sys1);
    free_fused(c.sys2);
    free_adjoint(c);
    if (c.arena) cudaFree(c.arena);
    if (c.h_scalars) cudaFreeHost(c.h_scalars);
    if (c.ev0) cudaEventDestroy(c.ev0);
    if (c.ev1) cudaEventDestroy(c.ev1);
    if (c.side_stream) cudaStreamDestroy(c.side_stream);
    if (c.coupling_stream) cudaStreamDestroy(c.coupling_stream);
    if (c.stream) cudaStreamDestroy(c.stream);
    delete h;
}

}  // extern "C"
