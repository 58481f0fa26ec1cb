// Krylov solvers for LHS1 (velocity) and LHS2 (Poisson), replacing
// cusp::krylov::bicgstab under cusp::monitor (NavierStokesSolver.cu:221-271).
//
// GB300 design:
//  * every scalar of the recurrence (rho, alpha, omega, beta, norms, status,
//    iteration count) lives in device memory; no host round trip per iteration;
//  * each kernel fuses its vector update with the dot products that follow it:
//    per-block partial sums, then the last block to arrive (atomic counter)
//    reduces the partials in a fixed order - deterministic, one launch;
//  * the iteration loop is a CUDA-graph WHILE node: the kernel that tests
//    convergence sets the graph conditional, so a whole solve (and a whole time
//    step) is one graph launch with no host synchronisation;
//  * the Jacobi preconditioner is applied on the fly inside the operator rows.
//
// Semantics kept from the reference: stop when ||b - A x||_2 <= tol*||b||_2 or at
// maxIterations (status MAXIT, reported as CUIBM_ERR_NOT_CONVERGED where the
// reference calls std::exit(-1)); warm start from the current x; the iteration
// count is that of cusp::monitor (full iterations; BiCGSTAB's exit on the
// half-step residual does not count one).
//
// BiCGSTAB: right-preconditioned (van der Vorst 1992).  CG: on the symmetrised
// system (W A) x = W b with W = diag(w) the row weights that make the staggered
// operators symmetric (cell or face areas); convergence is still measured on the
// original residual b - A x = W^-1 r_sym.
#include <cmath>
#include <vector>

#include "amg.h"
#include "operators.cuh"
#include "solver.h"

namespace cuibm {

// ---- operators seen by the solver -------------------------------------------
struct Op1 {
    Lhs1Coef c;
    Grid g;
    const double *w;  // symmetrisation weights or nullptr
    template <class X>
    __device__ __forceinline__ double row(int i, const X &x) const
    {
        double y = lhs1_row_f(c, g, i, x);
        return w ? w[i] * y : y;
    }
};
struct Op2 {
    Lhs2Coef c;
    Grid g;
    const double *w;
    template <class X>
    __device__ __forceinline__ double row(int i, const X &x) const
    {
        double y = lhs2_row_f(c, g, i, x);
        return w ? w[i] * y : y;
    }
};

struct ScaledAccess {
    const double *__restrict__ p, *__restrict__ d;
    __device__ __forceinline__ double operator()(int j) const { return p[j] * d[j]; }
};

// ---- deterministic fused reduction --------------------------------------------
template <int NV>
__device__ __forceinline__ bool reduce_arrive(double (&v)[NV], double *partials, unsigned int *arrive,
                                              double (&tot)[NV])
{
    __shared__ double sh[NV][32];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double a = v[k];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) sh[k][wid] = a;
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double a = lane < nw ? sh[k][lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
            if (lane == 0) partials[blockIdx.x * 4 + k] = a;
        }
    }
    __threadfence();
    if (threadIdx.x == 0) is_last = (atomicAdd(arrive, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
    // fixed-order sum of the per-block partials
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double a = 0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) a += __ldcg(partials + b * 4 + k);
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) sh[k][wid] = a;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double a = 0;
        for (int q = 0; q < nw; ++q) a += sh[k][q];
        tot[k] = a;
    }
    if (threadIdx.x == 0) *arrive = 0;
    return true;
}

__device__ __forceinline__ void set_cond(cudaGraphConditionalHandle h, int use, unsigned int v)
{
    if (use) cudaGraphSetConditional(h, v);
}

__device__ __forceinline__ void finish_status(KrylovScalars *ks, int *err_word, int which)
{
    if (ks->status == KS_RUNNING) {
        // a non-finite residual or right-hand side (an overflowed field passes
        // ||r|| <= tol ||b|| as inf <= inf) is reported, not taken as convergence
        if (!isfinite(ks->rnorm) || !isfinite(ks->tol)) ks->status = KS_NAN;
        else if (ks->rnorm <= ks->tol) ks->status = KS_CONVERGED;
        else if (ks->it >= ks->maxit) ks->status = KS_MAXIT;
    }
    if ((ks->status == KS_MAXIT || ks->status == KS_NAN) && err_word && *err_word == 0)
        *err_word = which * 16 + ks->status;
}

// ---- BiCGSTAB -------------------------------------------------------------------
// PC: 0 none, 1 Jacobi (fused), 2 external (Mp / Ms written by a V-cycle beforehand)
template <class Op>
__global__ void __launch_bounds__(256) k_bicg_init(Op A, int n, const double *__restrict__ b, const double *x,
                                                   double *r, double *rs, double *p, double *partials,
                                                   KrylovScalars *ks, int *err, int which,
                                                   cudaGraphConditionalHandle h, int use_cond)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[3] = {0, 0, 0};
    if (i < n) {
        double bi = b[i], ri = bi - A.row(i, PtrAccess{x});
        r[i] = ri;
        rs[i] = ri;
        p[i] = ri;
        v[0] = ri * ri;
        v[1] = bi * bi;
    }
    double t[3];
    if (reduce_arrive<3>(v, partials, &ks->arrive, t) && threadIdx.x == 0) {
        ks->rho = t[0];
        ks->rnorm = sqrt(t[0]);
        ks->bnorm = sqrt(t[1]);
        ks->tol = ks->rtol * ks->bnorm;
        ks->it = 0;
        ks->s_done = 0;
        ks->body_runs = 0;
        ks->status = KS_RUNNING;
        finish_status(ks, err, which);
        set_cond(h, use_cond, ks->status == KS_RUNNING);
    }
}

template <class Op, int PC>
__global__ void __launch_bounds__(256) k_bicg_1(Op A, int n, const double *p, const double *__restrict__ dinv,
                                                double *Mp, double *AMp, const double *__restrict__ rs,
                                                double *partials, KrylovScalars *ks)
{
    if (ks->status != KS_RUNNING) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {0};
    if (i < n) {
        double a;
        if (PC == 1) {
            Mp[i] = p[i] * dinv[i];
            a = A.row(i, ScaledAccess{p, dinv});
        } else if (PC == 0) {
            Mp[i] = p[i];
            a = A.row(i, PtrAccess{p});
        } else {
            a = A.row(i, PtrAccess{Mp});
        }
        AMp[i] = a;
        v[0] = rs[i] * a;
    }
    double t[1];
    if (reduce_arrive<1>(v, partials, &ks->arrive, t) && threadIdx.x == 0) {
        ks->alpha = ks->rho / t[0];
        ks->s_done = 0;
        ks->body_runs += 1;
    }
}

__global__ void __launch_bounds__(256) k_bicg_2(int n, const double *__restrict__ r, const double *__restrict__ AMp,
                                                double *s, double *partials, KrylovScalars *ks)
{
    if (ks->status != KS_RUNNING) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double alpha = ks->alpha;
    double v[1] = {0};
    if (i < n) {
        double si = r[i] - alpha * AMp[i];
        s[i] = si;
        v[0] = si * si;
    }
    double t[1];
    if (reduce_arrive<1>(v, partials, &ks->arrive, t) && threadIdx.x == 0) {
        ks->snorm = sqrt(t[0]);
        ks->s_done = ks->snorm <= ks->tol;
    }
}

template <class Op, int PC>
__global__ void __launch_bounds__(256) k_bicg_3(Op A, int n, const double *s, const double *__restrict__ dinv,
                                                double *Ms, double *AMs, double *partials, KrylovScalars *ks)
{
    if (ks->status != KS_RUNNING || ks->s_done) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[2] = {0, 0};
    if (i < n) {
        double a;
        if (PC == 1) {
            Ms[i] = s[i] * dinv[i];
            a = A.row(i, ScaledAccess{s, dinv});
        } else if (PC == 0) {
            Ms[i] = s[i];
            a = A.row(i, PtrAccess{s});
        } else {
            a = A.row(i, PtrAccess{Ms});
        }
        AMs[i] = a;
        v[0] = a * s[i];
        v[1] = a * a;
    }
    double t[2];
    if (reduce_arrive<2>(v, partials, &ks->arrive, t) && threadIdx.x == 0) ks->omega = t[0] / t[1];
}

__global__ void __launch_bounds__(256) k_bicg_4(int n, double *x, double *r, const double *__restrict__ rs,
                                                const double *__restrict__ s, const double *__restrict__ Mp,
                                                const double *__restrict__ Ms, const double *__restrict__ AMs,
                                                double *partials, KrylovScalars *ks, int *err, int which,
                                                cudaGraphConditionalHandle h, int use_cond)
{
    if (ks->status != KS_RUNNING) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double alpha = ks->alpha, omega = ks->omega;
    const int sd = ks->s_done;
    double v[2] = {0, 0};
    if (i < n) {
        if (sd) {
            x[i] += alpha * Mp[i];
        } else {
            x[i] += alpha * Mp[i] + omega * Ms[i];
            double ri = s[i] - omega * AMs[i];
            r[i] = ri;
            v[0] = rs[i] * ri;
            v[1] = ri * ri;
        }
    }
    double t[2];
    if (reduce_arrive<2>(v, partials, &ks->arrive, t) && threadIdx.x == 0) {
        if (sd) {
            ks->rnorm = ks->snorm;
            ks->status = KS_CONVERGED;
        } else {
            ks->beta = (t[0] / ks->rho) * (alpha / omega);
            ks->rho = t[0];
            ks->it += 1;
            ks->rnorm = sqrt(t[1]);
            finish_status(ks, err, which);
        }
        set_cond(h, use_cond, ks->status == KS_RUNNING);
    }
}

__global__ void __launch_bounds__(256) k_bicg_5(int n, double *p, const double *__restrict__ r,
                                                const double *__restrict__ AMp, const KrylovScalars *ks)
{
    if (ks->status != KS_RUNNING) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = r[i] + ks->beta * (p[i] - ks->omega * AMp[i]);
}

// ---- CG on the symmetrised system -------------------------------------------------
template <class Op, int PC>
__global__ void __launch_bounds__(256) k_cg_init(Op A, int n, const double *__restrict__ b,
                                                 const double *__restrict__ w, const double *x, double *r,
                                                 double *z, double *p, const double *__restrict__ dinv,
                                                 double *partials, KrylovScalars *ks, int *err, int which,
                                                 cudaGraphConditionalHandle h, int use_cond)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[3] = {0, 0, 0};
    if (i < n) {
        double bi = b[i], ri = w[i] * bi - A.row(i, PtrAccess{x});
        r[i] = ri;
        double ro = ri / w[i];
        v[0] = ro * ro;
        v[1] = bi * bi;
        if (PC != 2) {
            double zi = PC == 1 ? ri * dinv[i] : ri;
            z[i] = zi;
            p[i] = zi;
            v[2] = ri * zi;
        }
    }
    double t[3];
    if (reduce_arrive<3>(v, partials, &ks->arrive, t) && threadIdx.x == 0) {
        ks->rnorm = sqrt(t[0]);
        ks->bnorm = sqrt(t[1]);
        ks->rho = t[2];
        ks->tol = ks->rtol * ks->bnorm;
        ks->it = 0;
        ks->body_runs = 0;
        ks->status = KS_RUNNING;
        finish_status(ks, err, which);
        set_cond(h, use_cond, ks->status == KS_RUNNING);
    }
}

template <class Op>
__global__ void __launch_bounds__(256) k_cg_1(Op A, int n, const double *p, double *q, double *partials,
                                              KrylovScalars *ks)
{
    if (ks->status != KS_RUNNING) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {0};
    if (i < n) {
        double qi = A.row(i, PtrAccess{p});
        q[i] = qi;
        v[0] = p[i] * qi;
    }
    double t[1];
    if (reduce_arrive<1>(v, partials, &ks->arrive, t) && threadIdx.x == 0) {
        ks->alpha = ks->rho / t[0];
        ks->body_runs += 1;
    }
}

// x += alpha p; r -= alpha q; (PC<2) z = M r and r.z; residual norm of the original system
template <int PC>
__global__ void __launch_bounds__(256) k_cg_2(int n, double *x, double *r, double *z, const double *__restrict__ p,
                                              const double *__restrict__ q, const double *__restrict__ w,
                                              const double *__restrict__ dinv, double *partials,
                                              KrylovScalars *ks, int *err, int which,
                                              cudaGraphConditionalHandle h, int use_cond)
{
    if (ks->status != KS_RUNNING) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double alpha = ks->alpha;
    double v[2] = {0, 0};
    if (i < n) {
        x[i] += alpha * p[i];
        double ri = r[i] - alpha * q[i];
        r[i] = ri;
        double ro = ri / w[i];
        v[0] = ro * ro;
        if (PC != 2) {
            double zi = PC == 1 ? ri * dinv[i] : ri;
            z[i] = zi;
            v[1] = ri * zi;
        }
    }
    double t[2];
    if (reduce_arrive<2>(v, partials, &ks->arrive, t) && threadIdx.x == 0) {
        ks->it += 1;
        ks->rnorm = sqrt(t[0]);
        if (PC != 2) {
            ks->beta = t[1] / ks->rho;
            ks->rho = t[1];
        }
        finish_status(ks, err, which);
        set_cond(h, use_cond, ks->status == KS_RUNNING);
    }
}

// external preconditioner: rho_new = r.z, beta (first=1: p = z, rho = r.z)
__global__ void __launch_bounds__(256) k_cg_rz(int n, const double *__restrict__ r, const double *__restrict__ z,
                                               double *partials, KrylovScalars *ks)
{
    if (ks->status != KS_RUNNING) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {0};
    if (i < n) v[0] = r[i] * z[i];
    double t[1];
    if (reduce_arrive<1>(v, partials, &ks->arrive, t) && threadIdx.x == 0) {
        ks->beta = ks->it == 0 ? 0.0 : t[0] / ks->rho;
        ks->rho = t[0];
    }
}

__global__ void __launch_bounds__(256) k_cg_3(int n, double *p, const double *__restrict__ z,
                                              const KrylovScalars *ks)
{
    if (ks->status != KS_RUNNING) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = ks->it == 0 ? z[i] : z[i] + ks->beta * p[i];
}

// Jacobi of the (possibly symmetrised) operator: dinv = 1 / (w a_ii)
template <class Op>
__global__ void k_dinv(Op A, int n, double *dinv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double d = A.row(i, [&](int j) { return j == i ? 1.0 : 0.0; });
    dinv[i] = d != 0 ? 1.0 / d : 1.0;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static Op1 op1(Context &c, const double *w) { return Op1{c.l1, c.g, w}; }
static Op2 op2(Context &c, const double *w) { return Op2{c.l2, c.g, w}; }

// Row weights that make the operators symmetric: LHS1 u rows (dx[I]+dx[I+1])/2*dy[J],
// v rows dx[I]*(dy[J]+dy[J+1])/2; LHS2 rows dx[I]*dy[J].
static std::vector<double> sym_weights(Context &c, int which)
{
    const int nx = c.g.nx, ny = c.g.ny;
    const auto &dx = c.gx.width, &dy = c.gy.width;
    std::vector<double> w;
    if (which == 1) {
        w.resize(c.g.nUV);
        for (int J = 0; J < ny; ++J)
            for (int I = 0; I < nx - 1; ++I) w[J * (nx - 1) + I] = (dx[I] + dx[I + 1]) * 0.5 * dy[J];
        for (int J = 0; J < ny - 1; ++J)
            for (int I = 0; I < nx; ++I) w[c.g.nU + J * nx + I] = dx[I] * (dy[J] + dy[J + 1]) * 0.5;
    } else {
        w.resize(c.g.nP);
        for (int J = 0; J < ny; ++J)
            for (int I = 0; I < nx; ++I) w[J * nx + I] = dx[I] * dy[J];
    }
    return w;
}

void setup_system(Context &c, LinearSystem &S)
{
    const LinearSolve &L = S.which == 1 ? c.P.velocity : c.P.poisson;
    S.n = S.which == 1 ? c.g.nUV : c.g.nP;
    S.krylov = S.which == 1 ? c.P.krylovVelocity : c.P.krylovPoisson;
    S.precond = L.precond;
    S.rtol = L.tolerance;
    S.maxit = L.maxIterations;
    S.precision = L.precision;
    // unset threshold: CUSP's 0, but 0.05 for a moving embedded body (its SA-preconditioned
    // Poisson solves stalled or broke down with 0 on the oscillating-cylinder cases)
    S.strength = L.strength >= 0 ? L.strength
                                 : (c.P.solverType == ST_OSC && c.has_body && body_moves(c) ? 0.05 : 0.0);
    if (S.precond == PC_AINV)
        throw InputError("preconditioner AINV is not implemented by libcuibm_gb300; use DIAGONAL or SMOOTHED_AGGREGATION");
    const int n = S.n;
    S.r = c.carve<double>(n);
    S.rs = c.carve<double>(n);
    S.p = c.carve<double>(n);
    S.Mp = c.carve<double>(n);
    S.AMp = c.carve<double>(n);
    S.s = c.carve<double>(n);
    S.Ms = c.carve<double>(n);
    S.AMs = c.carve<double>(n);
    S.z = S.Ms;
    S.q = S.AMs;
    S.dinv = c.carve<double>(n);
    S.partials = c.carve<double>(4 * (size_t)blocks_for(n) + 4);
    S.ks = c.carve<KrylovScalars>(1);
    {
        KrylovScalars hk{};
        hk.rtol = S.rtol;
        hk.maxit = S.maxit;
        // mixed precision by refinement: each FP32 solve is asked for a 1e-3 reduction at
        // least and stops after 100 iterations (FP32 recurrences stall near their
        // attainable accuracy; the FP64 refinement then goes on from a fresh residual)
        hk.inner_rtol = 1e-3;
        hk.inner_maxit = 100;
        hk.status = KS_CONVERGED;
        CUIBM_TRY(cudaMemcpy(S.ks, &hk, sizeof(hk), cudaMemcpyHostToDevice));
    }
    S.w = nullptr;
    if (S.krylov == KRYLOV_CG) {
        std::vector<double> w = sym_weights(c, S.which);
        S.w = c.carve<double>(n);
        CUIBM_TRY(cudaMemcpyAsync(S.w, w.data(), n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    }
    if (S.which == 1)
        k_dinv<<<blocks_for(n), kBlock, 0, c.stream>>>(op1(c, S.w), n, S.dinv);
    else
        k_dinv<<<blocks_for(n), kBlock, 0, c.stream>>>(op2(c, S.w), n, S.dinv);
    CUIBM_TRY(cudaGetLastError());
    if (S.precond == PC_SMOOTHED_AGGREGATION) build_sa_hierarchy(c, S);
    setup_fused(c, S);
}

// level 0 of the SA hierarchy: Jacobi smoother tables from the operator's new diagonal
// (the hierarchy below keeps the operator it was built from)
__global__ void k_sa_level0_tables(int n, const double *__restrict__ dinv, double omega, double *__restrict__ l0dinv,
                                   double *__restrict__ l0wd)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    l0dinv[i] = dinv[i];
    if (l0wd) l0wd[i] = omega * dinv[i];
}

// The operator's rows changed (the embedded method's rows after a body moved): the
// Jacobi table, the persistent solver's diagonal and the SA smoother's level-0 tables
// follow.  The reference rebuilds its whole preconditioner each step; here the SA
// hierarchy is rebuilt between steps when the set of patched rows changes
// (rebuild_hierarchies in context.cu).
void refresh_system_diagonals(Context &c, LinearSystem &S)
{
    const int n = S.n;
    if (S.which == 1)
        k_dinv<<<blocks_for(n), kBlock, 0, c.stream>>>(op1(c, S.w), n, S.dinv);
    else
        k_dinv<<<blocks_for(n), kBlock, 0, c.stream>>>(op2(c, S.w), n, S.dinv);
    CUIBM_TRY(cudaGetLastError());
    refresh_fused_diag(c, S);
    if (!S.amg.empty() && S.amg[0]->n == n) {
        SaLevel *L = S.amg[0];
        k_sa_level0_tables<<<blocks_for(n), kBlock, 0, c.stream>>>(n, S.dinv, L->omega, L->dinv, L->wd);
        CUIBM_TRY(cudaGetLastError());
        refresh_fused_level0(c, S);
    }
}

struct SolveLauncher {
    Context &c;
    LinearSystem &S;
    const double *b;
    double *x;
    int *err;
    cudaGraphConditionalHandle h;
    int use_cond;

    template <class Op>
    void init(Op A)
    {
        const int n = S.n, nb = blocks_for(n);
        if (S.krylov == KRYLOV_BICGSTAB) {
            k_bicg_init<<<nb, kBlock, 0, c.stream>>>(A, n, b, x, S.r, S.rs, S.p, S.partials, S.ks, err, S.which, h,
                                                     use_cond);
        } else if (S.precond == PC_SMOOTHED_AGGREGATION) {
            k_cg_init<Op, 2><<<nb, kBlock, 0, c.stream>>>(A, n, b, S.w, x, S.r, S.z, S.p, S.dinv, S.partials, S.ks,
                                                         err, S.which, h, use_cond);
        } else if (S.precond == PC_DIAGONAL) {
            k_cg_init<Op, 1><<<nb, kBlock, 0, c.stream>>>(A, n, b, S.w, x, S.r, S.z, S.p, S.dinv, S.partials, S.ks,
                                                         err, S.which, h, use_cond);
        } else {
            k_cg_init<Op, 0><<<nb, kBlock, 0, c.stream>>>(A, n, b, S.w, x, S.r, S.z, S.p, S.dinv, S.partials, S.ks,
                                                         err, S.which, h, use_cond);
        }
        CUIBM_TRY(cudaGetLastError());
        if (S.krylov == KRYLOV_CG && S.precond == PC_SMOOTHED_AGGREGATION) {
            // z = M r, rho = r.z, p = z
            launch_vcycle(c, S, S.r, S.z);
            k_cg_rz<<<nb, kBlock, 0, c.stream>>>(n, S.r, S.z, S.partials, S.ks);
            k_cg_3<<<nb, kBlock, 0, c.stream>>>(n, S.p, S.z, S.ks);
            CUIBM_TRY(cudaGetLastError());
        }
    }

    template <class Op>
    void body(Op A)
    {
        const int n = S.n, nb = blocks_for(n);
        if (S.krylov == KRYLOV_BICGSTAB) {
            if (S.precond == PC_SMOOTHED_AGGREGATION) {
                launch_vcycle(c, S, S.p, S.Mp);
                k_bicg_1<Op, 2><<<nb, kBlock, 0, c.stream>>>(A, n, S.p, S.dinv, S.Mp, S.AMp, S.rs, S.partials, S.ks);
            } else if (S.precond == PC_DIAGONAL) {
                k_bicg_1<Op, 1><<<nb, kBlock, 0, c.stream>>>(A, n, S.p, S.dinv, S.Mp, S.AMp, S.rs, S.partials, S.ks);
            } else {
                k_bicg_1<Op, 0><<<nb, kBlock, 0, c.stream>>>(A, n, S.p, S.dinv, S.Mp, S.AMp, S.rs, S.partials, S.ks);
            }
            k_bicg_2<<<nb, kBlock, 0, c.stream>>>(n, S.r, S.AMp, S.s, S.partials, S.ks);
            if (S.precond == PC_SMOOTHED_AGGREGATION) {
                launch_vcycle(c, S, S.s, S.Ms);
                k_bicg_3<Op, 2><<<nb, kBlock, 0, c.stream>>>(A, n, S.s, S.dinv, S.Ms, S.AMs, S.partials, S.ks);
            } else if (S.precond == PC_DIAGONAL) {
                k_bicg_3<Op, 1><<<nb, kBlock, 0, c.stream>>>(A, n, S.s, S.dinv, S.Ms, S.AMs, S.partials, S.ks);
            } else {
                k_bicg_3<Op, 0><<<nb, kBlock, 0, c.stream>>>(A, n, S.s, S.dinv, S.Ms, S.AMs, S.partials, S.ks);
            }
            k_bicg_4<<<nb, kBlock, 0, c.stream>>>(n, x, S.r, S.rs, S.s, S.Mp, S.Ms, S.AMs, S.partials, S.ks, err,
                                                  S.which, h, use_cond);
            k_bicg_5<<<nb, kBlock, 0, c.stream>>>(n, S.p, S.r, S.AMp, S.ks);
        } else {
            k_cg_1<<<nb, kBlock, 0, c.stream>>>(A, n, S.p, S.q, S.partials, S.ks);
            if (S.precond == PC_SMOOTHED_AGGREGATION) {
                k_cg_2<2><<<nb, kBlock, 0, c.stream>>>(n, x, S.r, S.z, S.p, S.q, S.w, S.dinv, S.partials, S.ks, err,
                                                       S.which, h, use_cond);
                launch_vcycle(c, S, S.r, S.z);
                k_cg_rz<<<nb, kBlock, 0, c.stream>>>(n, S.r, S.z, S.partials, S.ks);
            } else if (S.precond == PC_DIAGONAL) {
                k_cg_2<1><<<nb, kBlock, 0, c.stream>>>(n, x, S.r, S.z, S.p, S.q, S.w, S.dinv, S.partials, S.ks, err,
                                                       S.which, h, use_cond);
            } else {
                k_cg_2<0><<<nb, kBlock, 0, c.stream>>>(n, x, S.r, S.z, S.p, S.q, S.w, S.dinv, S.partials, S.ks, err,
                                                       S.which, h, use_cond);
            }
            k_cg_3<<<nb, kBlock, 0, c.stream>>>(n, S.p, S.z, S.ks);
        }
        CUIBM_TRY(cudaGetLastError());
    }
};

// Launch a full solve on c.stream.  in_graph: the stream is being captured; the
// iteration loop becomes a WHILE conditional node.  Otherwise the host drives
// the loop and polls the status every few iterations.
void launch_solve(Context &c, LinearSystem &S, const double *b, double *x, bool in_graph)
{
    int *err = c.err_word;
    // a hierarchy without the body's rows (sa_body_free) cycles with the stepwise kernels,
    // whose level-0 residual is the current operator's (the persistent cycle's stored
    // A0 P is the hierarchy's own level-0 operator)
    if (c.fused_solve && S.fused_fn && !S.sa_body_free) {
        launch_fused_solve(c, S, b, x);
        S.body_kernels = 0;
        return;
    }
    if (in_graph) {
        cudaStreamCaptureStatus st;
        cudaGraph_t graph;
        const cudaGraphNode_t *deps = nullptr;
        size_t ndeps = 0;
        CUIBM_TRY(cudaStreamGetCaptureInfo(c.stream, &st, nullptr, &graph, &deps, nullptr, &ndeps));
        cudaGraphConditionalHandle h;
        CUIBM_TRY(cudaGraphConditionalHandleCreate(&h, graph, 0, 0));
        SolveLauncher L{c, S, b, x, err, h, 1};
        if (S.which == 1) L.init(op1(c, S.w)); else L.init(op2(c, S.w));
        // WHILE node after the init kernels
        CUIBM_TRY(cudaStreamGetCaptureInfo(c.stream, &st, nullptr, &graph, &deps, nullptr, &ndeps));
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        CUIBM_TRY(cudaGraphAddNode(&node, graph, deps, nullptr, ndeps, &cp));
        cudaGraph_t bodyg = cp.conditional.phGraph_out[0];
        // capture one iteration into the body graph on a side stream
        cudaStream_t side = c.side_stream;
        cudaStream_t main = c.stream;
        CUIBM_TRY(cudaStreamBeginCaptureToGraph(side, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
        c.stream = side;
        try {
            if (S.which == 1) L.body(op1(c, S.w)); else L.body(op2(c, S.w));
        } catch (...) {
            c.stream = main;
            cudaGraph_t dummy;
            cudaStreamEndCapture(side, &dummy);
            throw;
        }
        c.stream = main;
        cudaGraph_t got;
        CUIBM_TRY(cudaStreamEndCapture(side, &got));
        S.body_kernels = count_kernel_nodes(got);
        CUIBM_TRY(cudaStreamUpdateCaptureDependencies(c.stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    } else {
        SolveLauncher L{c, S, b, x, err, 0, 0};
        if (S.which == 1) L.init(op1(c, S.w)); else L.init(op2(c, S.w));
        KrylovScalars host{};
        const int chunk = 4;
        for (int done = 0; done <= S.maxit + chunk; done += chunk) {
            for (int k = 0; k < chunk; ++k) {
                if (S.which == 1) L.body(op1(c, S.w)); else L.body(op2(c, S.w));
            }
            CUIBM_TRY(cudaMemcpyAsync(&host, S.ks, sizeof(host), cudaMemcpyDeviceToHost, c.stream));
            CUIBM_TRY(cudaStreamSynchronize(c.stream));
            if (host.status != KS_RUNNING) break;
        }
    }
}

int count_kernel_nodes(cudaGraph_t g)
{
    size_t n = 0;
    CUIBM_TRY(cudaGraphGetNodes(g, nullptr, &n));
    std::vector<cudaGraphNode_t> nodes(n);
    if (n) CUIBM_TRY(cudaGraphGetNodes(g, nodes.data(), &n));
    int k = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        CUIBM_TRY(cudaGraphNodeGetType(nd, &t));
        if (t == cudaGraphNodeTypeKernel) ++k;
    }
    return k;
}

int read_body_runs(Context &c, LinearSystem &S)
{
    KrylovScalars host{};
    CUIBM_TRY(cudaMemcpyAsync(&host, S.ks, sizeof(host), cudaMemcpyDeviceToHost, c.stream));
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
    return host.body_runs;
}

int read_solve_status(Context &c, LinearSystem &S, int *iterations)
{
    KrylovScalars host{};
    FusedSyncState fs{};
    CUIBM_TRY(cudaMemcpyAsync(&host, S.ks, sizeof(host), cudaMemcpyDeviceToHost, c.stream));
    if (S.fsync) CUIBM_TRY(cudaMemcpyAsync(&fs, S.fsync, sizeof(fs), cudaMemcpyDeviceToHost, c.stream));
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
    if (iterations) *iterations = host.it;
    return fs.abort ? KS_TIMEOUT : host.status;
}

// ---- transposed solves (discrete adjoint) -------------------------------------------
__global__ void k_apply_op(Op1T A, int n, const double *__restrict__ x, double *__restrict__ y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = A.row(i, PtrAccess{x});
}
__global__ void k_apply_op(Op2T A, int n, const double *__restrict__ x, double *__restrict__ y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = A.row(i, PtrAccess{x});
}

// The transposed system S of the forward system F: its own Krylov vectors and scalars,
// F's Jacobi table (A and A^T share their diagonal) and, for the Poisson system, F's SA
// hierarchy.  Allocated with cudaMalloc (the context's arena is sized at initialise);
// the pointers go to allocs for the caller to free.
void setup_transposed_system(Context &c, const LinearSystem &F, LinearSystem &S, std::vector<void *> &allocs)
{
    auto dalloc = [&](size_t bytes) {
        void *p = nullptr;
        CUIBM_TRY(cudaMalloc(&p, bytes));
        allocs.push_back(p);
        return p;
    };
    S.which = F.which;
    S.n = F.n;
    S.krylov = KRYLOV_BICGSTAB;
    S.precond = F.precond == PC_SMOOTHED_AGGREGATION && !F.amg.empty() ? PC_SMOOTHED_AGGREGATION : PC_DIAGONAL;
    const size_t n = S.n;
    double *blk = static_cast<double *>(dalloc(8 * n * sizeof(double)));
    S.r = blk;
    S.rs = blk + n;
    S.p = blk + 2 * n;
    S.Mp = blk + 3 * n;
    S.AMp = blk + 4 * n;
    S.s = blk + 5 * n;
    S.Ms = blk + 6 * n;
    S.AMs = blk + 7 * n;
    S.z = S.Ms;
    S.q = S.AMs;
    S.dinv = F.dinv;
    S.w = nullptr;
    S.partials = static_cast<double *>(dalloc((4 * (size_t)blocks_for(S.n) + 4) * sizeof(double)));
    S.ks = static_cast<KrylovScalars *>(dalloc(sizeof(KrylovScalars)));
    KrylovScalars hk{};
    hk.rtol = S.rtol;
    hk.maxit = S.maxit;
    hk.status = KS_CONVERGED;
    CUIBM_TRY(cudaMemcpy(S.ks, &hk, sizeof(hk), cudaMemcpyHostToDevice));
    S.amg = F.amg;
}

template <class Op>
static void transposed_iterations(Context &c, LinearSystem &S, Op A, const TransposeList &T, const double *b,
                                  double *x)
{
    const int n = S.n, nb = blocks_for(n);
    const bool sa = S.precond == PC_SMOOTHED_AGGREGATION;
    auto precond = [&](const double *in, double *out) { launch_vcycle_transposed(c, S, T, in, out); };
    k_bicg_init<<<nb, kBlock, 0, c.stream>>>(A, n, b, x, S.r, S.rs, S.p, S.partials, S.ks, nullptr, S.which, 0, 0);
    CUIBM_TRY(cudaGetLastError());
    KrylovScalars host{};
    const int chunk = 4;
    for (int done = 0; done <= S.maxit + chunk; done += chunk) {
        for (int k = 0; k < chunk; ++k) {
            if (sa) {
                precond(S.p, S.Mp);
                k_bicg_1<Op, 2><<<nb, kBlock, 0, c.stream>>>(A, n, S.p, S.dinv, S.Mp, S.AMp, S.rs, S.partials, S.ks);
            } else {
                k_bicg_1<Op, 1><<<nb, kBlock, 0, c.stream>>>(A, n, S.p, S.dinv, S.Mp, S.AMp, S.rs, S.partials, S.ks);
            }
            k_bicg_2<<<nb, kBlock, 0, c.stream>>>(n, S.r, S.AMp, S.s, S.partials, S.ks);
            if (sa) {
                precond(S.s, S.Ms);
                k_bicg_3<Op, 2><<<nb, kBlock, 0, c.stream>>>(A, n, S.s, S.dinv, S.Ms, S.AMs, S.partials, S.ks);
            } else {
                k_bicg_3<Op, 1><<<nb, kBlock, 0, c.stream>>>(A, n, S.s, S.dinv, S.Ms, S.AMs, S.partials, S.ks);
            }
            k_bicg_4<<<nb, kBlock, 0, c.stream>>>(n, x, S.r, S.rs, S.s, S.Mp, S.Ms, S.AMs, S.partials, S.ks,
                                                  nullptr, S.which, 0, 0);
            k_bicg_5<<<nb, kBlock, 0, c.stream>>>(n, S.p, S.r, S.AMp, S.ks);
        }
        CUIBM_TRY(cudaGetLastError());
        CUIBM_TRY(cudaMemcpyAsync(&host, S.ks, sizeof(host), cudaMemcpyDeviceToHost, c.stream));
        CUIBM_TRY(cudaStreamSynchronize(c.stream));
        if (host.status != KS_RUNNING) break;
    }
}

// A^T x = b for system S.which, warm-started from x; returns the KStatus and the
// iteration count.  The Poisson system's preconditioner is the transposed cycle of the
// forward SA hierarchy (the same aggregates and prolongators, transposed level matrices).
int launch_solve_transposed(Context &c, LinearSystem &S, LinearSystem &F, const TransposeList &T, const double *b,
                            double *x, int *iterations)
{
    S.amg = F.amg;  // the forward hierarchy (rebuilt for a moving body between steps)
    if (S.precond == PC_SMOOTHED_AGGREGATION) ensure_transposed_levels(c, F);
    KrylovScalars hk{};
    CUIBM_TRY(cudaMemcpyAsync(&hk, S.ks, sizeof(hk), cudaMemcpyDeviceToHost, c.stream));
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
    hk.rtol = S.rtol;
    hk.maxit = S.maxit;
    CUIBM_TRY(cudaMemcpyAsync(S.ks, &hk, sizeof(hk), cudaMemcpyHostToDevice, c.stream));
    if (S.which == 1)
        transposed_iterations(c, S, Op1T{c.l1, c.g, T}, T, b, x);
    else
        transposed_iterations(c, S, Op2T{c.l2, c.g, T}, T, b, x);
    KrylovScalars host{};
    CUIBM_TRY(cudaMemcpyAsync(&host, S.ks, sizeof(host), cudaMemcpyDeviceToHost, c.stream));
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
    if (iterations) *iterations = host.it;
    return host.status;
}

// y = A^T x (which 1: LHS1, 2: LHS2)
void launch_apply_transposed(Context &c, int which, const TransposeList &T, const double *x, double *y)
{
    if (which == 1)
        k_apply_op<<<blocks_for(c.g.nUV), kBlock, 0, c.stream>>>(Op1T{c.l1, c.g, T}, c.g.nUV, x, y);
    else
        k_apply_op<<<blocks_for(c.g.nP), kBlock, 0, c.stream>>>(Op2T{c.l2, c.g, T}, c.g.nP, x, y);
    CUIBM_TRY(cudaGetLastError());
}

}  // namespace cuibm
