#pragma once
// Persistent linear solves, the device side (shared by the translation units that
// instantiate the kernels - fused_op1.cu, fused_op2.cu, fused_mixed_op1.cu,
// fused_mixed_op2.cu; the host side is fused_solve.cu).  One cooperative launch runs
// a whole Krylov solve of LHS1 or LHS2 - BiCGSTAB or CG, with no, Jacobi or smoothed-aggregation
// V-cycle preconditioning - replacing cusp::krylov::bicgstab under
// cusp::monitor (NavierStokesSolver.cu:221-271) and CUSP's SA cycle.
//
// Why: at the sizes the solver runs (10^4..10^6 unknowns) one Krylov
// iteration is a few microseconds of memory and FP64 work split over a dozen
// dependent phases (SpMV, dot products, one sweep per multigrid level), so a
// launch per phase is dominated by launch and drain latency.  Here the blocks
// of one co-resident grid (cudaLaunchAttributeCooperative, so all of them are
// on the GPU at once) stay alive for the whole solve and meet at grid-wide
// barriers between phases.  Dot products reduce in a fixed order (per-block
// partials, then every block sums the partials of all blocks in index order), so
// every block holds the same scalars and takes the same branch, and results are
// deterministic run to run.
//
// GB300 issues about two FP64 operations per clock per SM, so at these sizes a
// phase costs its barrier plus roughly 0.1-0.2 us per FP64 operation per row;
// the layout of the work follows from that:
//  * per-row tables replace arithmetic: the operator diagonal (summed once in
//    the reference's order), omega D^-1 per multigrid level, 1 / w for CG;
//  * vector updates are folded into the phase that consumes them (the new
//    BiCGSTAB direction r + beta (p - omega A M p) and the half step
//    r - alpha A M p are formed at the stencil points of the next operator
//    application; vectors updated that way are double-buffered);
//  * the V-cycle has one barrier per level on the way up: x_l = w D^-1 b_l +
//    P x_l+1 and the post-smoothing residual b_l - A_l x_l = r_l - (A_l P_l)
//    x_l+1 use the residual r_l kept from the way down and the product A_l P_l
//    formed at set-up, so no row needs its neighbours' new values;
//  * CSR rows of the coarse levels are split over groups of lanes, so their
//    loads overlap instead of forming one dependent chain per row.
// Recurrences, stopping rule (||b - A x||_2 <= tol*||b||_2, the residual of the
// original system for CG on the symmetrised one), warm start and iteration
// count are those of the stepwise kernels in krylov.cu; results agree with them
// to rounding.
//
// Mixed precision (a linear solver's `precision: MIXED`).  The Krylov code is also
// instantiated for float vectors, operator tables and multigrid levels (dot products
// still reduce in double), in two arrangements:
//  * with the SA preconditioner (k_fused_mixed): an FP64 BiCGSTAB - residuals, dot
//    products, updates and the stopping rule in FP64 - whose V-cycles run in FP32
//    except the coarsest dense solve.  The pressure operator is nearly singular (its
//    near-null space is the constant, pinned at one cell), and FP32 rounding inside
//    the cycle leaves a spurious constant in its output; each preconditioned vector z
//    therefore gets its constant component re-solved in FP64, z = y + c e with
//    c = (e.r - w.y) / E, w = A^T e, E = e^T A e - the coarse correction of the
//    constant mode, which makes e^T (A z - r) = 0 whatever y's constant;
//  * otherwise (k_fused_ir): iterative refinement around FP32 Krylov solves - the
//    residual r = b - A x, its norm and the stopping test in FP64, an FP32 solve of
//    A d = r to a relative tolerance of max(tol / (2 ||r||), 1e-3) in at most 100
//    iterations, x += d in FP64 - until the FP64 residual meets the tolerance.
// The FP64 work moves out of the preconditioner (most of an SA iteration) or out of
// the whole iteration (refinement), and FP32 vectors and matrix values take half the
// bytes; GB300's FP32 rate is about fifty times its FP64 rate.
//
// Barrier waits are bounded: a block that waits more than kBarrierTimeoutNs
// sets the abort word and returns, every other block leaves at its next
// barrier, and the host reports the failure.  Vectors written inside the
// kernel are read with ld.global.cg (L2, coherent across blocks); only tables
// that no block writes go through L1.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <vector>

#include "amg.h"
#include "operators.cuh"
#include "structured.cuh"
#include "solver.h"

namespace cuibm {

constexpr int kFT = 512;  // threads per block at most (the default; -solverThreads asks fewer)
constexpr int kMaxLevels = 10;
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;  // 2 s
constexpr int kGroupR = 8;  // lanes per restriction row (15-30 entries)
constexpr int kGroupA = 4;  // lanes per coarse-operator row (9-25 entries)

template <class T>
struct CsrV {
    int n, nnz;
    const int *ptr, *col;
    const T *val;
};

template <class T>
struct FLevel {
    int n;
    CsrV<T> A, P, R, AP;
    const T *wd;  // omega D^-1
    T *x, *b, *r, *t;
    const double *inv;  // coarsest level: dense inverse, FP64 in every precision (dense_solve)
    // structured hierarchy (structured.cuh): the level's grid, its 9-point operator
    // (below level 0) and its prolongator's weights
    int nx, ny;
    const T *c9, *pw;
    int fz;  // structured: prolongation and smoothing sweep in one phase
    int rg;  // structured: the restriction into this level's coarser one, 8 lanes a coarse node
};

// Everything a solve needs except its right-hand side and solution, built once
// per system and kept in device memory (the kernel reads it through a pointer:
// a struct this size indexed by level would otherwise be copied to local memory).
template <class T>
struct FArgs {
    int n;
    T *r, *rs, *p, *p2, *Mp, *AMp, *AMp2, *s, *Ms, *AMs, *z, *q;
    const T *dinv, *w, *winv, *diag;
    double *partials;  // 2 x gridDim x 4
    FusedSyncState *sync;
    unsigned long long *trace;  // [count, stamps...] of kTraceLen, or null
    KrylovScalars *ks;
    int *err;
    int which;
    int nlev;
    int st;  // the hierarchy is the structured one
    // the level-0 first sweep of the BiCGSTAB cycles in a phase of its own, from the
    // stored direction or half step, instead of recomputing them at its stencil points
    // inside the phase that writes them (large FP64 systems: the recomputation costs
    // more FP64 issue than the extra barrier)
    int split0;
    // Jacobi BiCGSTAB: the direction and the half step folded into the phases that apply
    // A to their scaled values, recomputed at the stencil points (FP32 solves; FP64 below
    // kFoldMax unknowns, none by default)
    int fold1;
    FLevel<T> lev[kMaxLevels];
    // mixed precision, float side: the FP32 cycle's input (SA) or the inner system's
    // right-hand side and solution (refinement)
    T *bin, *xin;
    // mixed precision with SA, FP64 side: the FP32 cycle's output and the constant-mode
    // correction (wdef = A^T e, Edef = e^T A e; wdef null: no correction)
    double *ym;
    const double *wdef;
    const double *aedef;  // A e: A (y + c e) = A y + c A e, without adding c at every stencil point
    double Edef;
};

// coefficient tables of the structured operators in the solver's precision
template <class T>
struct Lhs1T {
    const T *uE, *uW, *uN, *uS, *vE, *vW, *vN, *vS;
    RowPatch patch;
    const T *rscale;
};
template <class T>
struct Lhs2T {
    const T *E, *W, *N, *S;
    int pin0, pinc;
    RowPatch patch;
};

static Lhs1T<double> tab64(const Lhs1Coef &c)
{
    return Lhs1T<double>{c.uE, c.uW, c.uN, c.uS, c.vE, c.vW, c.vN, c.vS, c.patch, c.rscale};
}
static Lhs2T<double> tab64(const Lhs2Coef &c) { return Lhs2T<double>{c.E, c.W, c.N, c.S, c.pin0, c.pinc, c.patch}; }

// a patched row (FP64 entries, applied in T)
template <class T, class X>
__device__ __forceinline__ T patch_row_t(const RowPatch &P, int k, T xi, const X &x)
{
    T y = (T)P.pdiag[k] * xi;
#pragma unroll
    for (int m = 0; m < 5; ++m) {
        const int j = P.pcol[5 * k + m];
        if (j >= 0) y += (T)P.pval[5 * k + m] * x(j);
    }
    return y;
}

// ---- operators with a precomputed diagonal ---------------------------------------
template <class T>
struct Op1D {
    Lhs1T<T> c;
    Grid g;
    const T *diag, *w;
    template <class X>
    __device__ __forceinline__ T row(int i, const X &x) const
    {
        return row_x(i, x(i), x);
    }
    // the row with the own value given (it is often at hand already)
    template <class X>
    __device__ __forceinline__ T row_x(int i, T xi, const X &x) const
    {
        if (c.patch.pid) {
            const int k = c.patch.pid[i];
            if (k >= 0) {
                const T y = patch_row_t<T>(c.patch, k, xi, x);
                return w ? w[i] * y : y;
            }
        }
        const int wu = g.nx - 1;
        // embedded method: the off-diagonal part is scaled by rscale (diag[i] carries it
        // already); the other methods sum the row in the order of lhs1_row_f
        const T *rs = c.rscale;
        T o = rs ? T(0) : diag[i] * xi;
        if (i < g.nU) {
            const int I = i % wu, J = i / wu;
            if (I != g.nx - 2) o -= c.uE[I] * x(i + 1);
            if (I != 0) o -= c.uW[I] * x(i - 1);
            if (J != g.ny - 1) o -= c.uN[J] * x(i + wu);
            if (J != 0) o -= c.uS[J] * x(i - wu);
        } else {
            const int k = i - g.nU, I = k % g.nx, J = k / g.nx;
            if (I != g.nx - 1) o -= c.vE[I] * x(i + 1);
            if (I != 0) o -= c.vW[I] * x(i - 1);
            if (J != g.ny - 2) o -= c.vN[J] * x(i + g.nx);
            if (J != 0) o -= c.vS[J] * x(i - g.nx);
        }
        const T y = rs ? diag[i] * xi + o * rs[i] : o;
        return w ? w[i] * y : y;
    }
};
template <class T>
struct Op2D {
    Lhs2T<T> c;
    Grid g;
    const T *diag, *w;
    template <class X>
    __device__ __forceinline__ T row(int i, const X &x) const
    {
        return row_x(i, x(i), x);
    }
    template <class X>
    __device__ __forceinline__ T row_x(int i, T xi, const X &x) const
    {
        if (c.patch.pid) {
            const int k = c.patch.pid[i];
            if (k >= 0) {
                const T y = patch_row_t<T>(c.patch, k, xi, x);
                return w ? w[i] * y : y;
            }
        }
        const int I = i % g.nx, J = i / g.nx;
        T y = diag[i] * xi;
        if (I != g.nx - 1) y -= c.E[I] * x(i + 1);
        if (I != 0) y -= c.W[I] * x(i - 1);
        if (J != g.ny - 1) y -= c.N[J] * x(i + g.nx);
        if (J != 0) y -= c.S[J] * x(i - g.nx);
        return w ? w[i] * y : y;
    }
};

// ---- vector access inside the persistent kernel ----------------------------------
template <class T>
struct LdAcc {
    const T *p;
    __device__ __forceinline__ T operator()(int j) const { return __ldcg(p + j); }
};
template <class T>
__device__ __forceinline__ LdAcc<T> acc(const T *p)
{
    return LdAcc<T>{p};
}
struct LdShift {  // y + c (the FP32 cycle's output with its constant re-solved)
    const double *y;
    double c;
    __device__ __forceinline__ double operator()(int j) const { return __ldcg(y + j) + c; }
};
template <class F, class T>
struct LdScale {  // f .* d (right Jacobi, or the first damped-Jacobi sweep with d = omega D^-1)
    F f;
    const T *d;
    __device__ __forceinline__ T operator()(int j) const { return d[j] * f(j); }
};
template <class F, class T>
__device__ __forceinline__ LdScale<F, T> scaled(const F &f, const T *d)
{
    return LdScale<F, T>{f, d};
}
template <class T>
struct LdPnew {  // CG direction z + beta p
    const T *z, *p;
    T beta;
    __device__ __forceinline__ T operator()(int j) const { return __ldcg(z + j) + beta * __ldcg(p + j); }
};
template <class T>
struct LdAxpy {  // u - a v: the CG residual r - alpha q, the BiCGSTAB half step r - alpha A M p
    const T *u, *v;
    T a;
    __device__ __forceinline__ T operator()(int j) const { return __ldcg(u + j) - a * __ldcg(v + j); }
};
template <class T>
struct LdBicgDir {  // BiCGSTAB direction r + beta (p - omega A M p)
    const T *r, *p, *AMp;
    T beta, omega;
    __device__ __forceinline__ T operator()(int j) const
    {
        return __ldcg(r + j) + beta * (__ldcg(p + j) - omega * __ldcg(AMp + j));
    }
};

template <class T, class X>
__device__ __forceinline__ T csr_row(const CsrV<T> &M, int i, const X &x)
{
    T s = 0;
    const int k1 = M.ptr[i + 1];
#pragma unroll 4
    for (int k = M.ptr[i]; k < k1; ++k) s += M.val[k] * x(M.col[k]);
    return s;
}

template <int G>
__device__ __forceinline__ unsigned group_mask()
{
    return G == 32 ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
}

// one CSR row split over G lanes; every lane of the group gets the sum
template <int G, class T, class X>
__device__ __forceinline__ T csr_row_g(const CsrV<T> &M, int i, const X &x)
{
    const int sub = threadIdx.x & (G - 1);
    T s = 0;
    const int k1 = M.ptr[i + 1];
    for (int k = M.ptr[i] + sub; k < k1; k += G) s += M.val[k] * x(M.col[k]);
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(group_mask<G>(), s, o);
    return s;
}

#define FOR_ROWS(i, n) for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

// The rows of a grid-stride loop U at a time: ld(i) gathers and computes row i's values
// without storing (so the U rows' loads are in flight together - a store between them
// would keep the next row's loads behind it, the compiler not knowing that the arrays do
// not overlap), st(i, v) stores and accumulates.  Rows are taken in the order FOR_ROWS
// takes them, so per-thread sums are the same.
template <int U = 2, class Ld, class St>
__device__ __forceinline__ void rows2(int n, const Ld &ld, const St &st)
{
    const int stride = gridDim.x * blockDim.x;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + (U - 1) * stride < n; i += U * stride) {
        decltype(ld(i)) u[U];
#pragma unroll
        for (int k = 0; k < U; ++k) u[k] = ld(i + k * stride);
#pragma unroll
        for (int k = 0; k < U; ++k) st(i + k * stride, u[k]);
    }
    for (; i < n; i += stride) st(i, ld(i));
}
template <class T>
struct V2 {
    T a, b;
};
template <class T>
struct V3 {
    T a, b, c;
};
template <class T>
struct V4 {
    T a, b, c, d;
};
#define FOR_GROUP_ROWS(G, i, n) \
    for (int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) / G); i < (n); i += (int)((gridDim.x * blockDim.x) / G))

// ---- grid-wide barrier and reduction ------------------------------------------------
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// entry k: the source line of the barrier's call site in the top 16 bits, the
// global timer (ns) in the low 48
__device__ __forceinline__ void trace_stamp(unsigned long long *trace, int site)
{
    if (trace && blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned long long k = trace[0] + 1;
        if (k < (unsigned long long)kTraceLen) {
            trace[k] = ((unsigned long long)(site & 0xffff) << 48) | (global_ns() & 0xffffffffffffull);
            trace[0] = k;
        }
    }
}

// Arrivals count up from zero (reset by the host before each launch); barrier k
// is complete when the counter reaches k * gridDim.x.  Returns false when this
// block gave up waiting or saw another block give up.
static __device__ bool grid_sync(FusedSyncState *st, unsigned long long *trace, int site = __builtin_LINE())
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int good = 1;
        __threadfence();
        const unsigned long long nb = gridDim.x;
        const unsigned long long old = atomicAdd(&st->arrivals, 1ull);
        const unsigned long long target = (old / nb + 1) * nb;
        unsigned long long t0 = 0;
        for (unsigned int spin = 0;; ++spin) {
            if (*(volatile unsigned long long *)&st->arrivals >= target) break;
            if ((spin & 127) == 127) {
                if (*(volatile int *)&st->abort) {
                    good = 0;
                    break;
                }
                const unsigned long long t = global_ns();
                if (t0 == 0) {
                    t0 = t;
                } else if (t - t0 > kBarrierTimeoutNs || spin > (1u << 30)) {
                    atomicExch(&st->abort, 1);
                    good = 0;
                    break;
                }
            }
        }
        __threadfence();
        ok = good;
    }
    trace_stamp(trace, site);
    __syncthreads();
    return ok;
}

// Sum NV per-thread values over the grid.  Thread 0 of every block turns the
// totals into NO scalars with fn - the same arithmetic in every block, so every
// block takes the same decisions - and the block reads them from shared memory
// (the square roots and divisions of the recurrences run once per block, not
// once per thread: FP64 issue is the scarce resource).  The per-thread values
// are summed in double whatever the vectors' precision.
template <int NV, int NO, class A, class Fn>
__device__ bool grid_reduce(const double (&v)[NV], const A &a, int &parity, const Fn &fn, double (&o)[NO],
                            int site = __builtin_LINE())
{
    __shared__ double sh[NV][32];
    __shared__ double res[NO];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double t = v[k];
        for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
        if (lane == 0) sh[k][wid] = t;
    }
    __syncthreads();
    double *part = a.partials + (size_t)parity * gridDim.x * 4;
    parity ^= 1;
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = lane < nw ? sh[k][lane] : 0.0;
            for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
            if (lane == 0) part[blockIdx.x * 4 + k] = t;
        }
    }
    if (!grid_sync(a.sync, a.trace, site)) return false;
    if (wid == 0) {
        double tot[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = 0;
            for (int b = lane; b < (int)gridDim.x; b += 32) t += __ldcg(part + b * 4 + k);
            for (int off = 16; off > 0; off >>= 1) t += __shfl_down_sync(0xffffffffu, t, off);
            tot[k] = t;
        }
        if (lane == 0) {
            double out[NO];
            fn(tot, out);
#pragma unroll
            for (int k = 0; k < NO; ++k) res[k] = out[k];
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NO; ++k) o[k] = res[k];
    return true;
}

// per-thread partial sums kept in T, handed to the reduction in double
template <class T, int N>
__device__ __forceinline__ void to_double(const T (&v)[N], double (&d)[N])
{
#pragma unroll
    for (int k = 0; k < N; ++k) d[k] = (double)v[k];
}

// An FP32 inner solve (refinement) stops at a breakdown - a non-finite or zero
// recurrence scalar - keeping the iterate it has; the FP64 refinement around it
// measures the true residual and goes on.  FP64 solves keep the reference's
// behaviour (the non-finite residual is reported).
template <class T>
__device__ __forceinline__ bool inner_breakdown(double v)
{
    return sizeof(T) == 4 && !(isfinite(v) && v != 0.0);
}

__device__ __forceinline__ int solve_state(double rnorm, double tol, int it, int maxit)
{
    // a non-finite residual or right-hand side (an overflowed field passes
    // ||r|| <= tol ||b|| as inf <= inf) is reported, not taken as convergence
    if (!isfinite(rnorm) || !isfinite(tol)) return KS_NAN;
    if (rnorm <= tol) return KS_CONVERGED;
    if (it >= maxit) return KS_MAXIT;
    return KS_RUNNING;
}

// ---- V-cycle ----------------------------------------------------------------------
// z = V(b_0): the cycle of launch_vcycle in amg.cu.  Down: x_l = w D^-1 b_l (not
// stored), r_l = b_l - A_l x_l, b_l+1 = R_l r_l.  Coarsest: x = A^-1 b (dense).
// Up: x_l = w D^-1 b_l + P_l x_l+1, out_l = x_l + w D^-1 (r_l - (A_l P_l) x_l+1).

// First phase on level 0 for one row, with the input given by an accessor:
// r_0 = b - A (w D^-1 b).  The caller adds its own per-row work and the barrier.
template <class Op, class T, class B>
__device__ __forceinline__ void vcycle_residual0_row(const Op &A, const FLevel<T> &V, int i, const B &b, T bi)
{
    V.r[i] = bi - A.row_x(i, V.wd[i] * bi, scaled(b, V.wd));
}

// Coarsest level: x = A^-1 b with the dense inverse.  Each block stages b in
// shared memory; a warp per row then streams the row of the inverse with many
// loads in flight (they do not depend on one another).  The product runs in FP64
// for the FP32 cycle too: the coarse pressure operator is nearly singular, its
// inverse has entries of order 1/lambda_min, and an FP32 product of it is noise.
constexpr int kDenseMax = 1536;  // the coarsest level's size limit (kCoarse in amg.cu is below it)

template <class T>
__device__ __forceinline__ void dense_solve(const FLevel<T> &C, const T *b, T *x)
{
    __shared__ double sb[kDenseMax];
    const int n = C.n;
    for (int k = threadIdx.x; k < n; k += blockDim.x) sb[k] = (double)__ldcg(b + k);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    // rows dealt to the blocks in turn (row r to block r mod grid), so that every SM
    // streams its share of the inverse rather than the first n / 16 blocks all of it
    const int nw = blockDim.x >> 5;
    for (int row = blockIdx.x + gridDim.x * (threadIdx.x >> 5); row < n; row += gridDim.x * nw) {
        const double *a = C.inv + (size_t)row * n;
        double acc0 = 0, acc1 = 0;
        int k = lane;
#pragma unroll 8
        for (; k + 32 < n; k += 64) {
            acc0 += a[k] * sb[k];
            acc1 += a[k + 32] * sb[k + 32];
        }
        if (k < n) acc0 += a[k] * sb[k];
        double s = acc0 + acc1;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) x[row] = (T)s;
    }
}

// The end of a cycle on level l = 0: out = x + w D^-1 (b - A x) written to zout, with
// b0 . out (dot) or wdot . out reduced, or a plain barrier
template <class T>
__device__ __forceinline__ bool cycle_end(const FArgs<T> &a, T v0, double vw, bool dot, const double *wdot,
                                          double rho_prev, double &rz, double &beta, int &parity, double *wz)
{
    if (dot) {
        T v[1] = {v0};
        double vd[1], q[2];
        to_double(v, vd);
        if (!grid_reduce<1, 2>(vd, a, parity, [&](const double (&t)[1], double (&o)[2]) {
                o[0] = t[0];
                o[1] = t[0] / rho_prev;
            }, q))
            return false;
        rz = q[0];
        beta = q[1];
    } else if (wdot) {
        double vd[1] = {vw}, q[1];
        if (!grid_reduce<1, 1>(vd, a, parity, [&](const double (&t)[1], double (&o)[1]) { o[0] = t[0]; }, q))
            return false;
        *wz = q[0];
    } else if (!grid_sync(a.sync, a.trace)) {
        return false;
    }
    return true;
}

// The folded up-sweep works on tiles of kTW x kTH fine nodes with a halo of one node:
// x_l = w D^-1 b_l + P x_l+1 on the tile and its halo goes to shared memory, then
// out_l = x_l + w D^-1 (b_l - A_l x_l) reads its stencil values from there.
constexpr int kTW = 32, kTH = 16, kTP = kTW + 2;

// a tile's x_l as the stencil of node i (tile slot li) sees it: a neighbour j = i + dy nx
// + dx, |dx|, |dy| <= 1, told from the index difference where nx >= 3 and from j's
// coordinates otherwise (a level one or two nodes wide; the tile's first node (x0, y0))
template <class T>
struct TileAcc {
    const T *xs;
    int li, i, nx, x0, y0;
    __device__ __forceinline__ T operator()(int j) const
    {
        if (nx >= 3) {
            const int d = j - i;
            const int dy = d >= nx - 1 ? 1 : (d <= 1 - nx ? -1 : 0);
            return xs[li + dy * kTP + (d - dy * nx)];
        }
        const int jy = j / nx, jx = j - jy * nx;
        return xs[(jy - y0 + 1) * kTP + (jx - x0 + 1)];
    }
};

// The level's up-sweep in one phase (no barrier inside; the caller ends the phase):
// row(i, x_i, acc) applies A_l, out(i, o) takes out_l at node i
template <class T, class RowFn, class OutFn>
__device__ __forceinline__ void st_up_tiles(const FLevel<T> &V, int cnx, int cny, const T *bb, const T *xc,
                                            const RowFn &row, const OutFn &out)
{
    __shared__ T xs[(kTH + 2) * kTP];
    const int nx = V.nx, ny = V.ny;
    const int tx = (nx + kTW - 1) / kTW, ty = (ny + kTH - 1) / kTH;
    for (int t = blockIdx.x; t < tx * ty; t += gridDim.x) {
        const int x0 = (t % tx) * kTW, y0 = (t / tx) * kTH;
        for (int k = threadIdx.x; k < (kTH + 2) * kTP; k += blockDim.x) {
            const int hy = k / kTP, hx = k - hy * kTP;
            const int ix = x0 - 1 + hx, iy = y0 - 1 + hy;
            T v = 0;
            if (ix >= 0 && ix < nx && iy >= 0 && iy < ny) {
                const int i = iy * nx + ix;
                v = V.wd[i] * __ldcg(bb + i) + st_prolong_xy(nx, ny, cnx, cny, V.pw, ix, iy, acc(xc));
            }
            xs[k] = v;
        }
        __syncthreads();
        for (int k = threadIdx.x; k < kTH * kTW; k += blockDim.x) {
            const int ly = k / kTW, lx = k - ly * kTW;
            const int ix = x0 + lx, iy = y0 + ly;
            if (ix < nx && iy < ny) {
                const int i = iy * nx + ix, li = (ly + 1) * kTP + lx + 1;
                const T xi = xs[li];
                out(i, xi + V.wd[i] * (__ldcg(bb + i) - row(i, xi, TileAcc<T>{xs, li, i, nx, x0, y0})));
            }
        }
        __syncthreads();
    }
}

// The structured hierarchy's cycle after its first phase: the same cycle as below
// (one damped-Jacobi sweep from zero down, one up, R = P^T), with the prolongator as
// four weights a node and 9-point coarse operators, so that no phase loads a column
// index.  Down, r_l then its restriction (a coarse node's sum over the 5 x 5 nodes
// around its aggregate: recomputing r_l there, 9 points each, would leave a few
// thousand threads with hundreds of loads apiece).  Up, on the levels below 0 (fz set),
// one phase over shared-memory tiles (st_up_tiles: x_l computed once a node, a halo row
// and column twice); on level 0, x_l = w D^-1 b_l + P x_l+1 stored (one phase), then
// out_l (the next) - there the tiles' two dependent stages per tile, one tile after
// another in each block, cost more than the barrier they save (52 against 33 us at
// 850k unknowns in FP64, 33 against about 20 in FP32).
template <int U, class Op, class T, class TO>
__device__ __forceinline__ bool vcycle_rest_st(const Op &A, const FArgs<T> &a, const T *b0, TO *zout, bool dot,
                                               double rho_prev, double &rz, double &beta, int &parity,
                                               const double *wdot, double *wz)
{
    const int L = a.nlev;
    for (int l = 0; l < L - 1; ++l) {
        const FLevel<T> &V = a.lev[l];
        const FLevel<T> &C = a.lev[l + 1];
        if (l > 0) {
            FOR_ROWS(i, V.n) V.r[i] = __ldcg(V.b + i) - st_row9(V.nx, V.ny, V.c9, i, scaled(acc(V.b), V.wd));
            if (!grid_sync(a.sync, a.trace)) return false;
        }
        if (V.rg) {
            // a small coarse level: a coarse node's region rows over 8 lanes (rows 0-6), so
            // that a few thousand nodes do not leave each thread a long chain of loads
            FOR_GROUP_ROWS(8, J, C.n)
            {
                T v = st_restrict_row(V.nx, V.ny, C.nx, C.ny, V.pw, J, acc(V.r), threadIdx.x & 7);
#pragma unroll
                for (int o = 4; o > 0; o >>= 1) v += __shfl_xor_sync(group_mask<8>(), v, o);
                if ((threadIdx.x & 7) == 0) C.b[J] = v;
            }
        } else {
            FOR_ROWS(J, C.n) C.b[J] = st_restrict(V.nx, V.ny, C.nx, C.ny, V.pw, J, acc(V.r));
        }
        if (!grid_sync(a.sync, a.trace)) return false;
    }
    const FLevel<T> &C = a.lev[L - 1];
    dense_solve(C, C.b, C.x);
    if (!grid_sync(a.sync, a.trace)) return false;
    const T *xc = C.x;
    for (int l = L - 2; l >= 0; --l) {
        const FLevel<T> &V = a.lev[l];
        const FLevel<T> &Cn = a.lev[l + 1];
        const T *bb = l == 0 ? b0 : V.b;
        if (V.fz) {
            T v0 = 0;
            double vw = 0;
            if (l == 0) {
                st_up_tiles(
                    V, Cn.nx, Cn.ny, bb, xc,
                    [&](int i, T xi, const TileAcc<T> &x) { return A.row_x(i, xi, x); },
                    [&](int i, T o) {
                        zout[i] = (TO)o;
                        if (dot) v0 += __ldcg(b0 + i) * o;
                        if (wdot) vw += wdot[i] * (double)o;
                    });
                if (!cycle_end(a, v0, vw, dot, wdot, rho_prev, rz, beta, parity, wz)) return false;
            } else {
                st_up_tiles(
                    V, Cn.nx, Cn.ny, bb, xc,
                    [&](int i, T, const TileAcc<T> &x) { return st_row9(V.nx, V.ny, V.c9, i, x); },
                    [&](int i, T o) { V.t[i] = o; });
                if (!grid_sync(a.sync, a.trace)) return false;
            }
            xc = V.t;
            continue;
        }
        rows2<U>(
            V.n,
            [&](int i) { return V.wd[i] * __ldcg(bb + i) + st_prolong(V.nx, V.ny, Cn.nx, Cn.ny, V.pw, i, acc(xc)); },
            [&](int i, T xi) { V.x[i] = xi; });
        if (!grid_sync(a.sync, a.trace)) return false;
        if (l == 0) {
            T v0 = 0;
            double vw = 0;
            rows2(
                V.n,
                [&](int i) {
                    const T xi = __ldcg(V.x + i);
                    const T o = xi + V.wd[i] * (__ldcg(bb + i) - A.row_x(i, xi, acc((const T *)V.x)));
                    return V3<double>{(double)o, dot ? (double)__ldcg(b0 + i) : 0.0, wdot ? wdot[i] : 0.0};
                },
                [&](int i, const V3<double> &u) {
                    zout[i] = (TO)u.a;
                    if (dot) v0 += (T)u.b * (T)u.a;
                    if (wdot) vw += u.c * u.a;
                });
            if (!cycle_end(a, v0, vw, dot, wdot, rho_prev, rz, beta, parity, wz)) return false;
        } else {
            FOR_ROWS(i, V.n)
            {
                const T xi = __ldcg(V.x + i);
                V.t[i] = xi + V.wd[i] * (__ldcg(bb + i) - st_row9(V.nx, V.ny, V.c9, i, acc((const T *)V.x)));
            }
            if (!grid_sync(a.sync, a.trace)) return false;
        }
        xc = V.t;
    }
    return true;
}

// The cycle after its first phase (r_0 written, barrier passed).  b0 is the
// cycle's input (stored); the output zout may have another precision.  With dot,
// returns b0 . z; with wdot (and no dot), returns wdot . z in *wz.
template <int U = 4, class Op, class T, class TO>
__device__ __forceinline__ bool vcycle_rest(const Op &A, const FArgs<T> &a, const T *b0, TO *zout, bool dot,
                                            double rho_prev, double &rz, double &beta, int &parity,
                                            const double *wdot = nullptr, double *wz = nullptr)
{
    // U == 1 is the build for two blocks per SM, which leaves the structured cycle out (a
    // system solved by it never gets the structured hierarchy: amg.cu)
    if constexpr (U > 1) {
        if (a.st) return vcycle_rest_st<U>(A, a, b0, zout, dot, rho_prev, rz, beta, parity, wdot, wz);
    }
    const int L = a.nlev;
    for (int l = 0; l < L - 1; ++l) {
        const FLevel<T> &V = a.lev[l];
        const FLevel<T> &C = a.lev[l + 1];
        if (l > 0) {
            FOR_GROUP_ROWS(kGroupA, i, V.n)
            {
                const T ax = csr_row_g<kGroupA>(V.A, i, scaled(acc(V.b), V.wd));
                if ((threadIdx.x & (kGroupA - 1)) == 0) V.r[i] = __ldcg(V.b + i) - ax;
            }
            if (!grid_sync(a.sync, a.trace)) return false;
        }
        FOR_GROUP_ROWS(kGroupR, i, C.n)
        {
            const T bi = csr_row_g<kGroupR>(V.R, i, acc(V.r));
            if ((threadIdx.x & (kGroupR - 1)) == 0) C.b[i] = bi;
        }
        if (!grid_sync(a.sync, a.trace)) return false;
    }
    const FLevel<T> &C = a.lev[L - 1];
    dense_solve(C, C.b, C.x);
    if (!grid_sync(a.sync, a.trace)) return false;
    const T *xc = C.x;
    for (int l = L - 2; l >= 0; --l) {
        const FLevel<T> &V = a.lev[l];
        const T *bb = l == 0 ? b0 : V.b;
        T *out = V.t;  // levels above 0 (level 0 writes zout, in the output's precision)
        T v[1] = {0};
        double vw = 0;
        if (l == 0) {
            FOR_ROWS(i, V.n)
            {
                const T wdi = V.wd[i];
                const T xi = wdi * __ldcg(bb + i) + csr_row(V.P, i, acc(xc));
                const T o = xi + wdi * (__ldcg(V.r + i) - csr_row(V.AP, i, acc(xc)));
                zout[i] = (TO)o;
                if (dot) v[0] += __ldcg(b0 + i) * o;
                if (wdot) vw += wdot[i] * (double)o;
            }
        } else {
            FOR_GROUP_ROWS(kGroupA, i, V.n)
            {
                const T px = csr_row_g<kGroupA>(V.P, i, acc(xc));
                const T apx = csr_row_g<kGroupA>(V.AP, i, acc(xc));
                if ((threadIdx.x & (kGroupA - 1)) == 0) {
                    const T wdi = V.wd[i];
                    const T xi = wdi * __ldcg(bb + i) + px;
                    out[i] = xi + wdi * (__ldcg(V.r + i) - apx);
                }
            }
        }
        if (dot && l == 0) {
            double vd[1], q[2];
            to_double(v, vd);
            if (!grid_reduce<1, 2>(vd, a, parity, [&](const double (&t)[1], double (&o)[2]) {
                    o[0] = t[0];
                    o[1] = t[0] / rho_prev;
                }, q))
                return false;
            rz = q[0];
            beta = q[1];
        } else if (wdot && l == 0) {
            double vd[1] = {vw}, q[1];
            if (!grid_reduce<1, 1>(vd, a, parity, [&](const double (&t)[1], double (&o)[1]) { o[0] = t[0]; }, q))
                return false;
            *wz = q[0];
        } else if (!grid_sync(a.sync, a.trace)) {
            return false;
        }
        xc = out;
    }
    return true;
}

// (A (y + c e))_i for the cycle's output y and its constant-mode shift c: A y + c A e
// where A e is stored (five FP64 additions a row fewer), else with c added at every
// stencil point
template <class Op, class T>
__device__ __forceinline__ T shifted_row(const Op &A, const FArgs<T> &a, int i, double yi, double c)
{
    if (a.aedef) return A.row_x(i, (T)yi, acc((const T *)a.ym)) + (T)(c * a.aedef[i]);
    return A.row_x(i, (T)(yi + c), LdShift{a.ym, c});
}

// The cycle's first phase for a stored input b: r_0 = b - A (w D^-1 b), then the barrier
template <int U = 4, class Op, class T>
__device__ __forceinline__ bool first_sweep(const Op &A, const FArgs<T> &a, const T *b)
{
    const FLevel<T> &V = a.lev[0];
    rows2<U>(
        V.n,
        [&](int i) {
            const T bi = __ldcg(b + i);
            return bi - A.row_x(i, V.wd[i] * bi, scaled(acc(b), V.wd));
        },
        [&](int i, T r) { V.r[i] = r; });
    return grid_sync(a.sync, a.trace);
}

// The same first phase when the phase that wrote b also wrote t_0 = w D^-1 b (level 0's
// t): r_0 = b - A t_0, without scaling b at every stencil point again (FP64 issue)
template <int U = 4, class Op, class T>
__device__ __forceinline__ bool first_sweep_scaled(const Op &A, const FArgs<T> &a, const T *b)
{
    const FLevel<T> &V = a.lev[0];
    rows2<U>(
        V.n, [&](int i) { return __ldcg(b + i) - A.row_x(i, __ldcg(V.t + i), acc((const T *)V.t)); },
        [&](int i, T r) { V.r[i] = r; });
    return grid_sync(a.sync, a.trace);
}

// z = V(b) for a stored input; with dot also rz = b . z and beta = rz / rho_prev.
// A one-level hierarchy is the dense solve alone.
template <int U = 4, class Op, class T>
__device__ __forceinline__ bool vcycle(const Op &A, const FArgs<T> &a, const T *b, T *zout, bool dot,
                                       double rho_prev, double &rz, double &beta, int &parity)
{
    if (a.nlev == 1) {
        dense_solve(a.lev[0], b, zout);
        if (!grid_sync(a.sync, a.trace)) return false;
        if (!dot) return true;
        T v[1] = {0};
        double vd[1], q[2];
        FOR_ROWS(i, a.lev[0].n) v[0] += __ldcg(b + i) * __ldcg(zout + i);
        to_double(v, vd);
        if (!grid_reduce<1, 2>(vd, a, parity, [&](const double (&t)[1], double (&o)[2]) {
                o[0] = t[0];
                o[1] = t[0] / rho_prev;
            }, q))
            return false;
        rz = q[0];
        beta = q[1];
        return true;
    }
    FOR_ROWS(i, a.lev[0].n) vcycle_residual0_row(A, a.lev[0], i, acc(b), __ldcg(b + i));
    if (!grid_sync(a.sync, a.trace)) return false;
    return vcycle_rest<U>(A, a, b, zout, dot, rho_prev, rz, beta, parity);
}

// Mixed precision with SA: y = V(b32) in FP32 from b32, the float copy of an FP64
// vector b that the caller wrote (with eb = e . b reduced) before its barrier; y goes
// to the FP64 vector y.  The preconditioned vector is z = y + c e: with wdef set,
// c = (e . b - wdef . y) / Edef re-solves its constant component in FP64.
template <class Op32>
__device__ __forceinline__ bool vcycle_mixed(const Op32 &A32, const FArgs<float> &f, const float *b32, double *y,
                                             const double *wdef, double Edef, double eb, double &c, int &parity)
{
    if (!first_sweep(A32, f, b32)) return false;
    double d0 = 0, d1 = 0, wy = 0;
    if (!vcycle_rest(A32, f, b32, y, false, 1.0, d0, d1, parity, wdef, &wy)) return false;
    c = wdef ? (eb - wy) / Edef : 0.0;
    return true;
}

// ---- CG on the symmetrised system (W A) x = W b ---------------------------------------
// With the SA preconditioner the update x += alpha p, r -= alpha q runs in the
// same phase as the V-cycle's first sweep (which forms r - alpha q at its stencil
// points; the residual is double-buffered).
template <class Op, int PC, class T, int U = 4>
__device__ __forceinline__ bool cg_solve(const Op &A, const FArgs<T> &a, const T *b, T *x, double rtol, int maxit,
                                         int &parity, double (&out)[4], int &it_out, int &status_out)
{
    const bool merge = PC == 2 && a.nlev >= 2;
    T v[3] = {0, 0, 0};
    double vd[3], o[5];
    FOR_ROWS(i, a.n)
    {
        const T bi = b[i];
        const T ri = a.w[i] * bi - A.row(i, acc(x));
        a.r[i] = ri;
        const T ro = ri * a.winv[i];
        v[0] += ro * ro;
        v[1] += bi * bi;
        if (PC != 2) {
            const T zi = PC == 1 ? ri * a.dinv[i] : ri;
            a.z[i] = zi;
            v[2] += ri * zi;
        }
    }
    to_double(v, vd);
    if (!grid_reduce<3, 5>(vd, a, parity, [&](const double (&t)[3], double (&q)[5]) {
            q[0] = sqrt(t[0]);
            q[1] = sqrt(t[1]);
            q[2] = rtol * q[1];
            q[3] = t[2];
            q[4] = solve_state(q[0], q[2], 0, maxit);
        }, o))
        return false;
    double rnorm = o[0];
    const double bnorm = o[1], tol = o[2];
    double rho = o[3], beta = 0;
    int it = 0;
    int status = (int)o[4];
    T *r = a.r, *rn = a.rs;
    if (status == KS_RUNNING && PC == 2 && !vcycle<U>(A, a, (const T *)r, a.z, true, 1.0, rho, beta, parity))
        return false;
    T *p = a.p, *pn = a.p2;
    bool first = true;
    while (status == KS_RUNNING) {
        // direction pn = z + beta p, q = A pn, pn . q
        const T bt = (T)beta;
        T v1[1] = {0};
        double v1d[1], o1[1];
        FOR_ROWS(i, a.n)
        {
            const T zi = __ldcg(a.z + i);
            T pi, qi;
            if (first) {
                pi = zi;
                qi = A.row_x(i, pi, acc((const T *)a.z));
            } else {
                pi = zi + bt * __ldcg(p + i);
                qi = A.row_x(i, pi, LdPnew<T>{a.z, p, bt});
            }
            pn[i] = pi;
            a.q[i] = qi;
            v1[0] += pi * qi;
        }
        to_double(v1, v1d);
        if (!grid_reduce<1, 1>(v1d, a, parity, [&](const double (&t)[1], double (&q)[1]) { q[0] = rho / t[0]; }, o1))
            return false;
        const double alpha = o1[0];
        if (inner_breakdown<T>(alpha)) {
            status = KS_STALLED;
            break;
        }
        const T at = (T)alpha;
        {
            T *tmp = p;
            p = pn;
            pn = tmp;
        }
        first = false;
        if (merge) {
            const LdAxpy<T> rnew{r, a.q, at};
            T v2[1] = {0};
            double v2d[1], o2[2];
            FOR_ROWS(i, a.n)
            {
                x[i] = __ldcg(x + i) + at * __ldcg(p + i);
                const T ri = rnew(i);
                rn[i] = ri;
                const T ro = ri * a.winv[i];
                v2[0] += ro * ro;
                vcycle_residual0_row(A, a.lev[0], i, rnew, ri);
            }
            to_double(v2, v2d);
            if (!grid_reduce<1, 2>(v2d, a, parity, [&](const double (&t)[1], double (&q)[2]) {
                    q[0] = sqrt(t[0]);
                    q[1] = solve_state(q[0], tol, it + 1, maxit);
                }, o2))
                return false;
            {
                T *tmp = r;
                r = rn;
                rn = tmp;
            }
            ++it;
            rnorm = o2[0];
            status = (int)o2[1];
            if (status != KS_RUNNING) break;
            double rz = 0;
            if (!vcycle_rest<U>(A, a, (const T *)r, a.z, true, rho, rz, beta, parity)) return false;
            rho = rz;
            if (inner_breakdown<T>(beta)) {
                status = KS_STALLED;
                break;
            }
            continue;
        }
        T v2[2] = {0, 0};
        double v2d[2], o2[4];
        FOR_ROWS(i, a.n)
        {
            x[i] = __ldcg(x + i) + at * __ldcg(p + i);
            const T ri = __ldcg(r + i) - at * __ldcg(a.q + i);
            r[i] = ri;
            const T ro = ri * a.winv[i];
            v2[0] += ro * ro;
            if (PC != 2) {
                const T zi = PC == 1 ? ri * a.dinv[i] : ri;
                a.z[i] = zi;
                v2[1] += ri * zi;
            }
        }
        to_double(v2, v2d);
        if (!grid_reduce<2, 4>(v2d, a, parity, [&](const double (&t)[2], double (&q)[4]) {
                q[0] = sqrt(t[0]);
                q[1] = solve_state(q[0], tol, it + 1, maxit);
                q[2] = PC != 2 ? t[1] / rho : 0.0;
                q[3] = t[1];
            }, o2))
            return false;
        ++it;
        rnorm = o2[0];
        status = (int)o2[1];
        if (PC != 2) {
            beta = o2[2];
            rho = o2[3];
        }
        if (status != KS_RUNNING) break;
        if (PC == 2) {
            double rz = 0;
            if (!vcycle<U>(A, a, (const T *)r, a.z, true, rho, rz, beta, parity)) return false;
            rho = rz;
        }
        if (inner_breakdown<T>(beta)) {
            status = KS_STALLED;
            break;
        }
    }
    out[0] = rnorm;
    out[1] = bnorm;
    out[2] = tol;
    out[3] = rho;
    it_out = it;
    status_out = status;
    return true;
}

// ---- BiCGSTAB, right-preconditioned --------------------------------------------------------
// One iteration: Mp = M p; alpha = rho / (rs . A Mp); s = r - alpha A Mp (stop
// here when ||s|| <= tol); Ms = M s; omega = (A Ms . s) / (A Ms . A Ms);
// x += alpha Mp + omega Ms; r = s - omega A Ms; beta = (rs . r / rho)(alpha / omega);
// p = r + beta (p - omega A Mp).
// Phases per iteration: Jacobi or none - 3 (the direction update rides on the
// next A M p, the half step on A M s); SA - 2 V-cycles + 3 (the direction
// update rides on the first V-cycle sweep, the half step on the second).
// MX (mixed precision with SA, T = double): the V-cycles run in FP32 (A32, f) on
// float copies written in the direction and half-step phases, their outputs get the
// constant-mode correction, and M p, M s are written in the phases that apply A.
template <class Op, int PC, class T, bool MX = false, class Op32 = Op, int U = 4>
__device__ __forceinline__ bool bicg_solve(const Op &A, const FArgs<T> &a, const T *b, T *x, double rtol, int maxit,
                                           int &parity, double (&out)[4], int &it_out, int &status_out,
                                           const Op32 *A32 = nullptr, const FArgs<float> *f = nullptr)
{
    const bool sa_multi = PC == 2 && a.nlev >= 2;
    // FP64 cycle with the constant-mode correction (the Poisson system): its output goes
    // to ym, the corrected vector is written where A is applied to it
    const bool defl = !MX && sa_multi && a.wdef != nullptr;
    T v[2] = {0, 0};
    double vd[2], o[5];
    FOR_ROWS(i, a.n)
    {
        const T bi = b[i];
        const T ri = bi - A.row(i, acc(x));
        a.r[i] = ri;
        a.rs[i] = ri;
        a.p[i] = ri;
        v[0] += ri * ri;
        v[1] += bi * bi;
    }
    to_double(v, vd);
    if (!grid_reduce<2, 5>(vd, a, parity, [&](const double (&t)[2], double (&q)[5]) {
            q[0] = t[0];
            q[1] = sqrt(t[0]);
            q[2] = sqrt(t[1]);
            q[3] = rtol * q[2];
            q[4] = solve_state(q[1], q[3], 0, maxit);
        }, o))
        return false;
    double rho = o[0], rnorm = o[1];
    const double bnorm = o[2], tol = o[3];
    int it = 0;
    int status = (int)o[4];
    // p and A M p are double-buffered: the direction update reads the old ones
    // at the stencil points of the phase that writes the new ones
    T *p = a.p, *pn = a.p2, *amp = a.AMp, *ampn = a.AMp2;
    double beta = 0, omega = 1;
    bool first = true;
    double dummy = 0, dummy2 = 0, cmx = 0;
    while (status == KS_RUNNING) {
        // ---- new direction (folded), Mp = M p, A Mp, rs . A Mp
        const LdBicgDir<T> dir{a.r, p, amp, (T)beta, (T)omega};
        if (PC == 2) {
            if (MX) {
                T ve[1] = {0};
                rows2(
                    a.n, [&](int i) { return first ? __ldcg(p + i) : dir(i); },
                    [&](int i, T pi) {
                        if (!first) pn[i] = pi;
                        f->bin[i] = (float)pi;
                        ve[0] += pi;
                    });
                double ved[1], eb[1];
                to_double(ve, ved);
                if (!grid_reduce<1, 1>(ved, a, parity, [&](const double (&t)[1], double (&q)[1]) { q[0] = t[0]; },
                                       eb))
                    return false;
                if (!first) {
                    T *tmp = p;
                    p = pn;
                    pn = tmp;
                }
                if (!vcycle_mixed(*A32, *f, f->bin, a.ym, a.wdef, a.Edef, eb[0], cmx, parity)) return false;
            } else if (sa_multi) {
                T ve[1] = {0};
                FOR_ROWS(i, a.n)
                {
                    T pi;
                    if (first) {
                        pi = __ldcg(p + i);
                        if (!a.split0) vcycle_residual0_row(A, a.lev[0], i, acc((const T *)p), pi);
                    } else {
                        pi = dir(i);
                        pn[i] = pi;
                        if (!a.split0) vcycle_residual0_row(A, a.lev[0], i, dir, pi);
                    }
                    if (a.split0) a.lev[0].t[i] = a.lev[0].wd[i] * pi;  // the first sweep's w D^-1 b
                    ve[0] += pi;
                }
                double eb[1] = {0};
                if (defl) {
                    double ved[1];
                    to_double(ve, ved);
                    if (!grid_reduce<1, 1>(ved, a, parity, [&](const double (&t)[1], double (&q)[1]) { q[0] = t[0]; },
                                           eb))
                        return false;
                } else if (!grid_sync(a.sync, a.trace)) {
                    return false;
                }
                if (!first) {
                    T *tmp = p;
                    p = pn;
                    pn = tmp;
                }
                if (a.split0 && !first_sweep_scaled<U>(A, a, (const T *)p)) return false;
                if (defl) {
                    double wy = 0;
                    if (!vcycle_rest<U>(A, a, (const T *)p, a.ym, false, 1.0, dummy, dummy2, parity, a.wdef, &wy))
                        return false;
                    cmx = (eb[0] - wy) / a.Edef;
                } else if (!vcycle_rest<U>(A, a, (const T *)p, a.Mp, false, 1.0, dummy, dummy2, parity)) {
                    return false;
                }
            } else {
                if (!first) {
                    FOR_ROWS(i, a.n) pn[i] = dir(i);
                    if (!grid_sync(a.sync, a.trace)) return false;
                    T *tmp = p;
                    p = pn;
                    pn = tmp;
                }
                if (!vcycle<U>(A, a, (const T *)p, a.Mp, false, 1.0, dummy, dummy2, parity)) return false;
            }
        }
        T v1[1] = {0};
        double v1d[1], o1[1];
        // Jacobi or none: the new direction and M p are stored in one phase and A M p read
        // back in the next; or (fold1: the FP32 solves) one phase that recomputes the
        // direction and its scaling at the four stencil neighbours - about 22 operations
        // a row against 9, which FP64 issue does not repay (the values are the same:
        // M p_j = D^-1_j p_j either way)
        const bool fold = PC != 2 && a.fold1;
        if (PC != 2 && !fold) {
            FOR_ROWS(i, a.n)
            {
                const T pi = first ? __ldcg(p + i) : dir(i);
                if (!first) pn[i] = pi;
                a.Mp[i] = PC == 1 ? a.dinv[i] * pi : pi;
            }
            if (!grid_sync(a.sync, a.trace)) return false;
        }
        if (fold) {
            auto mp = [&](int j) {
                const T pj = first ? __ldcg(p + j) : dir(j);
                return PC == 1 ? a.dinv[j] * pj : pj;
            };
            rows2(
                a.n,
                [&](int i) {
                    const T pi = first ? __ldcg(p + i) : dir(i);
                    const T mi = PC == 1 ? a.dinv[i] * pi : pi;
                    return V4<T>{pi, mi, A.row_x(i, mi, mp), __ldcg(a.rs + i)};
                },
                [&](int i, const V4<T> &u) {
                    if (!first) pn[i] = u.a;
                    a.Mp[i] = u.b;
                    ampn[i] = u.c;
                    v1[0] += u.d * u.c;
                });
        } else if (PC == 2 && (MX || defl)) {
            rows2(
                a.n,
                [&](int i) {
                    const double yi = __ldcg(a.ym + i);
                    return V3<T>{(T)(yi + cmx), shifted_row(A, a, i, yi, cmx), __ldcg(a.rs + i)};
                },
                [&](int i, const V3<T> &u) {
                    a.Mp[i] = u.a;
                    ampn[i] = u.b;
                    v1[0] += u.c * u.b;
                });
        } else {
            rows2(
                a.n, [&](int i) { return V2<T>{A.row(i, acc((const T *)a.Mp)), __ldcg(a.rs + i)}; },
                [&](int i, const V2<T> &u) {
                    ampn[i] = u.a;
                    v1[0] += u.b * u.a;
                });
        }
        to_double(v1, v1d);
        if (!grid_reduce<1, 1>(v1d, a, parity, [&](const double (&t)[1], double (&q)[1]) { q[0] = rho / t[0]; }, o1))
            return false;
        if (PC != 2 && !first) {
            T *tmp = p;
            p = pn;
            pn = tmp;
        }
        {
            T *tmp = amp;
            amp = ampn;
            ampn = tmp;
        }
        first = false;
        const double alpha = o1[0];
        if (inner_breakdown<T>(alpha)) {
            status = KS_STALLED;
            break;
        }
        const T at = (T)alpha;
        // ---- half step s = r - alpha A Mp (folded into the application of M and A to s)
        const LdAxpy<T> snew{a.r, amp, at};
        double o3[3];  // snorm, half-step convergence, omega
        if (PC == 2) {
            T v2[2] = {0, 0};
            double v2d[2], o2[2];
            if (MX) {
                rows2(
                    a.n, [&](int i) { return snew(i); },
                    [&](int i, T si) {
                        a.s[i] = si;
                        v2[0] += si * si;
                        v2[1] += si;
                        f->bin[i] = (float)si;
                    });
            } else if (sa_multi) {
                FOR_ROWS(i, a.n)
                {
                    const T si = snew(i);
                    a.s[i] = si;
                    v2[0] += si * si;
                    v2[1] += si;
                    if (!a.split0) vcycle_residual0_row(A, a.lev[0], i, snew, si);
                    else a.lev[0].t[i] = a.lev[0].wd[i] * si;
                }
            } else {
                FOR_ROWS(i, a.n)
                {
                    const T si = snew(i);
                    a.s[i] = si;
                    v2[0] += si * si;
                }
            }
            to_double(v2, v2d);
            if (!grid_reduce<2, 2>(v2d, a, parity, [&](const double (&t)[2], double (&q)[2]) {
                    q[0] = sqrt(t[0]);
                    q[1] = t[1];
                }, o2))
                return false;
            o3[0] = o2[0];
            o3[1] = o2[0] <= tol;
            if (o3[1] != 0) {
                FOR_ROWS(i, a.n) x[i] = __ldcg(x + i) + at * __ldcg(a.Mp + i);
                rnorm = o3[0];
                status = KS_CONVERGED;
                break;
            }
            if (sa_multi && !MX && a.split0 && !first_sweep_scaled<U>(A, a, (const T *)a.s)) return false;
            if (MX) {
                if (!vcycle_mixed(*A32, *f, f->bin, a.ym, a.wdef, a.Edef, o2[1], cmx, parity)) return false;
            } else if (defl) {
                double wy = 0;
                if (!vcycle_rest<U>(A, a, (const T *)a.s, a.ym, false, 1.0, dummy, dummy2, parity, a.wdef, &wy))
                    return false;
                cmx = (o2[1] - wy) / a.Edef;
            } else if (sa_multi) {
                if (!vcycle_rest<U>(A, a, (const T *)a.s, a.Ms, false, 1.0, dummy, dummy2, parity)) return false;
            } else if (!vcycle<U>(A, a, (const T *)a.s, a.Ms, false, 1.0, dummy, dummy2, parity)) {
                return false;
            }
            T v3[2] = {0, 0};
            double v3d[2], o4[1];
            if (MX || defl) {
                rows2(
                    a.n,
                    [&](int i) {
                        const double yi = __ldcg(a.ym + i);
                        return V3<T>{(T)(yi + cmx), shifted_row(A, a, i, yi, cmx), __ldcg(a.s + i)};
                    },
                    [&](int i, const V3<T> &u) {
                        a.Ms[i] = u.a;
                        a.AMs[i] = u.b;
                        v3[0] += u.b * u.c;
                        v3[1] += u.b * u.b;
                    });
            } else {
                rows2(
                    a.n, [&](int i) { return V2<T>{A.row(i, acc((const T *)a.Ms)), __ldcg(a.s + i)}; },
                    [&](int i, const V2<T> &u) {
                        a.AMs[i] = u.a;
                        v3[0] += u.a * u.b;
                        v3[1] += u.a * u.a;
                    });
            }
            to_double(v3, v3d);
            if (!grid_reduce<2, 1>(v3d, a, parity, [&](const double (&t)[2], double (&q)[1]) { q[0] = t[0] / t[1]; },
                                   o4))
                return false;
            o3[2] = o4[0];
        } else {
            T v3[3] = {0, 0, 0};
            double v3d[3];
            // as for the direction: s and M s stored, then A M s in the next phase; or (fold1)
            // one phase with s and its scaling recomputed at the stencil points
            if (fold) {
                auto ms = [&](int j) {
                    const T sj = snew(j);
                    return PC == 1 ? a.dinv[j] * sj : sj;
                };
                rows2(
                    a.n,
                    [&](int i) {
                        const T si = snew(i);
                        const T mi = PC == 1 ? a.dinv[i] * si : si;
                        return V3<T>{si, mi, A.row_x(i, mi, ms)};
                    },
                    [&](int i, const V3<T> &u) {
                        a.s[i] = u.a;
                        a.Ms[i] = u.b;
                        a.AMs[i] = u.c;
                        v3[0] += u.c * u.a;
                        v3[1] += u.c * u.c;
                        v3[2] += u.a * u.a;
                    });
            } else {
                FOR_ROWS(i, a.n)
                {
                    const T si = snew(i);
                    a.s[i] = si;
                    a.Ms[i] = PC == 1 ? a.dinv[i] * si : si;
                }
                if (!grid_sync(a.sync, a.trace)) return false;
                FOR_ROWS(i, a.n)
                {
                    const T si = __ldcg(a.s + i);
                    const T ai = A.row(i, acc((const T *)a.Ms));
                    a.AMs[i] = ai;
                    v3[0] += ai * si;
                    v3[1] += ai * ai;
                    v3[2] += si * si;
                }
            }
            to_double(v3, v3d);
            if (!grid_reduce<3, 3>(v3d, a, parity, [&](const double (&t)[3], double (&q)[3]) {
                    q[0] = sqrt(t[2]);
                    q[1] = q[0] <= tol;
                    q[2] = t[0] / t[1];
                }, o3))
                return false;
            if (o3[1] != 0) {
                FOR_ROWS(i, a.n) x[i] = __ldcg(x + i) + at * __ldcg(a.Mp + i);
                rnorm = o3[0];
                status = KS_CONVERGED;
                break;
            }
        }
        omega = o3[2];
        if (inner_breakdown<T>(omega)) {  // keep the half step
            FOR_ROWS(i, a.n) x[i] = __ldcg(x + i) + at * __ldcg(a.Mp + i);
            status = KS_STALLED;
            break;
        }
        const T ot = (T)omega;
        // ---- x, r and the dots that give beta
        T v4[2] = {0, 0};
        double v4d[2], o5[4];
        rows2<U>(
            a.n,
            [&](int i) {
                return V3<T>{__ldcg(x + i) + (at * __ldcg(a.Mp + i) + ot * __ldcg(a.Ms + i)),
                             __ldcg(a.s + i) - ot * __ldcg(a.AMs + i), __ldcg(a.rs + i)};
            },
            [&](int i, const V3<T> &u) {
                x[i] = u.a;
                a.r[i] = u.b;
                v4[0] += u.c * u.b;
                v4[1] += u.b * u.b;
            });
        to_double(v4, v4d);
        if (!grid_reduce<2, 4>(v4d, a, parity, [&](const double (&t)[2], double (&q)[4]) {
                q[0] = (t[0] / rho) * (alpha / omega);
                q[1] = t[0];
                q[2] = sqrt(t[1]);
                q[3] = solve_state(q[2], tol, it + 1, maxit);
            }, o5))
            return false;
        beta = o5[0];
        rho = o5[1];
        ++it;
        rnorm = o5[2];
        status = (int)o5[3];
        if (status == KS_RUNNING && inner_breakdown<T>(beta)) status = KS_STALLED;
    }
    out[0] = rnorm;
    out[1] = bnorm;
    out[2] = tol;
    out[3] = rho;
    it_out = it;
    status_out = status;
    return true;
}

// MINB: blocks per SM the kernel is built for (2: at most 64 registers a thread, for
// batched instances whose solves share the SMs)
template <class Op, int PC, int KRY, int MINB = 1>
__global__ void __launch_bounds__(kFT, MINB) k_fused_solve(Op A, const FArgs<double> *__restrict__ ap,
                                                           const double *b, double *x)
{
    const FArgs<double> &a = *ap;
    if (a.trace && blockIdx.x == 0 && threadIdx.x == 0) {
        a.trace[0] = 1;
        a.trace[1] = global_ns() & 0xffffffffffffull;  // the start (site 0)
    }
    double res[4];
    int it = 0, status = KS_RUNNING, parity = 0;
    // rows taken four at a time, one at a time where the kernel is built for two blocks per
    // SM (64 registers a thread: batched rows would spill)
    constexpr int U = MINB == 2 ? 1 : 4;
    const bool ok = KRY == KRYLOV_CG
                        ? cg_solve<Op, PC, double, U>(A, a, b, x, a.ks->rtol, a.ks->maxit, parity, res, it, status)
                        : bicg_solve<Op, PC, double, false, Op, U>(A, a, b, x, a.ks->rtol, a.ks->maxit, parity, res, it,
                                                                   status);
    trace_stamp(a.trace, __LINE__);
    if (threadIdx.x != 0) return;
    if (!ok) {
        atomicCAS(a.err, 0, a.which * 16 + KS_TIMEOUT);
        return;
    }
    if (blockIdx.x != 0) return;
    KrylovScalars *ks = a.ks;
    ks->rnorm = res[0];
    ks->bnorm = res[1];
    ks->tol = res[2];
    ks->rho = res[3];
    ks->it = it;
    ks->body_runs = it;
    ks->status = status;
    if ((status == KS_MAXIT || status == KS_NAN) && a.err) atomicCAS(a.err, 0, a.which * 16 + status);
}

// Mixed precision with the SA preconditioner: FP64 BiCGSTAB whose two V-cycles per
// iteration run in FP32 (the constant mode re-solved in FP64).
template <class Op64, class Op32>
__global__ void __launch_bounds__(kFT, 1) k_fused_mixed(Op64 A, Op32 A32, const FArgs<double> *__restrict__ ap,
                                                        const FArgs<float> *__restrict__ fp, const double *b,
                                                        double *x)
{
    const FArgs<double> &a = *ap;
    if (a.trace && blockIdx.x == 0 && threadIdx.x == 0) {
        a.trace[0] = 1;
        a.trace[1] = global_ns() & 0xffffffffffffull;  // the start (site 0)
    }
    double res[4];
    int it = 0, status = KS_RUNNING, parity = 0;
    const bool ok = bicg_solve<Op64, 2, double, true, Op32>(A, a, b, x, a.ks->rtol, a.ks->maxit, parity, res, it,
                                                            status, &A32, fp);
    trace_stamp(a.trace, __LINE__);
    if (threadIdx.x != 0) return;
    if (!ok) {
        atomicCAS(a.err, 0, a.which * 16 + KS_TIMEOUT);
        return;
    }
    if (blockIdx.x != 0) return;
    KrylovScalars *ks = a.ks;
    ks->rnorm = res[0];
    ks->bnorm = res[1];
    ks->tol = res[2];
    ks->rho = res[3];
    ks->it = it;
    ks->body_runs = it;
    ks->status = status;
    if ((status == KS_MAXIT || status == KS_NAN) && a.err) atomicCAS(a.err, 0, a.which * 16 + status);
}

// Mixed precision without SA: iterative refinement in FP64 around FP32 Krylov solves,
// in one launch.  A64 is the original (unweighted) operator; A32 the FP32 operator the
// inner solver iterates on (symmetrised for CG).  The iteration count is the sum of the
// inner iterations.
template <class Op64, class Op32, int PC, int KRY>
__global__ void __launch_bounds__(kFT, 1) k_fused_ir(Op64 A, Op32 A32, const FArgs<double> *__restrict__ ap,
                                                     const FArgs<float> *__restrict__ fp, const double *b, double *x)
{
    const FArgs<double> &a = *ap;
    const FArgs<float> &f = *fp;
    if (a.trace && blockIdx.x == 0 && threadIdx.x == 0) {
        a.trace[0] = 1;
        a.trace[1] = global_ns() & 0xffffffffffffull;  // the start (site 0)
    }
    const double rtol = a.ks->rtol, floor_in = a.ks->inner_rtol;
    const int maxit = a.ks->maxit, maxit_in = a.ks->inner_maxit;
    int parity = 0, its = 0, status = KS_RUNNING;
    double bnorm = 0, tol = 0, rnorm = 0;
    bool ok = true, first = true;
    while (ok) {
        // outer residual of the original system in FP64; the inner right-hand side and
        // a zero inner start
        double v[2] = {0, 0}, o[5];
        FOR_ROWS(i, a.n)
        {
            const double bi = b[i];
            const double ri = bi - A.row(i, acc((const double *)x));
            f.bin[i] = (float)ri;
            f.xin[i] = 0.f;
            v[0] += ri * ri;
            v[1] += bi * bi;
        }
        const double bn0 = bnorm, tl0 = tol;
        ok = grid_reduce<2, 5>(v, a, parity, [&](const double (&t)[2], double (&q)[5]) {
            q[0] = sqrt(t[0]);
            q[1] = first ? sqrt(t[1]) : bn0;
            q[2] = first ? rtol * q[1] : tl0;
            q[3] = solve_state(q[0], q[2], its, maxit);
            q[4] = fmax(0.5 * q[2] / q[0], floor_in);  // the inner solve's relative tolerance
        }, o);
        if (!ok) break;
        rnorm = o[0];
        bnorm = o[1];
        tol = o[2];
        status = (int)o[3];
        first = false;
        if (status != KS_RUNNING) break;
        double res[4];
        int it_in = 0, st_in = KS_RUNNING;
        const int cap = min(maxit - its, maxit_in);
        ok = KRY == KRYLOV_CG ? cg_solve<Op32, PC, float>(A32, f, f.bin, f.xin, o[4], cap, parity, res, it_in, st_in)
                              : bicg_solve<Op32, PC, float>(A32, f, f.bin, f.xin, o[4], cap, parity, res, it_in, st_in);
        if (!ok) break;
        its += it_in > 0 ? it_in : 1;
        if (st_in == KS_NAN) {
            status = KS_NAN;
            break;
        }
        if (st_in == KS_STALLED && it_in == 0) {  // a breakdown before any progress: give up
            status = KS_MAXIT;
            break;
        }
        FOR_ROWS(i, a.n) x[i] = __ldcg(x + i) + (double)__ldcg(f.xin + i);
        ok = grid_sync(a.sync, a.trace);
    }
    trace_stamp(a.trace, __LINE__);
    if (threadIdx.x != 0) return;
    if (!ok) {
        atomicCAS(a.err, 0, a.which * 16 + KS_TIMEOUT);
        return;
    }
    if (blockIdx.x != 0) return;
    KrylovScalars *ks = a.ks;
    ks->rnorm = rnorm;
    ks->bnorm = bnorm;
    ks->tol = tol;
    ks->it = its;
    ks->body_runs = its;
    ks->status = status;
    if ((status == KS_MAXIT || status == KS_NAN) && a.err) atomicCAS(a.err, 0, a.which * 16 + status);
}

template <class Op>
static void *pick_kernel(int precond, int krylov, int pack)
{
    if (pack == 2 && (precond == PC_SMOOTHED_AGGREGATION || precond == PC_DIAGONAL)) {
        if (krylov == KRYLOV_CG)
            return precond == PC_SMOOTHED_AGGREGATION ? (void *)k_fused_solve<Op, 2, KRYLOV_CG, 2>
                                                      : (void *)k_fused_solve<Op, 1, KRYLOV_CG, 2>;
        return precond == PC_SMOOTHED_AGGREGATION ? (void *)k_fused_solve<Op, 2, KRYLOV_BICGSTAB, 2>
                                                  : (void *)k_fused_solve<Op, 1, KRYLOV_BICGSTAB, 2>;
    }
    if (krylov == KRYLOV_CG) {
        if (precond == PC_SMOOTHED_AGGREGATION) return (void *)k_fused_solve<Op, 2, KRYLOV_CG>;
        if (precond == PC_DIAGONAL) return (void *)k_fused_solve<Op, 1, KRYLOV_CG>;
        return (void *)k_fused_solve<Op, 0, KRYLOV_CG>;
    }
    if (precond == PC_SMOOTHED_AGGREGATION) return (void *)k_fused_solve<Op, 2, KRYLOV_BICGSTAB>;
    if (precond == PC_DIAGONAL) return (void *)k_fused_solve<Op, 1, KRYLOV_BICGSTAB>;
    return (void *)k_fused_solve<Op, 0, KRYLOV_BICGSTAB>;
}

// mixed precision: BiCGSTAB with a multilevel SA hierarchy keeps the FP64 Krylov
// around FP32 V-cycles; everything else is refined around FP32 solves
static bool mixed_vcycle(const LinearSystem &S)
{
    return S.precond == PC_SMOOTHED_AGGREGATION && S.krylov == KRYLOV_BICGSTAB && S.amg.size() >= 2;
}

template <class Op64, class Op32>
static void *pick_mixed_kernel(const LinearSystem &S)
{
    if (mixed_vcycle(S)) return (void *)k_fused_mixed<Op64, Op32>;
    if (S.krylov == KRYLOV_CG) {
        if (S.precond == PC_SMOOTHED_AGGREGATION) return (void *)k_fused_ir<Op64, Op32, 2, KRYLOV_CG>;
        if (S.precond == PC_DIAGONAL) return (void *)k_fused_ir<Op64, Op32, 1, KRYLOV_CG>;
        return (void *)k_fused_ir<Op64, Op32, 0, KRYLOV_CG>;
    }
    if (S.precond == PC_SMOOTHED_AGGREGATION) return (void *)k_fused_ir<Op64, Op32, 2, KRYLOV_BICGSTAB>;
    if (S.precond == PC_DIAGONAL) return (void *)k_fused_ir<Op64, Op32, 1, KRYLOV_BICGSTAB>;
    return (void *)k_fused_ir<Op64, Op32, 0, KRYLOV_BICGSTAB>;
}

// the kernels for one operator type, in their own translation units (compiled in parallel)
void *fused_pick_op1(int precond, int krylov, int pack);
void *fused_pick_op2(int precond, int krylov, int pack);
void *fused_pick_mixed_op1(const LinearSystem &S);
void *fused_pick_mixed_op2(const LinearSystem &S);

}  // namespace cuibm
