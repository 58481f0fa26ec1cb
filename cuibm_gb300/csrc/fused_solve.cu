// Persistent linear solves: one cooperative launch runs a whole Krylov solve
// of LHS1 or LHS2 - BiCGSTAB or CG, with no, Jacobi or smoothed-aggregation
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
#include "solver.h"

namespace cuibm {

constexpr int kFT = 512;  // threads per block
constexpr int kMaxLevels = 10;
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull;  // 2 s
constexpr int kGroupR = 8;  // lanes per restriction row (15-30 entries)
constexpr int kGroupA = 4;  // lanes per coarse-operator row (9-25 entries)

struct FLevel {
    int n;
    DevCsr A, P, R, AP;
    const double *wd;  // omega D^-1
    double *x, *b, *r, *t;
    const double *inv;  // coarsest level: dense inverse
};

// Everything a solve needs except its right-hand side and solution, built once
// per system and kept in device memory (the kernel reads it through a pointer:
// a struct this size indexed by level would otherwise be copied to local memory).
struct FArgs {
    int n;
    double *r, *rs, *p, *p2, *Mp, *AMp, *AMp2, *s, *Ms, *AMs, *z, *q;
    const double *dinv, *w, *winv, *diag;
    double *partials;  // 2 x gridDim x 4
    FusedSyncState *sync;
    unsigned long long *trace;  // [count, stamps...] of kTraceLen, or null
    KrylovScalars *ks;
    int *err;
    int which;
    int nlev;
    FLevel lev[kMaxLevels];
};

// ---- operators with a precomputed diagonal ---------------------------------------
struct Op1D {
    Lhs1Coef c;
    Grid g;
    const double *diag, *w;
    template <class X>
    __device__ __forceinline__ double row(int i, const X &x) const
    {
        return row_x(i, x(i), x);
    }
    // the row with the own value given (it is often at hand already)
    template <class X>
    __device__ __forceinline__ double row_x(int i, double xi, const X &x) const
    {
        if (c.patch.pid) {
            const int k = c.patch.pid[i];
            if (k >= 0) {
                const double y = patch_row(c.patch, k, xi, x);
                return w ? w[i] * y : y;
            }
        }
        const int wu = g.nx - 1;
        // embedded method: the off-diagonal part is scaled by rscale (diag[i] carries it
        // already); the other methods sum the row in the order of lhs1_row_f
        const double *rs = c.rscale;
        double o = rs ? 0.0 : diag[i] * xi;
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
        const double y = rs ? diag[i] * xi + o * rs[i] : o;
        return w ? w[i] * y : y;
    }
};
struct Op2D {
    Lhs2Coef c;
    Grid g;
    const double *diag, *w;
    template <class X>
    __device__ __forceinline__ double row(int i, const X &x) const
    {
        return row_x(i, x(i), x);
    }
    template <class X>
    __device__ __forceinline__ double row_x(int i, double xi, const X &x) const
    {
        if (c.patch.pid) {
            const int k = c.patch.pid[i];
            if (k >= 0) {
                const double y = patch_row(c.patch, k, xi, x);
                return w ? w[i] * y : y;
            }
        }
        const int I = i % g.nx, J = i / g.nx;
        double y = diag[i] * xi;
        if (I != g.nx - 1) y -= c.E[I] * x(i + 1);
        if (I != 0) y -= c.W[I] * x(i - 1);
        if (J != g.ny - 1) y -= c.N[J] * x(i + g.nx);
        if (J != 0) y -= c.S[J] * x(i - g.nx);
        return w ? w[i] * y : y;
    }
};

// ---- vector access inside the persistent kernel ----------------------------------
struct LdAcc {
    const double *p;
    __device__ __forceinline__ double operator()(int j) const { return __ldcg(p + j); }
};
template <class F>
struct LdScale {  // f .* d (right Jacobi, or the first damped-Jacobi sweep with d = omega D^-1)
    F f;
    const double *d;
    __device__ __forceinline__ double operator()(int j) const { return d[j] * f(j); }
};
struct LdPnew {  // CG direction z + beta p
    const double *z, *p;
    double beta;
    __device__ __forceinline__ double operator()(int j) const { return __ldcg(z + j) + beta * __ldcg(p + j); }
};
struct LdAxpy {  // u - a v: the CG residual r - alpha q, the BiCGSTAB half step r - alpha A M p
    const double *u, *v;
    double a;
    __device__ __forceinline__ double operator()(int j) const { return __ldcg(u + j) - a * __ldcg(v + j); }
};
struct LdBicgDir {  // BiCGSTAB direction r + beta (p - omega A M p)
    const double *r, *p, *AMp;
    double beta, omega;
    __device__ __forceinline__ double operator()(int j) const
    {
        return __ldcg(r + j) + beta * (__ldcg(p + j) - omega * __ldcg(AMp + j));
    }
};

template <class X>
__device__ __forceinline__ double csr_row(const DevCsr &M, int i, const X &x)
{
    double s = 0;
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
template <int G, class X>
__device__ __forceinline__ double csr_row_g(const DevCsr &M, int i, const X &x)
{
    const int sub = threadIdx.x & (G - 1);
    double s = 0;
    const int k1 = M.ptr[i + 1];
    for (int k = M.ptr[i] + sub; k < k1; k += G) s += M.val[k] * x(M.col[k]);
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(group_mask<G>(), s, o);
    return s;
}

#define FOR_ROWS(i, n) for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)
#define FOR_GROUP_ROWS(G, i, n) \
    for (int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) / G); i < (n); i += (int)((gridDim.x * blockDim.x) / G))

// ---- grid-wide barrier and reduction ------------------------------------------------
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void trace_stamp(unsigned long long *trace)
{
    if (trace && blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned long long k = trace[0] + 1;
        if (k < (unsigned long long)kTraceLen) {
            trace[k] = global_ns();
            trace[0] = k;
        }
    }
}

// Arrivals count up from zero (reset by the host before each launch); barrier k
// is complete when the counter reaches k * gridDim.x.  Returns false when this
// block gave up waiting or saw another block give up.
__device__ bool grid_sync(FusedSyncState *st, unsigned long long *trace)
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
    trace_stamp(trace);
    __syncthreads();
    return ok;
}

// Sum NV per-thread values over the grid.  Thread 0 of every block turns the
// totals into NO scalars with fn - the same arithmetic in every block, so every
// block takes the same decisions - and the block reads them from shared memory
// (the square roots and divisions of the recurrences run once per block, not
// once per thread: FP64 issue is the scarce resource).
template <int NV, int NO, class Fn>
__device__ bool grid_reduce(const double (&v)[NV], const FArgs &a, int &parity, const Fn &fn, double (&o)[NO])
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
    if (!grid_sync(a.sync, a.trace)) return false;
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

template <int NV>
__device__ __forceinline__ bool grid_sum(const double (&v)[NV], double (&tot)[NV], const FArgs &a, int &parity)
{
    return grid_reduce<NV, NV>(v, a, parity, [](const double (&t)[NV], double (&o)[NV]) {
#pragma unroll
        for (int k = 0; k < NV; ++k) o[k] = t[k];
    }, tot);
}

__device__ __forceinline__ int solve_state(double rnorm, double tol, int it, int maxit)
{
    if (!(rnorm == rnorm)) return KS_NAN;
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
template <class Op, class B>
__device__ __forceinline__ void vcycle_residual0_row(const Op &A, const FLevel &V, int i, const B &b, double bi)
{
    V.r[i] = bi - A.row_x(i, V.wd[i] * bi, LdScale<B>{b, V.wd});
}

// Coarsest level: x = A^-1 b with the dense inverse.  Each block stages b in
// shared memory; a warp per row then streams the row of the inverse with many
// loads in flight (they do not depend on one another).
constexpr int kDenseMax = 1536;  // the coarsest level's size limit (kCoarse in amg.cu is below it)

__device__ __forceinline__ void dense_solve(const FLevel &C, const double *b, double *x)
{
    __shared__ double sb[kDenseMax];
    const int n = C.n;
    for (int k = threadIdx.x; k < n; k += blockDim.x) sb[k] = __ldcg(b + k);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int row = warp; row < n; row += nwarps) {
        const double *a = C.inv + (size_t)row * n;
        double acc0 = 0, acc1 = 0;
        int k = lane;
#pragma unroll 8
        for (; k + 32 < n; k += 64) {
            acc0 += a[k] * sb[k];
            acc1 += a[k + 32] * sb[k + 32];
        }
        if (k < n) acc0 += a[k] * sb[k];
        double acc = acc0 + acc1;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) x[row] = acc;
    }
}

// The cycle after its first phase (r_0 written, barrier passed).  b0 is the
// cycle's input (stored).  With dot, returns b0 . z.
template <class Op>
__device__ __forceinline__ bool vcycle_rest(const Op &A, const FArgs &a, const double *b0, double *zout, bool dot,
                                            double rho_prev, double &rz, double &beta, int &parity)
{
    const int L = a.nlev;
    for (int l = 0; l < L - 1; ++l) {
        const FLevel &V = a.lev[l];
        const FLevel &C = a.lev[l + 1];
        if (l > 0) {
            FOR_GROUP_ROWS(kGroupA, i, V.n)
            {
                const double ax = csr_row_g<kGroupA>(V.A, i, LdScale<LdAcc>{LdAcc{V.b}, V.wd});
                if ((threadIdx.x & (kGroupA - 1)) == 0) V.r[i] = __ldcg(V.b + i) - ax;
            }
            if (!grid_sync(a.sync, a.trace)) return false;
        }
        FOR_GROUP_ROWS(kGroupR, i, C.n)
        {
            const double bi = csr_row_g<kGroupR>(V.R, i, LdAcc{V.r});
            if ((threadIdx.x & (kGroupR - 1)) == 0) C.b[i] = bi;
        }
        if (!grid_sync(a.sync, a.trace)) return false;
    }
    const FLevel &C = a.lev[L - 1];
    dense_solve(C, C.b, C.x);
    if (!grid_sync(a.sync, a.trace)) return false;
    const double *xc = C.x;
    for (int l = L - 2; l >= 0; --l) {
        const FLevel &V = a.lev[l];
        const double *bb = l == 0 ? b0 : V.b;
        double *out = l == 0 ? zout : V.t;
        double v[1] = {0};
        if (l == 0) {
            FOR_ROWS(i, V.n)
            {
                const double wdi = V.wd[i];
                const double xi = wdi * __ldcg(bb + i) + csr_row(V.P, i, LdAcc{xc});
                const double o = xi + wdi * (__ldcg(V.r + i) - csr_row(V.AP, i, LdAcc{xc}));
                out[i] = o;
                if (dot) v[0] += __ldcg(b0 + i) * o;
            }
        } else {
            FOR_GROUP_ROWS(kGroupA, i, V.n)
            {
                const double px = csr_row_g<kGroupA>(V.P, i, LdAcc{xc});
                const double apx = csr_row_g<kGroupA>(V.AP, i, LdAcc{xc});
                if ((threadIdx.x & (kGroupA - 1)) == 0) {
                    const double wdi = V.wd[i];
                    const double xi = wdi * __ldcg(bb + i) + px;
                    out[i] = xi + wdi * (__ldcg(V.r + i) - apx);
                }
            }
        }
        if (dot && l == 0) {
            double q[2];
            if (!grid_reduce<1, 2>(v, a, parity, [&](const double (&t)[1], double (&o)[2]) {
                    o[0] = t[0];
                    o[1] = t[0] / rho_prev;
                }, q))
                return false;
            rz = q[0];
            beta = q[1];
        } else if (!grid_sync(a.sync, a.trace)) {
            return false;
        }
        xc = out;
    }
    return true;
}

// z = V(b) for a stored input; with dot also rz = b . z and beta = rz / rho_prev.
// A one-level hierarchy is the dense solve alone.
template <class Op>
__device__ __forceinline__ bool vcycle(const Op &A, const FArgs &a, const double *b, double *zout, bool dot,
                                       double rho_prev, double &rz, double &beta, int &parity)
{
    if (a.nlev == 1) {
        dense_solve(a.lev[0], b, zout);
        if (!grid_sync(a.sync, a.trace)) return false;
        if (!dot) return true;
        double v[1] = {0}, q[2];
        FOR_ROWS(i, a.lev[0].n) v[0] += __ldcg(b + i) * __ldcg(zout + i);
        if (!grid_reduce<1, 2>(v, a, parity, [&](const double (&t)[1], double (&o)[2]) {
                o[0] = t[0];
                o[1] = t[0] / rho_prev;
            }, q))
            return false;
        rz = q[0];
        beta = q[1];
        return true;
    }
    FOR_ROWS(i, a.lev[0].n) vcycle_residual0_row(A, a.lev[0], i, LdAcc{b}, __ldcg(b + i));
    if (!grid_sync(a.sync, a.trace)) return false;
    return vcycle_rest(A, a, b, zout, dot, rho_prev, rz, beta, parity);
}

// ---- CG on the symmetrised system (W A) x = W b ---------------------------------------
// With the SA preconditioner the update x += alpha p, r -= alpha q runs in the
// same phase as the V-cycle's first sweep (which forms r - alpha q at its stencil
// points; the residual is double-buffered).
template <class Op, int PC>
__device__ __forceinline__ bool cg_solve(const Op &A, const FArgs &a, const double *b, double *x, double (&out)[4],
                                         int &it_out, int &status_out)
{
    int parity = 0;
    const double rtol = a.ks->rtol;
    const int maxit = a.ks->maxit;
    const bool merge = PC == 2 && a.nlev >= 2;
    double v[3] = {0, 0, 0}, o[5];
    FOR_ROWS(i, a.n)
    {
        const double bi = b[i];
        const double ri = a.w[i] * bi - A.row(i, LdAcc{x});
        a.r[i] = ri;
        const double ro = ri * a.winv[i];
        v[0] += ro * ro;
        v[1] += bi * bi;
        if (PC != 2) {
            const double zi = PC == 1 ? ri * a.dinv[i] : ri;
            a.z[i] = zi;
            v[2] += ri * zi;
        }
    }
    if (!grid_reduce<3, 5>(v, a, parity, [&](const double (&t)[3], double (&q)[5]) {
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
    double *r = a.r, *rn = a.rs;
    if (status == KS_RUNNING && PC == 2 && !vcycle(A, a, r, a.z, true, 1.0, rho, beta, parity)) return false;
    double *p = a.p, *pn = a.p2;
    bool first = true;
    while (status == KS_RUNNING) {
        // direction pn = z + beta p, q = A pn, pn . q
        double v1[1] = {0}, o1[1];
        FOR_ROWS(i, a.n)
        {
            const double zi = __ldcg(a.z + i);
            double pi, qi;
            if (first) {
                pi = zi;
                qi = A.row_x(i, pi, LdAcc{a.z});
            } else {
                pi = zi + beta * __ldcg(p + i);
                qi = A.row_x(i, pi, LdPnew{a.z, p, beta});
            }
            pn[i] = pi;
            a.q[i] = qi;
            v1[0] += pi * qi;
        }
        if (!grid_reduce<1, 1>(v1, a, parity, [&](const double (&t)[1], double (&q)[1]) { q[0] = rho / t[0]; }, o1))
            return false;
        const double alpha = o1[0];
        {
            double *tmp = p;
            p = pn;
            pn = tmp;
        }
        first = false;
        if (merge) {
            const LdAxpy rnew{r, a.q, alpha};
            double v2[1] = {0}, o2[2];
            FOR_ROWS(i, a.n)
            {
                x[i] = __ldcg(x + i) + alpha * __ldcg(p + i);
                const double ri = rnew(i);
                rn[i] = ri;
                const double ro = ri * a.winv[i];
                v2[0] += ro * ro;
                vcycle_residual0_row(A, a.lev[0], i, rnew, ri);
            }
            if (!grid_reduce<1, 2>(v2, a, parity, [&](const double (&t)[1], double (&q)[2]) {
                    q[0] = sqrt(t[0]);
                    q[1] = solve_state(q[0], tol, it + 1, maxit);
                }, o2))
                return false;
            {
                double *tmp = r;
                r = rn;
                rn = tmp;
            }
            ++it;
            rnorm = o2[0];
            status = (int)o2[1];
            if (status != KS_RUNNING) break;
            double rz = 0;
            if (!vcycle_rest(A, a, r, a.z, true, rho, rz, beta, parity)) return false;
            rho = rz;
            continue;
        }
        double v2[2] = {0, 0}, o2[4];
        FOR_ROWS(i, a.n)
        {
            x[i] = __ldcg(x + i) + alpha * __ldcg(p + i);
            const double ri = __ldcg(r + i) - alpha * __ldcg(a.q + i);
            r[i] = ri;
            const double ro = ri * a.winv[i];
            v2[0] += ro * ro;
            if (PC != 2) {
                const double zi = PC == 1 ? ri * a.dinv[i] : ri;
                a.z[i] = zi;
                v2[1] += ri * zi;
            }
        }
        if (!grid_reduce<2, 4>(v2, a, parity, [&](const double (&t)[2], double (&q)[4]) {
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
            if (!vcycle(A, a, r, a.z, true, rho, rz, beta, parity)) return false;
            rho = rz;
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
template <class Op, int PC>
__device__ __forceinline__ bool bicg_solve(const Op &A, const FArgs &a, const double *b, double *x,
                                           double (&out)[4], int &it_out, int &status_out)
{
    int parity = 0;
    const double rtol = a.ks->rtol;
    const int maxit = a.ks->maxit;
    const bool sa_multi = PC == 2 && a.nlev >= 2;
    double v[2] = {0, 0}, o[5];
    FOR_ROWS(i, a.n)
    {
        const double bi = b[i];
        const double ri = bi - A.row(i, LdAcc{x});
        a.r[i] = ri;
        a.rs[i] = ri;
        a.p[i] = ri;
        v[0] += ri * ri;
        v[1] += bi * bi;
    }
    if (!grid_reduce<2, 5>(v, a, parity, [&](const double (&t)[2], double (&q)[5]) {
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
    double *p = a.p, *pn = a.p2, *amp = a.AMp, *ampn = a.AMp2;
    double beta = 0, omega = 1;
    bool first = true;
    double dummy = 0, dummy2 = 0;
    while (status == KS_RUNNING) {
        // ---- new direction (folded), Mp = M p, A Mp, rs . A Mp
        const LdBicgDir dir{a.r, p, amp, beta, omega};
        if (PC == 2) {
            if (sa_multi) {
                FOR_ROWS(i, a.n)
                {
                    if (first) {
                        vcycle_residual0_row(A, a.lev[0], i, LdAcc{p}, __ldcg(p + i));
                    } else {
                        const double pi = dir(i);
                        pn[i] = pi;
                        vcycle_residual0_row(A, a.lev[0], i, dir, pi);
                    }
                }
                if (!grid_sync(a.sync, a.trace)) return false;
                if (!first) {
                    double *tmp = p;
                    p = pn;
                    pn = tmp;
                }
                if (!vcycle_rest(A, a, p, a.Mp, false, 1.0, dummy, dummy2, parity)) return false;
            } else {
                if (!first) {
                    FOR_ROWS(i, a.n) pn[i] = dir(i);
                    if (!grid_sync(a.sync, a.trace)) return false;
                    double *tmp = p;
                    p = pn;
                    pn = tmp;
                }
                if (!vcycle(A, a, p, a.Mp, false, 1.0, dummy, dummy2, parity)) return false;
            }
        }
        double v1[1] = {0}, o1[1];
        FOR_ROWS(i, a.n)
        {
            double ai;
            if (PC == 2) {
                ai = A.row(i, LdAcc{a.Mp});
            } else if (first) {
                const double pi = __ldcg(p + i);
                const double mpi = PC == 1 ? a.dinv[i] * pi : pi;
                a.Mp[i] = mpi;
                ai = PC == 1 ? A.row_x(i, mpi, LdScale<LdAcc>{LdAcc{p}, a.dinv}) : A.row_x(i, mpi, LdAcc{p});
            } else {
                const double pi = dir(i);
                pn[i] = pi;
                const double mpi = PC == 1 ? a.dinv[i] * pi : pi;
                a.Mp[i] = mpi;
                ai = PC == 1 ? A.row_x(i, mpi, LdScale<LdBicgDir>{dir, a.dinv}) : A.row_x(i, mpi, dir);
            }
            ampn[i] = ai;
            v1[0] += __ldcg(a.rs + i) * ai;
        }
        if (!grid_reduce<1, 1>(v1, a, parity, [&](const double (&t)[1], double (&q)[1]) { q[0] = rho / t[0]; }, o1))
            return false;
        if (PC != 2 && !first) {
            double *tmp = p;
            p = pn;
            pn = tmp;
        }
        {
            double *tmp = amp;
            amp = ampn;
            ampn = tmp;
        }
        first = false;
        const double alpha = o1[0];
        // ---- half step s = r - alpha A Mp (folded into the application of M and A to s)
        const LdAxpy snew{a.r, amp, alpha};
        double o3[3];  // snorm, half-step convergence, omega
        if (PC == 2) {
            double v2[1] = {0};
            if (sa_multi) {
                FOR_ROWS(i, a.n)
                {
                    const double si = snew(i);
                    a.s[i] = si;
                    v2[0] += si * si;
                    vcycle_residual0_row(A, a.lev[0], i, snew, si);
                }
            } else {
                FOR_ROWS(i, a.n)
                {
                    const double si = snew(i);
                    a.s[i] = si;
                    v2[0] += si * si;
                }
            }
            if (!grid_reduce<1, 3>(v2, a, parity, [&](const double (&t)[1], double (&q)[3]) {
                    q[0] = sqrt(t[0]);
                    q[1] = q[0] <= tol;
                    q[2] = 0;
                }, o3))
                return false;
            if (o3[1] != 0) {
                FOR_ROWS(i, a.n) x[i] = __ldcg(x + i) + alpha * __ldcg(a.Mp + i);
                rnorm = o3[0];
                status = KS_CONVERGED;
                break;
            }
            if (sa_multi) {
                if (!vcycle_rest(A, a, a.s, a.Ms, false, 1.0, dummy, dummy2, parity)) return false;
            } else if (!vcycle(A, a, a.s, a.Ms, false, 1.0, dummy, dummy2, parity)) {
                return false;
            }
            double v3[2] = {0, 0}, o4[1];
            FOR_ROWS(i, a.n)
            {
                const double ai = A.row(i, LdAcc{a.Ms});
                a.AMs[i] = ai;
                const double si = __ldcg(a.s + i);
                v3[0] += ai * si;
                v3[1] += ai * ai;
            }
            if (!grid_reduce<2, 1>(v3, a, parity, [&](const double (&t)[2], double (&q)[1]) { q[0] = t[0] / t[1]; },
                                   o4))
                return false;
            o3[2] = o4[0];
        } else {
            double v3[3] = {0, 0, 0};
            FOR_ROWS(i, a.n)
            {
                const double si = snew(i);
                a.s[i] = si;
                const double msi = PC == 1 ? a.dinv[i] * si : si;
                a.Ms[i] = msi;
                const double ai = PC == 1 ? A.row_x(i, msi, LdScale<LdAxpy>{snew, a.dinv}) : A.row_x(i, msi, snew);
                a.AMs[i] = ai;
                v3[0] += ai * si;
                v3[1] += ai * ai;
                v3[2] += si * si;
            }
            if (!grid_reduce<3, 3>(v3, a, parity, [&](const double (&t)[3], double (&q)[3]) {
                    q[0] = sqrt(t[2]);
                    q[1] = q[0] <= tol;
                    q[2] = t[0] / t[1];
                }, o3))
                return false;
            if (o3[1] != 0) {
                FOR_ROWS(i, a.n) x[i] = __ldcg(x + i) + alpha * __ldcg(a.Mp + i);
                rnorm = o3[0];
                status = KS_CONVERGED;
                break;
            }
        }
        omega = o3[2];
        // ---- x, r and the dots that give beta
        double v4[2] = {0, 0}, o5[4];
        FOR_ROWS(i, a.n)
        {
            x[i] = __ldcg(x + i) + (alpha * __ldcg(a.Mp + i) + omega * __ldcg(a.Ms + i));
            const double ri = __ldcg(a.s + i) - omega * __ldcg(a.AMs + i);
            a.r[i] = ri;
            v4[0] += __ldcg(a.rs + i) * ri;
            v4[1] += ri * ri;
        }
        if (!grid_reduce<2, 4>(v4, a, parity, [&](const double (&t)[2], double (&q)[4]) {
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
    }
    out[0] = rnorm;
    out[1] = bnorm;
    out[2] = tol;
    out[3] = rho;
    it_out = it;
    status_out = status;
    return true;
}

template <class Op, int PC, int KRY>
__global__ void __launch_bounds__(kFT, 1) k_fused_solve(Op A, const FArgs *__restrict__ ap, const double *b, double *x)
{
    const FArgs &a = *ap;
    if (a.trace && blockIdx.x == 0 && threadIdx.x == 0) {
        a.trace[0] = 1;
        a.trace[1] = global_ns();
    }
    double res[4];
    int it = 0, status = KS_RUNNING;
    const bool ok = KRY == KRYLOV_CG ? cg_solve<Op, PC>(A, a, b, x, res, it, status)
                                     : bicg_solve<Op, PC>(A, a, b, x, res, it, status);
    trace_stamp(a.trace);
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

// unscaled operator diagonal, summed as the stepwise row functions sum it
template <class Op>
__global__ void k_fused_diag(Op A, int n, double *diag)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    diag[i] = A.row(i, [&](int j) { return j == i ? 1.0 : 0.0; });
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct Op1Plain {
    Lhs1Coef c;
    Grid g;
    template <class X>
    __device__ __forceinline__ double row(int i, const X &x) const
    {
        return lhs1_row_f(c, g, i, x);
    }
};
struct Op2Plain {
    Lhs2Coef c;
    Grid g;
    template <class X>
    __device__ __forceinline__ double row(int i, const X &x) const
    {
        return lhs2_row_f(c, g, i, x);
    }
};

// the operator diagonal the persistent solver's rows use (rows may change when a body moves)
void refresh_fused_diag(Context &c, LinearSystem &S)
{
    if (!S.diag) return;
    if (S.which == 1)
        k_fused_diag<<<blocks_for(S.n), kBlock, 0, c.stream>>>(Op1Plain{c.l1, c.g}, S.n, S.diag);
    else
        k_fused_diag<<<blocks_for(S.n), kBlock, 0, c.stream>>>(Op2Plain{c.l2, c.g}, S.n, S.diag);
    CUIBM_TRY(cudaGetLastError());
}

template <class Op>
static void *pick_kernel(int precond, int krylov)
{
    if (krylov == KRYLOV_CG) {
        if (precond == PC_SMOOTHED_AGGREGATION) return (void *)k_fused_solve<Op, 2, KRYLOV_CG>;
        if (precond == PC_DIAGONAL) return (void *)k_fused_solve<Op, 1, KRYLOV_CG>;
        return (void *)k_fused_solve<Op, 0, KRYLOV_CG>;
    }
    if (precond == PC_SMOOTHED_AGGREGATION) return (void *)k_fused_solve<Op, 2, KRYLOV_BICGSTAB>;
    if (precond == PC_DIAGONAL) return (void *)k_fused_solve<Op, 1, KRYLOV_BICGSTAB>;
    return (void *)k_fused_solve<Op, 0, KRYLOV_BICGSTAB>;
}

template <class Op>
static void launch_fused_op(Context &c, LinearSystem &S, Op A, const double *b, double *x)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(S.fused_grid);
    cfg.blockDim = dim3(kFT);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = c.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    using Fn = void (*)(Op, const FArgs *, const double *, double *);
    const FArgs *args = static_cast<const FArgs *>(S.fargs);
    CUIBM_TRY(cudaLaunchKernelEx(&cfg, reinterpret_cast<Fn>(S.fused_fn), A, args, b, x));
}

// Upload the solver's arguments (after the SA hierarchy exists).
static void upload_fargs(Context &c, LinearSystem &S)
{
    FArgs a = {};
    a.n = S.n;
    a.r = S.r;
    a.rs = S.rs;
    a.p = S.p;
    a.p2 = S.p2;
    a.Mp = S.Mp;
    a.AMp = S.AMp;
    a.AMp2 = S.AMp2;
    a.s = S.s;
    a.Ms = S.Ms;
    a.AMs = S.AMs;
    a.z = S.z;
    a.q = S.q;
    a.dinv = S.dinv;
    a.w = S.w;
    a.winv = S.winv;
    a.diag = S.diag;
    a.partials = S.fpartials;
    a.sync = S.fsync;
    a.trace = c.trace_solve ? c.solve_trace + (S.which - 1) * kTraceLen : nullptr;
    a.ks = S.ks;
    a.err = c.err_word;
    a.which = S.which;
    a.nlev = (int)S.amg.size();
    for (int l = 0; l < a.nlev; ++l) {
        const SaLevel *L = S.amg[l];
        FLevel &F = a.lev[l];
        F.n = L->n;
        F.A = L->A;
        F.P = L->P;
        F.R = L->R;
        F.AP = L->AP;
        F.wd = L->wd;
        F.x = L->x;
        F.b = L->b;
        F.r = L->r;
        F.t = L->t;
        F.inv = L->coarse_inv;
    }
    FArgs *d = S.fargs ? static_cast<FArgs *>(S.fargs) : c.carve<FArgs>(1);
    CUIBM_TRY(cudaMemcpyAsync(d, &a, sizeof(FArgs), cudaMemcpyHostToDevice, c.stream));
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
    S.fargs = d;
}

void launch_fused_solve(Context &c, LinearSystem &S, const double *b, double *x)
{
    CUIBM_TRY(cudaMemsetAsync(S.fsync, 0, sizeof(FusedSyncState), c.stream));
    if (S.which == 1)
        launch_fused_op(c, S, Op1D{c.l1, c.g, S.diag, S.w}, b, x);
    else
        launch_fused_op(c, S, Op2D{c.l2, c.g, S.diag, S.w}, b, x);
}

void set_fused_trace(Context &c, LinearSystem &S, bool on)
{
    (void)on;  // read from c.trace_solve
    if (S.fused_fn) upload_fargs(c, S);
}

// Algorithmic bytes of one solve of `it` iterations as the persistent kernel
// does it: 8 bytes per vector value each phase reads or writes (every vector
// once per phase), 12 per matrix entry (value and column) and 4 per row pointer.
// Used to report achieved bandwidth; the phases are latency- and FP64-issue-
// bound, so this is a floor on traffic, not the bound.
double solve_bytes(const LinearSystem &S, int it)
{
    const double n = S.n, D = 8;
    auto csr = [](const DevCsr &M) { return 12.0 * M.nnz + 4.0 * (M.n + 1); };
    double vc = 0;  // one V-cycle without its first sweep's vector reads
    const int L = (int)S.amg.size();
    if (L == 1) {
        vc = D * (double)S.amg[0]->n * S.amg[0]->n + 2 * D * S.amg[0]->n;
    } else if (L > 1) {
        vc += 2 * D * n;  // first sweep: omega D^-1 and r_0 (its input is counted by the caller)
        for (int l = 0; l < L - 1; ++l) {
            const SaLevel *V = S.amg[l], *C = S.amg[l + 1];
            if (l > 0) vc += 3 * D * V->n + csr(V->A);
            vc += D * V->n + csr(V->R) + D * C->n;                           // restriction
            vc += 4 * D * V->n + csr(V->P) + csr(V->AP) + D * C->n;          // prolongation and sweep
        }
        const double nc = S.amg[L - 1]->n;
        vc += D * nc * nc + 2 * D * nc;
    }
    double per_it, init;
    if (S.krylov == KRYLOV_CG) {
        init = 6 * D * n + (S.precond == PC_SMOOTHED_AGGREGATION ? vc + D * n : 0);
        per_it = 6 * D * n + 7 * D * n + (S.precond == PC_SMOOTHED_AGGREGATION ? vc : 2 * D * n);
    } else {
        init = 6 * D * n;
        if (S.precond == PC_SMOOTHED_AGGREGATION)
            per_it = 7 * D * n + 4 * D * n + 6 * D * n + 4 * D * n + 8 * D * n + 2 * vc;
        else
            per_it = 9 * D * n + 7 * D * n + 8 * D * n;
    }
    return init + it * per_it;
}

// Decide whether the system can use the persistent solver, size its grid (one
// block per SM unless CUIBM_FUSED_BLOCKS_PER_SM asks for more and the kernel's
// registers allow it) and build its tables.
void setup_fused(Context &c, LinearSystem &S)
{
    S.fused_fn = nullptr;
    S.fused_grid = 0;
    if (S.precond == PC_SMOOTHED_AGGREGATION &&
        (S.amg.empty() || (int)S.amg.size() > kMaxLevels || sa_coarsest_size(S) > kDenseMax))
        return;
    void *fn = S.which == 1 ? pick_kernel<Op1D>(S.precond, S.krylov) : pick_kernel<Op2D>(S.precond, S.krylov);
    int dev = 0, sms = 0, coop = 0, per_sm = 0;
    CUIBM_TRY(cudaGetDevice(&dev));
    CUIBM_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CUIBM_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    CUIBM_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kFT, 0));
    if (!coop || per_sm < 1) return;
    int want = 1;
    if (const char *e = getenv("CUIBM_FUSED_BLOCKS_PER_SM")) want = std::max(1, atoi(e));
    S.fused_grid = sms * std::min(per_sm, want);
    S.fused_fn = fn;
    const int n = S.n;
    S.p2 = c.carve<double>(n);
    S.AMp2 = c.carve<double>(n);
    S.fpartials = c.carve<double>((size_t)2 * 4 * S.fused_grid);
    S.fsync = c.carve<FusedSyncState>(1);
    S.diag = c.carve<double>(n);
    CUIBM_TRY(cudaMemsetAsync(S.fsync, 0, sizeof(FusedSyncState), c.stream));
    refresh_fused_diag(c, S);
    S.winv = nullptr;
    if (S.w) {
        std::vector<double> w(n), wi(n);
        CUIBM_TRY(cudaMemcpyAsync(w.data(), S.w, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        CUIBM_TRY(cudaStreamSynchronize(c.stream));
        for (int i = 0; i < n; ++i) wi[i] = 1.0 / w[i];
        S.winv = c.carve<double>(n);
        CUIBM_TRY(cudaMemcpyAsync(S.winv, wi.data(), n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        CUIBM_TRY(cudaStreamSynchronize(c.stream));
    }
    upload_fargs(c, S);
}

}  // namespace cuibm
