// Discrete adjoint of the embedded method's time step (SolverType OSC_CYLINDER, the
// reference's luo_iter step, luo_iter/intermediateVelocity.cu:17-198, luo_iter/poisson.cu:
// 15-152, luo_base/projectVelocity.cu:11-53, luo_base/calculateForce.cu:21-74) with a
// prescribed body motion.  No counterpart in the reference, which has no derivatives.
//
// Objective: J = sum over the steps n of wx[n] Fx^n + wy[n] Fy^n, the control-volume
// force of each step (the period-averaged drag is wx = 2 / nt, wy = 0).  Parameters:
// the viscosity nu, the amplitude uCoefficient of the prescribed body velocity (the
// prescribed path, xCoefficient, is a separate input and stays fixed, so tags and
// interpolation weights do not depend on any parameter: they are frozen at their
// forward values) and per-point offsets of the body velocity (CUIBM_F_BODY_VELOCITY_
// OFFSET).  The reference's kernels read the first point's velocity only (uB[0]), so
// the other points' offsets have zero gradient, exactly.
//
// The step as a map of (u, N, xp) - the velocity, the convection term that the next
// step's Adams-Bashforth reads, the convective-outflow boundary - and the body velocity
// qb = (uB[0], vB[0]) of the step:
//   xp' = R(u, xp)                  Robin outflow (updateRobinBoundary)
//   u1  = Ins(u, qb)                inside velocity (setInsideVelocity)
//   N'  = Nc(u1, xp'), r = u1 + dt (0.5 N - 1.5 N' + 0.5 L(u1, xp', nu)) + B1(u1, xp', nu)
//   rhs1 = r rscale(nu) | r pns(nu) + pint(qb) | 2 qb - sum w q (ghost rows)
//   uhat = A1(nu)^-1 rhs1,  rhs2 = s (-D uhat + boundary),  p = A2^-1 rhs2
//   u2  = uhat - G p,  u3 = Ghost(u2, qb),  u4 = Ins(u3, qb),  F = Force(u4, u1, p, nu)
// The adjoint runs the transposes of these maps in reverse order:
//  * transposed stencils: the convection Jacobian, diffusion and boundary terms
//    (k_adj_rhs1), the divergence (k_adj_rhs2), the gradient (k_adj_project), the
//    force (k_adj_force) - each a local Jacobian taken with forward-mode duals of K
//    slots (MD<K>) over the same expressions as the forward kernels, scattered with
//    atomic adds (so adjoint results agree run to run to rounding, not bit for bit);
//  * transposed interpolation: the ghost-node values after the projection
//    (k_adj_ghost) and the inside velocity (k_adj_inside) over the interpolation
//    plan of the forward step (tags frozen);
//  * transposed solves: BiCGSTAB on A1^T (Jacobi) and on A2^T preconditioned by the
//    transposed V-cycle of the forward SA hierarchy - the same aggregates and
//    prolongators, the level matrices transposed (P^T A^T P = (P^T A P)^T)
//    (krylov.cu launch_solve_transposed, amg.cu launch_vcycle_transposed);
//  * the nu-derivative of the operator A1 and of the row scales (k_adj_dA1nu, k_adj_rhs1).
// Checkpointing: binomial (Griewank's Revolve schedule) over `snapshots` stored states;
// each step's intermediates are recomputed from the nearest stored state (the "tape"
// step) just before its adjoint.
#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/cuibm.h"
#include "amg.h"
#include "ib_plan.h"
#include "operators.cuh"
#include "solver.h"

namespace cuibm {

// ---- forward-mode duals with K derivative slots (local Jacobians) -------------------
template <int K>
struct MD {
    double v;
    double d[K];
};
template <int K>
__device__ __forceinline__ MD<K> mdc(double a)
{
    MD<K> r;
    r.v = a;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = 0;
    return r;
}
template <int K>
__device__ __forceinline__ MD<K> operator+(const MD<K> &a, const MD<K> &b)
{
    MD<K> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ MD<K> operator-(const MD<K> &a, const MD<K> &b)
{
    MD<K> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ MD<K> operator-(const MD<K> &a)
{
    MD<K> r;
    r.v = -a.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = -a.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ MD<K> operator*(const MD<K> &a, const MD<K> &b)
{
    MD<K> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
template <int K>
__device__ __forceinline__ MD<K> operator*(const MD<K> &a, double b)
{
    MD<K> r;
    r.v = a.v * b;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] * b;
    return r;
}
template <int K>
__device__ __forceinline__ MD<K> operator*(double b, const MD<K> &a)
{
    return a * b;
}
template <int K>
__device__ __forceinline__ MD<K> operator/(const MD<K> &a, double b)
{
    MD<K> r;
    r.v = a.v / b;
#pragma unroll
    for (int k = 0; k < K; ++k) r.d[k] = a.d[k] / b;
    return r;
}
template <int K>
__device__ __forceinline__ MD<K> operator+(const MD<K> &a, double b)
{
    MD<K> r = a;
    r.v += b;
    return r;
}
template <int K>
__device__ __forceinline__ MD<K> operator+(double b, const MD<K> &a)
{
    return a + b;
}
template <int K>
__device__ __forceinline__ MD<K> operator-(double b, const MD<K> &a)
{
    return (-a) + b;
}
template <int K>
__device__ __forceinline__ MD<K> operator-(const MD<K> &a, double b)
{
    return a + (-b);
}

// Each traced input takes the next slot; after the evaluation the gradient of the
// objective goes back to the recorded (array, index) pairs.
template <int K>
struct Trace {
    int n = 0;
    int idx[K];
    int arr[K];
    __device__ __forceinline__ MD<K> in(double value, int a, int i)
    {
        MD<K> r = mdc<K>(value);
        if (n < K) {
            r.d[n] = 1.0;
            idx[n] = i;
            arr[n] = a;
            ++n;
        }
        return r;
    }
    __device__ __forceinline__ void scatter(const MD<K> &f, double *const *targets) const
    {
        for (int s = 0; s < n; ++s)
            if (f.d[s] != 0) atomicAdd(targets[arr[s]] + idx[s], f.d[s]);
    }
};

__device__ __forceinline__ double warp_sum(double a)
{
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    return a;
}

// per-block sums of up to three scalars, then one atomic add each
__device__ __forceinline__ void block_add(double a, double b, double c, double *ta, double *tb, double *tc)
{
    __shared__ double sh[3][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    a = warp_sum(a);
    b = warp_sum(b);
    c = warp_sum(c);
    if (lane == 0) {
        sh[0][wid] = a;
        sh[1][wid] = b;
        sh[2][wid] = c;
    }
    __syncthreads();
    if (wid == 0) {
        a = lane < nw ? sh[0][lane] : 0.0;
        b = lane < nw ? sh[1][lane] : 0.0;
        c = lane < nw ? sh[2][lane] : 0.0;
        a = warp_sum(a);
        b = warp_sum(b);
        c = warp_sum(c);
        if (lane == 0) {
            if (ta && a != 0) atomicAdd(ta, a);
            if (tb && b != 0) atomicAdd(tb, b);
            if (tc && c != 0) atomicAdd(tc, c);
        }
    }
}

// ---- the transposed lists of the patched rows -------------------------------------
// Slots: velocity ghost [0, count[0]) and hybrid [cap1, cap1 + count[1]); pressure ghost
// [0, count[2]) and hybrid [cap2, cap2 + count[3]).  A slot counts only if the operator
// uses it (pid[row] == slot): a node tagged ghost and hybrid has a ghost slot that its
// row does not use.
__global__ void k_tlist_count(IbPlan P, int sys, int cap, const int *__restrict__ pid, const int *__restrict__ pcol,
                              int *prow, int *cnt, int *ent, int tmax, int *overflow)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int ng = P.count[sys == 1 ? 0 : 2], nh = P.count[sys == 1 ? 1 : 3];
    int slot, row;
    if (k < ng) {
        slot = k;
        row = sys == 1 ? P.gvNode[k] : P.gpNode[k];
    } else if (k < ng + nh) {
        slot = cap + (k - ng);
        row = sys == 1 ? P.hvNode[k - ng] : P.hpNode[k - ng];
    } else {
        return;
    }
    prow[slot] = row;
    if (pid[row] != slot) return;
    for (int m = 0; m < 5; ++m) {
        const int col = pcol[5 * slot + m];
        if (col < 0) continue;
        const int pos = atomicAdd(cnt + col, 1);
        if (pos < tmax) ent[(size_t)col * tmax + pos] = 5 * slot + m;
        else atomicExch(overflow, 1);
    }
}

// the entries of each column in ascending order (a fixed summation order)
__global__ void k_tlist_sort(int n, const int *cnt, int *ent, int tmax)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = cnt[i] < tmax ? cnt[i] : tmax;
    int *e = ent + (size_t)i * tmax;
    for (int a = 1; a < c; ++a) {
        const int v = e[a];
        int b = a - 1;
        while (b >= 0 && e[b] > v) {
            e[b + 1] = e[b];
            --b;
        }
        e[b + 1] = v;
    }
}

// ---- the force (k_force's items, ib_kernels.cu force_body) ------------------------
// The six sums' items, each an expression of a few field values: traced inputs are the
// step's final velocity (target 0), the velocity the projection kept as uold (target
// 1), the pressure (2) and nu (3, index 0).  The objective of an item is its weight
// (wx for the drag sums, wy for the lift sums) times its contribution.
constexpr int kForceK = 10;

__global__ void k_adj_force(int nx, int ny, const int *__restrict__ bb, const double *__restrict__ u,
                            const double *__restrict__ uold, const double *__restrict__ p,
                            const int *__restrict__ gtags, double nu_v, const double *__restrict__ dx,
                            const double *__restrict__ dy, double dt, double wx, double wy, double *ubar,
                            double *uoldbar, double *pbar, double *nubar)
{
    using T = MD<kForceK>;
    const int I = bb[0], J = bb[1], ncx = bb[2], ncy = bb[3];
    const int nU = (nx - 1) * ny;
    const int o1 = ncy, o3 = o1 + ncx + 1, o4 = o3 + ncy + 1, o2 = o4 + ncx, o5 = o2 + (ncx + 1) * ncy;
    const int total = o5 + ncx * (ncy + 1);
    double *const tg[4] = {ubar, uoldbar, pbar, nubar};
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
        Trace<kForceK> tr;
        auto U = [&](int i) { return tr.in(u[i], 0, i); };
        auto UO = [&](int i) { return tr.in(uold[i], 1, i); };
        auto PP = [&](int i) { return tr.in(p[i], 2, i); };
        T f = mdc<kForceK>(0.0);
        if (q < o1) {  // dragLeftRight
            const int idx = q;
            const int Ip = (J + idx) * nx + I, Iu = (J + idx) * (nx - 1) + I;
            const T nu = tr.in(nu_v, 3, 0);
            const T e1 = U(Iu + ncx), e0 = U(Iu + ncx - 1), w1 = U(Iu - 1), w0 = U(Iu);
            const T pe = PP(Ip + ncx), pw = PP(Ip);
            const T a = e1 + e0, b = w1 + w0;
            f = -((pe - pw) * dy[J + idx] + (a * a / 4 - b * b / 4) * dy[J + idx] -
                  nu * ((e1 - e0) / dx[I + ncx] - (w0 - w1) / dx[I]) * dy[J + idx]);
            f = f * wx;
        } else if (q < o3) {  // dragBottomTop
            const int idx = q - o1;
            const int Iu = J * (nx - 1) + (I - 1 + idx), Iv = nU + (J - 1) * nx + I + idx;
            const T nu = tr.in(nu_v, 3, 0);
            const T ut1 = U(Iu + ncy * (nx - 1)), ut0 = U(Iu + (ncy - 1) * (nx - 1));
            const T vt1 = U(Iv + ncy * nx), vt0 = U(Iv + ncy * nx - 1);
            const T ub1 = U(Iu), ub0 = U(Iu - (nx - 1)), vb1 = U(Iv), vb0 = U(Iv - 1);
            f = -((0.25 * (ut1 + ut0) * (vt1 + vt0) - 0.25 * (ub1 + ub0) * (vb1 + vb0)) -
                  nu * (((ut1 - ut0) / 2.0 / (dy[J + ncy] + dy[J + ncy - 1]) +
                         (vt1 - vt0) / 2.0 / (dx[I + idx] + dx[I + idx - 1])) -
                        ((ub1 - ub0) / 2.0 / (dy[J] + dy[J - 1]) + (vb1 - vb0) / 2.0 / (dx[I + idx] + dx[I + idx - 1])))) *
                0.5 * (dx[I + idx] + dx[I + idx - 1]);
            f = f * wx;
        } else if (q < o4) {  // liftLeftRight
            const int idx = q - o3;
            const int Iu = (J + idx) * (nx - 1) + (I - 1), Iv = nU + (J - 1 + idx) * nx + I;
            const T nu = tr.in(nu_v, 3, 0);
            const T ur1 = U(Iu + ncx), ur0 = U(Iu + ncx - (nx - 1)), vr1 = U(Iv + ncx), vr0 = U(Iv + ncx - 1);
            const T ul1 = U(Iu), ul0 = U(Iu - (nx - 1)), vl1 = U(Iv), vl0 = U(Iv - 1);
            f = -((0.25 * (ur1 + ur0) * (vr1 + vr0) - 0.25 * (ul1 + ul0) * (vl1 + vl0)) -
                  nu * (((ur1 - ur0) / 2.0 / (dy[J + idx] + dy[J - 1 + idx]) +
                         (vr1 - vr0) / 2.0 / (dx[I + ncx] + dx[I + ncx - 1])) -
                        ((ul1 - ul0) / 2.0 / (dy[J + idx] + dy[J - 1 + idx]) + (vl1 - vl0) / 2.0 / (dx[I] + dx[I - 1])))) *
                0.5 * (dy[J + idx] + dy[J - 1 + idx]);
            f = f * wy;
        } else if (q < o2) {  // liftBottomTop
            const int idx = q - o4;
            const int Ip = J * nx + I + idx, Iv = nU + (J - 1) * nx + I + idx;
            const T nu = tr.in(nu_v, 3, 0);
            const T t1 = U(Iv + (ncy + 1) * nx), t0 = U(Iv + ncy * nx), b1 = U(Iv), b0 = U(Iv - nx);
            const T pt = PP(Ip + ncy * nx), pb = PP(Ip - nx);
            const T a = t1 + t0, b = b1 + b0;
            f = -((pt - pb) * dx[I + idx] + (0.25 * a * a - 0.25 * b * b) * dx[I + idx] -
                  nu * ((t1 - t0) * dx[I + idx] / dy[J + ncy] - (b1 - b0) * dx[I] / dy[J - 1]));
            f = f * wy;
        } else if (q < o5) {  // dragUnsteady (fluid nodes only)
            const int idx = q - o2;
            const int i = idx % (ncx + 1), j = idx / (ncx + 1), Iu = (J + j) * (nx - 1) + (I - 1 + i);
            if (gtags[Iu] == -1) {
                const T a = U(Iu), b = UO(Iu);
                f = -((a * dy[J + j] - b * dy[J + j]) / dt * 0.5 * (dx[I + i] + dx[I - 1 + i]));
                f = f * wx;
            }
        } else {  // liftUnsteady
            const int idx = q - o5;
            const int i = idx % ncx, j = idx / ncx, Iv = (J - 1 + j) * nx + (I + i) + nU;
            if (gtags[Iv] == -1) {
                const T a = U(Iv), b = UO(Iv);
                f = -((a * dx[I + i] - b * dx[I + i]) / dt * 0.5 * (dy[J + j] + dy[J - 1 + j]));
                f = f * wy;
            }
        }
        tr.scatter(f, tg);
    }
}

// ---- inside velocity and ghost values (the interpolation plan, tags frozen) -------
// u = Ins(u, qb): the inside nodes take the body velocity.  Transposed: their adjoint
// goes to qb (u or v block) and is cleared.
__global__ void k_adj_inside(IbPlan P, int nU, double *ubar, double *qbar)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    double su = 0, sv = 0;
    if (k < P.count[4]) {
        const int n = P.inNode[k];
        const double a = ubar[n];
        ubar[n] = 0;
        if (n >= nU) sv = a;
        else su = a;
    }
    block_add(su, sv, 0, qbar, qbar + 1, nullptr);
}

// u3 = Ghost(u2, qb): each ghost node becomes 2 qb - sum_l w_l q_l, q_l the body value
// (masked corners) or u2 at the corner (read before any ghost node is written).
// Transposed, into u2bar (a copy of u3bar on entry).
__global__ void k_adj_ghost(IbPlan P, int nU, const double *__restrict__ u3bar, double *u2bar, double *qbar)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    double su = 0, sv = 0;
    if (k < P.count[0]) {
        const int n = P.gvNode[k], m = P.gvMask[k];
        const double a = u3bar[n];
        double cq = 2;
        for (int l = 0; l < 4; ++l) {
            const double w = P.gvW[4 * k + l];
            if (m >> l & 1) cq -= w;
            else atomicAdd(u2bar + P.gvIdx[4 * k + l], -w * a);
        }
        atomicAdd(u2bar + n, -a);  // the node's own value is overwritten
        if (n >= nU) sv = cq * a;
        else su = cq * a;
    }
    block_add(su, sv, 0, qbar, qbar + 1, nullptr);
}

// ---- projection u2 = uhat - G p (k_project) ------------------------------------------
__global__ void k_adj_project(Grid g, const double *__restrict__ gradU, const double *__restrict__ gradV,
                              const double *__restrict__ u2bar, double *uhbar, double *pbar)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < g.nUV) uhbar[t] = u2bar[t];
    if (t < g.nP) {
        const int nx = g.nx, ny = g.ny, I = t % nx, J = t / nx;
        double a = 0;
        if (I <= nx - 2) a += gradU[I] * u2bar[J * (nx - 1) + I];
        if (I >= 1) a -= gradU[I - 1] * u2bar[J * (nx - 1) + I - 1];
        if (J <= ny - 2) a += gradV[J] * u2bar[g.nU + J * nx + I];
        if (J >= 1) a -= gradV[J - 1] * u2bar[g.nU + (J - 1) * nx + I];
        pbar[t] += a;
    }
}

// ---- rhs2 = s (-D uhat) with the x+ boundary (k_rhs2) ---------------------------------
// s: the embedded rows' ns_rhs (pns) on patched rows below (nx-1) ny, else 1
__device__ __forceinline__ double rhs2_scale(const int *pid2, const double *pns2, int nx, int ny, int ip)
{
    if (!pid2 || ip >= (nx - 1) * ny) return 1.0;
    const int k = pid2[ip];
    return k >= 0 ? pns2[k] : 1.0;
}

__global__ void k_adj_rhs2(Grid g, const double *__restrict__ dx, const double *__restrict__ dy,
                           const int *__restrict__ pid2, const double *__restrict__ pns2,
                           const double *__restrict__ r2bar, double *uhbar, double *xpbar)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int nx = g.nx, ny = g.ny;
    if (t < g.nU) {
        const int I = t % (nx - 1), J = t / (nx - 1);
        const int c1 = J * nx + I, c2 = c1 + 1;  // east face of c1, west face of c2
        uhbar[t] += -rhs2_scale(pid2, pns2, nx, ny, c1) * r2bar[c1] / dx[I] +
                    rhs2_scale(pid2, pns2, nx, ny, c2) * r2bar[c2] / dx[I + 1];
    } else if (t < g.nUV) {
        const int k = t - g.nU, I = k % nx, J = k / nx;
        const int c1 = J * nx + I, c2 = c1 + nx;  // north face of c1, south face of c2
        uhbar[t] += -rhs2_scale(pid2, pns2, nx, ny, c1) * r2bar[c1] / dy[J] +
                    rhs2_scale(pid2, pns2, nx, ny, c2) * r2bar[c2] / dy[J + 1];
    }
    if (t < ny) {  // the x+ boundary velocity stands in for the east face of the last column
        const int c = t * nx + nx - 1;
        xpbar[t] += -rhs2_scale(pid2, pns2, nx, ny, c) * r2bar[c] / dx[nx - 1];
    }
}

// ---- the hybrid rows' coefficients (embedded.cu k_emb_rows) ------------------------
// c[0..3] the unblended N, E, S, W coefficients of node n's momentum row, c[4] its diagonal
__device__ __forceinline__ void hybrid_velocity_coefs(int n, int nx, int ny, double dt, double nu, const double *dx,
                                                      const double *dy, double c[5])
{
    const int nU = (nx - 1) * ny;
    const bool v = n >= nU;
    const int I = v ? (n - nU) % nx : n % (nx - 1), J = v ? (n - nU) / nx : n / (nx - 1);
    c[0] = -dt * nu / (dy[J + 1] * (dy[J] + dy[J + 1]));
    c[1] = -dt * nu / (dx[I] * (dx[I] + dx[I + 1]));
    c[2] = -dt * nu / (dy[J] * (dy[J] + dy[J + 1]));
    c[3] = -dt * nu / (dx[I] * (dx[I] + dx[I - 1]));
    c[4] = 1 - c[0] - c[1] - c[2] - c[3];
}

// ---- d(A1 x)/d nu (the operator's viscosity dependence) ----------------------------
// Rows without a patch are s (d x_i - sum_j c_ij x_j) with c proportional to nu,
// d = 1 + sum c and s = 1/d on interior rows (1 on boundary rows): the derivative is
// s (s g - x_i) / nu with g the unscaled row.  A hybrid row's momentum part
// (1 - a) c_l / c4 has derivative (1 - a) c_l / (nu c4^2).  Ghost rows do not depend on nu.
// nubar -= sum_i r1bar_i (dA1/dnu x)_i
__global__ void k_adj_dA1nu(Lhs1Coef cf, Grid g, IbPlan P, int cap1, double dt, double nu,
                            const double *__restrict__ dx, const double *__restrict__ dy,
                            const double *__restrict__ x, const double *__restrict__ r1bar, double *nubar)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double a = 0;
    if (i < g.nUV) {
        const int k = cf.patch.pid ? cf.patch.pid[i] : -1;
        if (k < 0) {
            Lhs1Coef raw = cf;
            raw.patch.pid = nullptr;
            raw.rscale = nullptr;
            const double gi = lhs1_row(raw, g, i, x);
            const double s = cf.rscale ? cf.rscale[i] : 1.0;
            a = r1bar[i] * s * (s * gi - x[i]) / nu;
        } else if (k >= cap1) {
            const int n = i, s = n >= g.nU ? g.nx : g.nx - 1;
            double c[5];
            hybrid_velocity_coefs(n, g.nx, g.ny, dt, nu, dx, dy, c);
            const double al = P.hvAlpha[k - cap1], f = (1 - al) / (nu * c[4] * c[4]);
            a = r1bar[i] * f * (c[0] * x[n + s] + c[1] * x[n + 1] + c[2] * x[n - s] + c[3] * x[n - 1]);
        }
    }
    block_add(-a, 0, 0, nubar, nullptr, nullptr);
}

// ---- the explicit right-hand side (ns_kernels.cu k_rhs1) -----------------------------
// N (convection), L (diffusion) and B1 (implicit-diffusion boundary terms) of node t as
// functions of the velocity (traced, target 0), the x+ boundary (traced, target 1) and nu
// (traced, target 2); the other boundaries are fixed inputs.
constexpr int kRhsK = 12;
struct BcPtrsA {
    const double *xm, *xp, *ym, *yp;
};

template <class TR>
__device__ __forceinline__ void rhs_terms(const RhsCoef &c, const Grid &g, const BcPtrsA &b, int t, double dt,
                                          const double *__restrict__ u, double nu_v, TR &tr, MD<kRhsK> &Nn,
                                          MD<kRhsK> &Ln, MD<kRhsK> &B1)
{
    using T = MD<kRhsK>;
    const int nx = g.nx, ny = g.ny, nU = g.nU;
    auto U = [&](int i) { return tr.in(u[i], 0, i); };
    auto XP = [&](int i) { return tr.in(b.xp[i], 1, i); };
    auto C = [&](double v) { return mdc<kRhsK>(v); };
    const T nu = tr.in(nu_v, 2, 0);
    const T hd = 0.5 * dt * nu;
    const T uc = U(t);
    B1 = C(0.0);
    if (t < nU) {
        const int I = t % (nx - 1), J = t / (nx - 1), iv = nU + nx * J + I;
        const T ue = (I == nx - 2) ? XP(J) : U(t + 1);
        const T uw = (I == 0) ? C(b.xm[J]) : U(t - 1);
        const T un = (J == ny - 1) ? C(0.0) : U(t + nx - 1);
        const T us = (J == 0) ? C(0.0) : U(t - nx + 1);
        const T vne = (J == ny - 1) ? C(b.yp[nx + I]) : U(iv + 1);
        const T vn = (J == ny - 1) ? C(b.yp[nx - 1 + I]) : U(iv);
        const T vse = (J == 0) ? C(b.ym[nx + I]) : U(iv - nx + 1);
        const T vs = (J == 0) ? C(b.ym[nx - 1 + I]) : U(iv - nx);
        const double a = c.uxA[I];
        const T vbar = ((vne - vn) * a + vn) / 2 + ((vse - vs) * a + vs) / 2;
        const T unc = (J == ny - 1) ? 2 * b.yp[I] - uc : un;
        const T usc = (J == 0) ? 2 * b.ym[I] - uc : us;
        Nn = uc * (ue * c.uxE[I] + uw * c.uxW[I] + uc * c.uxC[I]) + vbar * (unc * c.uyN[J] + usc * c.uyS[J] + uc * c.uyC[J]);
        const T unl = (J == ny - 1) ? C(b.yp[I]) : un;
        const T usl = (J == 0) ? C(b.ym[I]) : us;
        Ln = nu * ((ue - uc) * c.ulE[I] + (uw - uc) * c.ulW[I] + (unl - uc) * c.ulN[J] + (usl - uc) * c.ulS[J]);
        if (I == nx - 2) B1 = B1 + ue * hd * c.ulE[I];  // ue is the x+ boundary value here
        if (I == 0) B1 = B1 + b.xm[J] * hd * c.ulW[I];
        if (J == ny - 1) B1 = B1 + (2 * b.yp[I] - uc) * hd * (0.5 * c.ulN[J]);
        if (J == 0) B1 = B1 + (2 * b.ym[I] - uc) * hd * (0.5 * c.ulS[J]);
    } else {
        const int k = t - nU, I = k % nx, J = k / nx, iu = (nx - 1) * J + I;
        const T ve = (I == nx - 1) ? C(0.0) : U(t + 1);
        const T vw = (I == 0) ? C(0.0) : U(t - 1);
        const T vn = (J == ny - 2) ? C(b.yp[nx - 1 + I]) : U(t + nx);
        const T vs = (J == 0) ? C(b.ym[nx - 1 + I]) : U(t - nx);
        const T une = (I == nx - 1) ? XP(J + 1) : U(iu + nx - 1);
        const T ue = (I == nx - 1) ? XP(J) : U(iu);
        const T unw = (I == 0) ? C(b.xm[J + 1]) : U(iu + nx - 2);
        const T uw = (I == 0) ? C(b.xm[J]) : U(iu - 1);
        const double a = c.vyA[J];
        const T ubar = ((une - ue) * a + ue) / 2 + ((unw - uw) * a + uw) / 2;
        const T xpv = (I == nx - 1) ? XP(ny + J) : C(0.0);
        const T vec = (I == nx - 1) ? 2 * xpv - uc : ve;
        const T vwc = (I == 0) ? 2 * b.xm[ny + J] - uc : vw;
        Nn = ubar * (vec * c.vxE[I] + vwc * c.vxW[I] + uc * c.vxC[I]) + uc * (vn * c.vyN[J] + vs * c.vyS[J] + uc * c.vyC[J]);
        const T vel = (I == nx - 1) ? xpv : ve;
        const T vwl = (I == 0) ? C(b.xm[ny + J]) : vw;
        Ln = nu * ((vel - uc) * c.vlE[I] + (vwl - uc) * c.vlW[I] + (vn - uc) * c.vlN[J] + (vs - uc) * c.vlS[J]);
        if (I == nx - 1) B1 = B1 + (2 * xpv - uc) * hd * (0.5 * c.vlE[I]);
        if (I == 0) B1 = B1 + (2 * b.xm[ny + J] - uc) * hd * (0.5 * c.vlW[I]);
        if (J == ny - 2) B1 = B1 + b.yp[nx - 1 + I] * hd * c.vlN[J];
        if (J == 0) B1 = B1 + b.ym[nx - 1 + I] * hd * c.vlS[J];
    }
}

struct AdjRhs1 {
    const int *pid;
    const double *rscale, *pns;
    int cap;
    const int *gin;
    IbPlan P;
};

// Transposed rhs1: from r1bar (the adjoint of the step's rhs1) and Nbar (on entry the
// adjoint of this step's N through the next step's Nold; on exit the adjoint of this
// step's Nold), into u1bar (the velocity after the inside velocity), xpbar (the x+
// boundary after the Robin update), qbar (body velocity) and nubar.
__global__ void __launch_bounds__(256) k_adj_rhs1(RhsCoef c, Grid g, BcPtrsA b, double dt, double nu,
                                                  const double *__restrict__ u1, const double *__restrict__ Nold,
                                                  AdjRhs1 e, const double *__restrict__ dx,
                                                  const double *__restrict__ dy, const double *__restrict__ r1bar,
                                                  double *Nbar, double *u1bar, double *xpbar, double *qbar,
                                                  double *nubar)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double qu = 0, qv = 0, nb = 0;
    if (t < g.nUV) {
        const double rb = r1bar[t];
        const bool vnode = t >= g.nU;
        const int k = e.pid ? e.pid[t] : -1;
        double rbar;        // adjoint of the unscaled right-hand side r
        double dscale = 0;  // d(scale)/d nu
        double qcoef = 0;   // d rhs1 / d qb
        if (k < 0) {
            const double s = e.rscale ? e.rscale[t] : 1.0;
            rbar = rb * s;
            dscale = -s * (1 - s) / nu;
        } else if (k >= e.cap) {
            const int kk = k - e.cap;
            const double al = e.P.hvAlpha[kk];
            rbar = rb * e.pns[k];
            double cc[5];
            hybrid_velocity_coefs(t, g.nx, g.ny, dt, nu, dx, dy, cc);
            dscale = -(1 - al) / (cc[4] * cc[4]) * (cc[4] - 1) / nu;
            for (int l = 0; l < 4; ++l)
                if (e.P.hvIdx[4 * kk + l] == t) qcoef += e.P.hvW[4 * kk + l] * al;
        } else {
            rbar = 0;
            const int in = e.gin[k], m = e.P.gvMask[k];
            qcoef = 2;
            for (int l = 0; l < 4; ++l)
                if (in >> l & 1) {
                    const double w = e.P.gvW[4 * k + l];
                    if (m >> l & 1) qcoef -= w;
                    else atomicAdd(u1bar + e.P.gvIdx[4 * k + l], -w * rb);
                }
        }
        if (vnode) qv = qcoef * rb;
        else qu = qcoef * rb;
        Trace<kRhsK> tr;
        MD<kRhsK> Nn, Ln, B1;
        rhs_terms(c, g, b, t, dt, u1, nu, tr, Nn, Ln, B1);
        const double Nb = Nbar[t] - 1.5 * dt * rbar;
        const MD<kRhsK> f = Nn * Nb + Ln * (0.5 * dt * rbar) + B1 * rbar;
        double *const tg[3] = {u1bar, xpbar, nubar};
        tr.scatter(f, tg);
        atomicAdd(u1bar + t, rbar);  // the r = u1 + ... term
        Nbar[t] = 0.5 * dt * rbar;    // this step's Nold
        if (dscale != 0) {
            const double r = u1[t] + dt * (0.5 * Nold[t] - 1.5 * Nn.v + 0.5 * Ln.v) + B1.v;
            nb = rb * r * dscale;
        }
    }
    block_add(qu, qv, nb, qbar, qbar + 1, nubar);
}

// ---- Robin outflow xp' = (1 - beta) xp + beta u[last column] (k_ib_step PH_ROBIN) ----
__global__ void k_adj_robin(int nx, int ny, double dt, const double *__restrict__ dx, double *xpbar, double *ubar)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= 2 * ny - 1) return;
    const int nU = (nx - 1) * ny;
    const double beta = 1.0 * dt / dx[nx - 1];
    const double a = xpbar[r];
    const int i = r < ny ? r * (nx - 1) + nx - 2 : nU + (r - ny) * nx + nx - 1;
    ubar[i] += beta * a;
    xpbar[r] = (1 - beta) * a;
}

__global__ void k_accum_objective(const double *force, double wx, double wy, double *J)
{
    if (threadIdx.x == 0) *J += wx * force[0] + wy * force[1];
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

constexpr int kTransposeMax = 32;  // patched rows holding one column, at most

struct Snapshot {
    double *blk = nullptr;  // u, uhat, N (nUV each), p (nP), xp (2ny-1), body (6 nb), motion,
                            // the pressure nodes' intercepts and image points (4 nP)
    int *step = nullptr;    // the device step counter, then the force's box (4 ints): the first
                            // step's box is the initial body's, not the box of its position
    int timeStep = 0;
    int holds = -1;  // the step whose state it holds, -1 free
};

struct AdjointState {
    int nUV = 0, nP = 0, nxp = 0, nb = 0, steps_cap = 0;
    double *ubar = nullptr, *u1bar = nullptr, *u2bar = nullptr, *uhbar = nullptr, *r1bar = nullptr;
    double *pbar = nullptr, *r2bar = nullptr, *Nbar = nullptr, *xpbar = nullptr, *u2tape = nullptr;
    double *scal = nullptr;  // [0] nubar, [1] J, [2 + 2 n] qbar of step n (u, v)
    int *tcnt1 = nullptr, *tent1 = nullptr, *prow1 = nullptr;
    int *tcnt2 = nullptr, *tent2 = nullptr, *prow2 = nullptr;
    int *overflow = nullptr;
    LinearSystem S1T, S2T;
    std::vector<void *> allocs;
    std::vector<Snapshot> snaps;
    // two stashes of one step's solutions (uhat, then p) with the step they belong to
    // (-1 none): the solutions of a checkpoint step whose snapshot was released, or of
    // the last step of an advance, kept for the tape that comes next
    double *stash[2] = {nullptr, nullptr};
    int stash_step[2] = {-1, -1};
    // statistics of the last run
    long long forward_steps = 0, tape_steps = 0, solves_reused = 0;
    long long it1 = 0, it2 = 0;
};

AdjointState &adj(Context &c) { return *static_cast<AdjointState *>(c.adj); }

void *dalloc(AdjointState &A, size_t bytes)
{
    void *p = nullptr;
    CUIBM_TRY(cudaMalloc(&p, bytes));
    A.allocs.push_back(p);
    return p;
}

size_t snapshot_doubles(const AdjointState &A)
{
    return 3 * (size_t)A.nUV + 5 * (size_t)A.nP + A.nxp + 6 * (size_t)A.nb + kMotionLen;
}

void ensure_state(Context &c, int nsteps, int snapshots)
{
    if (!c.adj) c.adj = new AdjointState();
    AdjointState &A = adj(c);
    if (!A.ubar) {
        A.nUV = c.g.nUV;
        A.nP = c.g.nP;
        A.nxp = 2 * c.g.ny - 1;
        A.nb = c.body.total;
        const size_t UV = A.nUV, P = A.nP;
        double *blk = static_cast<double *>(dalloc(A, (7 * UV + 2 * P + (size_t)A.nxp) * sizeof(double)));
        A.ubar = blk;
        A.u1bar = blk + UV;
        A.u2bar = blk + 2 * UV;
        A.uhbar = blk + 3 * UV;
        A.r1bar = blk + 4 * UV;
        A.Nbar = blk + 5 * UV;
        A.u2tape = blk + 6 * UV;
        double *q = blk + 7 * UV;
        A.pbar = q;
        A.r2bar = q + P;
        A.xpbar = q + 2 * P;
        A.tcnt1 = static_cast<int *>(dalloc(A, UV * sizeof(int)));
        A.tent1 = static_cast<int *>(dalloc(A, UV * kTransposeMax * sizeof(int)));
        A.prow1 = static_cast<int *>(dalloc(A, 2 * (size_t)c.emb.cap1 * sizeof(int) + 4));
        A.tcnt2 = static_cast<int *>(dalloc(A, P * sizeof(int)));
        A.tent2 = static_cast<int *>(dalloc(A, P * kTransposeMax * sizeof(int)));
        A.prow2 = static_cast<int *>(dalloc(A, 2 * (size_t)c.emb.cap2 * sizeof(int) + 4));
        A.overflow = static_cast<int *>(dalloc(A, sizeof(int)));
        CUIBM_TRY(cudaMemset(A.overflow, 0, sizeof(int)));
        for (double *&st : A.stash) st = static_cast<double *>(dalloc(A, (UV + P) * sizeof(double)));
        A.S1T.rtol = A.S2T.rtol = 1e-10;
        A.S1T.maxit = c.sys1.maxit;
        A.S2T.maxit = c.sys2.maxit;
        setup_transposed_system(c, c.sys1, A.S1T, A.allocs);
        setup_transposed_system(c, c.sys2, A.S2T, A.allocs);
    }
    if (nsteps > A.steps_cap) {
        A.scal = static_cast<double *>(dalloc(A, (2 + 2 * (size_t)nsteps) * sizeof(double)));
        A.steps_cap = nsteps;
    }
    while ((int)A.snaps.size() < snapshots) {
        Snapshot s;
        s.blk = static_cast<double *>(dalloc(A, snapshot_doubles(A) * sizeof(double)));
        s.step = static_cast<int *>(dalloc(A, 5 * sizeof(int)));
        A.snaps.push_back(s);
    }
}

struct Runner {
    Context &c;
    AdjointState &A;
    const std::vector<double> &wx, &wy;
    int T;
    bool moving;

    void copy_state(Snapshot &s, bool save)
    {
        const size_t UV = A.nUV, P = A.nP, nb = A.nb;
        double *p = s.blk;
        // the pressure nodes' body intercepts and image points are arrays a tagging does not
        // refill (luo_base/tagPoints.cu:26-40): a re-tagging keeps their values where it
        // does not write, so the state holds them too
        double *f[] = {c.u, c.uhat, c.N, c.p, c.bc[XPLUS], c.ib.bx, c.ib.by, c.ib.uB, c.ib.vB, c.ib.uBk, c.ib.vBk,
                       c.ib.motion, c.ib.bipX, c.ib.bipY, c.ib.ippX, c.ib.ippY};
        const size_t n[] = {UV, UV, UV, P, (size_t)A.nxp, nb, nb, nb, nb, nb, nb, (size_t)kMotionLen, P, P, P, P};
        for (int k = 0; k < 16; ++k) {
            if (save) CUIBM_TRY(cudaMemcpyAsync(p, f[k], n[k] * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
            else CUIBM_TRY(cudaMemcpyAsync(f[k], p, n[k] * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
            p += n[k];
        }
        int *box = const_cast<int *>(force_box_dev(c));
        if (save) {
            CUIBM_TRY(cudaMemcpyAsync(s.step, c.step_counter_dev, sizeof(int), cudaMemcpyDeviceToDevice, c.stream));
            CUIBM_TRY(cudaMemcpyAsync(s.step + 1, box, 4 * sizeof(int), cudaMemcpyDeviceToDevice, c.stream));
            s.timeStep = c.timeStep;
        } else {
            CUIBM_TRY(cudaMemcpyAsync(c.step_counter_dev, s.step, sizeof(int), cudaMemcpyDeviceToDevice, c.stream));
            CUIBM_TRY(cudaMemcpyAsync(box, s.step + 1, 4 * sizeof(int), cudaMemcpyDeviceToDevice, c.stream));
            c.timeStep = s.timeStep;
        }
    }

    int save(int step)
    {
        for (size_t k = 0; k < A.snaps.size(); ++k)
            if (A.snaps[k].holds < 0) {
                copy_state(A.snaps[k], true);
                A.snaps[k].holds = step;
                return (int)k;
            }
        throw CudaError("adjoint checkpointing: no free snapshot");
    }

    void restore(int slot)
    {
        copy_state(A.snaps[slot], false);
        if (moving) launch_tag_points(c);  // the tags, plan and rows of the restored body position
    }

    void advance(int from, int to)
    {
        for (int s = from; s < to; ++s) {
            step_once(c);
            ++A.forward_steps;
        }
    }

    // keep the solutions of step n (uhat at src_uhat, p at src_p) in the stash the
    // next tape does not need (that one holds step keep)
    void stash_solutions(int n, const double *src_uhat, const double *src_p, int keep)
    {
        const int k = A.stash_step[0] == keep ? 1 : 0;
        launch_copy(c, A.stash[k], src_uhat, c.g.nUV);
        launch_copy(c, A.stash[k] + A.nUV, src_p, c.g.nP);
        A.stash_step[k] = n;
    }

    // the intermediates of step n (1-based) from the state after step n-1.  Where a
    // snapshot holds the state after step n, or a stash that step's solutions, its uhat
    // and p are that step's solutions (the embedded method changes neither after its
    // solve): they are copied, not solved again.
    void tape(int n)
    {
        launch_copy(c, c.p_old, c.p, c.g.nP);
        launch_copy(c, c.uold, c.u, c.g.nUV);
        launch_body_pre_step(c);
        phase_generate_rhs1(c, true);  // u := u1 (inside velocity), Nold := N, N, rhs1, x+ boundary
        const double *done_uhat = nullptr, *done_p = nullptr;
        for (const Snapshot &sn : A.snaps)
            if (sn.holds == n) {
                done_uhat = sn.blk + A.nUV;
                done_p = sn.blk + 3 * (size_t)A.nUV;
            }
        for (int k = 0; k < 2 && !done_uhat; ++k)
            if (A.stash_step[k] == n) {
                done_uhat = A.stash[k];
                done_p = A.stash[k] + A.nUV;
                A.stash_step[k] = -1;
            }
        if (done_uhat) {
            launch_copy(c, c.uhat, done_uhat, c.g.nUV);
            launch_copy(c, c.p, done_p, c.g.nP);
            ++A.solves_reused;
        } else {
            phase_solve_velocity(c, false);
            phase_generate_rhs2(c);
            phase_solve_poisson(c, false);
        }
        launch_project(c);  // uold := u1, u := u2
        launch_copy(c, A.u2tape, c.u, c.g.nUV);
        launch_ib_after_projection(c);  // u := u4
        launch_force(c);
        k_accum_objective<<<1, 32, 0, c.stream>>>(c.ib.forceOut, wx[n - 1], wy[n - 1], A.scal + 1);
        CUIBM_TRY(cudaGetLastError());
        ++A.tape_steps;
        const int errw = read_step_error(c);
        if (errw) throw CudaError("adjoint: a forward solve failed while recomputing step " + std::to_string(n));
    }

    void transpose_lists()
    {
        const IbPlan &P = ib_plan(c);
        const auto &E = c.emb;
        CUIBM_TRY(cudaMemsetAsync(A.tcnt1, 0, A.nUV * sizeof(int), c.stream));
        CUIBM_TRY(cudaMemsetAsync(A.tcnt2, 0, A.nP * sizeof(int), c.stream));
        k_tlist_count<<<blocks_for(2 * E.cap1 + 1), kBlock, 0, c.stream>>>(P, 1, E.cap1, E.pid1, E.pcol1, A.prow1,
                                                                          A.tcnt1, A.tent1, kTransposeMax,
                                                                          A.overflow);
        k_tlist_count<<<blocks_for(2 * E.cap2 + 1), kBlock, 0, c.stream>>>(P, 2, E.cap2, E.pid2, E.pcol2, A.prow2,
                                                                          A.tcnt2, A.tent2, kTransposeMax,
                                                                          A.overflow);
        k_tlist_sort<<<blocks_for(A.nUV), kBlock, 0, c.stream>>>(A.nUV, A.tcnt1, A.tent1, kTransposeMax);
        k_tlist_sort<<<blocks_for(A.nP), kBlock, 0, c.stream>>>(A.nP, A.tcnt2, A.tent2, kTransposeMax);
        CUIBM_TRY(cudaGetLastError());
    }

    // the adjoint of step n (1-based), its intermediates taped
    void reverse_step(int n)
    {
        const Grid &g = c.g;
        const IbPlan &P = ib_plan(c);
        const auto &E = c.emb;
        double *qbar = A.scal + 2 + 2 * (size_t)(n - 1);
        double *nubar = A.scal;
        transpose_lists();
        CUIBM_TRY(cudaMemsetAsync(A.pbar, 0, A.nP * sizeof(double), c.stream));
        CUIBM_TRY(cudaMemsetAsync(A.u1bar, 0, A.nUV * sizeof(double), c.stream));
        // force of this step
        k_adj_force<<<64, kBlock, 0, c.stream>>>(g.nx, g.ny, force_box_dev(c), c.u, c.uold, c.p, c.ib.ghostUV, c.P.nu,
                                                c.dx, c.dy, c.P.dt, wx[n - 1], wy[n - 1], A.ubar, A.u1bar, A.pbar,
                                                nubar);
        // inside velocity, ghost values, projection
        const int cin = std::max(1, P.cap_in), cv = std::max(1, P.cap_v);
        k_adj_inside<<<blocks_for(cin), kBlock, 0, c.stream>>>(P, g.nU, A.ubar, qbar);
        CUIBM_TRY(cudaMemcpyAsync(A.u2bar, A.ubar, A.nUV * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
        k_adj_ghost<<<blocks_for(cv), kBlock, 0, c.stream>>>(P, g.nU, A.ubar, A.u2bar, qbar);
        k_adj_project<<<blocks_for(std::max(A.nUV, A.nP)), kBlock, 0, c.stream>>>(g, c.gradU, c.gradV, A.u2bar,
                                                                                  A.uhbar, A.pbar);
        CUIBM_TRY(cudaGetLastError());
        // Poisson: r2bar = A2^-T pbar, then the divergence
        const TransposeList T2{A.tcnt2, A.tent2, A.prow2, kTransposeMax};
        int its = 0;
        int st = launch_solve_transposed(c, A.S2T, c.sys2, T2, A.pbar, A.r2bar, &its);
        A.it2 += its;
        if (st != KS_CONVERGED)
            throw CudaError("adjoint: the transposed Poisson solve of step " + std::to_string(n) +
                            " did not converge (status " + std::to_string(st) + ", " + std::to_string(its) +
                            " iterations)");
        k_adj_rhs2<<<blocks_for(A.nUV), kBlock, 0, c.stream>>>(g, c.dx, c.dy, E.pid2, E.pns2, A.r2bar, A.uhbar,
                                                              A.xpbar);
        CUIBM_TRY(cudaGetLastError());
        // velocity: r1bar = A1^-T uhbar, the operator's nu-dependence, then the explicit terms
        const TransposeList T1{A.tcnt1, A.tent1, A.prow1, kTransposeMax};
        st = launch_solve_transposed(c, A.S1T, c.sys1, T1, A.uhbar, A.r1bar, &its);
        A.it1 += its;
        if (st != KS_CONVERGED)
            throw CudaError("adjoint: the transposed velocity solve of step " + std::to_string(n) +
                            " did not converge (status " + std::to_string(st) + ", " + std::to_string(its) +
                            " iterations)");
        k_adj_dA1nu<<<blocks_for(A.nUV), kBlock, 0, c.stream>>>(c.l1, g, P, E.cap1, c.P.dt, c.P.nu, c.dx, c.dy,
                                                               c.uhat, A.r1bar, nubar);
        AdjRhs1 ea{E.pid1, E.rscale1, E.pns1, E.cap1, E.gin, P};
        BcPtrsA b{c.bc[XMINUS], c.bc[XPLUS], c.bc[YMINUS], c.bc[YPLUS]};
        k_adj_rhs1<<<blocks_for(A.nUV), kBlock, 0, c.stream>>>(c.rc, g, b, c.P.dt, c.P.nu, c.uold, c.Nold, ea, c.dx,
                                                              c.dy, A.r1bar, A.Nbar, A.u1bar, A.xpbar, qbar, nubar);
        // inside velocity of u1, then the Robin update: the adjoint of the step's initial u
        k_adj_inside<<<blocks_for(cin), kBlock, 0, c.stream>>>(P, g.nU, A.u1bar, qbar);
        CUIBM_TRY(cudaMemcpyAsync(A.ubar, A.u1bar, A.nUV * sizeof(double), cudaMemcpyDeviceToDevice, c.stream));
        k_adj_robin<<<blocks_for(A.nxp), kBlock, 0, c.stream>>>(g.nx, g.ny, c.P.dt, c.dx, A.xpbar, A.ubar);
        CUIBM_TRY(cudaGetLastError());
    }

    static double beta(int s, int r)
    {  // C(s + r, s), saturated; 0 for r < 0
        if (r < 0) return 0;
        double b = 1;
        for (int k = 1; k <= s; ++k) {
            b = b * (r + k) / k;
            if (b > 1e15) return 1e15;
        }
        return b;
    }

    // Reverse steps a+1..b; the state after step a is in snapshot slot_a; s more slots
    // free.  Binomial checkpointing (Griewank and Walther, "Algorithm 799: revolve", ACM
    // TOMS 26, 2000): with r the least repetition count for which beta(s, r) >= t = b - a
    // steps can be reversed, the checkpoint goes after m - a steps with m - a in
    //   [max(beta(s, r-2), t - beta(s-1, r)), min(beta(s, r-1), t - beta(s-1, r-1))],
    // the range where the right part (s - 1 free slots) and the left part (s slots)
    // together advance the fewest steps, r t - beta(s+1, r-1) in all.
    void reverse(int a, int b, int s, int slot_a)
    {
        if (b - a == 1) {
            restore(slot_a);
            tape(b);
            reverse_step(b);
            return;
        }
        if (s == 0) {
            for (int k = b; k > a; --k) {
                restore(slot_a);
                advance(a, k - 1);
                // the advance's last step is the one the next tape recomputes
                if (k - 1 > a) stash_solutions(k - 1, c.uhat, c.p, k);
                tape(k);
                reverse_step(k);
            }
            return;
        }
        const int t = b - a;
        int r = 1;
        while (beta(s, r) < t) ++r;
        const double lo = std::max(beta(s, r - 2), t - beta(s - 1, r));
        const int m = a + (int)std::min<double>(std::max(1.0, lo), t - 1);
        restore(slot_a);
        advance(a, m);
        const int slot_m = save(m);
        reverse(m, b, s - 1, slot_m);
        // the left part's first tape is step m: its solutions go to a stash, the slot is free
        Snapshot &sm = A.snaps[slot_m];
        stash_solutions(m, sm.blk + A.nUV, sm.blk + 3 * (size_t)A.nUV, -2);
        sm.holds = -1;
        reverse(a, m, s, slot_a);
    }
};

}  // namespace

// y = A^T x for system 1 (LHS1) or 2 (LHS2) with the current rows (CUIBM_OP_APPLY_LHS1_T/2_T)
void apply_transposed(Context &c, int which, const double *x, double *y)
{
    if (!(c.P.solverType == ST_OSC && c.has_body))
        throw InputError("the transposed operators are those of the embedded method (SolverType OSC_CYLINDER)");
    ensure_state(c, 1, 1);
    AdjointState &A = adj(c);
    std::vector<double> none;
    Runner R{c, A, none, none, 0, false};
    R.transpose_lists();
    const TransposeList T = which == 1 ? TransposeList{A.tcnt1, A.tent1, A.prow1, kTransposeMax}
                                       : TransposeList{A.tcnt2, A.tent2, A.prow2, kTransposeMax};
    launch_apply_transposed(c, which, T, x, y);
}

void free_adjoint(Context &c)
{
    if (!c.adj) return;
    AdjointState *A = static_cast<AdjointState *>(c.adj);
    for (void *p : A->allocs) cudaFree(p);
    delete A;
    c.adj = nullptr;
}

// Runs steps 1..nsteps from the context's current state (which must be its initial
// condition: cuibm_initialise and no step since), then the adjoint sweep; leaves the
// context at that initial state.
void run_adjoint(Context &c, int nsteps, int snapshots, const double *wx, const double *wy, double *J, double *grad,
                 size_t ngrad, double adjoint_rtol, AdjointStats *stats)
{
    if (!(c.P.solverType == ST_OSC && c.has_body))
        throw InputError("the adjoint covers the embedded method (SolverType OSC_CYLINDER) with a body");
    if (c.P.VIV != 0) throw InputError("the adjoint covers prescribed body motion only (VIV: 0)");
    if (c.force_method != 0) throw InputError("the adjoint differentiates the control-volume force (force_method 0)");
    if (c.timeStep != c.P.startStep)
        throw InputError("the adjoint starts from the initial condition: call it right after cuibm_initialise");
    const int nb = c.body.total;
    if (nsteps < 1) throw InputError("nsteps < 1");
    if (snapshots < 1) throw InputError("snapshots < 1");
    if (ngrad != 2 + 2 * (size_t)nb) throw InputError("grad must hold 2 + 2 * total_points values");
    ensure_state(c, nsteps, snapshots);
    AdjointState &A = adj(c);
    A.S1T.rtol = A.S2T.rtol = adjoint_rtol;
    A.forward_steps = A.tape_steps = A.solves_reused = A.it1 = A.it2 = 0;
    for (auto &s : A.snaps) s.holds = -1;
    A.stash_step[0] = A.stash_step[1] = -1;
    CUIBM_TRY(cudaMemsetAsync(A.scal, 0, (2 + 2 * (size_t)nsteps) * sizeof(double), c.stream));
    CUIBM_TRY(cudaMemsetAsync(A.ubar, 0, A.nUV * sizeof(double), c.stream));
    CUIBM_TRY(cudaMemsetAsync(A.Nbar, 0, A.nUV * sizeof(double), c.stream));
    CUIBM_TRY(cudaMemsetAsync(A.xpbar, 0, A.nxp * sizeof(double), c.stream));
    CUIBM_TRY(cudaMemsetAsync(A.r1bar, 0, A.nUV * sizeof(double), c.stream));
    CUIBM_TRY(cudaMemsetAsync(A.r2bar, 0, A.nP * sizeof(double), c.stream));
    CUIBM_TRY(cudaMemsetAsync(A.overflow, 0, sizeof(int), c.stream));
    std::vector<double> vx(wx, wx + nsteps), vy(wy, wy + nsteps);
    const int t0 = c.timeStep;
    Runner R{c, A, vx, vy, nsteps, body_moves(c)};
    cudaEvent_t e0, e1;
    CUIBM_TRY(cudaEventCreate(&e0));
    CUIBM_TRY(cudaEventCreate(&e1));
    CUIBM_TRY(cudaEventRecord(e0, c.stream));
    const int slot0 = R.save(0);
    try {
        R.reverse(0, nsteps, snapshots - 1, slot0);
        R.restore(slot0);
    } catch (...) {
        R.restore(slot0);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    CUIBM_TRY(cudaEventRecord(e1, c.stream));
    CUIBM_TRY(cudaEventSynchronize(e1));
    float ms = 0;
    CUIBM_TRY(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int overflow = 0;
    CUIBM_TRY(cudaMemcpy(&overflow, A.overflow, sizeof(int), cudaMemcpyDeviceToHost));
    if (overflow) throw CudaError("adjoint: more patched rows hold one column than the transposed lists keep");
    std::vector<double> sc(2 + 2 * (size_t)nsteps);
    CUIBM_TRY(cudaMemcpy(sc.data(), A.scal, sc.size() * sizeof(double), cudaMemcpyDeviceToHost));
    // the body velocity of step n was set by the motion at step index s_n: the initial
    // condition's (t0) for the first step, the end of step n - 1 (t0 + n - 2) after it
    const BodyState &B = c.body;
    double gu = 0, gv = 0, gc = 0;
    for (int n = 1; n <= nsteps; ++n) {
        const int s = n == 1 ? t0 : t0 + n - 2;
        const double cosine = std::cos(2 * M_PI * B.freq * (c.P.dt * s) + B.uPhase);
        const double qu = sc[2 + 2 * (size_t)(n - 1)], qv = sc[3 + 2 * (size_t)(n - 1)];
        gu += qu;
        gv += qv;
        gc += qu * cosine;
    }
    for (size_t k = 0; k < ngrad; ++k) grad[k] = 0;
    grad[0] = sc[0];
    grad[1] = gc;
    grad[2] = gu;
    grad[2 + nb] = gv;
    if (J) *J = sc[1];
    if (stats) {
        stats->ms = ms;
        stats->forward_steps = A.forward_steps;
        stats->tape_steps = A.tape_steps;
        stats->solves_reused = A.solves_reused;
        stats->velocity_iterations = A.it1;
        stats->poisson_iterations = A.it2;
    }
}

}  // namespace cuibm
