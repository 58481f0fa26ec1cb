// Structured smoothed aggregation on the pressure grid: the device side shared by
// the hierarchy's set-up and stepwise cycle (amg.cu) and the persistent solver
// (fused_solve.cu).
//
// The aggregates of a level with nx x ny unknowns (row-major, i = iy nx + ix) are
// blocks of 3 x 3 nodes: along each axis cn = max(1, n / 3) aggregates, aggregate a
// spanning [3a, 3a + 2] and the last one taking the remainder (3 to 5 nodes wide).
// The tentative prolongator is piecewise constant (entries 1: the near-null space,
// the constant, passes to every level exactly); the prolongator is its damped-Jacobi
// smoothing P = (I - w D^-1 A) T.  Row i of P has nonzeros only in the aggregates of
// i's stencil neighbours: its own aggregate, the one across its x edge (sx = -1 or
// +1 where i is the first or last column of its aggregate), the one across its y
// edge and the diagonal one - four weights a node, pw[k n + i], k = 0 own, 1 x side,
// 2 y side, 3 diagonal (zero where the side does not exist), and no column indices.
// With aggregates at least 3 wide, P's columns reach one node past their aggregate
// and A P's two, so the Galerkin operator P^T A P couples only neighbouring
// aggregates: every coarse level is a 9-point operator, stored as nine coefficient
// arrays c9[k n + i], k = 3 (dy + 1) + (dx + 1) for the neighbour (ix + dx, iy + dy).
#pragma once

namespace cuibm {

struct StAxis {
    int a, s;  // aggregate along the axis, side (-1, 0, +1) of the neighbouring aggregate
};

// aggregate and side of fine index x on an axis of n fine and cn coarse nodes
__host__ __device__ __forceinline__ StAxis st_axis(int x, int n, int cn)
{
    int a = x / 3;
    if (a > cn - 1) a = cn - 1;
    const int last = a == cn - 1 ? n - 1 : 3 * a + 2;
    int s = 0;
    if (x == 3 * a && a > 0) s = -1;
    else if (x == last && a < cn - 1) s = 1;
    return StAxis{a, s};
}

__host__ __device__ __forceinline__ int st_coarse(int n) { return n / 3 > 1 ? n / 3 : 1; }

// (P xc)_i for the fine node (ix, iy), i = iy nx + ix
template <class T, class X>
__device__ __forceinline__ T st_prolong_xy(int nx, int ny, int cnx, int cny, const T *__restrict__ pw, int ix,
                                           int iy, const X &xc)
{
    const int n = nx * ny, i = iy * nx + ix;
    const StAxis ax = st_axis(ix, nx, cnx), ay = st_axis(iy, ny, cny);
    const int J = ay.a * cnx + ax.a;
    T y = pw[i] * xc(J);
    if (ax.s) y += pw[n + i] * xc(J + ax.s);
    if (ay.s) y += pw[2 * n + i] * xc(J + ay.s * cnx);
    if (ax.s && ay.s) y += pw[3 * n + i] * xc(J + ax.s + ay.s * cnx);
    return y;
}

// (P xc)_i: the four weights of fine node i against the coarse values around it
template <class T, class X>
__device__ __forceinline__ T st_prolong(int nx, int ny, int cnx, int cny, const T *__restrict__ pw, int i,
                                        const X &xc)
{
    const int n = nx * ny;
    const int iy = i / nx, ix = i - iy * nx;
    const StAxis ax = st_axis(ix, nx, cnx), ay = st_axis(iy, ny, cny);
    const int J = ay.a * cnx + ax.a;
    T y = pw[i] * xc(J);
    if (ax.s) y += pw[n + i] * xc(J + ax.s);
    if (ay.s) y += pw[2 * n + i] * xc(J + ay.s * cnx);
    if (ax.s && ay.s) y += pw[3 * n + i] * xc(J + ax.s + ay.s * cnx);
    return y;
}

// One row of (P^T r)_J: row dy (0..6) of the region of aggregate J - its fine nodes and
// the ring around them - each node weighted by its row of P's weight that refers to J.
// An interior aggregate (3 x 3, with 3-wide aggregates or the last one around it) has a
// 5 x 5 region whose slots are fixed (the ring on the side slots); an aggregate on the
// grid's edge (up to 5 wide) has up to 7 x 7, its slots worked out first and then all
// the loads issued on a clamped index, weighted 0 or 1, so that no load waits for the
// one before it.
template <class T, class X>
__device__ __forceinline__ T st_restrict_row(int nx, int ny, int cnx, int cny, const T *__restrict__ pw, int J,
                                             const X &r, int dy)
{
    const int n = nx * ny;
    const int Jy = J / cnx, Jx = J - Jy * cnx;
    const int x0 = 3 * Jx, iy = 3 * Jy - 1 + dy;
    T s = 0;
    if (Jx >= 1 && Jx <= cnx - 2 && Jy >= 1 && Jy <= cny - 2) {
        if (dy >= 5) return s;
        const int base = iy * nx + x0 - 1, ky = dy == 0 || dy == 4 ? 2 : 0;
#pragma unroll
        for (int dx = 0; dx < 5; ++dx) {
            const int kx = dx == 0 || dx == 4 ? 1 : 0;
            s += pw[(kx + ky) * n + base + dx] * r(base + dx);
        }
        return s;
    }
    if (dy >= 7 || iy < 0 || iy >= ny) return s;
    const StAxis ay = st_axis(iy, ny, cny);
    const int ky = ay.a == Jy ? 0 : (ay.s && ay.a + ay.s == Jy ? 2 : -1);
    if (ky < 0) return s;
#pragma unroll
    for (int dx = 0; dx < 7; ++dx) {
        const int ix = x0 - 1 + dx;
        int kx = -1;
        if (ix >= 0 && ix < nx) {
            const StAxis ax = st_axis(ix, nx, cnx);
            kx = ax.a == Jx ? 0 : (ax.s && ax.a + ax.s == Jx ? 1 : -1);
        }
        const bool on = kx >= 0;
        const int i = on ? iy * nx + ix : 0;
        const T w = pw[(on ? kx + ky : 0) * n + i];
        const T v = r(i);
        if (on) s += w * v;
    }
    return s;
}

// (P^T r)_J: the interior 5 x 5 region in one unrolled sum, an edge aggregate row by row
template <class T, class X>
__device__ __forceinline__ T st_restrict(int nx, int ny, int cnx, int cny, const T *__restrict__ pw, int J,
                                         const X &r)
{
    const int n = nx * ny;
    const int Jy = J / cnx, Jx = J - Jy * cnx;
    T s = 0;
    if (Jx >= 1 && Jx <= cnx - 2 && Jy >= 1 && Jy <= cny - 2) {
        const int base = (3 * Jy - 1) * nx + 3 * Jx - 1;
#pragma unroll
        for (int dy = 0; dy < 5; ++dy) {
            const int ky = dy == 0 || dy == 4 ? 2 : 0;
#pragma unroll
            for (int dx = 0; dx < 5; ++dx) {
                const int kx = dx == 0 || dx == 4 ? 1 : 0;
                const int i = base + dy * nx + dx;
                s += pw[(kx + ky) * n + i] * r(i);
            }
        }
        return s;
    }
    for (int dy = 0; dy < 7; ++dy) s += st_restrict_row(nx, ny, cnx, cny, pw, J, r, dy);
    return s;
}

// row i of a 9-point level operator applied to x
template <class T, class X>
__device__ __forceinline__ T st_row9(int nx, int ny, const T *__restrict__ c9, int i, const X &x)
{
    const int n = nx * ny;
    const int iy = i / nx, ix = i - iy * nx;
    T y = 0;
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy) {
        if (iy + dy < 0 || iy + dy >= ny) continue;
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
            if (ix + dx < 0 || ix + dx >= nx) continue;
            y += c9[(3 * (dy + 1) + dx + 1) * n + i] * x(i + dy * nx + dx);
        }
    }
    return y;
}

}  // namespace cuibm
