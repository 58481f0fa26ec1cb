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

// (P^T r)_J: the fine nodes of aggregate J and the ring around it, each with the
// weight of its row of P that refers to J
template <class T, class X>
__device__ __forceinline__ T st_restrict(int nx, int ny, int cnx, int cny, const T *__restrict__ pw, int J,
                                         const X &r)
{
    const int n = nx * ny;
    const int Jy = J / cnx, Jx = J - Jy * cnx;
    if (Jx >= 1 && Jx <= cnx - 2 && Jy >= 1 && Jy <= cny - 2) {
        // an interior aggregate (3 x 3, with 3-wide aggregates or the last one around):
        // its 5 x 5 region, the ring's weights on the side slots, every load independent
        const int base = (3 * Jy - 1) * nx + 3 * Jx - 1;
        T s = 0;
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
    const int x0 = 3 * Jx, x1 = Jx == cnx - 1 ? nx - 1 : 3 * Jx + 2;
    const int y0 = 3 * Jy, y1 = Jy == cny - 1 ? ny - 1 : 3 * Jy + 2;
    const int xa = x0 > 0 ? x0 - 1 : 0, xb = x1 < nx - 1 ? x1 + 1 : nx - 1;
    const int ya = y0 > 0 ? y0 - 1 : 0, yb = y1 < ny - 1 ? y1 + 1 : ny - 1;
    T s = 0;
    for (int iy = ya; iy <= yb; ++iy) {
        const StAxis ay = st_axis(iy, ny, cny);
        // which of the row's aggregates along y is J's row: own (0) or the side (1)
        const int ky = ay.a == Jy ? 0 : (ay.s && ay.a + ay.s == Jy ? 1 : -1);
        if (ky < 0) continue;
        for (int ix = xa; ix <= xb; ++ix) {
            const StAxis ax = st_axis(ix, nx, cnx);
            const int kx = ax.a == Jx ? 0 : (ax.s && ax.a + ax.s == Jx ? 1 : -1);
            if (kx < 0) continue;
            const int i = iy * nx + ix;
            s += pw[(kx + 2 * ky) * n + i] * r(i);
        }
    }
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
