// Matrix-free rows of the reference's LHS1 (I - dt/2 nu L) and LHS2 (dt D G)
// COO matrices (NavierStokes/kernels/LHS1.cu, LHS2.cu), shared by the operator
// kernels and the Krylov solvers.  Diagonals are summed in the reference's
// order (1 + E + W + N + S; 0 + E + W + N + S), so diagonal values are bit-
// identical to the reference's matrix entries.
#pragma once
#include "solver.h"

namespace cuibm {

// ---------------------------------------------------------------------------
// operator rows (device)
// ---------------------------------------------------------------------------
// a patched row (RowPatch), the own value given
template <class X>
__device__ __forceinline__ double patch_row(const RowPatch &P, int k, double xi, const X &x)
{
    double y = P.pdiag[k] * xi;
#pragma unroll
    for (int m = 0; m < 5; ++m) {
        const int j = P.pcol[5 * k + m];
        if (j >= 0) y += P.pval[5 * k + m] * x(j);
    }
    return y;
}

template <class X>
__device__ __forceinline__ double lhs1_row_f(const Lhs1Coef &c, const Grid &g, int i, const X &x)
{
    if (c.patch.pid) {
        const int k = c.patch.pid[i];
        if (k >= 0) return patch_row(c.patch, k, x(i), x);
    }
    const int w = g.nx - 1;
    if (i < g.nU) {
        int I = i % w, J = i / w;
        double d = (((1 + c.uE[I]) + c.uW[I]) + c.uN[J]) + c.uS[J];
        double y = d * x(i);
        if (I != g.nx - 2) y -= c.uE[I] * x(i + 1);
        if (I != 0) y -= c.uW[I] * x(i - 1);
        if (J != g.ny - 1) y -= c.uN[J] * x(i + w);
        if (J != 0) y -= c.uS[J] * x(i - w);
        return c.rscale ? y * c.rscale[i] : y;
    }
    int k = i - g.nU, I = k % g.nx, J = k / g.nx;
    double d = (((1 + c.vE[I]) + c.vW[I]) + c.vN[J]) + c.vS[J];
    double y = d * x(i);
    if (I != g.nx - 1) y -= c.vE[I] * x(i + 1);
    if (I != 0) y -= c.vW[I] * x(i - 1);
    if (J != g.ny - 2) y -= c.vN[J] * x(i + g.nx);
    if (J != 0) y -= c.vS[J] * x(i - g.nx);
    return c.rscale ? y * c.rscale[i] : y;
}

template <class X>
__device__ __forceinline__ double lhs2_row_f(const Lhs2Coef &c, const Grid &g, int i, const X &x)
{
    if (c.patch.pid) {
        const int k = c.patch.pid[i];
        if (k >= 0) return patch_row(c.patch, k, x(i), x);
    }
    int I = i % g.nx, J = i / g.nx;
    double d = (((0 + c.E[I]) + c.W[I]) + c.N[J]) + c.S[J];
    if (i == c.pin0 || i == c.pinc) d += d;
    double y = d * x(i);
    if (I != g.nx - 1) y -= c.E[I] * x(i + 1);
    if (I != 0) y -= c.W[I] * x(i - 1);
    if (J != g.ny - 1) y -= c.N[J] * x(i + g.nx);
    if (J != 0) y -= c.S[J] * x(i - g.nx);
    return y;
}


struct PtrAccess {
    const double *__restrict__ p;
    __device__ __forceinline__ double operator()(int j) const { return p[j]; }
};

__device__ __forceinline__ double lhs1_row(const Lhs1Coef &c, const Grid &g, int i, const double *__restrict__ x)
{
    return lhs1_row_f(c, g, i, PtrAccess{x});
}

__device__ __forceinline__ double lhs2_row(const Lhs2Coef &c, const Grid &g, int i, const double *__restrict__ x)
{
    return lhs2_row_f(c, g, i, PtrAccess{x});
}

// ---- transposed operators (discrete adjoint) ---------------------------------------
// Row i of A^T is column i of A: the structured rows j next to i that are not patched
// contribute their coefficient towards i (times the row scale of LHS1's embedded rows),
// the diagonal is row i's own, and the patched rows holding column i are listed in
// TransposeList (built by the adjoint for each tagging).
struct Op1T {
    Lhs1Coef c;
    Grid g;
    TransposeList T;
    template <class X>
    __device__ __forceinline__ double row(int i, const X &x) const
    {
        const RowPatch &P = c.patch;
        auto patched = [&](int j) { return P.pid && P.pid[j] >= 0; };
        auto rs = [&](int j) { return c.rscale ? c.rscale[j] : 1.0; };
        const int ki = P.pid ? P.pid[i] : -1;
        double y;
        if (i < g.nU) {
            const int w = g.nx - 1, I = i % w, J = i / w;
            if (ki >= 0) y = P.pdiag[ki] * x(i);
            else y = ((((1 + c.uE[I]) + c.uW[I]) + c.uN[J]) + c.uS[J]) * rs(i) * x(i);
            if (I != 0 && !patched(i - 1)) y -= c.uE[I - 1] * rs(i - 1) * x(i - 1);
            if (I != g.nx - 2 && !patched(i + 1)) y -= c.uW[I + 1] * rs(i + 1) * x(i + 1);
            if (J != 0 && !patched(i - w)) y -= c.uN[J - 1] * rs(i - w) * x(i - w);
            if (J != g.ny - 1 && !patched(i + w)) y -= c.uS[J + 1] * rs(i + w) * x(i + w);
        } else {
            const int k = i - g.nU, w = g.nx, I = k % w, J = k / w;
            if (ki >= 0) y = P.pdiag[ki] * x(i);
            else y = ((((1 + c.vE[I]) + c.vW[I]) + c.vN[J]) + c.vS[J]) * rs(i) * x(i);
            if (I != 0 && !patched(i - 1)) y -= c.vE[I - 1] * rs(i - 1) * x(i - 1);
            if (I != g.nx - 1 && !patched(i + 1)) y -= c.vW[I + 1] * rs(i + 1) * x(i + 1);
            if (J != 0 && !patched(i - w)) y -= c.vN[J - 1] * rs(i - w) * x(i - w);
            if (J != g.ny - 2 && !patched(i + w)) y -= c.vS[J + 1] * rs(i + w) * x(i + w);
        }
        if (T.cnt) {
            const int n = T.cnt[i] < T.tmax ? T.cnt[i] : T.tmax;
            for (int t = 0; t < n; ++t) {
                const int e = T.ent[(size_t)i * T.tmax + t];
                y += P.pval[e] * x(T.prow[e / 5]);
            }
        }
        return y;
    }
};
struct Op2T {
    Lhs2Coef c;
    Grid g;
    TransposeList T;
    template <class X>
    __device__ __forceinline__ double row(int i, const X &x) const
    {
        const RowPatch &P = c.patch;
        auto patched = [&](int j) { return P.pid && P.pid[j] >= 0; };
        const int ki = P.pid ? P.pid[i] : -1;
        const int I = i % g.nx, J = i / g.nx;
        double y;
        if (ki >= 0) {
            y = P.pdiag[ki] * x(i);
        } else {
            double d = (((0 + c.E[I]) + c.W[I]) + c.N[J]) + c.S[J];
            if (i == c.pin0 || i == c.pinc) d += d;
            y = d * x(i);
        }
        if (I != 0 && !patched(i - 1)) y -= c.E[I - 1] * x(i - 1);
        if (I != g.nx - 1 && !patched(i + 1)) y -= c.W[I + 1] * x(i + 1);
        if (J != 0 && !patched(i - g.nx)) y -= c.N[J - 1] * x(i - g.nx);
        if (J != g.ny - 1 && !patched(i + g.nx)) y -= c.S[J + 1] * x(i + g.nx);
        if (T.cnt) {
            const int n = T.cnt[i] < T.tmax ? T.cnt[i] : T.tmax;
            for (int t = 0; t < n; ++t) {
                const int e = T.ent[(size_t)i * T.tmax + t];
                y += P.pval[e] * x(T.prow[e / 5]);
            }
        }
        return y;
    }
};

}  // namespace cuibm
