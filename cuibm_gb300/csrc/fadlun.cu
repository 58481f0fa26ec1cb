// The modified Fadlun immersed-boundary method (SolverType FADLUN):
// fadlunModified.cu with FadlunModified/kernels/LHS1.cu, LHS2.cu,
// intermediateVelocity.cu, intermediatePressure.cu and projectVelocity.cu.
//
// The body enters through the linear systems rather than through interpolated
// field values:
//  * LHS1: at a hybrid velocity node (first fluid node) the momentum row is
//    replaced by the linear interpolation u_i - d/(d+b) u_away = b/(d+b) u_body;
//    at a ghost node (first node inside) by u_i - c u_across = 0; all other rows,
//    the body interior included, are the plain I - dt/2 nu L rows;
//  * LHS2: at tagged pressure nodes the 5-point row drops the faces that cross the
//    body and uses the shortened face distance where the body cuts the cell;
//  * rhs1 gets the body terms of those rows, rhs2 the matching face fluxes, and the
//    projection applies no pressure gradient across a face touching a tagged cell.
// The operators stay matrix-free: the tagged rows are RowPatch rows (operators.cuh),
// built on the host once from the initial tags - the reference assembles its Fadlun
// matrices once in initialise and updateSolver never rebuilds them.  The patch
// values follow the reference's arithmetic, so the matrices are the reference's
// (tests compare them entry by entry with the oracle).
#include <algorithm>
#include <vector>

#include "solver.h"

namespace cuibm {

namespace {

struct HostTags {
    std::vector<int> hyb, hyb2, ghost, ghostP, hybP;
    std::vector<double> dn, db, du, dv;
};

template <class T>
std::vector<T> to_host(Context &c, const T *d, size_t n)
{
    std::vector<T> h(n);
    CUIBM_TRY(cudaMemcpyAsync(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost, c.stream));
    return h;
}

struct PatchBuilder {
    std::vector<int> pid, pcol;
    std::vector<double> pval, pdiag;
    explicit PatchBuilder(size_t n) : pid(n, -1) {}
    // a new patched row; entries with a zero value are dropped (they do not change the operator)
    void row(int i, double diag, const int *col, const double *val, int n)
    {
        const int k = (int)pdiag.size();
        pid[i] = k;
        pdiag.push_back(diag);
        int m = 0;
        for (int e = 0; e < n; ++e)
            if (val[e] != 0) {
                pcol.push_back(col[e]);
                pval.push_back(val[e]);
                ++m;
            }
        for (; m < 5; ++m) {
            pcol.push_back(-1);
            pval.push_back(0);
        }
    }
};

// LHS_mid_X (dir 0) / LHS_mid_Y (dir 1) at an interior row i of stride s: returns
// false for a plain row, else the patch (a diagonal and at most one off-diagonal)
bool velocity_patch(int dir, int i, int s, double dxI, const HostTags &T, double *diag, int *col, double *val)
{
    const int hyb = T.hyb[i], g = T.ghost[i];
    if ((hyb == -1 && g == -1) || g == 0) return false;
    *diag = 1;
    *col = 0;
    *val = 0;
    const bool tagged = dir == 0 ? hyb != -1 : hyb > 0;
    const bool inner = dir == 0 ? g > 0 : g != -1;
    if (tagged) {
        // the partner away from the surface; column 0 where no branch matches (the
        // reference's zero-initialised COO column)
        const int h2 = T.hyb2[i];
        if (hyb == h2 - 1) *col = i + 1;
        else if (hyb == h2 + 1) *col = i - 1;
        else if (hyb == h2 + s) *col = i - s;
        else if (hyb == h2 - s) *col = i + s;
        *val = dir == 0 ? -T.dn[i] / (T.dn[i] + T.db[i]) : -T.dn[i] / (T.db[i] + T.dn[i]);
        return true;
    }
    if (inner) {
        int nb = -1;
        if (T.hyb[i + 1] != -1) { nb = i + 1; *col = i - 1; }
        else if (T.hyb[i - 1] != -1) { nb = i - 1; *col = i + 1; }
        else if (T.hyb[i + s] != -1) { nb = i + s; *col = i - s; }
        else if (T.hyb[i - s] != -1) { nb = i - s; *col = i + s; }
        if (nb >= 0) *val = -(dxI - T.dn[nb]) / (dxI - T.dn[nb] + T.db[nb]);
        return true;
    }
    *diag = 0;  // no branch of the reference writes this row: it is empty
    return true;
}

}  // namespace

void setup_fadlun(Context &c)
{
    const int nx = c.g.nx, ny = c.g.ny, nU = c.g.nU, nUV = c.g.nUV, nP = c.g.nP;
    IbArrays &b = c.ib;
    HostTags T;
    T.hyb = to_host(c, b.hybridUV, nUV);
    T.hyb2 = to_host(c, b.hybrid2UV, nUV);
    T.ghost = to_host(c, b.ghostUV, nUV);
    T.dn = to_host(c, b.distNode, nUV);
    T.db = to_host(c, b.distBetween, nUV);
    T.ghostP = to_host(c, b.ghostP, nP);
    T.hybP = to_host(c, b.hybridP, nP);
    T.du = to_host(c, b.distU, nP);
    T.dv = to_host(c, b.distV, nP);
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
    const std::vector<double> &dx = c.gx.width, &dy = c.gy.width;

    // LHS1: interior rows of the u block, then of the v block
    PatchBuilder P1(nUV);
    for (int i = 0; i < nU; ++i) {
        const int I = i % (nx - 1), J = i / (nx - 1);
        if (I == 0 || I == nx - 2 || J == 0 || J == ny - 1) continue;
        double d, v;
        int col;
        if (velocity_patch(0, i, nx - 1, dx[I], T, &d, &col, &v)) P1.row(i, d, &col, &v, 1);
    }
    for (int k = 0; k < nx * (ny - 1); ++k) {
        const int I = k % nx, J = k / nx, i = k + nU;
        if (I == 0 || I == nx - 1 || J == 0 || J == ny - 2) continue;
        double d, v;
        int col;
        if (velocity_patch(1, i, nx, dx[I], T, &d, &col, &v)) P1.row(i, d, &col, &v, 1);
    }

    // LHS2 (LHS2_mid): tagged interior rows; the centre pin as the plain rows have it
    PatchBuilder P2(nP);
    const double dt = c.P.dt;
    const int centre = (ny / 2) * nx + nx / 2;
    for (int ip = 0; ip < nP; ++ip) {
        const int I = ip % nx, J = ip / nx;
        if (I == 0 || I == nx - 1 || J == 0 || J == ny - 1) continue;
        const bool hybrid = T.hybP[ip] != -1, inside = !hybrid && T.ghostP[ip] > 0;
        if (!hybrid && !inside) continue;
        const int nb[4] = {ip + 1, ip - 1, ip + nx, ip - nx};
        double val[4], t = 0;
        for (int k = 0; k < 4; ++k) {
            const double h = k < 2 ? dx[I] : dy[J];
            val[k] = 0;
            if (hybrid) {
                if (T.ghostP[nb[k]] == -1) {
                    const double d = k < 2 ? T.du[ip] : T.dv[ip];
                    const double e = (d > h / 2 && d < h) ? d : h;  // the face shortened by the body
                    val[k] = -dt / h / e;
                    t += dt / h / e;
                }
            } else if (T.ghostP[nb[k]] == 0) {
                val[k] = -dt / h / h;
                t += dt / h / h;
            }
        }
        if (ip == centre) t += t;
        P2.row(ip, t, nb, val, 4);
    }

    auto upload = [&](PatchBuilder &B, RowPatch &R, std::vector<int> &hid, std::vector<int> &hcol,
                      std::vector<double> &hval, std::vector<double> &hdiag) {
        const size_t n = B.pid.size(), np = std::max<size_t>(1, B.pdiag.size());
        int *pid = c.carve<int>(n);
        int *pcol = c.carve<int>(5 * np);
        double *pval = c.carve<double>(5 * np);
        double *pdiag = c.carve<double>(np);
        CUIBM_TRY(cudaMemcpy(pid, B.pid.data(), n * sizeof(int), cudaMemcpyHostToDevice));
        if (!B.pdiag.empty()) {
            CUIBM_TRY(cudaMemcpy(pcol, B.pcol.data(), B.pcol.size() * sizeof(int), cudaMemcpyHostToDevice));
            CUIBM_TRY(cudaMemcpy(pval, B.pval.data(), B.pval.size() * sizeof(double), cudaMemcpyHostToDevice));
            CUIBM_TRY(cudaMemcpy(pdiag, B.pdiag.data(), B.pdiag.size() * sizeof(double), cudaMemcpyHostToDevice));
        }
        R = RowPatch{pid, pcol, pval, pdiag};
        hid = B.pid;
        hcol = B.pcol;
        hval = B.pval;
        hdiag = B.pdiag;
    };
    upload(P1, c.l1.patch, c.fadlun.pid1, c.fadlun.pcol1, c.fadlun.pval1, c.fadlun.pdiag1);
    upload(P2, c.l2.patch, c.fadlun.pid2, c.fadlun.pcol2, c.fadlun.pval2, c.fadlun.pdiag2);
    std::vector<int> r, cc;
    std::vector<double> v;
    host_matrix_coo(c, 1, r, cc, v);
    c.fadlun.nnz1 = (int)r.size();
    host_matrix_coo(c, 2, r, cc, v);
    c.fadlun.nnz2 = (int)r.size();
}

// ---- right-hand sides and projection ------------------------------------------------
// updateRHS1forIBX/Y: hybrid rows get b/(d+b) uv, ghost rows 0 (the same expression)
__global__ void k_fadlun_rhs1(int nUV, const int *hyb, const int *ghost, double *rhs, const double *dn,
                              const double *db, const double *uv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nUV) return;
    rhs[i] = (hyb[i] == -1) * (ghost[i] <= 0) * (rhs[i]) + (hyb[i] != -1) * db[i] / (dn[i] + db[i]) * uv[i];
}

// intermediatePressure (FadlunModified): -D uhat with the faces of tagged cells as LHS2_mid has them
__global__ void k_fadlun_rhs2(int nx, int ny, const double *uhat, const int *ghostP, const int *hybP,
                              const double *du, const double *dv, const double *ym, const double *yp,
                              const double *xm, const double *xp, const double *dx, const double *dy, double *rhs2)
{
    const int ip = blockIdx.x * blockDim.x + threadIdx.x;
    if (ip >= nx * ny) return;
    const int I = ip % nx, J = ip / nx, iu = (nx - 1) * J + I, iv = (nx - 1) * ny + nx * J + I;
    double t = 0;
    if (hybP[ip] != -1) {
        const double eu = (du[ip] > dx[I] / 2 && du[ip] < dx[I]) ? du[ip] : dx[I];
        const double ev = (dv[ip] > dy[J] / 2 && dv[ip] < dy[J]) ? dv[ip] : dy[J];
        if (ghostP[ip + 1] == -1) t -= uhat[iu] / eu;
        if (ghostP[ip - 1] == -1) t += uhat[iu - 1] / eu;
        if (ghostP[ip + nx] == -1) t -= uhat[iv] / ev;
        if (ghostP[ip - nx] == -1) t += uhat[iv - nx] / ev;
    } else if (ghostP[ip] > 0) {
        if (ghostP[ip + 1] == 0) t -= uhat[iu] / dx[I];
        if (ghostP[ip - 1] == 0) t += uhat[iu - 1] / dx[I];
        if (ghostP[ip + nx] == 0) t -= uhat[iv] / dy[J];
        if (ghostP[ip - nx] == 0) t += uhat[iv - nx] / dy[J];
    } else {
        t -= (I != nx - 1 ? uhat[iu] : xp[J]) / dx[I];
        t += (I != 0 ? uhat[iu - 1] : xm[J]) / dx[I];
        t -= (J != ny - 1 ? uhat[iv] : yp[(nx - 1) + I]) / dy[J];
        t += (J != 0 ? uhat[iv - nx] : ym[(nx - 1) + I]) / dy[J];
    }
    rhs2[ip] = t;
}

// project_velocity_X/Y (FadlunModified): no gradient across faces touching a tagged cell
__global__ void k_fadlun_project(int nx, int ny, const double *uhat, const double *p, const int *ghostP,
                                 const double *dx, const double *dy, double dt, double *u)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nU = (nx - 1) * ny, nUV = nU + nx * (ny - 1);
    if (i >= nUV) return;
    if (i < nU) {
        const int I = i % (nx - 1), J = i / (nx - 1), ip = J * nx + I;
        u[i] = uhat[i] - (ghostP[ip + 1] == -1 && ghostP[ip] == -1) * dt * (p[ip + 1] - p[ip]) /
                             (0.5 * dx[I + 1] + 0.5 * dx[I]);
    } else {
        const int k = i - nU, I = k % nx, J = k / nx, ip = J * nx + I;
        u[i] = uhat[i] - (ghostP[ip + nx] == -1 && ghostP[ip] == -1) * dt * (p[ip + nx] - p[ip]) /
                             (0.5 * dy[J + 1] + 0.5 * dy[J]);
    }
}

void launch_fadlun_rhs1(Context &c)
{
    IbArrays &b = c.ib;
    k_fadlun_rhs1<<<blocks_for(c.g.nUV), kBlock, 0, c.stream>>>(c.g.nUV, b.hybridUV, b.ghostUV, c.rhs1, b.distNode,
                                                                b.distBetween, b.uvBody);
    CUIBM_TRY(cudaGetLastError());
}

void launch_fadlun_rhs2(Context &c)
{
    IbArrays &b = c.ib;
    k_fadlun_rhs2<<<blocks_for(c.g.nP), kBlock, 0, c.stream>>>(c.g.nx, c.g.ny, c.uhat, b.ghostP, b.hybridP, b.distU,
                                                              b.distV, c.bc[YMINUS], c.bc[YPLUS], c.bc[XMINUS],
                                                              c.bc[XPLUS], c.dx, c.dy, c.rhs2);
    CUIBM_TRY(cudaGetLastError());
}

void launch_fadlun_project(Context &c)
{
    k_fadlun_project<<<blocks_for(c.g.nUV), kBlock, 0, c.stream>>>(c.g.nx, c.g.ny, c.uhat, c.p, c.ib.ghostP, c.dx,
                                                                  c.dy, c.P.dt, c.u);
    CUIBM_TRY(cudaGetLastError());
}

}  // namespace cuibm
