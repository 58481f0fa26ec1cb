// Navier-Stokes stencils of the fractional step on the staggered grid.
//
// GB300 layout: one thread per unknown, u block then v block exactly as the
// reference's flat vectors, so every field is read and written with unit-stride
// coalesced accesses.  All grid metrics are precomputed once on the host into
// small 1-D tables (per column I / per row J): the reference evaluates ~12 FP64
// divisions per node per kernel (NavierStokes/kernels/N.cu:39-50), which on GB300's
// FP64 pipe would cost more than the HBM traffic itself.  The tables are a few KB
// and stay in L1/L2.
//
// Replaces (NavierStokes/kernels/):
//   k_rhs1     N.cu (Nmidx, Nbcx, Nmidy, Nbcy) + L.cu (Lmidx..Lbcy) + intermediateVelocity.cu
//              (bc1X, bc1Y, generateRHS), fused into one pass.  The reference's
//              NavierStokes/intermediateVelocity.cu:124 copy Nold = N is folded in too.
//   k_rhs2     intermediatePressure.cu (intermediatePressureNoBody; same as luoIBM's)
//   k_project  projectVelocity.cu (project_velocity_X/Y_nobody; same as luo_base's)
//   lhs1_row / lhs2_row   the COO matrices of LHS1.cu / LHS2.cu applied matrix-free
//   k_init_velocity  initialise.cu;  k_cfl  CFL.cu
#include <cmath>
#include <algorithm>
#include <vector>

#include "operators.cuh"
#include "solver.h"

namespace cuibm {

__global__ void k_apply_lhs1(Lhs1Coef c, Grid g, const double *__restrict__ x, double *__restrict__ y)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < g.nUV) y[i] = lhs1_row(c, g, i, x);
}

__global__ void k_apply_lhs2(Lhs2Coef c, Grid g, const double *__restrict__ x, double *__restrict__ y)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < g.nP) y[i] = lhs2_row(c, g, i, x);
}

// ---------------------------------------------------------------------------
// fused explicit right-hand side
// ---------------------------------------------------------------------------
struct BcPtrs {
    const double *xm, *xp, *ym, *yp;
};

// SHIFT: the step's form: N of the previous step moves to Nold while the new N is
// written (the reference's "Nold = N" copy).  DEBUG: also store L and bc1.
template <bool SHIFT, bool DEBUG>
__global__ void __launch_bounds__(256) k_rhs1(RhsCoef c, Grid g, BcPtrs b, const double *__restrict__ u,
                                              double *__restrict__ N, double *__restrict__ Nold,
                                              double *__restrict__ rhs, double *__restrict__ Lout,
                                              double *__restrict__ bc1out, double nu, double dt)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.nUV) return;
    const int nx = g.nx, ny = g.ny, nU = g.nU;
    const double hd = 0.5 * dt * nu;
    const double uc = u[t];
    double Nn, Ln, B1 = 0;
    if (t < nU) {
        const int I = t % (nx - 1), J = t / (nx - 1), iv = nU + nx * J + I;
        const double ue = (I == nx - 2) ? b.xp[J] : u[t + 1];
        const double uw = (I == 0) ? b.xm[J] : u[t - 1];
        const double un = (J == ny - 1) ? 0.0 : u[t + nx - 1];
        const double us = (J == 0) ? 0.0 : u[t - nx + 1];
        const double vne = (J == ny - 1) ? b.yp[nx + I] : u[iv + 1];
        const double vn = (J == ny - 1) ? b.yp[nx - 1 + I] : u[iv];
        const double vse = (J == 0) ? b.ym[nx + I] : u[iv - nx + 1];
        const double vs = (J == 0) ? b.ym[nx - 1 + I] : u[iv - nx];
        const double a = c.uxA[I];
        const double vbar = ((vne - vn) * a + vn) / 2 + ((vse - vs) * a + vs) / 2;
        const double unc = (J == ny - 1) ? 2 * b.yp[I] - uc : un;  // mirrored ghost value
        const double usc = (J == 0) ? 2 * b.ym[I] - uc : us;
        Nn = uc * (ue * c.uxE[I] + uw * c.uxW[I] + uc * c.uxC[I]) +
             vbar * (unc * c.uyN[J] + usc * c.uyS[J] + uc * c.uyC[J]);
        const double unl = (J == ny - 1) ? b.yp[I] : un;
        const double usl = (J == 0) ? b.ym[I] : us;
        Ln = nu * ((ue - uc) * c.ulE[I] + (uw - uc) * c.ulW[I] + (unl - uc) * c.ulN[J] + (usl - uc) * c.ulS[J]);
        if (I == nx - 2) B1 += b.xp[J] * hd * c.ulE[I];
        if (I == 0) B1 += b.xm[J] * hd * c.ulW[I];
        if (J == ny - 1) B1 += (2 * b.yp[I] - uc) * hd * (0.5 * c.ulN[J]);
        if (J == 0) B1 += (2 * b.ym[I] - uc) * hd * (0.5 * c.ulS[J]);
    } else {
        const int k = t - nU, I = k % nx, J = k / nx, iu = (nx - 1) * J + I;
        const double ve = (I == nx - 1) ? 0.0 : u[t + 1];
        const double vw = (I == 0) ? 0.0 : u[t - 1];
        const double vn = (J == ny - 2) ? b.yp[nx - 1 + I] : u[t + nx];
        const double vs = (J == 0) ? b.ym[nx - 1 + I] : u[t - nx];
        const double une = (I == nx - 1) ? b.xp[J + 1] : u[iu + nx - 1];
        const double ue = (I == nx - 1) ? b.xp[J] : u[iu];
        const double unw = (I == 0) ? b.xm[J + 1] : u[iu + nx - 2];
        const double uw = (I == 0) ? b.xm[J] : u[iu - 1];
        const double a = c.vyA[J];
        const double ubar = ((une - ue) * a + ue) / 2 + ((unw - uw) * a + uw) / 2;
        const double vec = (I == nx - 1) ? 2 * b.xp[ny + J] - uc : ve;
        const double vwc = (I == 0) ? 2 * b.xm[ny + J] - uc : vw;
        Nn = ubar * (vec * c.vxE[I] + vwc * c.vxW[I] + uc * c.vxC[I]) +
             uc * (vn * c.vyN[J] + vs * c.vyS[J] + uc * c.vyC[J]);
        const double vel = (I == nx - 1) ? b.xp[ny + J] : ve;
        const double vwl = (I == 0) ? b.xm[ny + J] : vw;
        Ln = nu * ((vel - uc) * c.vlE[I] + (vwl - uc) * c.vlW[I] + (vn - uc) * c.vlN[J] + (vs - uc) * c.vlS[J]);
        if (I == nx - 1) B1 += (2 * b.xp[ny + J] - uc) * hd * (0.5 * c.vlE[I]);
        if (I == 0) B1 += (2 * b.xm[ny + J] - uc) * hd * (0.5 * c.vlW[I]);
        if (J == ny - 2) B1 += b.yp[nx - 1 + I] * hd * c.vlN[J];
        if (J == 0) B1 += b.ym[nx - 1 + I] * hd * c.vlS[J];
    }
    const double Nprev = SHIFT ? N[t] : Nold[t];
    if (SHIFT) Nold[t] = Nprev;
    N[t] = Nn;
    rhs[t] = uc + dt * (0.5 * Nprev - 1.5 * Nn + 0.5 * Ln) + B1;
    if (DEBUG) {
        Lout[t] = Ln;
        bc1out[t] = B1;
    }
}

// rhs2 = -D uhat with boundary velocities on the domain edges
__global__ void k_rhs2(Grid g, BcPtrs b, const double *__restrict__ dx, const double *__restrict__ dy,
                       const double *__restrict__ uh, double *__restrict__ rhs2)
{
    const int ip = blockIdx.x * blockDim.x + threadIdx.x;
    if (ip >= g.nP) return;
    const int nx = g.nx, ny = g.ny, I = ip % nx, J = ip / nx;
    const int iu = (nx - 1) * J + I, iv = g.nU + nx * J + I;
    const double ue = (I != nx - 1) ? uh[iu] : b.xp[J];
    const double uw = (I != 0) ? uh[iu - 1] : b.xm[J];
    const double vn = (J != ny - 1) ? uh[iv] : b.yp[nx - 1 + I];
    const double vs = (J != 0) ? uh[iv - nx] : b.ym[nx - 1 + I];
    rhs2[ip] = (((0 - ue / dx[I]) + uw / dx[I]) - vn / dy[J]) + vs / dy[J];
}

// u = uhat - dt G p ; uold = u
__global__ void k_project(Grid g, const double *__restrict__ gradU, const double *__restrict__ gradV,
                          const double *__restrict__ p, const double *__restrict__ uh, double *__restrict__ u,
                          double *__restrict__ uold)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.nUV) return;
    const double uc = u[t];
    double un;
    if (t < g.nU) {
        const int I = t % (g.nx - 1), J = t / (g.nx - 1), ip = J * g.nx + I;
        un = uh[t] - (p[ip + 1] - p[ip]) * gradU[I];
    } else {
        const int k = t - g.nU, J = k / g.nx;
        un = uh[t] - (p[k + g.nx] - p[k]) * gradV[J];
    }
    uold[t] = uc;
    u[t] = un;
}

__global__ void k_init_velocity(Grid g, const double *xu, const double *yu, const double *xv, const double *yv,
                                double uI, double vI, double uP, double vP, double xmax, double xmin,
                                double ymax, double ymin, double *u)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.nUV) return;
    const double pi = M_PI;
    if (t < g.nU) {
        const int i = t % (g.nx - 1), j = t / (g.nx - 1);
        u[t] = uI + uP * cos(0.5 * pi * (2 * xu[i] - xmax - xmin) / (xmax - xmin)) *
                        sin(pi * (2 * yu[j] - ymax - ymin) / (ymax - ymin));
    } else {
        const int k = t - g.nU, i = k % g.nx, j = k / g.nx;
        u[t] = vI + vP * cos(0.5 * pi * (2 * yv[j] - ymax - ymin) / (ymax - ymin)) *
                        sin(pi * (2 * xv[i] - xmax - xmin) / (xmax - xmin));
    }
}

__global__ void k_cfl(Grid g, const double *__restrict__ u, const double *__restrict__ dx,
                      const double *__restrict__ dy, double dt, double *__restrict__ cfl)
{
    const int ip = blockIdx.x * blockDim.x + threadIdx.x;
    if (ip >= g.nP) return;
    const int I = ip % g.nx, J = ip / g.nx;
    if (I == g.nx - 1 || J == g.ny - 1) return;
    cfl[ip] = dt * (fabs(u[(g.nx - 1) * J + I]) / dx[I] + fabs(u[g.nU + g.nx * J + I]) / dy[J]);
}

__global__ void k_copy(double *__restrict__ dst, const double *__restrict__ src, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i];
}

// ---------------------------------------------------------------------------
// host: metric tables
// ---------------------------------------------------------------------------
void upload_ns_tables(Context &c)
{
    const int nx = c.g.nx, ny = c.g.ny;
    const std::vector<double> &dx = c.gx.width, &dy = c.gy.width;
    const double dt = c.P.dt, nu = c.P.nu;
    std::vector<double> h;  // all tables, concatenated
    auto table = [&](int n, auto f) {
        size_t off = h.size();
        for (int k = 0; k < n; ++k) h.push_back(f(k));
        return off;
    };
    // convection / diffusion, u nodes per I
    size_t o_uxE = table(nx - 1, [&](int I) { double a = dx[I], b = dx[I + 1]; return a / (b * (a + b)); });
    size_t o_uxW = table(nx - 1, [&](int I) { double a = dx[I], b = dx[I + 1]; return a / (a * (a + b)) - 1 / a; });
    size_t o_uxC = table(nx - 1, [&](int I) {
        double a = dx[I], b = dx[I + 1];
        return -a / (b * (a + b)) - (a / (a * (a + b)) - 1 / a);
    });
    size_t o_uxA = table(nx - 1, [&](int I) { double a = dx[I], b = dx[I + 1]; return a / (a + b); });
    size_t o_ulE = table(nx - 1, [&](int I) { return 1 / (dx[I + 1] * (dx[I + 1] + dx[I]) * 0.5); });
    size_t o_ulW = table(nx - 1, [&](int I) { return 1 / (dx[I] * (dx[I + 1] + dx[I]) * 0.5); });
    // u nodes per J (walls fold the mirrored spacing in)
    auto dyn = [&](int J) { return J < ny - 1 ? dy[J + 1] : dy[J]; };
    auto dys = [&](int J) { return J > 0 ? dy[J - 1] : dy[J]; };
    size_t o_uyN = table(ny, [&](int J) { double cc = dy[J]; return cc / (cc * (dyn(J) + cc)); });
    size_t o_uyS = table(ny, [&](int J) { double cc = dy[J], s = dys(J); return s / (cc * (cc + s)) - 1 / cc; });
    size_t o_uyC = table(ny, [&](int J) {
        double cc = dy[J], n_ = dyn(J), s = dys(J);
        return -cc / (cc * (n_ + cc)) - (s / (cc * (cc + s)) - 1 / cc);
    });
    size_t o_ulN = table(ny, [&](int J) {
        return J < ny - 1 ? 1 / (dy[J] * (dy[J + 1] + dy[J]) * 0.5) : 2 / (dy[J] * dy[J]);
    });
    size_t o_ulS = table(ny, [&](int J) { return J > 0 ? 1 / (dy[J] * (dy[J - 1] + dy[J]) * 0.5) : 2 / (dy[J] * dy[J]); });
    // v nodes per I
    auto dxe = [&](int I) { return I < nx - 1 ? dx[I + 1] : dx[I]; };
    auto dxw = [&](int I) { return I > 0 ? dx[I - 1] : dx[I]; };
    size_t o_vxE = table(nx, [&](int I) { double a = dx[I]; return a / (a * (a + dxe(I))); });
    size_t o_vxW = table(nx, [&](int I) { double a = dx[I], w = dxw(I); return w / (a * (a + w)) - 1 / a; });
    size_t o_vxC = table(nx, [&](int I) {
        double a = dx[I], e = dxe(I), w = dxw(I);
        return -a / (a * (a + e)) - (w / (a * (a + w)) - 1 / a);
    });
    size_t o_vlE = table(nx, [&](int I) { return I < nx - 1 ? 1 / (dx[I] * (dx[I] + dx[I + 1]) * 0.5) : 2 / (dx[I] * dx[I]); });
    size_t o_vlW = table(nx, [&](int I) { return I > 0 ? 1 / (dx[I] * (dx[I] + dx[I - 1]) * 0.5) : 2 / (dx[I] * dx[I]); });
    // v nodes per J
    size_t o_vyN = table(ny - 1, [&](int J) { double cc = dy[J], d = dy[J + 1]; return cc / (d * (d + cc)); });
    size_t o_vyS = table(ny - 1, [&](int J) { double cc = dy[J], d = dy[J + 1]; return cc / (cc * (d + cc)) - 1 / cc; });
    size_t o_vyC = table(ny - 1, [&](int J) {
        double cc = dy[J], d = dy[J + 1];
        return -cc / (d * (d + cc)) - (cc / (cc * (d + cc)) - 1 / cc);
    });
    size_t o_vyA = table(ny - 1, [&](int J) { double cc = dy[J], d = dy[J + 1]; return cc / (cc + d); });
    size_t o_vlN = table(ny - 1, [&](int J) { return 1 / (dy[J + 1] * (dy[J] + dy[J + 1]) * 0.5); });
    size_t o_vlS = table(ny - 1, [&](int J) { return 1 / (dy[J] * (dy[J] + dy[J + 1]) * 0.5); });
    // LHS1 (reference LHS1.cu expressions)
    size_t o_1uE = table(nx - 1, [&](int I) { return 0.5 * dt * nu * (1 / (dx[I + 1] * (dx[I + 1] + dx[I]) * 0.5)); });
    size_t o_1uW = table(nx - 1, [&](int I) { return 0.5 * dt * nu * (1 / (dx[I] * (dx[I + 1] + dx[I]) * 0.5)); });
    size_t o_1uN = table(ny, [&](int J) { return 0.5 * dt * nu * (1 / (dy[J] * (dyn(J) + dy[J]) * 0.5)); });
    size_t o_1uS = table(ny, [&](int J) { return 0.5 * dt * nu * (1 / (dy[J] * (dys(J) + dy[J]) * 0.5)); });
    size_t o_1vE = table(nx, [&](int I) { return 0.5 * dt * nu * (1 / (dx[I] * (dx[I] + dxe(I)) * 0.5)); });
    size_t o_1vW = table(nx, [&](int I) { return 0.5 * dt * nu * (1 / (dx[I] * (dx[I] + dxw(I)) * 0.5)); });
    size_t o_1vN = table(ny - 1, [&](int J) { return 0.5 * dt * nu * (1 / (dy[J + 1] * (dy[J] + dy[J + 1]) * 0.5)); });
    size_t o_1vS = table(ny - 1, [&](int J) { return 0.5 * dt * nu * (1 / (dy[J] * (dy[J] + dy[J + 1]) * 0.5)); });
    // LHS2 (reference LHS2.cu expressions; 0 where the neighbour does not exist)
    size_t o_2E = table(nx, [&](int I) { return I != nx - 1 ? dt / (dx[I] * (dx[I] + dx[I + 1]) * 0.5) : 0.0; });
    size_t o_2W = table(nx, [&](int I) { return I != 0 ? dt / (dx[I] * (dx[I] + dx[I - 1]) * 0.5) : 0.0; });
    size_t o_2N = table(ny, [&](int J) { return J != ny - 1 ? dt / (dy[J] * (dy[J] + dy[J + 1]) * 0.5) : 0.0; });
    size_t o_2S = table(ny, [&](int J) { return J != 0 ? dt / (dy[J] * (dy[J] + dy[J - 1]) * 0.5) : 0.0; });
    // projection
    size_t o_gU = table(nx - 1, [&](int I) { return dt / (0.5 * dx[I + 1] + 0.5 * dx[I]); });
    size_t o_gV = table(ny - 1, [&](int J) { return dt / (0.5 * dy[J + 1] + 0.5 * dy[J]); });

    c.htab = h;
    c.hoff = {{"1uE", o_1uE}, {"1uW", o_1uW}, {"1uN", o_1uN}, {"1uS", o_1uS}, {"1vE", o_1vE}, {"1vW", o_1vW},
              {"1vN", o_1vN}, {"1vS", o_1vS}, {"2E", o_2E},   {"2W", o_2W},   {"2N", o_2N},   {"2S", o_2S}};
    double *d = c.carve<double>(h.size());
    CUIBM_TRY(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    RhsCoef &r = c.rc;
    r.uxE = d + o_uxE; r.uxW = d + o_uxW; r.uxC = d + o_uxC; r.uxA = d + o_uxA;
    r.ulE = d + o_ulE; r.ulW = d + o_ulW;
    r.uyN = d + o_uyN; r.uyS = d + o_uyS; r.uyC = d + o_uyC; r.ulN = d + o_ulN; r.ulS = d + o_ulS;
    r.vxE = d + o_vxE; r.vxW = d + o_vxW; r.vxC = d + o_vxC; r.vlE = d + o_vlE; r.vlW = d + o_vlW;
    r.vyN = d + o_vyN; r.vyS = d + o_vyS; r.vyC = d + o_vyC; r.vyA = d + o_vyA; r.vlN = d + o_vlN; r.vlS = d + o_vlS;
    r.dx = c.dx; r.dy = c.dy;
    c.l1.uE = d + o_1uE; c.l1.uW = d + o_1uW; c.l1.uN = d + o_1uN; c.l1.uS = d + o_1uS;
    c.l1.vE = d + o_1vE; c.l1.vW = d + o_1vW; c.l1.vN = d + o_1vN; c.l1.vS = d + o_1vS;
    c.l2.E = d + o_2E; c.l2.W = d + o_2W; c.l2.N = d + o_2N; c.l2.S = d + o_2S;
    c.l2.pin0 = 0;
    // the centre pin exists in the plain and Fadlun operators only (LHS2_mid_nobody,
    // FadlunModified LHS2_mid), and only when the centre cell is not on the boundary
    int cidx = (ny / 2) * nx + nx / 2, cI = nx / 2, cJ = ny / 2;
    bool interior = cI != 0 && cI != nx - 1 && cJ != 0 && cJ != ny - 1;
    c.l2.pinc = ((c.P.solverType == ST_NAVIERSTOKES || c.P.solverType == ST_FADLUN) && interior) ? cidx : -1;
    c.gradU = d + o_gU;
    c.gradV = d + o_gV;
}

// The reference's COO matrices rebuilt from the host copy of the coefficient
// tables, entries in the reference's order (LHS1.cu / LHS2.cu numE offsets: per
// row E, W, N, S, centre, rows in increasing order).  The same table values feed
// the device rows, so this is exactly the operator the solvers apply.
void host_matrix_coo(Context &c, int which, std::vector<int> &row, std::vector<int> &col, std::vector<double> &val)
{
    const int nx = c.g.nx, ny = c.g.ny;
    const double *t = c.htab.data();
    auto T = [&](const char *k) { return t + c.hoff.at(k); };
    row.clear();
    col.clear();
    val.clear();
    auto push = [&](int r, int cc, double v) {
        row.push_back(r);
        col.push_back(cc);
        val.push_back(v);
    };
    // a patched row of the modified Fadlun method: its entries in column order (the
    // reference sorts its Fadlun matrices by row and column; zero entries dropped)
    auto patched = [&](int i, const std::vector<int> &pid, const std::vector<int> &pcol,
                       const std::vector<double> &pval, const std::vector<double> &pdiag) {
        if (pid.empty() || pid[i] < 0) return false;
        const int k = pid[i];
        std::vector<std::pair<int, double>> e;
        if (pdiag[k] != 0) e.push_back({i, pdiag[k]});
        for (int m = 0; m < 5; ++m)
            if (pcol[5 * k + m] >= 0) e.push_back({pcol[5 * k + m], pval[5 * k + m]});
        std::sort(e.begin(), e.end(), [](const std::pair<int, double> &a, const std::pair<int, double> &b) {
            return a.first < b.first;
        });
        for (auto &q : e) push(i, q.first, q.second);
        return true;
    };
    const auto &F = c.fadlun;
    if (which == 1) {
        const double *E = T("1uE"), *W = T("1uW"), *Nn = T("1uN"), *S = T("1uS");
        for (int J = 0; J < ny; ++J)
            for (int I = 0; I < nx - 1; ++I) {
                int i = J * (nx - 1) + I;
                if (patched(i, F.pid1, F.pcol1, F.pval1, F.pdiag1)) continue;
                if (I != nx - 2) push(i, i + 1, -E[I]);
                if (I != 0) push(i, i - 1, -W[I]);
                if (J != ny - 1) push(i, i + nx - 1, -Nn[J]);
                if (J != 0) push(i, i - (nx - 1), -S[J]);
                push(i, i, (((1 + E[I]) + W[I]) + Nn[J]) + S[J]);
            }
        const double *vE = T("1vE"), *vW = T("1vW"), *vN = T("1vN"), *vS = T("1vS");
        for (int J = 0; J < ny - 1; ++J)
            for (int I = 0; I < nx; ++I) {
                int i = c.g.nU + J * nx + I;
                if (patched(i, F.pid1, F.pcol1, F.pval1, F.pdiag1)) continue;
                if (I != nx - 1) push(i, i + 1, -vE[I]);
                if (I != 0) push(i, i - 1, -vW[I]);
                if (J != ny - 2) push(i, i + nx, -vN[J]);
                if (J != 0) push(i, i - nx, -vS[J]);
                push(i, i, (((1 + vE[I]) + vW[I]) + vN[J]) + vS[J]);
            }
    } else {
        const double *E = T("2E"), *W = T("2W"), *Nn = T("2N"), *S = T("2S");
        for (int J = 0; J < ny; ++J)
            for (int I = 0; I < nx; ++I) {
                int i = J * nx + I;
                if (patched(i, F.pid2, F.pcol2, F.pval2, F.pdiag2)) continue;
                if (I != nx - 1) push(i, i + 1, -E[I]);
                if (I != 0) push(i, i - 1, -W[I]);
                if (J != ny - 1) push(i, i + nx, -Nn[J]);
                if (J != 0) push(i, i - nx, -S[J]);
                double d = (((0 + E[I]) + W[I]) + Nn[J]) + S[J];
                if (i == c.l2.pin0 || i == c.l2.pinc) d += d;
                push(i, i, d);
            }
    }
}

// CSR of the operator the solver iterates on (row weights w applied when given)
void host_operator_csr(Context &c, int which, const double *w, std::vector<int> &ptr, std::vector<int> &col,
                       std::vector<double> &val)
{
    std::vector<int> row;
    host_matrix_coo(c, which, row, col, val);
    const int n = which == 1 ? c.g.nUV : c.g.nP;
    ptr.assign(n + 1, 0);
    for (int r : row) ptr[r + 1]++;
    for (int i = 0; i < n; ++i) ptr[i + 1] += ptr[i];
    if (w)
        for (size_t k = 0; k < row.size(); ++k) val[k] *= w[row[k]];
}

static BcPtrs bc_ptrs(Context &c) { return BcPtrs{c.bc[XMINUS], c.bc[XPLUS], c.bc[YMINUS], c.bc[YPLUS]}; }

void launch_rhs1(Context &c, bool debug_terms)
{
    int nb = blocks_for(c.g.nUV);
    if (debug_terms)
        k_rhs1<false, true><<<nb, kBlock, 0, c.stream>>>(c.rc, c.g, bc_ptrs(c), c.u, c.N, c.Nold, c.rhs1, c.L, c.bc1,
                                                         c.P.nu, c.P.dt);
    else
        k_rhs1<true, false><<<nb, kBlock, 0, c.stream>>>(c.rc, c.g, bc_ptrs(c), c.u, c.N, c.Nold, c.rhs1, nullptr,
                                                         nullptr, c.P.nu, c.P.dt);
    CUIBM_TRY(cudaGetLastError());
}

void launch_rhs2(Context &c, const double *uh)
{
    k_rhs2<<<blocks_for(c.g.nP), kBlock, 0, c.stream>>>(c.g, bc_ptrs(c), c.dx, c.dy, uh, c.rhs2);
    CUIBM_TRY(cudaGetLastError());
}

void launch_project(Context &c)
{
    k_project<<<blocks_for(c.g.nUV), kBlock, 0, c.stream>>>(c.g, c.gradU, c.gradV, c.p, c.uhat, c.u, c.uold);
    CUIBM_TRY(cudaGetLastError());
}

void launch_initial_velocity(Context &c)
{
    const int nx = c.g.nx, ny = c.g.ny;
    k_init_velocity<<<blocks_for(c.g.nUV), kBlock, 0, c.stream>>>(
        c.g, c.xu, c.yu, c.xv, c.yv, c.P.uInitial, c.P.vInitial, c.P.uPerturb, c.P.vPerturb, c.gx.centre[nx - 1],
        c.gx.centre[0], c.gy.centre[ny - 1], c.gy.centre[0], c.u);
    CUIBM_TRY(cudaGetLastError());
}

void launch_apply(Context &c, int which, const double *xin, double *yout)
{
    if (which == 1)
        k_apply_lhs1<<<blocks_for(c.g.nUV), kBlock, 0, c.stream>>>(c.l1, c.g, xin, yout);
    else
        k_apply_lhs2<<<blocks_for(c.g.nP), kBlock, 0, c.stream>>>(c.l2, c.g, xin, yout);
    CUIBM_TRY(cudaGetLastError());
}

void launch_cfl(Context &c)
{
    k_cfl<<<blocks_for(c.g.nP), kBlock, 0, c.stream>>>(c.g, c.u, c.dx, c.dy, c.P.dt, c.cfl);
    CUIBM_TRY(cudaGetLastError());
}

void launch_copy(Context &c, double *dst, const double *src, int n)
{
    k_copy<<<blocks_for(n), kBlock, 0, c.stream>>>(dst, src, n);
    CUIBM_TRY(cudaGetLastError());
}

}  // namespace cuibm
