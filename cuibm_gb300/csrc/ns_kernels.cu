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

#include "ib_plan.h"
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

// The embedded method's update of rhs1 (luo_iter/kernels/intermediateVelocity.cu
// update_rhs1_x/y with the ns_rhs and interp_rhs of LHS1_mid_iter_X/Y): interior rows
// without a patch are divided by their diagonal (rhs * rscale); a hybrid row becomes
// rhs * pns + pint; a ghost row becomes its interp_rhs 2 u_B - sum_l w_l q_l over the
// interpolation corners that are ghost nodes, q_l the body velocity where the
// interpolation substituted the corner, else the field there.  pid is null for the
// other methods.
struct EmbRhs1 {
    const int *pid;
    const double *rscale, *pns, *pint;
    int cap;  // slots below cap are ghost rows
    const int *gin, *gIdx, *gMask;
    const double *gW, *uB, *vB;
};

__device__ __forceinline__ double emb_rhs1(const EmbRhs1 &e, int t, int nU, double r, const double *__restrict__ u)
{
    const int k = e.pid[t];
    if (k < 0) return r * e.rscale[t];
    if (k >= e.cap) return __dadd_rn(__dmul_rn(r, e.pns[k]), e.pint[k]);
    const double qb = t >= nU ? e.vB[0] : e.uB[0];
    const int in = e.gin[k], m = e.gMask[k];
    double temp = 0;
    for (int l = 0; l < 4; ++l)
        if (in >> l & 1) {
            const double q = (m >> l & 1) ? qb : u[e.gIdx[4 * k + l]];
            temp = __dsub_rn(temp, __dmul_rn(e.gW[4 * k + l], q));
        }
    return __dadd_rn(2 * qb, temp);
}

// SHIFT: the step's form: N of the previous step moves to Nold while the new N is
// written (the reference's "Nold = N" copy).  DEBUG: also store L and bc1.
template <bool SHIFT, bool DEBUG>
__global__ void __launch_bounds__(256) k_rhs1(RhsCoef c, Grid g, BcPtrs b, const double *__restrict__ u,
                                              double *__restrict__ N, double *__restrict__ Nold,
                                              double *__restrict__ rhs, double *__restrict__ Lout,
                                              double *__restrict__ bc1out, double nu, double dt, EmbRhs1 e)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.nUV) return;
    const int nx = g.nx, ny = g.ny, nU = g.nU;
    const double hd = 0.5 * dt * nu;
    const double uc = u[t];
    double Nn, Lr, B1 = 0;  // Lr: the diffusion term over nu
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
        // ((vne - vn) a + vn) / 2 + ((vse - vs) a + vs) / 2, folded
        const double vbar = c.uhA[I] * (vne + vse) + c.uhB[I] * (vn + vs);
        const double unc = (J == ny - 1) ? 2 * b.yp[I] - uc : un;  // mirrored ghost value
        const double usc = (J == 0) ? 2 * b.ym[I] - uc : us;
        Nn = uc * (ue * c.uxE[I] + uw * c.uxW[I] + uc * c.uxC[I]) +
             vbar * (unc * c.uyN[J] + usc * c.uyS[J] + uc * c.uyC[J]);
        const double unl = (J == ny - 1) ? b.yp[I] : un;
        const double usl = (J == 0) ? b.ym[I] : us;
        Lr = (ue - uc) * c.ulE[I] + (uw - uc) * c.ulW[I] + (unl - uc) * c.ulN[J] + (usl - uc) * c.ulS[J];
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
        const double ubar = c.vhA[J] * (une + unw) + c.vhB[J] * (ue + uw);
        const double vec = (I == nx - 1) ? 2 * b.xp[ny + J] - uc : ve;
        const double vwc = (I == 0) ? 2 * b.xm[ny + J] - uc : vw;
        Nn = ubar * (vec * c.vxE[I] + vwc * c.vxW[I] + uc * c.vxC[I]) +
             uc * (vn * c.vyN[J] + vs * c.vyS[J] + uc * c.vyC[J]);
        const double vel = (I == nx - 1) ? b.xp[ny + J] : ve;
        const double vwl = (I == 0) ? b.xm[ny + J] : vw;
        Lr = (vel - uc) * c.vlE[I] + (vwl - uc) * c.vlW[I] + (vn - uc) * c.vlN[J] + (vs - uc) * c.vlS[J];
        if (I == nx - 1) B1 += (2 * b.xp[ny + J] - uc) * hd * (0.5 * c.vlE[I]);
        if (I == 0) B1 += (2 * b.xm[ny + J] - uc) * hd * (0.5 * c.vlW[I]);
        if (J == ny - 2) B1 += b.yp[nx - 1 + I] * hd * c.vlN[J];
        if (J == 0) B1 += b.ym[nx - 1 + I] * hd * c.vlS[J];
    }
    const double Nprev = SHIFT ? N[t] : Nold[t];
    if (SHIFT) Nold[t] = Nprev;
    N[t] = Nn;
    // uc + dt (0.5 Nold - 1.5 N + 0.5 L) + B1 with L = nu Lr
    const double r = uc + (0.5 * dt) * Nprev - (1.5 * dt) * Nn + hd * Lr + B1;
    rhs[t] = e.pid ? emb_rhs1(e, t, nU, r, u) : r;
    if (DEBUG) {
        Lout[t] = nu * Lr;
        bc1out[t] = B1;
    }
}

// The embedded method's update of rhs2 (luo_iter/kernels/pressure.cu update_rhs2, whose
// threads stop at (nx-1)*ny): a patched row becomes rhs * pns + interp_rhs, where
// interp_rhs (the dp/dn and Neumann-corner terms of LHS2_mid_iter) is linear in the
// body acceleration (uB - uBk)/dt; the other rows keep rhs (ns_rhs 1, interp_rhs 0).
struct EmbRhs2 {
    const int *pid;
    const double *pns, *pAu, *pAv;
    const double *uB, *uBk, *vB, *vBk;
    double dt;
};

// rhs2 = -D uhat with boundary velocities on the domain edges (1/dx, 1/dy tables)
__global__ void k_rhs2(Grid g, BcPtrs b, const double *__restrict__ rdx, const double *__restrict__ rdy,
                       const double *__restrict__ uh, double *__restrict__ rhs2, EmbRhs2 e)
{
    const int ip = blockIdx.x * blockDim.x + threadIdx.x;
    if (ip >= g.nP) return;
    const int nx = g.nx, ny = g.ny, I = ip % nx, J = ip / nx;
    const int iu = (nx - 1) * J + I, iv = g.nU + nx * J + I;
    const double ue = (I != nx - 1) ? uh[iu] : b.xp[J];
    const double uw = (I != 0) ? uh[iu - 1] : b.xm[J];
    const double vn = (J != ny - 1) ? uh[iv] : b.yp[nx - 1 + I];
    const double vs = (J != 0) ? uh[iv - nx] : b.ym[nx - 1 + I];
    // -(ue - uw)/dx - (vn - vs)/dy with reciprocal tables (FP64 divides are the slow path)
    double r = (uw - ue) * rdx[I] + (vs - vn) * rdy[J];
    if (e.pid && ip < (nx - 1) * ny) {
        const int k = e.pid[ip];
        if (k >= 0) {
            const double dudt = (e.uB[0] - e.uBk[0]) / e.dt, dvdt = (e.vB[0] - e.vBk[0]) / e.dt;
            const double in = __dadd_rn(__dmul_rn(dudt, e.pAu[k]), __dmul_rn(dvdt, e.pAv[k]));
            r = __dadd_rn(__dmul_rn(r, e.pns[k]), in);
        }
    }
    rhs2[ip] = r;
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

// FP64 issue peak: 8 independent chains of kFmaIters fused multiply-adds per thread
// (2 FLOPs each), the result kept live through one store per thread
constexpr int kFmaIters = 4096;
__global__ void __launch_bounds__(256) k_fp64_fma(double a, double b, double sink, double *out)
{
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-9 + k;
    for (int it = 0; it < kFmaIters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
    }
    double s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += x[k];
    // the sum is compared with a value it never takes (a NaN): every FMA is needed for
    // the comparison, and nothing is written
    if (s == sink) out[0] = s;
}

// one launch of k_fp64_fma over blocks x 256 threads (out: one double, never written);
// returns the FLOPs it performs
double launch_fp64_fma(Context &c, int blocks, double *out)
{
    k_fp64_fma<<<blocks, 256, 0, c.stream>>>(0.999999, 1e-7, std::nan(""), out);
    CUIBM_TRY(cudaGetLastError());
    return 2.0 * 8 * kFmaIters * 256.0 * blocks;
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
    // folded tables of the fused right-hand side (see RhsCoef)
    size_t o_uhA = table(nx - 1, [&](int I) { double a = dx[I], b = dx[I + 1]; return 0.5 * (a / (a + b)); });
    size_t o_uhB = table(nx - 1, [&](int I) { double a = dx[I], b = dx[I + 1]; return 0.5 * (1 - a / (a + b)); });
    size_t o_vhA = table(ny - 1, [&](int J) { double cc = dy[J], d = dy[J + 1]; return 0.5 * (cc / (cc + d)); });
    size_t o_vhB = table(ny - 1, [&](int J) { double cc = dy[J], d = dy[J + 1]; return 0.5 * (1 - cc / (cc + d)); });
    size_t o_rdx = table(nx, [&](int I) { return 1 / dx[I]; });
    size_t o_rdy = table(ny, [&](int J) { return 1 / dy[J]; });
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
    r.uhA = d + o_uhA; r.uhB = d + o_uhB;
    r.vhA = d + o_vhA; r.vhB = d + o_vhB;
    r.rdx = d + o_rdx; r.rdy = d + o_rdy;
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
void host_matrix_coo(Context &c, int which, std::vector<int> &row, std::vector<int> &col, std::vector<double> &val,
                     bool body_free)
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
    // a patched row (modified Fadlun or embedded method): its entries in column order
    // (the reference sorts these matrices by row and column; zero entries dropped)
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
    // the embedded method's patched rows live on the device (rebuilt at every tagging)
    Context::FadlunRows F = c.fadlun;
    const bool emb = c.emb.pid1 != nullptr;
    if (body_free) F = Context::FadlunRows{};  // no patched rows
    if (emb && !body_free) {
        auto down = [&](auto &v, const auto *src, size_t n) {
            v.resize(n);
            CUIBM_TRY(cudaMemcpyAsync(v.data(), src, n * sizeof(v[0]), cudaMemcpyDeviceToHost, c.stream));
        };
        const size_t s1 = 2 * (size_t)c.emb.cap1, s2 = 2 * (size_t)c.emb.cap2;
        down(F.pid1, c.emb.pid1, c.g.nUV);
        down(F.pcol1, c.emb.pcol1, 5 * s1);
        down(F.pval1, c.emb.pval1, 5 * s1);
        down(F.pdiag1, c.emb.pdiag1, s1);
        down(F.pid2, c.emb.pid2, c.g.nP);
        down(F.pcol2, c.emb.pcol2, 5 * s2);
        down(F.pval2, c.emb.pval2, 5 * s2);
        down(F.pdiag2, c.emb.pdiag2, s2);
        CUIBM_TRY(cudaStreamSynchronize(c.stream));
    }
    const double *dx = c.gx.width.data(), *dy = c.gy.width.data(), dt = c.P.dt, nu = c.P.nu;
    // an interior row of the embedded LHS1 without a patch: the momentum row over its
    // diagonal (LHS1_mid_iter_X/Y, luo_iter/kernels/LHS1.cu), entries E, W, N, S, centre
    auto scaled_u = [&](int i, int I, int J) {
        const double temp = 1 + 0.5 * dt * nu * (1 / (dx[I + 1] * (dx[I + 1] + dx[I]) * 0.5)) +
                            0.5 * dt * nu * (1 / (dx[I] * (dx[I + 1] + dx[I]) * 0.5)) +
                            0.5 * dt * nu * (1 / (dy[J] * (dy[J + 1] + dy[J]) * 0.5)) +
                            0.5 * dt * nu * (1 / (dy[J] * (dy[J - 1] + dy[J]) * 0.5));
        push(i, i + 1, -0.5 * dt * nu * (1 / (dx[I + 1] * (dx[I + 1] + dx[I]) * 0.5)) / temp);
        push(i, i - 1, -0.5 * dt * nu * (1 / (dx[I] * (dx[I + 1] + dx[I]) * 0.5)) / temp);
        push(i, i + (nx - 1), -0.5 * dt * nu * (1 / (dy[J] * (dy[J + 1] + dy[J]) * 0.5)) / temp);
        push(i, i - (nx - 1), -0.5 * dt * nu * (1 / (dy[J] * (dy[J - 1] + dy[J]) * 0.5)) / temp);
        push(i, i, 1);
    };
    auto scaled_v = [&](int i, int I, int J) {
        const double temp = 1 + 0.5 * dt * nu * (1 / (dx[I] * (dx[I] + dx[I + 1]) * 0.5)) +
                            0.5 * dt * nu * (1 / (dx[I] * (dx[I] + dx[I - 1]) * 0.5)) +
                            0.5 * dt * nu * (1 / (dy[J + 1] * (dy[J] + dy[J + 1]) * 0.5)) +
                            0.5 * dt * nu * (1 / (dy[J] * (dy[J] + dy[J + 1]) * 0.5));
        push(i, i + 1, -0.5 * dt * nu * (1 / (dx[I] * (dx[I] + dx[I + 1]) * 0.5)) / temp);
        push(i, i - 1, -0.5 * dt * nu * (1 / (dx[I] * (dx[I] + dx[I - 1]) * 0.5)) / temp);
        push(i, i + nx, -0.5 * dt * nu * (1 / (dy[J + 1] * (dy[J] + dy[J + 1]) * 0.5)) / temp);
        push(i, i - nx, -0.5 * dt * nu * (1 / (dy[J] * (dy[J] + dy[J + 1]) * 0.5)) / temp);
        push(i, i, 1);
    };
    if (which == 1) {
        const double *E = T("1uE"), *W = T("1uW"), *Nn = T("1uN"), *S = T("1uS");
        for (int J = 0; J < ny; ++J)
            for (int I = 0; I < nx - 1; ++I) {
                int i = J * (nx - 1) + I;
                if (patched(i, F.pid1, F.pcol1, F.pval1, F.pdiag1)) continue;
                if (emb && I != 0 && I != nx - 2 && J != 0 && J != ny - 1) {
                    scaled_u(i, I, J);
                    continue;
                }
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
                if (emb && I != 0 && I != nx - 1 && J != 0 && J != ny - 2) {
                    scaled_v(i, I, J);
                    continue;
                }
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
    if (emb) {
        // the embedded matrices as the reference leaves them after its per-step sort: rows
        // and columns ascending, and as many entries as it sized them (the plain operator's
        // plus one per hybrid node); the positions its kernels leave unwritten hold zero
        // entries at (0, 0), which sort first
        std::vector<size_t> order(row.size());
        for (size_t k = 0; k < order.size(); ++k) order[k] = k;
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
            return row[a] != row[b] ? row[a] < row[b] : col[a] < col[b];
        });
        const size_t plain = which == 1 ? (size_t)(nx - 1) * ny * 5 - 2 * ny - 2 * (nx - 1) + (size_t)nx * (ny - 1) * 5 -
                                              2 * nx - 2 * (ny - 1)
                                        : (size_t)nx * ny * 5 - 2 * nx - 2 * ny;
        const size_t want = plain + embedded_hybrid_count(c, which);
        const size_t pad = want > row.size() ? want - row.size() : 0;
        std::vector<int> r2(pad, 0), c2(pad, 0);
        std::vector<double> v2(pad, 0.0);
        for (size_t k : order) {
            r2.push_back(row[k]);
            c2.push_back(col[k]);
            v2.push_back(val[k]);
        }
        row.swap(r2);
        col.swap(c2);
        val.swap(v2);
    }
}

// CSR of the operator the solver iterates on (row weights w applied when given)
void host_operator_csr(Context &c, int which, const double *w, std::vector<int> &ptr, std::vector<int> &col,
                       std::vector<double> &val, bool body_free)
{
    std::vector<int> row;
    host_matrix_coo(c, which, row, col, val, body_free);
    const int n = which == 1 ? c.g.nUV : c.g.nP;
    ptr.assign(n + 1, 0);
    for (int r : row) ptr[r + 1]++;
    for (int i = 0; i < n; ++i) ptr[i + 1] += ptr[i];
    if (w)
        for (size_t k = 0; k < row.size(); ++k) val[k] *= w[row[k]];
}

static BcPtrs bc_ptrs(Context &c) { return BcPtrs{c.bc[XMINUS], c.bc[XPLUS], c.bc[YMINUS], c.bc[YPLUS]}; }

static EmbRhs1 emb_rhs1_args(Context &c)
{
    const auto &E = c.emb;
    if (!E.pid1) return EmbRhs1{};
    const IbPlan &P = ib_plan(c);
    return EmbRhs1{E.pid1, E.rscale1, E.pns1, E.pint1, E.cap1, E.gin, P.gvIdx, P.gvMask, P.gvW, c.ib.uB, c.ib.vB};
}

// shift = false: a later sub-iteration of a strongly coupled step, whose Nold is
// already the previous step's N (luoIBM/intermediateVelocity.cu:38 keeps Nold)
void launch_rhs1(Context &c, bool debug_terms, bool shift)
{
    int nb = blocks_for(c.g.nUV);
    const EmbRhs1 e = debug_terms ? EmbRhs1{} : emb_rhs1_args(c);
    if (debug_terms)
        k_rhs1<false, true><<<nb, kBlock, 0, c.stream>>>(c.rc, c.g, bc_ptrs(c), c.u, c.N, c.Nold, c.rhs1, c.L, c.bc1,
                                                         c.P.nu, c.P.dt, e);
    else if (shift)
        k_rhs1<true, false><<<nb, kBlock, 0, c.stream>>>(c.rc, c.g, bc_ptrs(c), c.u, c.N, c.Nold, c.rhs1, nullptr,
                                                         nullptr, c.P.nu, c.P.dt, e);
    else
        k_rhs1<false, false><<<nb, kBlock, 0, c.stream>>>(c.rc, c.g, bc_ptrs(c), c.u, c.N, c.Nold, c.rhs1, nullptr,
                                                          nullptr, c.P.nu, c.P.dt, e);
    CUIBM_TRY(cudaGetLastError());
}

void launch_rhs2(Context &c, const double *uh)
{
    const auto &E = c.emb;
    const EmbRhs2 e = E.pid2 ? EmbRhs2{E.pid2, E.pns2, E.pAu2, E.pAv2, c.ib.uB, c.ib.uBk, c.ib.vB, c.ib.vBk, c.P.dt}
                             : EmbRhs2{};
    k_rhs2<<<blocks_for(c.g.nP), kBlock, 0, c.stream>>>(c.g, bc_ptrs(c), c.rc.rdx, c.rc.rdy, uh, c.rhs2, e);
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
