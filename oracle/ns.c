/*
 * Navier-Stokes operators of the fractional step (oracle restatement; test
 * infrastructure only).  Association order follows the reference kernels so
 * that, with -ffp-contract=off, results are bit-identical to them.
 *
 * or_generateN        NavierStokes/kernels/N.cu (Nmidx, Nbcx, Nmidy, Nbcy)
 * or_generateL        NavierStokes/kernels/L.cu (Lmidx, Lbcx, Lmidy, Lbcy)
 * or_generateBC1      NavierStokes/kernels/intermediateVelocity.cu (bc1X, bc1Y)
 * or_generateRHS      NavierStokes/kernels/intermediateVelocity.cu (generateRHS)
 * or_lhs1_coo         NavierStokes/kernels/LHS1.cu (LHS_mid_X/Y_nobody, LHS_BC_X/Y)
 *                     (identical rows: luoIBM/kernels/LHS1.cu)
 * or_lhs2_coo         NavierStokes/kernels/LHS2.cu (LHS2_mid_nobody, LHS2_BC);
 *                     centre_pin=0 gives luoIBM/kernels/LHS2.cu (LHS2_mid_luo)
 * or_generateRHS2     NavierStokes/kernels/intermediatePressure.cu (intermediatePressureNoBody)
 *                     (identical: luoIBM/kernels/intermediatePressure.cu)
 * or_project          NavierStokes/kernels/projectVelocity.cu (identical: luo_base/kernels/projectVelocity.cu)
 * or_initialiseVelocity NavierStokes/kernels/initialise.cu
 * or_calculateCFL     NavierStokes/kernels/CFL.cu (calculateCFL)
 */
#include <math.h>
#include "oracle.h"

/* ---- convection ---------------------------------------------------------- */

/* x-direction part of u-convection at a u node (N.cu Nmidx), with the east/west
 * neighbour values substituted at the boundaries */
static inline double conv_ux(double uc, double ue, double uw, double a, double b)
{
    /* a = dx[I], b = dx[I+1] */
    return ue * a / (b * (a + b)) + uw * (a / (a * (a + b)) - 1 / a) +
           uc * (-a / (b * (a + b)) - (a / (a * (a + b)) - 1 / a));
}

/* y-direction part of u-convection; dn replaces dy[J+1], ds replaces dy[J-1] */
static inline double conv_uy(double uc, double un, double us, double c, double dn, double ds)
{
    return un * c / (c * (dn + c)) + us * (ds / (c * (c + ds)) - 1 / c) +
           uc * (-c / (c * (dn + c)) - (ds / (c * (c + ds)) - 1 / c));
}

/* v interpolated to a u node from the four surrounding v values */
static inline double vbar_at_u(double vne, double vn, double vse, double vs, double a, double b)
{
    return ((vne - vn) * a / (a + b) + vn) / 2 + ((vse - vs) * a / (a + b) + vs) / 2;
}

/* x-direction part of v-convection (N.cu Nmidy); de replaces dx[I+1], dw replaces dx[I-1] */
static inline double conv_vx(double vc, double ve, double vw, double a, double de, double dw)
{
    return ve * a / (a * (a + de)) + vw * (dw / (a * (a + dw)) - 1 / a) +
           vc * (-a / (a * (a + de)) - (dw / (a * (a + dw)) - 1 / a));
}

/* y-direction part of v-convection: c = dy[J], d = dy[J+1] */
static inline double conv_vy(double vc, double vn, double vs, double c, double d)
{
    return vn * c / (d * (d + c)) + vs * (c / (c * (d + c)) - 1 / c) +
           vc * (-c / (d * (d + c)) - (c / (c * (d + c)) - 1 / c));
}

static inline double ubar_at_v(double une, double ue, double unw, double uw, double c, double d)
{
    return ((une - ue) * c / (c + d) + ue) / 2 + ((unw - uw) * c / (c + d) + uw) / 2;
}

void or_generateN(double *N, const double *u, const double *dx, const double *dy, const double *ym,
                  const double *yp, const double *xm, const double *xp, int nx, int ny)
{
    const int nU = (nx - 1) * ny;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nU; ++i) {
        int I = i % (nx - 1), J = i / (nx - 1), iv = nU + nx * J + I;
        double a = dx[I], b = dx[I + 1];
        double ue = (I == nx - 2) ? xp[J] : u[i + 1];
        double uw = (I == 0) ? xm[J] : u[i - 1];
        double tx = u[i] * conv_ux(u[i], ue, uw, a, b);
        double vbar, ty;
        if (J == ny - 1) {
            vbar = vbar_at_u(yp[(nx - 1) + I + 1], yp[(nx - 1) + I], u[iv - nx + 1], u[iv - nx], a, b);
            ty = vbar * conv_uy(u[i], 2 * yp[I] - u[i], u[i - nx + 1], dy[J], dy[J], dy[J - 1]);
        } else if (J == 0) {
            vbar = vbar_at_u(u[iv + 1], u[iv], ym[(nx - 1) + I + 1], ym[(nx - 1) + I], a, b);
            ty = vbar * conv_uy(u[i], u[i + nx - 1], 2 * ym[I] - u[i], dy[J], dy[J + 1], dy[J]);
        } else {
            vbar = vbar_at_u(u[iv + 1], u[iv], u[iv - nx + 1], u[iv - nx], a, b);
            ty = vbar * conv_uy(u[i], u[i + nx - 1], u[i - nx + 1], dy[J], dy[J + 1], dy[J - 1]);
        }
        /* interior nodes: one expression (Nmidx); edges accumulate from 0 (Nbcx) */
        if (I == 0 || I == nx - 2 || J == 0 || J == ny - 1)
            N[i] = (0 + tx) + ty;
        else
            N[i] = tx + ty;
    }
    const int nV = nx * (ny - 1);
#pragma omp parallel for schedule(static)
    for (int ip = 0; ip < nV; ++ip) {
        int I = ip % nx, J = ip / nx, iu = (nx - 1) * J + I, iv = ip + nU;
        double c = dy[J], d = dy[J + 1];
        double ubar, tx;
        if (I == nx - 1) {
            ubar = ubar_at_v(xp[J + 1], xp[J], u[iu + (nx - 1) - 1], u[iu - 1], c, d);
            tx = ubar * conv_vx(u[iv], 2 * xp[ny + J] - u[iv], u[iv - 1], dx[I], dx[I], dx[I - 1]);
        } else if (I == 0) {
            ubar = ubar_at_v(u[iu + (nx - 1)], u[iu], xm[J + 1], xm[J], c, d);
            tx = ubar * conv_vx(u[iv], u[iv + 1], 2 * xm[ny + J] - u[iv], dx[I], dx[I + 1], dx[I]);
        } else {
            ubar = ubar_at_v(u[iu + (nx - 1)], u[iu], u[iu + (nx - 1) - 1], u[iu - 1], c, d);
            tx = ubar * conv_vx(u[iv], u[iv + 1], u[iv - 1], dx[I], dx[I + 1], dx[I - 1]);
        }
        double vn = (J == ny - 2) ? yp[(nx - 1) + I] : u[iv + nx];
        double vs = (J == 0) ? ym[(nx - 1) + I] : u[iv - nx];
        double ty = u[iv] * conv_vy(u[iv], vn, vs, c, d);
        if (I == 0 || I == nx - 1 || J == 0 || J == ny - 2)
            N[iv] = (0 + tx) + ty;
        else
            N[iv] = tx + ty;
    }
}

/* ---- diffusion ----------------------------------------------------------- */

void or_generateL(double *L, const double *u, const double *dx, const double *dy, const double *ym,
                  const double *yp, const double *xm, const double *xp, int nx, int ny, double nu)
{
    const int nU = (nx - 1) * ny;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nU; ++i) {
        int I = i % (nx - 1), J = i / (nx - 1);
        if (I != 0 && I != nx - 2 && J != 0 && J != ny - 1) {
            L[i] = nu * ((u[i + 1] - u[i]) / (dx[I + 1] * (dx[I + 1] + dx[I]) * 0.5) +
                         (u[i - 1] - u[i]) / (dx[I] * (dx[I + 1] + dx[I]) * 0.5) +
                         (u[i + (nx - 1)] - u[i]) / (dy[J] * (dy[J + 1] + dy[J]) * 0.5) +
                         (u[i - (nx - 1)] - u[i]) / (dy[J] * (dy[J - 1] + dy[J]) * 0.5));
            continue;
        }
        double t = 0;
        t += nu * (((I != nx - 2) ? u[i + 1] : xp[J]) - u[i]) / (dx[I + 1] * (dx[I + 1] + dx[I]) * 0.5);
        t += nu * (((I != 0) ? u[i - 1] : xm[J]) - u[i]) / (dx[I] * (dx[I + 1] + dx[I]) * 0.5);
        if (J != ny - 1)
            t += nu * (u[i + (nx - 1)] - u[i]) / (dy[J] * (dy[J + 1] + dy[J]) * 0.5);
        else
            t += nu * (2 * yp[I] - 2 * u[i]) / (dy[J] * dy[J]);
        if (J != 0)
            t += nu * (u[i - (nx - 1)] - u[i]) / (dy[J] * (dy[J - 1] + dy[J]) * 0.5);
        else
            t += nu * (2 * ym[I] - 2 * u[i]) / (dy[J] * dy[J]);
        L[i] = t;
    }
    const int nV = nx * (ny - 1);
#pragma omp parallel for schedule(static)
    for (int ip = 0; ip < nV; ++ip) {
        int I = ip % nx, J = ip / nx, iv = ip + nU;
        if (I != 0 && I != nx - 1 && J != 0 && J != ny - 2) {
            L[iv] = nu * ((u[iv + 1] - u[iv]) / (dx[I] * (dx[I] + dx[I + 1]) * 0.5) +
                          (u[iv - 1] - u[iv]) / (dx[I] * (dx[I] + dx[I - 1]) * 0.5) +
                          (u[iv + nx] - u[iv]) / (dy[J + 1] * (dy[J] + dy[J + 1]) * 0.5) +
                          (u[iv - nx] - u[iv]) / (dy[J] * (dy[J] + dy[J + 1]) * 0.5));
            continue;
        }
        double t = 0;
        if (I != nx - 1)
            t += nu * (u[iv + 1] - u[iv]) / (dx[I] * (dx[I] + dx[I + 1]) * 0.5);
        else
            t += nu * (2 * xp[ny + J] - 2 * u[iv]) / (dx[I] * dx[I]);
        if (I != 0)
            t += nu * (u[iv - 1] - u[iv]) / (dx[I] * (dx[I] + dx[I - 1]) * 0.5);
        else
            t += nu * (2 * xm[ny + J] - 2 * u[iv]) / (dx[I] * dx[I]);
        t += nu * (((J != ny - 2) ? u[iv + nx] : yp[nx - 1 + I]) - u[iv]) / (dy[J + 1] * (dy[J] + dy[J + 1]) * 0.5);
        t += nu * (((J != 0) ? u[iv - nx] : ym[nx - 1 + I]) - u[iv]) / (dy[J] * (dy[J] + dy[J + 1]) * 0.5);
        L[iv] = t;
    }
}

/* ---- boundary terms of the implicit half and the RHS sum ------------------ */

void or_generateBC1(const double *u, double *bc1, const double *ym, const double *yp, const double *xm,
                    const double *xp, const double *dx, const double *dy, double nu, double dt, int nx, int ny)
{
    const int nU = (nx - 1) * ny;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nU; ++i) {
        int I = i % (nx - 1), J = i / (nx - 1);
        double t = 0;
        if (I == nx - 2) t += xp[J] * 0.5 * dt * nu * (1 / (dx[I + 1] * (dx[I + 1] + dx[I]) * 0.5));
        if (I == 0) t += xm[J] * 0.5 * dt * nu * (1 / (dx[I] * (dx[I + 1] + dx[I]) * 0.5));
        if (J == ny - 1) t += (2 * yp[I] - u[i]) * nu * dt * 0.5 / dy[J] / dy[J];
        if (J == 0) t += (2 * ym[I] - u[i]) * nu * dt * 0.5 / dy[J] / dy[J];
        bc1[i] = t;
    }
    const int nV = nx * (ny - 1);
#pragma omp parallel for schedule(static)
    for (int ip = 0; ip < nV; ++ip) {
        int I = ip % nx, J = ip / nx, iv = ip + nU;
        double t = 0;
        if (I == nx - 1) t += (2 * xp[ny + J] - u[iv]) * nu * dt * 0.5 / dx[I] / dx[I];
        if (I == 0) t += (2 * xm[ny + J] - u[iv]) * nu * dt * 0.5 / dx[I] / dx[I];
        if (J == ny - 2) t += yp[(nx - 1) + I] * 0.5 * dt * nu * (1 / (dy[J + 1] * (dy[J] + dy[J + 1]) * 0.5));
        if (J == 0) t += ym[(nx - 1) + I] * 0.5 * dt * nu * (1 / (dy[J] * (dy[J] + dy[J + 1]) * 0.5));
        bc1[iv] = t;
    }
}

void or_generateRHS(double *rhs, const double *L, const double *Nold, const double *N, const double *u,
                    const double *bc1, double dt, int n)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) rhs[i] = u[i] + dt * (0.5 * Nold[i] - 1.5 * N[i] + 0.5 * L[i]) + bc1[i];
}

/* ---- LHS1 = I - 0.5 dt nu Laplacian, COO at the reference's entry offsets ---- */

/* Entry offset of the first entry of u-row (I,J); rows on the boundary have 4
 * entries (corners 3), interior rows 5 (LHS1.cu numE formulas). */
static int lhs_row_offset(int I, int J, int w, int h)
{
    if (J == 0) return I * 4 - (I != 0);
    if (J == h - 1) return w * 4 - 2 + (J - 1) * (5 * w - 2) + I * 4 - (I != 0);
    return w * 4 - 2 + (J - 1) * (5 * w - 2) + I * 5 - (I != 0);
}

void or_lhs1_coo(int *row, int *col, double *val, const double *dx, const double *dy, double dt, double nu,
                 int nx, int ny)
{
    const int nU = (nx - 1) * ny, w = nx - 1;
    const int offV = (nx - 1) * ny * 5 - 2 * ny - 2 * (nx - 1);
    for (int i = 0; i < nU; ++i) {
        int I = i % w, J = i / w, e = lhs_row_offset(I, J, w, ny);
        double t = 1, ce = 0.5 * dt * nu * (1 / (dx[I + 1] * (dx[I + 1] + dx[I]) * 0.5));
        double cw = 0.5 * dt * nu * (1 / (dx[I] * (dx[I + 1] + dx[I]) * 0.5));
        double cn = 0.5 * dt * nu * (1 / (dy[J] * (((J != ny - 1) ? dy[J + 1] : dy[J]) + dy[J]) * 0.5));
        double cs = 0.5 * dt * nu * (1 / (dy[J] * (((J != 0) ? dy[J - 1] : dy[J]) + dy[J]) * 0.5));
        if (I != nx - 2) { row[e] = i; col[e] = i + 1; val[e] = -ce; e++; }
        t += ce;
        if (I != 0) { row[e] = i; col[e] = i - 1; val[e] = -cw; e++; }
        t += cw;
        if (J != ny - 1) { row[e] = i; col[e] = i + w; val[e] = -cn; e++; }
        t += cn;
        if (J != 0) { row[e] = i; col[e] = i - w; val[e] = -cs; e++; }
        t += cs;
        row[e] = i; col[e] = i; val[e] = t;
    }
    const int nV = nx * (ny - 1);
    for (int ip = 0; ip < nV; ++ip) {
        int I = ip % nx, J = ip / nx, i = ip + nU, e = offV + lhs_row_offset(I, J, nx, ny - 1);
        double t = 1;
        double ce = 0.5 * dt * nu * (1 / (dx[I] * (dx[I] + ((I != nx - 1) ? dx[I + 1] : dx[I])) * 0.5));
        double cw = 0.5 * dt * nu * (1 / (dx[I] * (dx[I] + ((I != 0) ? dx[I - 1] : dx[I])) * 0.5));
        double cn = 0.5 * dt * nu * (1 / (dy[J + 1] * (dy[J] + dy[J + 1]) * 0.5));
        double cs = 0.5 * dt * nu * (1 / (dy[J] * (dy[J] + dy[J + 1]) * 0.5));
        if (I != nx - 1) { row[e] = i; col[e] = i + 1; val[e] = -ce; e++; }
        t += ce;
        if (I != 0) { row[e] = i; col[e] = i - 1; val[e] = -cw; e++; }
        t += cw;
        if (J != ny - 2) { row[e] = i; col[e] = i + nx; val[e] = -cn; e++; }
        t += cn;
        if (J != 0) { row[e] = i; col[e] = i - nx; val[e] = -cs; e++; }
        t += cs;
        row[e] = i; col[e] = i; val[e] = t;
    }
}

/* ---- LHS2 = dt * D G (the "QTBNQ" operator) ------------------------------ */
void or_lhs2_coo(int centre_pin, int *row, int *col, double *val, const double *dx, const double *dy, int nx,
                 int ny, double dt)
{
    for (int ip = 0; ip < nx * ny; ++ip) {
        int I = ip % nx, J = ip / nx, e = lhs_row_offset(I, J, nx, ny);
        double t = 0, c;
        if (I != nx - 1) {
            c = dt / (dx[I] * (dx[I] + dx[I + 1]) * 0.5);
            row[e] = ip; col[e] = ip + 1; val[e] = -c; e++; t += c;
        }
        if (I != 0) {
            c = dt / (dx[I] * (dx[I] + dx[I - 1]) * 0.5);
            row[e] = ip; col[e] = ip - 1; val[e] = -c; e++; t += c;
        }
        if (J != ny - 1) {
            c = dt / (dy[J] * (dy[J] + dy[J + 1]) * 0.5);
            row[e] = ip; col[e] = ip + nx; val[e] = -c; e++; t += c;
        }
        if (J != 0) {
            c = dt / (dy[J] * (dy[J] + dy[J - 1]) * 0.5);
            row[e] = ip; col[e] = ip - nx; val[e] = -c; e++; t += c;
        }
        row[e] = ip; col[e] = ip; val[e] = t;
        /* pins that make the singular Neumann operator invertible: the diagonal
         * is doubled at ip = 0 (LHS2_BC) and, for the plain solver, at the
         * centre cell (LHS2_mid_nobody) */
        if (ip == 0) val[e] += val[e];
        if (centre_pin && ip == (ny / 2) * nx + nx / 2 && !(I == 0 || I == nx - 1 || J == 0 || J == ny - 1))
            val[e] += val[e];
    }
}

/* ---- rhs2 = -D uhat ------------------------------------------------------- */
void or_generateRHS2(double *rhs2, const double *uhat, const double *ym, const double *yp, const double *xm,
                     const double *xp, const double *dx, const double *dy, int nx, int ny)
{
    const int nU = (nx - 1) * ny;
#pragma omp parallel for schedule(static)
    for (int ip = 0; ip < nx * ny; ++ip) {
        int I = ip % nx, J = ip / nx, iu = (nx - 1) * J + I, iv = nU + nx * J + I;
        double t = 0;
        t -= ((I != nx - 1) ? uhat[iu] : xp[J]) / dx[I];
        t += ((I != 0) ? uhat[iu - 1] : xm[J]) / dx[I];
        t -= ((J != ny - 1) ? uhat[iv] : yp[(nx - 1) + I]) / dy[J];
        t += ((J != 0) ? uhat[iv - nx] : ym[(nx - 1) + I]) / dy[J];
        rhs2[ip] = t;
    }
}

/* ---- projection u = uhat - dt G p ----------------------------------------- */
void or_project(double *u, const double *uhat, double *uold, const double *p, const double *dx,
                const double *dy, double dt, int nx, int ny)
{
    const int nU = (nx - 1) * ny, nV = nx * (ny - 1);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nU; ++i) {
        int I = i % (nx - 1), J = i / (nx - 1), ip = J * nx + I;
        uold[i] = u[i];
        u[i] = uhat[i] - dt * (p[ip + 1] - p[ip]) / (0.5 * dx[I + 1] + 0.5 * dx[I]);
    }
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nV; ++k) {
        int J = k / nx, ip = k, i = k + nU;
        uold[i] = u[i];
        u[i] = uhat[i] - dt * (p[ip + nx] - p[ip]) / (0.5 * dy[J + 1] + 0.5 * dy[J]);
    }
}

void or_initialiseVelocity(double *u, const double *xu, const double *yu, const double *xv, const double *yv,
                           double uI, double vI, double uP, double vP, double xmax, double xmin, double ymax,
                           double ymin, int nx, int ny)
{
    const int nU = (nx - 1) * ny, nV = nx * (ny - 1);
    const double pi = M_PI;
    for (int k = 0; k < nU; ++k) {
        int i = k % (nx - 1), j = k / (nx - 1);
        u[k] = uI + uP * cos(0.5 * pi * (2 * xu[i] - xmax - xmin) / (xmax - xmin)) *
                        sin(pi * (2 * yu[j] - ymax - ymin) / (ymax - ymin));
    }
    for (int k = 0; k < nV; ++k) {
        int i = k % nx, j = k / nx;
        u[nU + k] = vI + vP * cos(0.5 * pi * (2 * yv[j] - ymax - ymin) / (ymax - ymin)) *
                             sin(pi * (2 * xv[i] - xmax - xmin) / (xmax - xmin));
    }
}

void or_calculateCFL(double *cfl, const double *u, const double *dx, const double *dy, int nx, int ny,
                     double dt)
{
    const int nU = (nx - 1) * ny;
    for (int ip = 0; ip < nx * ny; ++ip) {
        int I = ip % nx, J = ip / nx, iu = (nx - 1) * J + I, iv = nU + nx * J + I;
        if (I == nx - 1 || J == ny - 1) continue;
        cfl[ip] = dt * (fabs(u[iu]) / dx[I] + fabs(u[iv]) / dy[J]);
    }
}
