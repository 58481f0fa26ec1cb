/*
 * The modified-Fadlun immersed-boundary method on the CPU (TEST INFRASTRUCTURE).
 *
 * Restates FadlunModified/kernels/LHS1.cu (LHS_mid_X, LHS_mid_Y),
 * FadlunModified/kernels/LHS2.cu (LHS2_mid), FadlunModified/kernels/
 * intermediateVelocity.cu (updateRHS1forIBX/Y), FadlunModified/kernels/
 * intermediatePressure.cu (intermediatePressure) and FadlunModified/kernels/
 * projectVelocity.cu (project_velocity_X/Y), as fadlunModified.cu launches them.
 *
 * Matrices are produced as the reference leaves them before its
 * sort_by_row_and_column: COO arrays value-initialised to zero (a resized
 * cusp::coo_matrix), boundary rows from the plain operator (LHS_BC_X/Y,
 * LHS2_BC), interior rows from the Fadlun kernels at the reference's entry
 * offsets.  Entries a Fadlun row does not write stay (0, 0, 0.0); entries it
 * writes with a zero value keep their (sometimes odd) column, e.g. the
 * 1 + nx of LHS_mid_Y.  Tagged rows:
 *   hybrid velocity node  u_i - d/(d+b) u_away = (b/(d+b)) uv_i    (rhs1 update)
 *   ghost velocity node   u_i - c u_across = 0                      (rhs1 update)
 * where "away"/"across" is chosen from the hybrid tags as in the reference.
 */
#include <math.h>
#include <string.h>

#include "oracle.h"

/* first entry of interior row (I, J) of a block of width w (LHS1.cu / LHS2.cu numE) */
static int mid_offset(int I, int J, int w) { return w * 4 - 2 + (J - 1) * (5 * w - 2) + I * 5 - 1; }

static void put(int *row, int *col, double *val, int e, int r, int c, double v)
{
    row[e] = r;
    col[e] = c;
    val[e] = v;
}

/* one interior velocity row of LHS_mid_X (dir 0) or LHS_mid_Y (dir 1).
 * i: row index, s: the row stride of the block (nx-1 for u, nx for v),
 * the plain coefficients ce, cw, cn, cs as the reference computes them */
static void fadlun_velocity_row(int dir, int *row, int *col, double *val, int e, int i, int s, double ce, double cw,
                                double cn, double cs, const int *hyb, const int *hyb2, const int *ghost,
                                const double *dn, const double *db, double dxI)
{
    const int tagged = dir == 0 ? hyb[i] != -1 : hyb[i] > 0;
    const int inner = dir == 0 ? ghost[i] > 0 : ghost[i] != -1;
    /* the zero entries' third column: i + s and i - s, written 1 + nx / 1 - nx by LHS_mid_Y */
    const int up = dir == 0 ? i + s : 1 + s, down = dir == 0 ? i - s : 1 - s;
    if ((hyb[i] == -1 && ghost[i] == -1) || ghost[i] == 0) {
        double t = 1;
        put(row, col, val, e++, i, i + 1, -ce); t += ce;
        put(row, col, val, e++, i, i - 1, -cw); t += cw;
        put(row, col, val, e++, i, i + s, -cn); t += cn;
        put(row, col, val, e++, i, i - s, -cs); t += cs;
        put(row, col, val, e, i, i, t);
        return;
    }
    if (tagged) {
        int far = 0;  /* column of the interpolation partner; 0 (zero-initialised) when no branch matches */
        if (hyb[i] == hyb2[i] - 1) {
            put(row, col, val, e++, i, i - 1, 0); put(row, col, val, e++, i, i - s, 0);
            put(row, col, val, e++, i, up, 0); far = i + 1;
        } else if (hyb[i] == hyb2[i] + 1) {
            put(row, col, val, e++, i, i + 1, 0); put(row, col, val, e++, i, i - s, 0);
            put(row, col, val, e++, i, up, 0); far = i - 1;
        } else if (hyb[i] == hyb2[i] + s) {
            put(row, col, val, e++, i, i - 1, 0); put(row, col, val, e++, i, i + 1, 0);
            put(row, col, val, e++, i, up, 0); far = i - s;
        } else if (hyb[i] == hyb2[i] - s) {
            put(row, col, val, e++, i, i - 1, 0); put(row, col, val, e++, i, i + 1, 0);
            put(row, col, val, e++, i, down, 0); far = i + s;
        }
        col[e] = far;
        row[e] = i;
        val[e] = dir == 0 ? -dn[i] / (dn[i] + db[i]) : -dn[i] / (db[i] + dn[i]);
        e++;
        put(row, col, val, e, i, i, 1);
        return;
    }
    if (inner) {
        int nb = -1, far = 0;
        if (hyb[i + 1] != -1) {
            put(row, col, val, e++, i, i + 1, 0); put(row, col, val, e++, i, i - s, 0);
            put(row, col, val, e++, i, up, 0); far = i - 1; nb = i + 1;
        } else if (hyb[i - 1] != -1) {
            put(row, col, val, e++, i, i - 1, 0); put(row, col, val, e++, i, i - s, 0);
            put(row, col, val, e++, i, up, 0); far = i + 1; nb = i - 1;
        } else if (hyb[i + s] != -1) {
            put(row, col, val, e++, i, i - 1, 0); put(row, col, val, e++, i, i + 1, 0);
            put(row, col, val, e++, i, up, 0); far = i - s; nb = i + s;
        } else if (hyb[i - s] != -1) {
            put(row, col, val, e++, i, i - 1, 0); put(row, col, val, e++, i, i + 1, 0);
            put(row, col, val, e++, i, down, 0); far = i + s; nb = i - s;
        }
        if (nb >= 0) {
            col[e] = far;
            val[e] = -(dxI - dn[nb]) / (dxI - dn[nb] + db[nb]);
        }
        row[e] = i;
        e++;
        put(row, col, val, e, i, i, 1);
    }
}

/* fadlunModified::generateLHS1 (nnz = the plain operator's, whose boundary rows it keeps) */
void or_fadlun_lhs1_coo(int *row, int *col, double *val, int nnz, const int *hyb, const int *hyb2, const int *ghost,
                        const double *dn, const double *db, const double *dx, const double *dy, double dt,
                        double nu, int nx, int ny)
{
    or_lhs1_coo(row, col, val, dx, dy, dt, nu, nx, ny);  /* boundary rows */
    const int nU = (nx - 1) * ny, w = nx - 1;
    const int offV = (nx - 1) * ny * 5 - 2 * ny - 2 * (nx - 1);
    /* clear the interior rows' entries: the Fadlun kernels write them on zeroed arrays */
    for (int i = 0; i < nU; ++i) {
        int I = i % w, J = i / w;
        if (I == 0 || I == nx - 2 || J == 0 || J == ny - 1) continue;
        int e = mid_offset(I, J, w);
        for (int k = 0; k < 5; ++k) put(row, col, val, e + k, 0, 0, 0);
    }
    for (int ip = 0; ip < nx * (ny - 1); ++ip) {
        int I = ip % nx, J = ip / nx;
        if (I == 0 || I == nx - 1 || J == 0 || J == ny - 2) continue;
        int e = offV + mid_offset(I, J, nx);
        for (int k = 0; k < 5; ++k) put(row, col, val, e + k, 0, 0, 0);
    }
    (void)nnz;
    for (int i = 0; i < nU; ++i) {
        int I = i % w, J = i / w;
        if (I == 0 || I == nx - 2 || J == 0 || J == ny - 1) continue;
        double ce = 0.5 * dt * nu * (1 / (dx[I + 1] * (dx[I + 1] + dx[I]) * 0.5));
        double cw = 0.5 * dt * nu * (1 / (dx[I] * (dx[I + 1] + dx[I]) * 0.5));
        double cn = 0.5 * dt * nu * (1 / (dy[J] * (dy[J + 1] + dy[J]) * 0.5));
        double cs = 0.5 * dt * nu * (1 / (dy[J] * (dy[J - 1] + dy[J]) * 0.5));
        fadlun_velocity_row(0, row, col, val, mid_offset(I, J, w), i, w, ce, cw, cn, cs, hyb, hyb2, ghost, dn, db,
                            dx[I]);
    }
    for (int ip = 0; ip < nx * (ny - 1); ++ip) {
        int I = ip % nx, J = ip / nx, i = ip + nU;
        if (I == 0 || I == nx - 1 || J == 0 || J == ny - 2) continue;
        double ce = 0.5 * dt * nu * (1 / (dx[I] * (dx[I] + dx[I + 1]) * 0.5));
        double cw = 0.5 * dt * nu * (1 / (dx[I] * (dx[I] + dx[I - 1]) * 0.5));
        double cn = 0.5 * dt * nu * (1 / (dy[J + 1] * (dy[J] + dy[J + 1]) * 0.5));
        double cs = 0.5 * dt * nu * (1 / (dy[J] * (dy[J] + dy[J + 1]) * 0.5));
        fadlun_velocity_row(1, row, col, val, offV + mid_offset(I, J, nx), i, nx, ce, cw, cn, cs, hyb, hyb2,
                            ghost, dn, db, dx[I]);
    }
}

/* fadlunModified::generateLHS2: values zeroed, LHS2_mid (Fadlun) on interior rows,
 * the plain operator's boundary rows (LHS2_BC, with its pin at cell 0) */
void or_fadlun_lhs2_coo(int *row, int *col, double *val, const double *du, const double *dv, const int *ghostP,
                        const int *hybP, const double *dx, const double *dy, int nx, int ny, double dt)
{
    or_lhs2_coo(0, row, col, val, dx, dy, nx, ny, dt);  /* boundary rows */
    for (int ip = 0; ip < nx * ny; ++ip) {
        const int I = ip % nx, J = ip / nx;
        if (I == 0 || I == nx - 1 || J == 0 || J == ny - 1) continue;
        int e = mid_offset(I, J, nx);
        double t = 0;
        const int nb[4] = {ip + 1, ip - 1, ip + nx, ip - nx};
        if (hybP[ip] != -1) {
            for (int k = 0; k < 4; ++k) {
                const double d = k < 2 ? du[ip] : dv[ip], h = k < 2 ? dx[I] : dy[J];
                if (ghostP[nb[k]] == -1) {
                    if (d > h / 2 && d < h) {
                        put(row, col, val, e, ip, nb[k], -dt / h / d);
                        t += dt / h / d;
                    } else {
                        put(row, col, val, e, ip, nb[k], -dt / h / h);
                        t += dt / h / h;
                    }
                } else {
                    put(row, col, val, e, ip, nb[k], 0);
                }
                e++;
            }
        } else if (ghostP[ip] > 0) {
            for (int k = 0; k < 4; ++k) {
                const double h = k < 2 ? dx[I] : dy[J];
                if (ghostP[nb[k]] == 0) {
                    put(row, col, val, e, ip, nb[k], -dt / h / h);
                    t += dt / h / h;
                } else {
                    put(row, col, val, e, ip, nb[k], 0);
                }
                e++;
            }
        } else {
            double c;
            c = dt / (dx[I] * (dx[I] + dx[I + 1]) * 0.5);
            put(row, col, val, e++, ip, ip + 1, -c); t += c;
            c = dt / (dx[I] * (dx[I] + dx[I - 1]) * 0.5);
            put(row, col, val, e++, ip, ip - 1, -c); t += c;
            c = dt / (dy[J] * (dy[J] + dy[J + 1]) * 0.5);
            put(row, col, val, e++, ip, ip + nx, -c); t += c;
            c = dt / (dy[J] * (dy[J] + dy[J - 1]) * 0.5);
            put(row, col, val, e++, ip, ip - nx, -c); t += c;
        }
        put(row, col, val, e, ip, ip, t);
        /* the centre pin of LHS2_mid (as the plain solver's) */
        if (ip == (ny / 2) * nx + nx / 2) val[e] += val[e];
    }
}

/* updateRHS1forIBX/Y: hybrid rows get their body term, ghost rows 0 */
void or_fadlun_update_rhs1(const int *hyb, const int *ghost, double *rhs, const double *dn, const double *db,
                           const double *uv, int nx, int ny)
{
    const int nUV = (nx - 1) * ny + nx * (ny - 1);
    for (int i = 0; i < nUV; ++i)
        rhs[i] = (hyb[i] == -1) * (ghost[i] <= 0) * (rhs[i]) + (hyb[i] != -1) * db[i] / (dn[i] + db[i]) * uv[i];
}

/* FadlunModified/kernels/intermediatePressure.cu intermediatePressure */
void or_fadlun_rhs2(double *rhs2, const double *uhat, const int *ghostP, const int *hybP, const double *du,
                    const double *dv, const double *ym, const double *yp, const double *xm, const double *xp,
                    const double *dx, const double *dy, int nx, int ny)
{
    for (int ip = 0; ip < nx * ny; ++ip) {
        const int I = ip % nx, J = ip / nx, iu = (nx - 1) * J + I, iv = (nx - 1) * ny + nx * J + I;
        double t = 0;
        if (hybP[ip] != -1) {
            /* next to the body on the fluid side: faces toward fluid nodes, the
             * face distance shortened where the body cuts the cell */
            const int near_u = du[ip] > dx[I] / 2 && du[ip] < dx[I];
            const int near_v = dv[ip] > dy[J] / 2 && dv[ip] < dy[J];
            if (ghostP[ip + 1] == -1) t -= uhat[iu] / (near_u ? du[ip] : dx[I]);
            if (ghostP[ip - 1] == -1) t += uhat[iu - 1] / (near_u ? du[ip] : dx[I]);
            if (ghostP[ip + nx] == -1) t -= uhat[iv] / (near_v ? dv[ip] : dy[J]);
            if (ghostP[ip - nx] == -1) t += uhat[iv - nx] / (near_v ? dv[ip] : dy[J]);
        } else if (ghostP[ip] > 0) {
            /* just inside: faces toward interior nodes only */
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
}

/* FadlunModified/kernels/projectVelocity.cu: no pressure gradient across a face
 * that touches a tagged pressure node */
void or_fadlun_project(double *u, const double *uhat, const double *p, const int *ghostP, const double *dx,
                       const double *dy, double dt, int nx, int ny)
{
    const int nU = (nx - 1) * ny, nV = nx * (ny - 1);
    for (int i = 0; i < nU; ++i) {
        const int I = i % (nx - 1), J = i / (nx - 1), ip = J * nx + I;
        u[i] = uhat[i] - (ghostP[ip + 1] == -1 && ghostP[ip] == -1) * dt * (p[ip + 1] - p[ip]) /
                             (0.5 * dx[I + 1] + 0.5 * dx[I]);
    }
    for (int k = 0; k < nV; ++k) {
        const int I = k % nx, J = k / nx, ip = J * nx + I, i = k + nU;
        u[i] = uhat[i] - (ghostP[ip + nx] == -1 && ghostP[ip] == -1) * dt * (p[ip + nx] - p[ip]) /
                             (0.5 * dy[J + 1] + 0.5 * dy[J]);
    }
}
