/*
 * The embedded ghost-node method (SolverType OSC_CYLINDER, the reference's luo_iter)
 * on the CPU (TEST INFRASTRUCTURE).
 *
 * Restates luo_iter/kernels/weight.cu (alpha_u, alpha_v, alpha_p),
 * luo_iter/kernels/intermediateVelocity.cu (size_LHS1, update_rhs1_x/y),
 * luo_iter/kernels/LHS1.cu (LHS1_mid_iter_X/Y), luo_iter/kernels/pressure.cu
 * (size_LHS2, update_rhs2) and luo_iter/kernels/LHS2.cu (LHS2_mid_iter), as
 * luo_iter/intermediateVelocity.cu and luo_iter/poisson.cu launch them.
 *
 * Each step the operators are rebuilt from the current tags and the current
 * interpolation stencils (index, coefficient and corner value of the
 * luo_base bilinear fits):
 *   plain interior rows   the momentum row divided by its diagonal (LHS1;
 *                         rhs1 scaled by 1/diagonal), the plain row (LHS2);
 *   hybrid rows           (1 - alpha) (the row over its diagonal) + alpha (the
 *                         interpolation row); interpolation corners at the four
 *                         diagonal neighbours get one extra entry (the last such
 *                         corner), corners elsewhere are dropped;
 *   ghost rows            node + interpolation = 2 u_body (LHS1) or
 *                         node - interpolation = dp/dn (LHS2), the corners that
 *                         are ghost nodes or the node itself moved to the rhs.
 * Matrices are built as the reference builds them on zero-initialised arrays:
 * the extra entries after the plain operator's nnz, at the hybrid node's rank in
 * the box scan.  (The reference reuses its previous step's sorted COO arrays
 * without clearing the LHS1 values; entries a step does not write then keep
 * stale values of the previous sorted matrix.  That artefact is not reproduced:
 * every step here starts from zero, which is the reference's first step.)
 */
#include <math.h>
#include <string.h>

#include "oracle.h"

static int mid_offset(int I, int J, int w) { return w * 4 - 2 + (J - 1) * (5 * w - 2) + I * 5 - 1; }

static void put(int *row, int *col, double *val, int e, int r, int c, double v)
{
    row[e] = r;
    col[e] = c;
    val[e] = v;
}

/* alpha_u (kind 0), alpha_v (1), alpha_p (2) over the threads whose node lies in the grid */
void or_iter_alpha(int kind, double *alpha, const int *ghost, const int *hybrid, const double *yc, const double *xc,
                   const double *bix, const double *biy, int i_start, int j_start, int width, int nx, int ny)
{
    const int nU = (nx - 1) * ny;
    const int nthreads = kind == 2 ? nx * ny : nU; /* the reference's launch grids */
    const int ngrid = ((int)((nthreads - 0.5) / 256) + 1) * 256;
    for (int idx = 0; idx < ngrid; ++idx) {
        const int I = i_start + idx % width, J = j_start + idx / width;
        int n, sv;
        if (kind == 0) {
            if (J >= ny || I >= nx - 1) continue;
            n = J * (nx - 1) + I;
            sv = nx - 1;
        } else if (kind == 1) {
            if (J * nx + I > nx * (ny - 1) || J >= ny - 1) continue;
            n = J * nx + I + nU;
            sv = nx;
        } else {
            if (J * nx + I > nx * ny || J >= ny) continue;
            n = J * nx + I;
            sv = nx;
        }
        if (hybrid[n] <= 0) continue;
        double d1 = 0, d2 = 0;
        const double dx = xc[I] - xc[I - 1], dy = yc[J] - yc[J - 1];
        if (ghost[n - 1] > 0)
            d1 = sqrt(pow(bix[n - 1] - xc[I - 1], 2) + pow(biy[n - 1] - yc[J], 2));
        else if (ghost[n + 1] > 0)
            d1 = sqrt(pow(bix[n + 1] - xc[I + 1], 2) + pow(biy[n + 1] - yc[J], 2));
        if (ghost[n - sv] > 0) d2 = sqrt(pow(bix[n - sv] - xc[I], 2) + pow(biy[n - sv] - yc[J - 1], 2));
        if (ghost[n + sv] > 0) d2 = sqrt(pow(bix[n + sv] - xc[I], 2) + pow(biy[n + sv] - yc[J + 1], 2));
        alpha[n] = sqrt(pow(d1 / dx, 2) + pow(d2 / dy, 2));
    }
}

/* size_LHS1 / size_LHS2: rank of each hybrid node in the box scan (u rows, then v rows) */
static int box_ranks(const int *hyb, int *count, int i_start, int j_start, int width, int height, int nx, int ny,
                     int velocity)
{
    int counter = 0;
    for (int pass = 0; pass < (velocity ? 2 : 1); ++pass)
        for (int j = j_start; j < j_start + height; ++j)
            for (int i = i_start; i < i_start + width; ++i) {
                const int n = velocity ? (pass == 0 ? j * (nx - 1) + i : j * nx + i + (nx - 1) * ny) : j * nx + i;
                if (hyb[n] > 0) count[n] = ++counter;
            }
    return counter;
}

/* one interior row of LHS1_mid_iter_X/Y (s: stride of the block) */
static void iter_velocity_row(int *row, int *col, double *val, int e, int extra_base, int i, int s, double cn,
                              double ce, double cs, double cw, double temp_plain, const double plain[4],
                              const int *hyb, const int *ghost, double *ns_rhs, double *interp_rhs,
                              const int *count, const int idx[4], const double coef[4], const double q[4],
                              double alpha, double ubody)
{
    if (hyb[i] > 0) {
        double Cns[5] = {cn, ce, cs, cw, 0}, CI[4];
        Cns[4] = 1 - Cns[0] - Cns[1] - Cns[2] - Cns[3];
        for (int l = 0; l < 4; ++l) {
            Cns[l] = Cns[l] * (1 - alpha) / Cns[4];
            CI[l] = coef[l] * alpha;
        }
        const int st[9] = {i + s - 1, i + s, i + s + 1, i - 1, i, i + 1, i - s - 1, i - s, i - s + 1};
        double sv[9] = {0, Cns[0], 0, Cns[3], 1, Cns[1], 0, Cns[2], 0};
        const int used[9] = {0, 1, 0, 1, 1, 1, 0, 1, 0};
        for (int n = 0; n < 4; ++n)
            for (int m = 0; m < 9; ++m)
                if (st[m] == idx[n] && m != 4) sv[m] -= CI[n];
        for (int m = 0; m < 9; ++m)
            if (used[m]) put(row, col, val, e++, i, st[m], sv[m]);
        ns_rhs[i] = (1 - alpha) / Cns[4];
        interp_rhs[i] = 0;
        const int x = extra_base + count[i] - 1;
        for (int n = 0; n < 4; ++n)
            for (int m = 0; m < 9; ++m) {
                if (st[m] == idx[n] && !used[m]) put(row, col, val, x, i, idx[n], -CI[n]);
                else if (st[m] == idx[n] && idx[n] == i) interp_rhs[i] += CI[n] * q[n];
            }
        return;
    }
    if (ghost[i] > 0) {
        const int ns[5] = {i + s, i + 1, i - s, i - 1, i};
        int overlap[5] = {0, 0, 0, 0, 1}, in[4] = {0, 0, 0, 0}, counter = 0;
        double temp = 0;
        for (int l = 0; l < 4; ++l) {
            if (ghost[idx[l]] > 0) {
                counter += 1;
                in[l] = 1;
            }
            for (int n = 0; n < 5; ++n)
                if (idx[l] == ns[n]) overlap[n] = 1;
        }
        put(row, col, val, e++, i, i, 1);
        for (int l = 0; l < 4; ++l) {
            if (!in[l] && idx[l] != i) put(row, col, val, e++, i, idx[l], coef[l]);
            else temp -= coef[l] * q[l];
        }
        int c2 = 0;
        for (int n = 0; n < 5; ++n) {
            if (c2 >= counter) break;
            if (!overlap[n]) {
                put(row, col, val, e++, i, ns[n], 0);
                c2++;
            }
        }
        ns_rhs[i] = 0;
        interp_rhs[i] = 2 * ubody + temp;
        return;
    }
    put(row, col, val, e++, i, i + 1, plain[0] / temp_plain);
    put(row, col, val, e++, i, i - 1, plain[1] / temp_plain);
    put(row, col, val, e++, i, i + s, plain[2] / temp_plain);
    put(row, col, val, e++, i, i - s, plain[3] / temp_plain);
    put(row, col, val, e, i, i, 1);
    ns_rhs[i] = 1 / temp_plain;
    interp_rhs[i] = 0;
}

/* luo_iter::intermediate_velocity_size_lhs + intermediate_velocity_calculate_lhs on zeroed
 * arrays of nnz = the plain operator's + the number of hybrid nodes.  idx/coef/q: the four
 * corners of each node's fit (index1..4, q1coef..4, q1..4). */
int or_iter_lhs1(int *row, int *col, double *val, int nnz, const double *dx, const double *dy, double dt, double nu,
                 int nx, int ny, const int *hyb, const int *ghost, double *ns_rhs, double *interp_rhs, int *count,
                 const int *i1, const int *i2, const int *i3, const int *i4, const double *alpha, double uB0,
                 double vB0, const double *c1, const double *c2, const double *c3, const double *c4,
                 const double *q1, const double *q2, const double *q3, const double *q4, int i_start, int j_start,
                 int width, int height)
{
    const int nU = (nx - 1) * ny, w = nx - 1;
    const int base = (nx - 1) * ny * 5 - 2 * ny - 2 * (nx - 1) + nx * (ny - 1) * 5 - 2 * nx - 2 * (ny - 1);
    const int offV = (nx - 1) * ny * 5 - 2 * ny - 2 * (nx - 1);
    const int nh = box_ranks(hyb, count, i_start, j_start, width, height, nx, ny, 1);
    if (base + nh > nnz) return -1;
    or_lhs1_coo(row, col, val, dx, dy, dt, nu, nx, ny); /* boundary rows (LHS_BC_X/Y) */
    for (int k = base; k < nnz; ++k) put(row, col, val, k, 0, 0, 0);
    for (int i = 0; i < nU; ++i) {
        const int I = i % w, J = i / w;
        if (I == 0 || I == nx - 2 || J == 0 || J == ny - 1) continue;
        const int e = mid_offset(I, J, w);
        for (int k = 0; k < 5; ++k) put(row, col, val, e + k, 0, 0, 0);
        const double pe = -0.5 * dt * nu * (1 / (dx[I + 1] * (dx[I + 1] + dx[I]) * 0.5));
        const double pw = -0.5 * dt * nu * (1 / (dx[I] * (dx[I + 1] + dx[I]) * 0.5));
        const double pn = -0.5 * dt * nu * (1 / (dy[J] * (dy[J + 1] + dy[J]) * 0.5));
        const double ps = -0.5 * dt * nu * (1 / (dy[J] * (dy[J - 1] + dy[J]) * 0.5));
        const double temp = 1 + 0.5 * dt * nu * (1 / (dx[I + 1] * (dx[I + 1] + dx[I]) * 0.5)) +
                            0.5 * dt * nu * (1 / (dx[I] * (dx[I + 1] + dx[I]) * 0.5)) +
                            0.5 * dt * nu * (1 / (dy[J] * (dy[J + 1] + dy[J]) * 0.5)) +
                            0.5 * dt * nu * (1 / (dy[J] * (dy[J - 1] + dy[J]) * 0.5));
        const double plain[4] = {pe, pw, pn, ps};
        const int idx[4] = {i1[i], i2[i], i3[i], i4[i]};
        const double coef[4] = {c1[i], c2[i], c3[i], c4[i]}, q[4] = {q1[i], q2[i], q3[i], q4[i]};
        iter_velocity_row(row, col, val, e, base, i, w, -dt * nu / (dy[J + 1] * (dy[J] + dy[J + 1])),
                          -dt * nu / (dx[I] * (dx[I] + dx[I + 1])), -dt * nu / (dy[J] * (dy[J] + dy[J + 1])),
                          -dt * nu / (dx[I] * (dx[I] + dx[I - 1])), temp, plain, hyb, ghost, ns_rhs, interp_rhs,
                          count, idx, coef, q, alpha[i], uB0);
    }
    for (int k = 0; k < nx * (ny - 1); ++k) {
        const int I = k % nx, J = k / nx, i = k + nU;
        if (I == 0 || I == nx - 1 || J == 0 || J == ny - 2) continue;
        const int e = offV + mid_offset(I, J, nx);
        for (int m = 0; m < 5; ++m) put(row, col, val, e + m, 0, 0, 0);
        const double pe = -0.5 * dt * nu * (1 / (dx[I] * (dx[I] + dx[I + 1]) * 0.5));
        const double pw = -0.5 * dt * nu * (1 / (dx[I] * (dx[I] + dx[I - 1]) * 0.5));
        const double pn = -0.5 * dt * nu * (1 / (dy[J + 1] * (dy[J] + dy[J + 1]) * 0.5));
        const double ps = -0.5 * dt * nu * (1 / (dy[J] * (dy[J] + dy[J + 1]) * 0.5));
        const double temp = 1 + 0.5 * dt * nu * (1 / (dx[I] * (dx[I] + dx[I + 1]) * 0.5)) +
                            0.5 * dt * nu * (1 / (dx[I] * (dx[I] + dx[I - 1]) * 0.5)) +
                            0.5 * dt * nu * (1 / (dy[J + 1] * (dy[J] + dy[J + 1]) * 0.5)) +
                            0.5 * dt * nu * (1 / (dy[J] * (dy[J] + dy[J + 1]) * 0.5));
        const double plain[4] = {pe, pw, pn, ps};
        const int idx[4] = {i1[i], i2[i], i3[i], i4[i]};
        const double coef[4] = {c1[i], c2[i], c3[i], c4[i]}, q[4] = {q1[i], q2[i], q3[i], q4[i]};
        iter_velocity_row(row, col, val, e, base, i, nx, -dt * nu / (dy[J + 1] * (dy[J] + dy[J + 1])),
                          -dt * nu / (dx[I] * (dx[I] + dx[I + 1])), -dt * nu / (dy[J] * (dy[J] + dy[J + 1])),
                          -dt * nu / (dx[I] * (dx[I] + dx[I - 1])), temp, plain, hyb, ghost, ns_rhs, interp_rhs,
                          count, idx, coef, q, alpha[i], vB0);
    }
    return base + nh;
}

/* update_rhs1_x over the u rows, update_rhs1_y launched on the u grid (numU threads) */
void or_iter_update_rhs1(double *rhs1, const double *ns_rhs, const double *interp_rhs, int nx, int ny)
{
    const int nU = (nx - 1) * ny, threads = ((int)((nU - 0.5) / 256) + 1) * 256;
    for (int i = 0; i < nU; ++i) {
        const int I = i % (nx - 1), J = i / (nx - 1);
        if (I == 0 || I == nx - 2 || J == 0 || J == ny - 1) continue;
        rhs1[i] = rhs1[i] * ns_rhs[i] + interp_rhs[i];
    }
    for (int k = 0; k < nx * (ny - 1) && k < threads; ++k) {
        const int I = k % nx, J = k / nx, i = k + nU;
        if (I == 0 || I == nx - 1 || J == 0 || J == ny - 2) continue;
        rhs1[i] = rhs1[i] * ns_rhs[i] + interp_rhs[i];
    }
}

/* luo_iter::poisson_size_lhs + poisson_calculate_lhs (values zeroed, LHS2_mid_iter,
 * LHS2_BC) on zeroed arrays of nnz = the plain operator's + the number of hybrid nodes */
int or_iter_lhs2(int *row, int *col, double *val, int nnz, const double *dx, const double *dy, int nx, int ny,
                 double dt, int *count, double *ns_rhs, double *interp_rhs, const int *hyb, const int *ghost,
                 const double *alpha, const double *dpdn, const int *i1, const int *i2, const int *i3, const int *i4,
                 const double *c1, const double *c2, const double *c3, const double *c4, const double *q1,
                 const double *q2, const double *q3, const double *q4, int i_start, int j_start, int width,
                 int height)
{
    const int base = nx * ny * 5 - 2 * nx - 2 * ny;
    const int nh = box_ranks(hyb, count, i_start, j_start, width, height, nx, ny, 0);
    if (base + nh > nnz) return -1;
    or_lhs2_coo(0, row, col, val, dx, dy, nx, ny, dt); /* boundary rows (LHS2_BC, pin at cell 0) */
    for (int k = base; k < nnz; ++k) put(row, col, val, k, 0, 0, 0);
    for (int ip = 0; ip < nx * ny; ++ip) {
        const int I = ip % nx, J = ip / nx;
        if (I == 0 || I == nx - 1 || J == 0 || J == ny - 1) continue;
        int e = mid_offset(I, J, nx);
        for (int k = 0; k < 5; ++k) put(row, col, val, e + k, 0, 0, 0);
        const int idx[4] = {i1[ip], i2[ip], i3[ip], i4[ip]};
        const double coef[4] = {c1[ip], c2[ip], c3[ip], c4[ip]}, q[4] = {q1[ip], q2[ip], q3[ip], q4[ip]};
        if (hyb[ip] > 0) {
            double Cns[5], CI[4];
            Cns[0] = -dt / (dy[J] * (dy[J] + dy[J + 1]) * 0.5);
            Cns[1] = -dt / (dx[I] * (dx[I] + dx[I + 1]) * 0.5);
            Cns[2] = -dt / (dy[J] * (dy[J] + dy[J - 1]) * 0.5);
            Cns[3] = -dt / (dx[I] * (dx[I] + dx[I - 1]) * 0.5);
            Cns[4] = -Cns[0] - Cns[1] - Cns[2] - Cns[3];
            for (int l = 0; l < 4; ++l) {
                Cns[l] = (1 - alpha[ip]) * Cns[l] / Cns[4];
                CI[l] = alpha[ip] * coef[l];
            }
            const int st[9] = {ip + nx - 1, ip + nx, ip + nx + 1, ip - 1, ip, ip + 1, ip - nx - 1, ip - nx, ip - nx + 1};
            double sv[9] = {0, Cns[0], 0, Cns[3], 1, Cns[1], 0, Cns[2], 0};
            const int used[9] = {0, 1, 0, 1, 1, 1, 0, 1, 0};
            for (int n = 0; n < 4; ++n)
                for (int m = 0; m < 9; ++m)
                    if (st[m] == idx[n] && m != 4) sv[m] -= CI[n];
            for (int m = 0; m < 9; ++m)
                if (used[m]) put(row, col, val, e++, ip, st[m], sv[m]);
            ns_rhs[ip] = (1 - alpha[ip]) / Cns[4];
            interp_rhs[ip] = 0;
            const int x = base + count[ip] - 1;
            for (int n = 0; n < 4; ++n)
                for (int m = 0; m < 9; ++m) {
                    if (st[m] == idx[n] && !used[m]) put(row, col, val, x, ip, idx[n], -CI[n]);
                    else if (st[m] == ip && idx[n] == ip) interp_rhs[ip] += CI[n] * q[n];
                }
        } else if (ghost[ip] > 0) {
            const int ns[5] = {ip + nx, ip + 1, ip - nx, ip - 1, ip};
            int overlap[5] = {0, 0, 0, 0, 1}, in[4] = {0, 0, 0, 0}, counter = 0;
            double temp = 0;
            for (int l = 0; l < 4; ++l) {
                if (ghost[idx[l]] > 0) {
                    counter += 1;
                    in[l] = 1;
                }
                for (int n = 0; n < 5; ++n)
                    if (idx[l] == ns[n]) overlap[n] = 1;
            }
            put(row, col, val, e++, ip, ip, 1);
            for (int l = 0; l < 4; ++l) {
                if (!in[l] && idx[l] != ip) put(row, col, val, e++, ip, idx[l], -coef[l]);
                else temp += coef[l] * q[l];
            }
            int c2 = 0;
            for (int n = 0; n < 5; ++n) {
                if (c2 >= counter) break;
                if (!overlap[n]) {
                    put(row, col, val, e++, ip, ns[n], 0);
                    c2++;
                }
            }
            ns_rhs[ip] = 0;
            interp_rhs[ip] = dpdn[ip] + temp;
        } else {
            double t = 0, c;
            c = dt / (dx[I] * (dx[I] + dx[I + 1]) * 0.5);
            put(row, col, val, e++, ip, ip + 1, -c); t += c;
            c = dt / (dx[I] * (dx[I] + dx[I - 1]) * 0.5);
            put(row, col, val, e++, ip, ip - 1, -c); t += c;
            c = dt / (dy[J] * (dy[J] + dy[J + 1]) * 0.5);
            put(row, col, val, e++, ip, ip + nx, -c); t += c;
            c = dt / (dy[J] * (dy[J] + dy[J - 1]) * 0.5);
            put(row, col, val, e++, ip, ip - nx, -c); t += c;
            put(row, col, val, e, ip, ip, t);
            ns_rhs[ip] = 1;
            interp_rhs[ip] = 0;
        }
    }
    return base + nh;
}

/* update_rhs2, launched over numP threads but bounded by (nx-1)*ny */
void or_iter_update_rhs2(double *rhs2, const double *ns_rhs, const double *interp_rhs, int nx, int ny)
{
    for (int ip = 0; ip < (nx - 1) * ny; ++ip) {
        const int I = ip % nx, J = ip / nx;
        if (I == 0 || I == nx - 1 || J == 0 || J == ny - 1) continue;
        rhs2[ip] = rhs2[ip] * ns_rhs[ip] + interp_rhs[ip];
    }
}
