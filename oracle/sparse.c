/*
 * Sparse operators and Krylov solvers of the oracle (test infrastructure only).
 *
 * The reference solves both systems with CUSP 0.5.1 (not vendored, not present):
 * cusp::krylov::bicgstab (NavierStokesSolver.cu:221-243 velocity, :249-271 Poisson)
 * under cusp::monitor(b, maxIters, relTol), i.e. stop when ||b - Ax||_2 <= relTol*||b||_2
 * or at maxIters, warm-started from the previous solution.  CUSP's iterates cannot
 * be reproduced without its source, so parity with it is "unpinned" at this
 * boundary: tests compare converged solutions.
 *
 * or_bicgstab: right-preconditioned BiCGSTAB (van der Vorst, SIAM J. Sci. Stat.
 *              Comput. 13(2), 1992), with the early exit on the half-step residual s
 *              and the iteration count of cusp::monitor (full iterations only).
 * or_cg:       preconditioned conjugate gradients on the symmetrised system
 *              (W A) x = W b, W = diag(w) > 0; convergence is measured on the
 *              residual of the ORIGINAL system, ||W^-1 r_sym|| <= rtol ||b||.
 * precond:     0 none, 1 diagonal (Jacobi), 2 smoothed aggregation (or_sa_build).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"


void or_sa_apply(void *amg, const double *r, double *z);

void or_coo_to_csr(int n, int nnz, const int *row, const int *col, const double *val, int *rowptr, int *colind,
                   double *vals)
{
    /* stable counting sort by row: entries keep their order inside each row */
    memset(rowptr, 0, sizeof(int) * (n + 1));
    for (int k = 0; k < nnz; ++k) rowptr[row[k] + 1]++;
    for (int i = 0; i < n; ++i) rowptr[i + 1] += rowptr[i];
    int *pos = (int *)malloc(sizeof(int) * n);
    memcpy(pos, rowptr, sizeof(int) * n);
    for (int k = 0; k < nnz; ++k) {
        int d = pos[row[k]]++;
        colind[d] = col[k];
        vals[d] = val[k];
    }
    free(pos);
}

void or_csr_spmv(int n, const int *rowptr, const int *colind, const double *vals, const double *x, double *y)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double s = 0;
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) s += vals[k] * x[colind[k]];
        y[i] = s;
    }
}

static double dot(int n, const double *a, const double *b)
{
    double s = 0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

typedef struct {
    int kind;
    int n;
    double *dinv;
    void *amg;
} pc_t;

static void pc_init(pc_t *M, int n, const int *rowptr, const int *colind, const double *vals, int kind, void *amg)
{
    M->kind = kind;
    M->n = n;
    M->dinv = NULL;
    M->amg = amg;
    if (kind == 1) {
        M->dinv = (double *)malloc(sizeof(double) * n);
        for (int i = 0; i < n; ++i) {
            double d = 0;
            for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
                if (colind[k] == i) d += vals[k];
            M->dinv[i] = (d != 0) ? 1.0 / d : 1.0;
        }
    }
}

static void pc_apply(const pc_t *M, const double *r, double *z)
{
    if (M->kind == 1) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < M->n; ++i) z[i] = M->dinv[i] * r[i];
    } else if (M->kind == 2) {
        or_sa_apply(M->amg, r, z);
    } else {
        memcpy(z, r, sizeof(double) * M->n);
    }
}

static void pc_free(pc_t *M) { free(M->dinv); }

int or_bicgstab(int n, const int *rowptr, const int *colind, const double *vals, const double *b, double *x,
                double rtol, int maxit, int precond, void *amg, double *resid_out)
{
    pc_t M;
    pc_init(&M, n, rowptr, colind, vals, precond, amg);
    double *r = malloc(sizeof(double) * n), *rs = malloc(sizeof(double) * n), *p = malloc(sizeof(double) * n);
    double *Mp = malloc(sizeof(double) * n), *AMp = malloc(sizeof(double) * n), *s = malloc(sizeof(double) * n);
    double *Ms = malloc(sizeof(double) * n), *AMs = malloc(sizeof(double) * n);
    double tol = rtol * sqrt(dot(n, b, b));
    or_csr_spmv(n, rowptr, colind, vals, x, r);
    for (int i = 0; i < n; ++i) {
        r[i] = b[i] - r[i];
        rs[i] = r[i];
        p[i] = r[i];
    }
    double rho = dot(n, rs, r), rn = sqrt(dot(n, r, r));
    int it = 0;
    while (!(rn <= tol) && it < maxit) {
        pc_apply(&M, p, Mp);
        or_csr_spmv(n, rowptr, colind, vals, Mp, AMp);
        double alpha = rho / dot(n, rs, AMp);
        for (int i = 0; i < n; ++i) s[i] = r[i] - alpha * AMp[i];
        double sn = sqrt(dot(n, s, s));
        if (sn <= tol) {
            for (int i = 0; i < n; ++i) x[i] += alpha * Mp[i];
            rn = sn;
            break;
        }
        pc_apply(&M, s, Ms);
        or_csr_spmv(n, rowptr, colind, vals, Ms, AMs);
        double omega = dot(n, AMs, s) / dot(n, AMs, AMs);
        for (int i = 0; i < n; ++i) {
            x[i] += alpha * Mp[i] + omega * Ms[i];
            r[i] = s[i] - omega * AMs[i];
        }
        double rho_new = dot(n, rs, r);
        double beta = (rho_new / rho) * (alpha / omega);
        rho = rho_new;
        for (int i = 0; i < n; ++i) p[i] = r[i] + beta * (p[i] - omega * AMp[i]);
        rn = sqrt(dot(n, r, r));
        ++it;
    }
    if (resid_out) *resid_out = (tol > 0) ? rn / (tol / rtol) : rn;
    free(r); free(rs); free(p); free(Mp); free(AMp); free(s); free(Ms); free(AMs);
    pc_free(&M);
    return (rn <= tol) ? it : -(it + 1);
}

int or_cg(int n, const int *rowptr, const int *colind, const double *vals, const double *w, const double *b,
          double *x, double rtol, int maxit, int precond, void *amg, double *resid_out)
{
    /* The caller passes the symmetrised matrix S = W A (rowptr/colind/vals) and
     * the row weights w; b is the ORIGINAL right-hand side. */
    pc_t M;
    pc_init(&M, n, rowptr, colind, vals, precond, amg);
    double *r = malloc(sizeof(double) * n), *z = malloc(sizeof(double) * n), *p = malloc(sizeof(double) * n);
    double *q = malloc(sizeof(double) * n);
    double tol = rtol * sqrt(dot(n, b, b));
    or_csr_spmv(n, rowptr, colind, vals, x, r);
    double rn2 = 0;
    for (int i = 0; i < n; ++i) {
        r[i] = w[i] * b[i] - r[i];
        double ro = r[i] / w[i];
        rn2 += ro * ro;
    }
    double rn = sqrt(rn2);
    int it = 0;
    pc_apply(&M, r, z);
    memcpy(p, z, sizeof(double) * n);
    double rz = dot(n, r, z);
    while (!(rn <= tol) && it < maxit) {
        or_csr_spmv(n, rowptr, colind, vals, p, q);
        double alpha = rz / dot(n, p, q);
        rn2 = 0;
        for (int i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * q[i];
            double ro = r[i] / w[i];
            rn2 += ro * ro;
        }
        rn = sqrt(rn2);
        ++it;
        if (rn <= tol) break;
        pc_apply(&M, r, z);
        double rz_new = dot(n, r, z);
        double beta = rz_new / rz;
        rz = rz_new;
        for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
    if (resid_out) *resid_out = (tol > 0) ? rn / (tol / rtol) : rn;
    free(r); free(z); free(p); free(q);
    pc_free(&M);
    return (rn <= tol) ? it : -(it + 1);
}
