/*
 * Smoothed-aggregation AMG of the oracle (test infrastructure only), standing
 * in for cusp::precond::aggregation::smoothed_aggregation (CUSP 0.5.1, not
 * available; selected in the reference by "preconditioner: SMOOTHED_AGGREGATION",
 * src/preconditioner.h:84-113).  Textbook algorithm (Vanek, Mandel, Brezina 1996):
 * greedy aggregation over the matrix graph, piecewise-constant tentative
 * prolongator, one damped-Jacobi prolongator smoothing step with
 * w = 4/(3 rho(D^-1 A)), Galerkin coarse operators R A P with R = P^T, dense LU
 * on the coarsest level; V(1,1) cycle with damped Jacobi.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

typedef struct {
    int n, m;
    int *ptr, *col;
    double *val;
} csr;

typedef struct {
    csr A, P, R;
    double *dinv, omega;
    double *x, *b, *r;
} level;

typedef struct {
    int nl;
    level L[32];
    int nc;
    double *lu; /* dense LU of the coarsest operator, row-major, with pivots */
    int *piv;
} sa_t;

static csr csr_copy(int n, int m, const int *ptr, const int *col, const double *val)
{
    csr A = {n, m, malloc(sizeof(int) * (n + 1)), malloc(sizeof(int) * ptr[n]), malloc(sizeof(double) * ptr[n])};
    memcpy(A.ptr, ptr, sizeof(int) * (n + 1));
    memcpy(A.col, col, sizeof(int) * ptr[n]);
    memcpy(A.val, val, sizeof(double) * ptr[n]);
    return A;
}

static void csr_free(csr *A)
{
    free(A->ptr);
    free(A->col);
    free(A->val);
}

static csr csr_transpose(const csr *A)
{
    csr T = {A->m, A->n, calloc(A->m + 1, sizeof(int)), malloc(sizeof(int) * A->ptr[A->n]),
             malloc(sizeof(double) * A->ptr[A->n])};
    for (int k = 0; k < A->ptr[A->n]; ++k) T.ptr[A->col[k] + 1]++;
    for (int i = 0; i < T.n; ++i) T.ptr[i + 1] += T.ptr[i];
    int *pos = malloc(sizeof(int) * (T.n + 1));
    memcpy(pos, T.ptr, sizeof(int) * (T.n + 1));
    for (int i = 0; i < A->n; ++i)
        for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) {
            int d = pos[A->col[k]]++;
            T.col[d] = i;
            T.val[d] = A->val[k];
        }
    free(pos);
    return T;
}

static csr csr_mult(const csr *A, const csr *B)
{
    int cap = A->ptr[A->n] * 4 + 16, nnz = 0;
    csr C = {A->n, B->m, malloc(sizeof(int) * (A->n + 1)), malloc(sizeof(int) * cap), malloc(sizeof(double) * cap)};
    int *mark = malloc(sizeof(int) * B->m);
    double *acc = malloc(sizeof(double) * B->m);
    int *cols = malloc(sizeof(int) * B->m);
    for (int j = 0; j < B->m; ++j) mark[j] = -1;
    C.ptr[0] = 0;
    for (int i = 0; i < A->n; ++i) {
        int nc = 0;
        for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) {
            int a = A->col[k];
            double av = A->val[k];
            for (int q = B->ptr[a]; q < B->ptr[a + 1]; ++q) {
                int j = B->col[q];
                if (mark[j] != i) {
                    mark[j] = i;
                    acc[j] = 0;
                    cols[nc++] = j;
                }
                acc[j] += av * B->val[q];
            }
        }
        if (nnz + nc > cap) {
            while (nnz + nc > cap) cap *= 2;
            C.col = realloc(C.col, sizeof(int) * cap);
            C.val = realloc(C.val, sizeof(double) * cap);
        }
        for (int t = 0; t < nc; ++t) {
            C.col[nnz] = cols[t];
            C.val[nnz++] = acc[cols[t]];
        }
        C.ptr[i + 1] = nnz;
    }
    free(mark);
    free(acc);
    free(cols);
    return C;
}

static void spmv(const csr *A, const double *x, double *y)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < A->n; ++i) {
        double s = 0;
        for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k) s += A->val[k] * x[A->col[k]];
        y[i] = s;
    }
}

static double *diag_inv(const csr *A)
{
    double *d = malloc(sizeof(double) * A->n);
    for (int i = 0; i < A->n; ++i) {
        double s = 0;
        for (int k = A->ptr[i]; k < A->ptr[i + 1]; ++k)
            if (A->col[k] == i) s += A->val[k];
        d[i] = s != 0 ? 1.0 / s : 1.0;
    }
    return d;
}

void *or_sa_build(int n, const int *rowptr, const int *colind, const double *vals, double theta, int coarse_n)
{
    (void)theta; /* every off-diagonal entry is treated as strong */
    sa_t *S = calloc(1, sizeof(sa_t));
    csr A = csr_copy(n, n, rowptr, colind, vals);
    for (;;) {
        level *L = &S->L[S->nl++];
        L->A = A;
        L->dinv = diag_inv(&A);
        L->x = calloc(A.n, sizeof(double));
        L->b = calloc(A.n, sizeof(double));
        L->r = calloc(A.n, sizeof(double));
        if (A.n <= coarse_n || S->nl == 32) break;
        /* rho(D^-1 A) by power iteration */
        double *x = malloc(sizeof(double) * A.n), *y = malloc(sizeof(double) * A.n), lam = 1;
        for (int i = 0; i < A.n; ++i) x[i] = 1.0 + 0.25 * sin(0.37 * i);
        for (int it = 0; it < 20; ++it) {
            spmv(&A, x, y);
            double ny = 0, nx = 0;
            for (int i = 0; i < A.n; ++i) {
                y[i] *= L->dinv[i];
                ny += y[i] * y[i];
                nx += x[i] * x[i];
            }
            lam = sqrt(ny / nx);
            for (int i = 0; i < A.n; ++i) x[i] = y[i] / sqrt(ny);
        }
        free(x);
        free(y);
        L->omega = 4.0 / (3.0 * lam);
        /* aggregation */
        int *agg = malloc(sizeof(int) * A.n), na = 0;
        for (int i = 0; i < A.n; ++i) agg[i] = -1;
        for (int i = 0; i < A.n; ++i) {
            if (agg[i] >= 0) continue;
            int ok = 1;
            for (int k = A.ptr[i]; k < A.ptr[i + 1] && ok; ++k)
                if (A.col[k] != i && A.val[k] != 0 && agg[A.col[k]] >= 0) ok = 0;
            if (!ok) continue;
            for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
                if (A.val[k] != 0) agg[A.col[k]] = na;
            agg[i] = na++;
        }
        int *agg1 = malloc(sizeof(int) * A.n);
        memcpy(agg1, agg, sizeof(int) * A.n);
        for (int i = 0; i < A.n; ++i) {
            if (agg1[i] >= 0) continue;
            double best = 0;
            for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
                if (A.col[k] != i && agg1[A.col[k]] >= 0 && fabs(A.val[k]) > best) {
                    best = fabs(A.val[k]);
                    agg[i] = agg1[A.col[k]];
                }
        }
        free(agg1);
        for (int i = 0; i < A.n; ++i) {
            if (agg[i] >= 0) continue;
            for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
                if (agg[A.col[k]] < 0) agg[A.col[k]] = na;
            agg[i] = na++;
        }
        int *cnt = calloc(na, sizeof(int));
        for (int i = 0; i < A.n; ++i) cnt[agg[i]]++;
        csr T = {A.n, na, malloc(sizeof(int) * (A.n + 1)), malloc(sizeof(int) * A.n), malloc(sizeof(double) * A.n)};
        for (int i = 0; i < A.n; ++i) {
            T.ptr[i] = i;
            T.col[i] = agg[i];
            T.val[i] = 1.0 / sqrt((double)cnt[agg[i]]);
        }
        T.ptr[A.n] = A.n;
        csr AT = csr_mult(&A, &T);
        for (int i = 0; i < AT.n; ++i)
            for (int k = AT.ptr[i]; k < AT.ptr[i + 1]; ++k) {
                AT.val[k] *= -L->omega * L->dinv[i];
                if (AT.col[k] == agg[i]) AT.val[k] += T.val[i];
            }
        L->P = AT;
        L->R = csr_transpose(&L->P);
        csr AP = csr_mult(&A, &L->P);
        csr Ac = csr_mult(&L->R, &AP);
        csr_free(&AP);
        csr_free(&T);
        free(cnt);
        free(agg);
        A = Ac;
    }
    /* dense LU with partial pivoting of the coarsest operator */
    level *C = &S->L[S->nl - 1];
    int nc = C->A.n;
    S->nc = nc;
    S->lu = calloc((size_t)nc * nc, sizeof(double));
    S->piv = malloc(sizeof(int) * nc);
    for (int i = 0; i < nc; ++i)
        for (int k = C->A.ptr[i]; k < C->A.ptr[i + 1]; ++k) S->lu[(size_t)i * nc + C->A.col[k]] += C->A.val[k];
    for (int c = 0; c < nc; ++c) {
        int p = c;
        for (int r = c + 1; r < nc; ++r)
            if (fabs(S->lu[(size_t)r * nc + c]) > fabs(S->lu[(size_t)p * nc + c])) p = r;
        S->piv[c] = p;
        if (p != c)
            for (int k = 0; k < nc; ++k) {
                double t = S->lu[(size_t)c * nc + k];
                S->lu[(size_t)c * nc + k] = S->lu[(size_t)p * nc + k];
                S->lu[(size_t)p * nc + k] = t;
            }
        double d = S->lu[(size_t)c * nc + c];
        if (d == 0) d = S->lu[(size_t)c * nc + c] = 1e-300;
        for (int r = c + 1; r < nc; ++r) {
            double f = S->lu[(size_t)r * nc + c] /= d;
            for (int k = c + 1; k < nc; ++k) S->lu[(size_t)r * nc + k] -= f * S->lu[(size_t)c * nc + k];
        }
    }
    return S;
}

static void coarse_solve(const sa_t *S, const double *b, double *x)
{
    int n = S->nc;
    for (int i = 0; i < n; ++i) x[i] = b[i];
    for (int c = 0; c < n; ++c) {
        int p = S->piv[c];
        if (p != c) {
            double t = x[c];
            x[c] = x[p];
            x[p] = t;
        }
        for (int r = c + 1; r < n; ++r) x[r] -= S->lu[(size_t)r * n + c] * x[c];
    }
    for (int c = n - 1; c >= 0; --c) {
        for (int k = c + 1; k < n; ++k) x[c] -= S->lu[(size_t)c * n + k] * x[k];
        x[c] /= S->lu[(size_t)c * n + c];
    }
}

static void vcycle(sa_t *S, int l, const double *b, double *x)
{
    level *L = &S->L[l];
    int n = L->A.n;
    if (l == S->nl - 1) {
        coarse_solve(S, b, x);
        return;
    }
    for (int i = 0; i < n; ++i) x[i] = L->omega * L->dinv[i] * b[i];
    spmv(&L->A, x, L->r);
    for (int i = 0; i < n; ++i) L->r[i] = b[i] - L->r[i];
    level *C = &S->L[l + 1];
    spmv(&L->R, L->r, C->b);
    vcycle(S, l + 1, C->b, C->x);
    double *t = malloc(sizeof(double) * n);
    spmv(&L->P, C->x, t);
    for (int i = 0; i < n; ++i) x[i] += t[i];
    spmv(&L->A, x, t);
    for (int i = 0; i < n; ++i) x[i] += L->omega * L->dinv[i] * (b[i] - t[i]);
    free(t);
}

void or_sa_apply(void *amg, const double *r, double *z) { vcycle((sa_t *)amg, 0, r, z); }

int or_sa_levels(void *amg) { return ((sa_t *)amg)->nl; }

void or_sa_free(void *amg)
{
    sa_t *S = amg;
    if (!S) return;
    for (int l = 0; l < S->nl; ++l) {
        level *L = &S->L[l];
        csr_free(&L->A);
        if (l < S->nl - 1) {
            csr_free(&L->P);
            csr_free(&L->R);
        }
        free(L->dinv);
        free(L->x);
        free(L->b);
        free(L->r);
    }
    free(S->lu);
    free(S->piv);
    free(S);
}
