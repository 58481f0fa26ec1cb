/*
 * CPU oracle: a plain-C restatement of cuIBM's fractional-step time step.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py load this library (through oracle/__init__.py),
 * and only as the test oracle or the CPU baseline.  The product never links it.
 *
 * Every function names the reference file and function it restates.  The
 * arithmetic keeps the reference's association order and the library is
 * compiled with -ffp-contract=off, so results are bit-identical to the
 * reference kernels run on the CPU (oracle/_ref) - the golden fixtures under
 * tests/golden pin this.
 *
 * Layout (same as the reference): velocity is one vector of numUV = nU + nV
 * doubles, u first (index J*(nx-1)+I) then v (nU + J*nx+I); pressure J*nx+I.
 * Boundary arrays: bc[XMINUS|XPLUS] have 2*ny-1 entries (u on 0..ny-1, v on
 * ny..2ny-2), bc[YMINUS|YPLUS] have 2*nx-1 (u on 0..nx-2, v on nx-1..2nx-2).
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- grid.c : io/parseDomainFile.cu, io/parseBodiesFile.cu, src/bodies.cu ---- */
int or_axis_count(double start, double mid_h, int nsub, const double *ends, const double *ratios);
void or_axis_fill(double start, double mid_h, int nsub, const double *ends, const double *ratios, double *c,
                  double *d, double *cs);
void or_circle_points(double cx, double cy, double R, int n, double *X, double *Y);
int or_circle_count(double R, int numPoints, int selfSize, double mid_h);
void or_body_place(int n, const double *X, const double *Y, double *x, double *y, double *midX, double *midY,
                   double *bdx, double *bdy);
void or_bounding_box(int n, const double *x, const double *y, const double *gx, const double *gy, double scale,
                     int *startI, int *startJ, int *ncx, int *ncy);

/* ---- ns.c : the NavierStokes/kernels sources ---- */
void or_generateN(double *N, const double *u, const double *dx, const double *dy, const double *ym,
                  const double *yp, const double *xm, const double *xp, int nx, int ny);
void or_generateL(double *L, const double *u, const double *dx, const double *dy, const double *ym,
                  const double *yp, const double *xm, const double *xp, int nx, int ny, double nu);
void or_generateBC1(const double *u, double *bc1, const double *ym, const double *yp, const double *xm,
                    const double *xp, const double *dx, const double *dy, double nu, double dt, int nx, int ny);
void or_generateRHS(double *rhs, const double *L, const double *Nold, const double *N, const double *u,
                    const double *bc1, double dt, int n);
void or_lhs1_coo(int *row, int *col, double *val, const double *dx, const double *dy, double dt, double nu,
                 int nx, int ny);
void or_lhs2_coo(int centre_pin, int *row, int *col, double *val, const double *dx, const double *dy, int nx,
                 int ny, double dt);
void or_generateRHS2(double *rhs2, const double *uhat, const double *ym, const double *yp, const double *xm,
                     const double *xp, const double *dx, const double *dy, int nx, int ny);
void or_project(double *u, const double *uhat, double *uold, const double *p, const double *dx,
                const double *dy, double dt, int nx, int ny);
void or_initialiseVelocity(double *u, const double *xu, const double *yu, const double *xv, const double *yv,
                           double uI, double vI, double uP, double vP, double xmax, double xmin, double ymax,
                           double ymin, int nx, int ny);
void or_calculateCFL(double *cfl, const double *u, const double *dx, const double *dy, int nx, int ny,
                     double dt);

/* ---- sparse.c : CSR operators and the Krylov solvers that replace CUSP ---- */
void or_coo_to_csr(int n, int nnz, const int *row, const int *col, const double *val, int *rowptr, int *colind,
                   double *vals);
void or_csr_spmv(int n, const int *rowptr, const int *colind, const double *vals, const double *x, double *y);
/* precond: 0 none, 1 diagonal (Jacobi), 2 smoothed aggregation (hierarchy built by or_sa_build) */
int or_bicgstab(int n, const int *rowptr, const int *colind, const double *vals, const double *b, double *x,
                double rtol, int maxit, int precond, void *amg, double *resid_out);
int or_cg(int n, const int *rowptr, const int *colind, const double *vals, const double *w, const double *b,
          double *x, double rtol, int maxit, int precond, void *amg, double *resid_out);
void *or_sa_build(int n, const int *rowptr, const int *colind, const double *vals, double theta, int coarse_n);
void or_sa_free(void *amg);
int or_sa_levels(void *amg);

/* ---- ib.c : luo_base / luoIBM / FadlunModified kernels ---- */
typedef struct {
    int *ghostTagsUV, *ghostTagsP, *hybridTagsUV, *hybridTagsP, *hybridTagsUV2;
    double *dist_node, *dist_between, *dist_u_body, *dist_v_body, *uv;
    double *bi_x, *bi_y, *ip_x, *ip_y;     /* numUV */
    double *bip_x, *bip_y, *ipp_x, *ipp_y; /* numP  */
} or_tags;

typedef struct {
    int *index1, *index2, *index3, *index4;
    double *q1coef, *q2coef, *q3coef, *q4coef;
    double *value; /* image_point_u (velocity) or body_intercept_p (pressure ghost) */
    double *dpdn;  /* pressure ghost only */
    double *q1, *q2, *q3, *q4; /* the corner values the fit used (field or substituted body values) */
} or_interp;

/* body intercept form of the tagging: 0 the reference's trigonometric form, 1 its
 * closed form (the default; the GPU's) */
void or_set_intercept_form(int form);
int or_get_intercept_form(void);
void or_tagPoints(or_tags *T, const double *bx, const double *by, const double *uB, const double *vB,
                  const double *xu, const double *yu, const double *xv, const double *yv, int i_start,
                  int j_start, int width, int height, int nx, int ny, int totalPoints, double midX, double midY);
void or_ghost_velocity(int dir, double *u, int set, const int *ghostTagsUV, double uB0, const double *yc,
                       const double *xc, const double *bi_x, const double *bi_y, const double *ip_x,
                       const double *ip_y, int i_start, int j_start, int width, int height, int nx, int ny,
                       or_interp *R);
void or_hybrid_velocity(int dir, const double *u, double *ustar, const int *hybridTagsUV, double uB0,
                        const double *yc, const double *xc, const double *bi_x, const double *bi_y,
                        const double *ip_x, const double *ip_y, int i_start, int j_start, int width, int height,
                        int nx, int ny, or_interp *R);
void or_hybrid_pressure(const double *p, double *pstar, const int *hybridTagsP, double dudt_u, double dudt_v,
                        const double *yu, const double *xv, const double *bip_x, const double *bip_y,
                        const double *ipp_x, const double *ipp_y, int i_start, int j_start, int width,
                        int height, int nx, int ny, or_interp *R);
void or_ghost_pressure(double *p, int set, const int *ghostTagsP, double dudt_u, double dudt_v,
                       const double *yu, const double *xv, const double *bip_x, const double *bip_y,
                       const double *ipp_x, const double *ipp_y, int i_start, int j_start, int width, int height,
                       int nx, int ny, or_interp *R);
void or_weight(int dir, double *f, const double *fstar, const int *ghostTags, const int *hybridTags,
               const double *yc, const double *xc, const double *bi_x, const double *bi_y, int i_start,
               int j_start, int width, int height, int nx, int ny);
void or_setInsideVelocity(const int *ghostTags, double *u, double uB0, double vB0, int nx, int ny);
void or_updateRobinBoundary(const double *u, double *xp, const double *dx, double dt, double Uinf, double Vinf,
                            int nx, int ny);
void or_calculateForce(const double *u, const double *uold, const double *p, const int *ghostTagsUV, double nu,
                       const double *dx, const double *dy, double dt, int nx, int ny, int I, int J, int ncx,
                       int ncy, double *fx, double *fy);
void or_surfaceForce(int mode, const double *bx, const double *by, int n, double uB0, double vB0, const double *u,
                     const double *bip, const double *bip_x, const double *bip_y, const int *ghostTagsP,
                     const double *xu, const double *yu, const double *xv, const double *yv, int startI,
                     int startJ, int nx, int ny, double midX, double midY, double nu, double mid_h, double *terms,
                     double *fx, double *fy);

/* ---- fadlun.c : FadlunModified kernels (modified Fadlun method) ---- */
void or_fadlun_lhs1_coo(int *row, int *col, double *val, int nnz, const int *hyb, const int *hyb2, const int *ghost,
                        const double *dn, const double *db, const double *dx, const double *dy, double dt,
                        double nu, int nx, int ny);
void or_fadlun_lhs2_coo(int *row, int *col, double *val, const double *du, const double *dv, const int *ghostP,
                        const int *hybP, const double *dx, const double *dy, int nx, int ny, double dt);
void or_fadlun_update_rhs1(const int *hyb, const int *ghost, double *rhs, const double *dn, const double *db,
                           const double *uv, int nx, int ny);
void or_fadlun_rhs2(double *rhs2, const double *uhat, const int *ghostP, const int *hybP, const double *du,
                    const double *dv, const double *ym, const double *yp, const double *xm, const double *xp,
                    const double *dx, const double *dy, int nx, int ny);
void or_fadlun_project(double *u, const double *uhat, const double *p, const int *ghostP, const double *dx,
                       const double *dy, double dt, int nx, int ny);

/* ---- embedded.c : luo_iter kernels (embedded method, SolverType OSC_CYLINDER) ---- */
void or_iter_alpha(int kind, double *alpha, const int *ghost, const int *hybrid, const double *yc, const double *xc,
                   const double *bix, const double *biy, int i_start, int j_start, int width, int nx, int ny);
int or_iter_lhs1(int *row, int *col, double *val, int nnz, const double *dx, const double *dy, double dt, double nu,
                 int nx, int ny, const int *hyb, const int *ghost, double *ns_rhs, double *interp_rhs, int *count,
                 const int *i1, const int *i2, const int *i3, const int *i4, const double *alpha, double uB0,
                 double vB0, const double *c1, const double *c2, const double *c3, const double *c4,
                 const double *q1, const double *q2, const double *q3, const double *q4, int i_start, int j_start,
                 int width, int height);
void or_iter_update_rhs1(double *rhs1, const double *ns_rhs, const double *interp_rhs, int nx, int ny);
int or_iter_lhs2(int *row, int *col, double *val, int nnz, const double *dx, const double *dy, int nx, int ny,
                 double dt, int *count, double *ns_rhs, double *interp_rhs, const int *hyb, const int *ghost,
                 const double *alpha, const double *dpdn, const int *i1, const int *i2, const int *i3, const int *i4,
                 const double *c1, const double *c2, const double *c3, const double *c4, const double *q1,
                 const double *q2, const double *q3, const double *q4, int i_start, int j_start, int width,
                 int height);
void or_iter_update_rhs2(double *rhs2, const double *ns_rhs, const double *interp_rhs, int nx, int ny);

#ifdef __cplusplus
}
#endif
