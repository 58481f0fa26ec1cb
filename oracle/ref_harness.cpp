/*
 * Serial CPU launcher for the reference's own kernel code (TEST INFRASTRUCTURE).
 *
 * oracle/Makefile compiles the reference kernel sources (read in place from the
 * reference tree, never copied) as host C++ through oracle/ref_shim.h and links
 * them with this file into oracle/_ref/libcuibm_refkernels.so.  Each extern "C"
 * entry point below reproduces one launch sequence of the reference's host code
 * (same grid size, same kernel order) and runs every thread of the grid one after
 * another, in increasing global thread index.  tests/golden/make_golden.py calls
 * these entry points to write the golden fixtures that pin the oracle.
 *
 * Race semantics (the reference kernels have cross-thread hazards):
 *  - write/write conflicts (tagging writes into neighbour nodes) resolve as
 *    "last thread in global index order wins" - the natural serial order;
 *  - read-neighbour/write-self kernels that update a field in place
 *    (interpolateVelocityToGhostNode*, interpolatePressureToGhostNode with
 *    set=true) are run with SNAPSHOT semantics: every thread reads the field as it
 *    was before the launch.  On the GPU every thread of those kernels loads its
 *    four corner values long before any thread stores, so this is the behaviour
 *    of the reference on hardware; serial order would instead chain updates.
 */
#include "ref_shim.h"
#include <vector>
#include <cstring>

thread_local ref_dim3 threadIdx, blockIdx, blockDim, gridDim;

#include "solvers/NavierStokes/NavierStokes/kernels/N.h"
#include "solvers/NavierStokes/NavierStokes/kernels/L.h"
#include "solvers/NavierStokes/NavierStokes/kernels/intermediateVelocity.h"
#include "solvers/NavierStokes/NavierStokes/kernels/intermediatePressure.h"
#include "solvers/NavierStokes/NavierStokes/kernels/projectVelocity.h"
#include "solvers/NavierStokes/NavierStokes/kernels/LHS1.h"
#include "solvers/NavierStokes/NavierStokes/kernels/LHS2.h"
#include "solvers/NavierStokes/NavierStokes/kernels/initialise.h"
#include "solvers/NavierStokes/NavierStokes/kernels/CFL.h"
#include "solvers/NavierStokes/luo_base/kernels/tagPoints.h"
#include "solvers/NavierStokes/luo_base/kernels/biLinearInterpolation.h"
#include "solvers/NavierStokes/luo_base/kernels/intermediateVelocity.h"
#include "solvers/NavierStokes/luo_base/kernels/projectVelocity.h"
#include "solvers/NavierStokes/luo_base/kernels/structure.h"
#include "solvers/NavierStokes/luo_base/kernels/calculateForce.h"
#include "solvers/NavierStokes/luoIBM/kernels/LHS1.h"
#include "solvers/NavierStokes/luoIBM/kernels/LHS2.h"
#include "solvers/NavierStokes/luoIBM/kernels/intermediatePressure.h"
#include "solvers/NavierStokes/luoIBM/kernels/weight.h"
#include "solvers/NavierStokes/FadlunModified/kernels/intermediateVelocity.h"
#include "solvers/NavierStokes/FadlunModified/kernels/calculateForce.h"
#include "solvers/NavierStokes/FadlunModified/kernels/LHS1.h"
#include "solvers/NavierStokes/FadlunModified/kernels/LHS2.h"
#include "solvers/NavierStokes/FadlunModified/kernels/intermediatePressure.h"
#include "solvers/NavierStokes/FadlunModified/kernels/projectVelocity.h"
#include "solvers/NavierStokes/luo_iter/kernels/LHS1.h"
#include "solvers/NavierStokes/luo_iter/kernels/LHS2.h"
#include "solvers/NavierStokes/luo_iter/kernels/intermediateVelocity.h"
#include "solvers/NavierStokes/luo_iter/kernels/pressure.h"
#include "solvers/NavierStokes/luo_iter/kernels/weight.h"

namespace {
const int BS = 256;

// grid size rule of the reference host code: int((count-0.5)/256)+1
inline int grid_for(double count) { return int((count - 0.5) / BS) + 1; }

template <class F>
void launch(int grid, int block, F f)
{
    blockDim = {(unsigned)block, 1, 1};
    gridDim = {(unsigned)grid, 1, 1};
    for (int b = 0; b < grid; ++b)
        for (int t = 0; t < block; ++t) {
            blockIdx = {(unsigned)b, 0, 0};
            threadIdx = {(unsigned)t, 0, 0};
            f();
        }
}

// Snapshot-semantics launch for kernels that read neighbours of `field` and
// write field[self]: each thread runs on the pre-launch field; the value it
// leaves at its own index is collected and applied after the launch.
template <class SelfIndex, class F>
void launch_snapshot(int grid, int block, double *field, int n, SelfIndex self_index, F f)
{
    std::vector<double> out(field, field + n);
    blockDim = {(unsigned)block, 1, 1};
    gridDim = {(unsigned)grid, 1, 1};
    for (int b = 0; b < grid; ++b)
        for (int t = 0; t < block; ++t) {
            blockIdx = {(unsigned)b, 0, 0};
            threadIdx = {(unsigned)t, 0, 0};
            int s = self_index(b * block + t);
            if (s < 0 || s >= n) { f(); continue; }
            double before = field[s];
            f();
            out[s] = field[s];
            field[s] = before;
        }
    std::memcpy(field, out.data(), sizeof(double) * n);
}
}  // namespace

extern "C" {

// ---- NavierStokes/intermediateVelocity.cu : generateN, generateL, generateBC1, generateRHS
void ref_generateN(double *N, double *u, double *dx, double *dy, double *ym, double *yp, double *xm,
                   double *xp, int nx, int ny)
{
    int gU = grid_for((nx - 1) * ny), gV = grid_for(nx * (ny - 1));
    launch(gU, BS, [&] { kernels::Nmidx(N, u, dx, dy, nx, ny); });
    launch(gU, BS, [&] { kernels::Nbcx(N, u, dx, dy, ym, yp, xm, xp, nx, ny); });
    launch(gV, BS, [&] { kernels::Nmidy(N, u, dx, dy, nx, ny); });
    launch(gV, BS, [&] { kernels::Nbcy(N, u, dx, dy, ym, yp, xm, xp, nx, ny); });
}

void ref_generateL(double *L, double *u, double *dx, double *dy, double *ym, double *yp, double *xm,
                   double *xp, int nx, int ny, double nu)
{
    int gU = grid_for((nx - 1) * ny), gV = grid_for(nx * (ny - 1));
    launch(gU, BS, [&] { kernels::Lmidx(L, u, dx, dy, nx, ny, nu); });
    launch(gU, BS, [&] { kernels::Lbcx(L, u, dx, dy, ym, yp, xm, xp, nx, ny, nu); });
    launch(gV, BS, [&] { kernels::Lmidy(L, u, dx, dy, nx, ny, nu); });
    launch(gV, BS, [&] { kernels::Lbcy(L, u, dx, dy, ym, yp, xm, xp, nx, ny, nu); });
}

void ref_generateBC1(double *u, double *bc1, double *ym, double *yp, double *xm, double *xp, double *dx,
                     double *dy, double nu, double dt, int nx, int ny)
{
    int gU = grid_for((nx - 1) * ny), gV = grid_for(nx * (ny - 1));
    launch(gU, BS, [&] { kernels::bc1X(u, bc1, ym, yp, xm, xp, dx, dy, nu, dt, nx, ny); });
    launch(gV, BS, [&] { kernels::bc1Y(u, bc1, ym, yp, xm, xp, dx, dy, nu, dt, nx, ny); });
}

void ref_generateRHS(double *rhs, double *L, double *Nold, double *N, double *u, double *bc1, double dt,
                     int nx, int ny)
{
    int g = grid_for((nx - 1) * ny + nx * (ny - 1));
    launch(g, BS, [&] { kernels::generateRHS(rhs, L, Nold, N, u, bc1, dt, nx, ny); });
}

// ---- NavierStokes/intermediateVelocity.cu generateLHS1 (base) and luoIBM/intermediateVelocity.cu (LUO)
void ref_generateLHS1(int luo, int *row, int *col, double *val, int *ghostTagsUV, double *dx, double *dy,
                      double dt, double nu, int nx, int ny)
{
    int gU = grid_for((nx - 1) * ny), gV = grid_for(nx * (ny - 1));
    if (luo) {
        launch(gU, BS, [&] { kernels::LHS1_mid_luo_X(row, col, val, ghostTagsUV, dx, dy, dt, nu, nx, ny); });
        launch(gV, BS, [&] { kernels::LHS1_mid_luo_Y(row, col, val, ghostTagsUV, dx, dy, dt, nu, nx, ny); });
    } else {
        launch(gU, BS, [&] { kernels::LHS_mid_X_nobody(row, col, val, dx, dy, dt, nu, nx, ny); });
        launch(gV, BS, [&] { kernels::LHS_mid_Y_nobody(row, col, val, dx, dy, dt, nu, nx, ny); });
    }
    launch(gU, BS, [&] { kernels::LHS_BC_X(row, col, val, dx, dy, dt, nu, nx, ny); });
    launch(gV, BS, [&] { kernels::LHS_BC_Y(row, col, val, dx, dy, dt, nu, nx, ny); });
}

// ---- NavierStokes/intermediatePressure.cu generateLHS2 (base) and luoIBM/intermediatePressure.cu (LUO)
void ref_generateLHS2(int luo, int *row, int *col, double *val, int nnz, double *dx, double *dy, int nx,
                      int ny, double dt)
{
    for (int k = 0; k < nnz; ++k) val[k] = 0;
    int g = grid_for(nx * ny);
    if (luo)
        launch(g, BS, [&] { kernels::LHS2_mid_luo(row, col, val, dx, dy, nx, ny, dt); });
    else
        launch(g, BS, [&] { kernels::LHS2_mid_nobody(row, col, val, dx, dy, nx, ny, dt); });
    launch(g, BS, [&] { kernels::LHS2_BC(row, col, val, dx, dy, nx, ny, dt); });
}

// ---- generateRHS2: NavierStokes (intermediatePressureNoBody) and luoIBM (intermediatePressure_luo)
void ref_generateRHS2(int luo, double *rhs2, double *uhat, double *ym, double *yp, double *xm, double *xp,
                      double *dx, double *dy, int nx, int ny)
{
    int g = grid_for(nx * ny);
    if (luo)
        launch(g, BS, [&] { kernels::intermediatePressure_luo(rhs2, uhat, ym, yp, xm, xp, dx, dy, nx, ny); });
    else
        launch(g, BS, [&] { kernels::intermediatePressureNoBody(rhs2, uhat, ym, yp, xm, xp, dx, dy, nx, ny); });
}

// ---- velocityProjection (base) / luo_base::_project_velocity first two launches
void ref_project(int luo, double *u, double *uhat, double *uold, double *p, double *dx, double *dy, double dt,
                 int nx, int ny)
{
    int gU = grid_for((nx - 1) * ny), gV = grid_for(nx * (ny - 1));
    if (luo) {
        launch(gU, BS, [&] { kernels::project_velocity_luo_X(u, uhat, uold, p, dx, dt, nx, ny); });
        launch(gV, BS, [&] { kernels::project_velocity_luo_Y(u, uhat, uold, p, dy, dt, nx, ny); });
    } else {
        launch(gU, BS, [&] { kernels::project_velocity_X_nobody(u, uhat, uold, p, dx, dt, nx, ny); });
        launch(gV, BS, [&] { kernels::project_velocity_Y_nobody(u, uhat, uold, p, dy, dt, nx, ny); });
    }
}

// ---- NavierStokesSolver::initialiseNoBody velocity initial condition
void ref_initialiseVelocity(double *u, double *xu, double *yu, double *xv, double *yv, double uI, double vI,
                            double uP, double vP, double xmax, double xmin, double ymax, double ymin, int nx,
                            int ny)
{
    int gU = grid_for((nx - 1) * ny), gV = grid_for(nx * (ny - 1));
    launch(gU, BS, [&] { kernels::initialiseU(u, xu, yu, uI, uP, M_PI, xmax, xmin, ymax, ymin, nx, ny); });
    launch(gV, BS, [&] { kernels::initialiseV(u, xv, yv, vI, vP, M_PI, xmax, xmin, ymax, ymin, nx, ny); });
}

void ref_calculateCFL(double *cfl, double *u, double *dx, double *dy, int nx, int ny, double dt)
{
    launch(grid_for(nx * ny), BS, [&] { kernels::calculateCFL(cfl, u, dx, dy, nx, ny, dt); });
}

// ---- luo_base/intermediateVelocity.cu updateRobinBoundary (Uinf = Vinf = 1 there)
void ref_updateRobinBoundary(double *u, double *xp, double *dx, double dt, double Uinf, double Vinf, int nx,
                             int ny)
{
    launch(int(ny / BS) + 1, BS, [&] { kernels::updateBoundaryX(u, xp, dx, dt, Uinf, nx, ny); });
    launch(int(nx / BS) + 1, BS, [&] { kernels::updateBoundaryY(u, xp, dx, dt, Vinf, nx, ny); });
}

// ---- luo_base/tagPoints.cu tagPoints(): fills, then tag_u/tag_v/tag_p and the three zero passes
struct RefTagArrays {
    int *ghostTagsUV, *ghostTagsP, *hybridTagsUV, *hybridTagsP, *hybridTagsUV2;
    double *distance_from_intersection_to_node, *distance_between_nodes_at_IB;
    double *distance_from_u_to_body, *distance_from_v_to_body, *uv;
    double *body_intercept_x, *body_intercept_y, *image_point_x, *image_point_y;
    double *body_intercept_p_x, *body_intercept_p_y, *image_point_p_x, *image_point_p_y;
    double *x1, *y1, *x2, *y2;          // numUV (velocity segment end points)
    double *x1_p, *y1_p, *x2_p, *y2_p;  // numP
    double *x1_ip, *y1_ip, *x2_ip, *y2_ip;
};

void ref_tagPoints(RefTagArrays *A, double *bx, double *by, double *uB, double *vB, double *xu, double *yu,
                   double *xv, double *yv, int i_start, int j_start, int width_i, int height_j, int nx, int ny,
                   int totalPoints, double midX, double midY)
{
    int numUV = (nx - 1) * ny + nx * (ny - 1), numP = nx * ny;
    for (int k = 0; k < numUV; ++k) {
        A->ghostTagsUV[k] = -1; A->hybridTagsUV[k] = -1; A->hybridTagsUV2[k] = -1;
        A->distance_from_intersection_to_node[k] = 1; A->distance_between_nodes_at_IB[k] = 1;
        A->x1_ip[k] = 0; A->y1_ip[k] = 0; A->x2_ip[k] = 0; A->y2_ip[k] = 0;
        A->body_intercept_x[k] = 0; A->body_intercept_y[k] = 0;
        A->image_point_x[k] = 0; A->image_point_y[k] = 0;
    }
    for (int k = 0; k < numP; ++k) { A->ghostTagsP[k] = -1; A->hybridTagsP[k] = -1; }
    int i_end = i_start + width_i, j_end = j_start + height_j;
    int g = int((double(width_i) * height_j - 0.5) / BS) + 1;
    int g0 = int((double(i_end - i_start) - 0.5) / BS) + 1;
    launch(g, BS, [&] {
        kernels::tag_u_luo(A->hybridTagsUV, A->ghostTagsUV, A->hybridTagsUV2, bx, by, uB, vB, yu, xu,
                           A->body_intercept_x, A->body_intercept_y, A->image_point_x, A->image_point_y,
                           A->x1, A->y1, A->x2, A->y2, A->distance_from_intersection_to_node,
                           A->distance_between_nodes_at_IB, A->distance_from_u_to_body,
                           A->distance_from_v_to_body, A->uv, i_start, j_start, i_end, j_end, nx, ny,
                           totalPoints, midX, midY);
    });
    launch(g, BS, [&] {
        kernels::tag_v_luo(A->hybridTagsUV, A->ghostTagsUV, A->hybridTagsUV2, bx, by, uB, vB, yv, xv,
                           A->body_intercept_x, A->body_intercept_y, A->image_point_x, A->image_point_y,
                           A->x1, A->y1, A->x2, A->y2, A->distance_from_intersection_to_node,
                           A->distance_between_nodes_at_IB, A->distance_from_u_to_body,
                           A->distance_from_v_to_body, A->uv, i_start, j_start, i_end, j_end, nx, ny,
                           totalPoints, midX, midY);
    });
    launch(g, BS, [&] {
        kernels::tag_p_luo(A->ghostTagsP, A->hybridTagsP, bx, by, yu, xv, A->body_intercept_p_x,
                           A->body_intercept_p_y, A->image_point_p_x, A->image_point_p_y, A->x1_p, A->y1_p,
                           A->x2_p, A->y2_p, i_start, j_start, i_end, j_end, nx, ny, totalPoints, midX,
                           midY);
    });
    launch(g0, BS, [&] { kernels::zero_pressure_luo(A->ghostTagsP, i_start, j_start, i_end, j_end, nx, ny); });
    launch(g0, BS, [&] { kernels::zero_x_luo(A->ghostTagsUV, i_start, j_start, i_end, j_end, nx, ny); });
    launch(g0, BS, [&] { kernels::zero_y_luo(A->ghostTagsUV, i_start, j_start, i_end, j_end, nx, ny); });
}

struct RefInterpArrays {
    int *index1, *index2, *index3, *index4;
    double *q1coef, *q2coef, *q3coef, *q4coef;
    double *x1, *x2, *x3, *x4, *y1, *y2, *y3, *y4, *q1, *q2, *q3, *q4;
    double *image_point_u, *a0, *a1, *a2, *a3;
};

// interpolateVelocityToGhostNodeX/Y over the bounding box (dir 0 = u, 1 = v); snapshot semantics when set
void ref_interpolateVelocityToGhostNode(int dir, double *u, int set, int *ghostTagsUV, double *bx, double *by,
                                        double *uB, double *yc, double *xc, double *bix, double *biy,
                                        double *ipx, double *ipy, int i_start, int j_start, int width,
                                        int height, int nx, int ny, RefInterpArrays *R)
{
    int g = int((double(width) * height - 0.5) / BS) + 1;
    int numUV = (nx - 1) * ny + nx * (ny - 1);
    auto call = [&] {
        if (dir == 0)
            kernels::interpolateVelocityToGhostNodeX(u, set != 0, ghostTagsUV, bx, by, uB, yc, xc, bix, biy, ipx,
                                                     ipy, &i_start, &j_start, width, nx, ny, R->index1,
                                                     R->index2, R->index3, R->index4, R->q1coef, R->q2coef,
                                                     R->q3coef, R->q4coef, R->x1, R->x2, R->x3, R->x4, R->y1,
                                                     R->y2, R->y3, R->y4, R->q1, R->q2, R->q3, R->q4,
                                                     R->image_point_u);
        else
            kernels::interpolateVelocityToGhostNodeY(u, set != 0, ghostTagsUV, bx, by, uB, yc, xc, bix, biy, ipx,
                                                     ipy, &i_start, &j_start, width, nx, ny, R->index1,
                                                     R->index2, R->index3, R->index4, R->q1coef, R->q2coef,
                                                     R->q3coef, R->q4coef, R->x1, R->x2, R->x3, R->x4, R->y1,
                                                     R->y2, R->y3, R->y4, R->q1, R->q2, R->q3, R->q4,
                                                     R->image_point_u);
    };
    auto self = [&](int idx) {
        int I = i_start + idx % width, J = j_start + idx / width;
        return dir == 0 ? J * (nx - 1) + I : J * nx + I + (nx - 1) * ny;
    };
    if (set)
        launch_snapshot(g, BS, u, numUV, self, call);
    else
        launch(g, BS, call);
}

void ref_interpolateVelocityToHybridNode(int dir, double *u, double *ustar, int *hybridTagsUV, double *bx,
                                         double *by, double *uB, double *yc, double *xc, double *bix,
                                         double *biy, double *ipx, double *ipy, int i_start, int j_start,
                                         int width, int height, int nx, int ny, RefInterpArrays *R)
{
    int g = int((double(width) * height - 0.5) / BS) + 1;
    launch(g, BS, [&] {
        if (dir == 0)
            kernels::interpolateVelocityToHybridNodeX(u, ustar, hybridTagsUV, bx, by, uB, yc, xc, bix, biy, ipx,
                                                      ipy, &i_start, &j_start, width, nx, ny, R->index1,
                                                      R->index2, R->index3, R->index4, R->q1coef, R->q2coef,
                                                      R->q3coef, R->q4coef, R->x1, R->x2, R->x3, R->x4, R->y1,
                                                      R->y2, R->y3, R->y4, R->q1, R->q2, R->q3, R->q4,
                                                      R->image_point_u);
        else
            kernels::interpolateVelocityToHybridNodeY(u, ustar, hybridTagsUV, bx, by, uB, yc, xc, bix, biy, ipx,
                                                      ipy, &i_start, &j_start, width, nx, ny, R->index1,
                                                      R->index2, R->index3, R->index4, R->q1coef, R->q2coef,
                                                      R->q3coef, R->q4coef, R->x1, R->x2, R->x3, R->x4, R->y1,
                                                      R->y2, R->y3, R->y4, R->q1, R->q2, R->q3, R->q4,
                                                      R->image_point_u);
    });
}

void ref_interpolatePressureToHybridNode(double *p, double *pstar, double *u, int *hybridTagsP, double *bx,
                                         double *by, double *uB, double *uB0, double *vB, double *vB0,
                                         double *yu, double *yv, double *xu, double *xv, double *bipx,
                                         double *bipy, double *ippx, double *ippy, int i_start, int j_start,
                                         int width, int height, int nx, int ny, double dt, RefInterpArrays *R)
{
    int g = int((double(width) * height - 0.5) / BS) + 1;
    launch(g, BS, [&] {
        kernels::interpolatePressureToHybridNode(p, pstar, u, hybridTagsP, bx, by, uB, uB0, vB, vB0, yu, yv, xu,
                                                 xv, bipx, bipy, ippx, ippy, &i_start, &j_start, width, nx, ny,
                                                 dt, R->index1, R->index2, R->index3, R->index4, R->q1coef,
                                                 R->q2coef, R->q3coef, R->q4coef, R->a0, R->a1, R->a2, R->a3,
                                                 R->x1, R->x2, R->x3, R->x4, R->y1, R->y2, R->y3, R->y4, R->q1,
                                                 R->q2, R->q3, R->q4);
    });
}

void ref_interpolatePressureToGhostNode(double *p, int set, double *u, int *ghostTagsP, double *bx, double *by,
                                        double *dpdn, double *uB, double *uB0, double *vB, double *vB0,
                                        double *yu, double *yv, double *xu, double *xv, double *bipx,
                                        double *bipy, double *ippx, double *ippy, double *body_intercept_p,
                                        int i_start, int j_start, int width, int height, int nx, int ny,
                                        double dt, RefInterpArrays *R)
{
    int g = int((double(width) * height - 0.5) / BS) + 1;
    auto call = [&] {
        kernels::interpolatePressureToGhostNode(p, set != 0, u, ghostTagsP, bx, by, dpdn, uB, uB0, vB, vB0, yu, yv,
                                                xu, xv, bipx, bipy, ippx, ippy, body_intercept_p, &i_start,
                                                &j_start, width, nx, ny, dt, R->index1, R->index2, R->index3,
                                                R->index4, R->q1coef, R->q2coef, R->q3coef, R->q4coef, R->a0,
                                                R->a1, R->a2, R->a3, R->x1, R->x2, R->x3, R->x4, R->y1, R->y2,
                                                R->y3, R->y4, R->q1, R->q2, R->q3, R->q4);
    };
    auto self = [&](int idx) { return (j_start + idx / width) * nx + i_start + idx % width; };
    if (set)
        launch_snapshot(g, BS, p, nx * ny, self, call);
    else
        launch(g, BS, call);
}

// luoIBM weightUhat (dir 0/1) and weightPressure's weightP (dir 2)
void ref_weight(int dir, double *f, double *fstar, int *ghostTags, int *hybridTags, double *yc, double *xc,
                double *bix, double *biy, double *ipx, double *ipy, int i_start, int j_start, int width,
                int height, int nx, int ny)
{
    int g = int((double(width) * height - 0.5) / BS) + 1;
    launch(g, BS, [&] {
        if (dir == 0)
            kernels::weightX(f, fstar, ghostTags, hybridTags, yc, xc, bix, biy, ipx, ipy, &i_start, &j_start,
                             width, nx, ny);
        else if (dir == 1)
            kernels::weightY(f, fstar, ghostTags, hybridTags, yc, xc, bix, biy, ipx, ipy, &i_start, &j_start,
                             width, nx, ny);
        else
            kernels::weightP(f, fstar, ghostTags, hybridTags, yc, xc, bix, biy, ipx, ipy, &i_start, &j_start,
                             width, nx, ny);
    });
}

// luoIBM::zeroVelocity / luo_base::_project_velocity setInsideVelocity (grid over numUV threads or numU)
void ref_setInsideVelocity(int *ghostTags, double *u, double *uB, double *vB, int nx, int ny, int grid_count)
{
    launch(grid_for(grid_count), BS, [&] {
        // The reference kernel indexes v with the u index map; for J = ny-1 its v index
        // lies past the end of u.  Those threads are skipped here (their access is
        // out of bounds in the reference as well and leaves the field unchanged).
        int i = threadIdx.x + blockDim.x * blockIdx.x;
        int I = i % (nx - 1), J = i / (nx - 1);
        if (i < (nx - 1) * ny && J * nx + I + (nx - 1) * ny >= (nx - 1) * ny + nx * (ny - 1)) {
            int iu = J * (nx - 1) + I;
            u[iu] = (ghostTags[iu] != 0) * u[iu] + (ghostTags[iu] == 0) * uB[0];
            return;
        }
        kernels::setInsideVelocity(ghostTags, u, uB, vB, nx, ny);
    });
}

// luo_base::calculateForce: six kernels, each reduced by a serial sum (thrust::reduce on the GPU)
void ref_calculateForce(double *u, double *uold, double *p, int *ghostTagsUV, double nu, double *dx, double *dy,
                        double dt, int nx, int ny, int I, int J, int ncx, int ncy, double *fx, double *fy)
{
    std::vector<double> FxX(ncy), FxY(ncx + 1), FxU((ncx + 1) * ncy);
    std::vector<double> FyX(ncy + 1), FyY(ncx), FyU((ncx + 1) * ncy);
    int g = int((double(ncx + ncy + 1) - 0.5) / BS) + 1;
    int gX = int((double((ncx + 1) * ncy) - 0.5) / BS) + 1;
    int gY = int((double(ncx * (ncy + 1)) - 0.5) / BS) + 1;
    launch(g, BS, [&] { kernels::dragLeftRight(FxX.data(), u, p, nu, dx, dy, nx, ny, I, J, ncx, ncy); });
    launch(g, BS, [&] { kernels::dragBottomTop(FxY.data(), u, nu, dx, dy, nx, ny, I, J, ncx, ncy); });
    launch(gX, BS, [&] {
        kernels::dragUnsteady(FxU.data(), u, uold, ghostTagsUV, dx, dy, dt, nx, ny, I, J, ncx, ncy);
    });
    double sxx = 0, sxy = 0, sxu = 0;
    for (double v : FxX) sxx += v;
    for (double v : FxY) sxy += v;
    for (double v : FxU) sxu += v;
    *fx = sxx + sxy + sxu;
    launch(g, BS, [&] { kernels::liftLeftRight(FyX.data(), u, nu, dx, dy, nx, ny, I, J, ncx, ncy); });
    launch(g, BS, [&] { kernels::liftBottomTop(FyY.data(), u, p, nu, dx, dy, nx, ny, I, J, ncx, ncy); });
    launch(gY, BS, [&] {
        kernels::liftUnsteady(FyU.data(), u, uold, ghostTagsUV, dx, dy, dt, nx, ny, I, J, ncx, ncy);
    });
    double syx = 0, syy = 0, syu = 0;
    for (double v : FyX) syx += v;
    for (double v : FyY) syy += v;
    for (double v : FyU) syu += v;
    *fy = syx + syy + syu;
}

// luo_base::luoForce (luo_base/calculateForce.cu:76-98, not called by the reference's
// step): its four kernels on a grid over the body points, with its arguments as
// written (the pressure kernel gets startI for both starts), forces summed serially
// (thrust::reduce on the GPU).  terms: pressure, du/dn, dv/dn per point.
void ref_luoForce(double *bip, double *bip_x, double *bip_y, double *bx, double *by, double *xu, double *yu,
                  double *xv, double *yv, int *ghostTagsP, double *u, double *uB, double *vB, int startI, int startJ,
                  int ncx, int ncy, int totalPoints, int nx, int ny, double midX, double midY, double nu,
                  double mid_h, double *terms, double *fx, double *fy)
{
    std::vector<double> fX(totalPoints), fY(totalPoints);
    double *pr = terms, *du = terms + totalPoints, *dv = terms + 2 * totalPoints;
    int sI = startI, sJ = startJ;
    int g = grid_for(totalPoints);
    launch(g, BS, [&] {
        kernels::force_pressure(pr, bip, bip_x, bip_y, bx, by, xv, yu, ghostTagsP, &sI, &sI, ncx, ncy, totalPoints,
                                nx, ny, midX, midY);
    });
    launch(g, BS, [&] {
        kernels::force_velocity_x(du, uB, u, bx, by, xu, yu, &sI, &sJ, ncx, ncy, totalPoints, nx, ny, midX, midY,
                                  mid_h);
    });
    launch(g, BS, [&] {
        kernels::force_velocity_y(dv, vB, u, bx, by, xv, yv, &sI, &sJ, ncx, ncy, totalPoints, nx, ny, midX, midY,
                                  mid_h);
    });
    launch(g, BS, [&] {
        kernels::force(fX.data(), fY.data(), pr, du, dv, bx, by, totalPoints, midX, midY, nu);
    });
    double sx = 0, sy = 0;
    for (double v : fX) sx += v;
    for (double v : fY) sy += v;
    *fx = sx;
    *fy = sy;
}

// luo_base::set_movement's update_body_viv (the reference grid also writes index totalPoints,
// one past the end; that write is dropped here)
void ref_update_body_viv(double *Bx, double *uB, double *Bdx, double unew, double midX, int totalPoints)
{
    launch(int(totalPoints / BS) + 1, BS, [&] {
        int i = threadIdx.x + blockDim.x * blockIdx.x;
        if (i >= totalPoints) return;
        kernels::update_body_viv(Bx, uB, Bdx, unew, midX, totalPoints);
    });
}

// ---- modified Fadlun (fadlunModified.cu, FadlunModified/*.cu) ----------------------------
// fadlunModified::generateLHS1 on zero-initialised COO arrays (the reference's
// cusp::coo_matrix resize value-initialises them): Fadlun mid rows, base boundary rows
void ref_fadlun_lhs1(int *row, int *col, double *val, int nnz, int *hybridTagsUV, int *hybridTagsUV2,
                     int *ghostTagsUV, double *dist_node, double *dist_between, double *dx, double *dy, double dt,
                     double nu, int nx, int ny)
{
    for (int k = 0; k < nnz; ++k) row[k] = col[k] = 0, val[k] = 0;
    int gU = grid_for((nx - 1) * ny), gV = grid_for(nx * (ny - 1));
    launch(gU, BS, [&] { kernels::LHS_mid_X(row, col, val, hybridTagsUV, hybridTagsUV2, ghostTagsUV, dist_node,
                                            dist_between, dx, dy, dt, nu, nx, ny); });
    launch(gV, BS, [&] { kernels::LHS_mid_Y(row, col, val, hybridTagsUV, hybridTagsUV2, ghostTagsUV, dist_node,
                                            dist_between, dx, dy, dt, nu, nx, ny); });
    launch(gU, BS, [&] { kernels::LHS_BC_X(row, col, val, dx, dy, dt, nu, nx, ny); });
    launch(gV, BS, [&] { kernels::LHS_BC_Y(row, col, val, dx, dy, dt, nu, nx, ny); });
}

// fadlunModified::generateLHS2: values filled with 0, Fadlun mid rows, base boundary rows
void ref_fadlun_lhs2(int *row, int *col, double *val, int nnz, double *dist_u, double *dist_v, int *ghostTagsP,
                     int *hybridTagsP, double *dx, double *dy, int nx, int ny, double dt)
{
    for (int k = 0; k < nnz; ++k) row[k] = col[k] = 0, val[k] = 0;
    int g = grid_for(nx * ny);
    launch(g, BS, [&] { kernels::LHS2_mid(row, col, val, dist_u, dist_v, ghostTagsP, hybridTagsP, dx, dy, nx, ny, dt); });
    launch(g, BS, [&] { kernels::LHS2_BC(row, col, val, dx, dy, nx, ny, dt); });
}

// the IB part of fadlunModified::generateRHS1 (after generateRHS)
void ref_fadlun_update_rhs1(int *hybridTagsUV, int *ghostTagsUV, double *rhs, double *dist_node,
                            double *dist_between, double *uv, int nx, int ny)
{
    int gU = grid_for((nx - 1) * ny), gV = grid_for(nx * (ny - 1));
    launch(gU, BS, [&] { kernels::updateRHS1forIBX(hybridTagsUV, ghostTagsUV, rhs, dist_node, dist_between, uv, nx, ny); });
    launch(gV, BS, [&] { kernels::updateRHS1forIBY(hybridTagsUV, ghostTagsUV, rhs, dist_node, dist_between, uv, nx, ny); });
}

// fadlunModified::generateRHS2
void ref_fadlun_rhs2(double *rhs2, double *uhat, int *ghostTagsP, int *hybridTagsP, int *ghostTagsUV,
                     double *dist_u, double *dist_v, double *ym, double *yp, double *xm, double *xp, double *dx,
                     double *dy, int nx, int ny)
{
    int g = grid_for(nx * ny);
    launch(g, BS, [&] { kernels::intermediatePressure(rhs2, uhat, ghostTagsP, hybridTagsP, ghostTagsUV, dist_u,
                                                      dist_v, ym, yp, xm, xp, dx, dy, nx, ny); });
}

// fadlunModified::_project_velocity
void ref_fadlun_project(double *u, double *uhat, double *uold, double *p, int *ghostTagsP, double *dx, double *dy,
                        double dt, int nx, int ny)
{
    int gU = grid_for((nx - 1) * ny), gV = grid_for(nx * (ny - 1));
    launch(gU, BS, [&] { kernels::project_velocity_X(u, uhat, uold, p, ghostTagsP, dx, dt, nx, ny); });
    launch(gV, BS, [&] { kernels::project_velocity_Y(u, uhat, uold, p, ghostTagsP, dy, dt, nx, ny); });
}

// ---- embedded method (luo_iter.cu, luo_iter/*.cu) -------------------------------------
// alpha_u (kind 0), alpha_v (1), alpha_p (2) on the reference's grid, running only the
// threads whose node lies in the grid (the others read past the arrays)
void ref_iter_alpha(int kind, double *alpha, int *ghost, int *hybrid, double *yc, double *xc, double *bix,
                    double *biy, double *ipx, double *ipy, int i_start, int j_start, int width, int nx, int ny)
{
    const int nU = (nx - 1) * ny;
    const int g = grid_for(kind == 2 ? nx * ny : nU);
    blockDim = {(unsigned)BS, 1, 1};
    gridDim = {(unsigned)g, 1, 1};
    for (int b = 0; b < g; ++b)
        for (int t = 0; t < BS; ++t) {
            const int idx = b * BS + t, I = i_start + idx % width, J = j_start + idx / width;
            if (kind == 0 && (J >= ny || I >= nx - 1)) continue;
            if (kind == 1 && (J * nx + I > nx * (ny - 1) || J >= ny - 1)) continue;
            if (kind == 2 && (J * nx + I > nx * ny || J >= ny)) continue;
            blockIdx = {(unsigned)b, 0, 0};
            threadIdx = {(unsigned)t, 0, 0};
            if (kind == 0)
                kernels::alpha_u(alpha, ghost, hybrid, yc, xc, bix, biy, ipx, ipy, &i_start, &j_start, width, nx, ny);
            else if (kind == 1)
                kernels::alpha_v(alpha, ghost, hybrid, yc, xc, bix, biy, ipx, ipy, &i_start, &j_start, width, nx, ny);
            else
                kernels::alpha_p(alpha, ghost, hybrid, yc, xc, bix, biy, ipx, ipy, &i_start, &j_start, width, nx, ny);
        }
}

// intermediate_velocity_size_lhs + intermediate_velocity_calculate_lhs on zeroed arrays of nnz
// entries; returns the reference's nnz (plain + max count)
int ref_iter_lhs1(int *row, int *col, double *val, int nnz, double *dx, double *dy, double dt, double nu, int nx,
                  int ny, int *hyb, int *ghost, double *ns_rhs, double *interp_rhs, int *count, int *i1, int *i2,
                  int *i3, int *i4, double *xu, double *yu, double *xv, double *yv, double *alpha, double *uB,
                  double *vB, double *c1, double *c2, double *c3, double *c4, double *q1, double *q2, double *q3,
                  double *q4, int i_start, int j_start, int width, int height)
{
    const int nUV = (nx - 1) * ny + nx * (ny - 1);
    for (int k = 0; k < nUV; ++k) count[k] = 0;
    launch(1, 1, [&] { kernels::size_LHS1(hyb, count, &i_start, &j_start, width, height, nx, ny); });
    int mx = 0;
    for (int k = 0; k < nUV; ++k) mx = count[k] > mx ? count[k] : mx;
    const int need = (nx - 1) * ny * 5 - 2 * (nx - 1) - ny * 2 + nx * (ny - 1) * 5 - 2 * nx - 2 * (ny - 1) + mx;
    if (need > nnz) return -need;
    for (int k = 0; k < need; ++k) row[k] = col[k] = 0, val[k] = 0;
    int gU = grid_for((nx - 1) * ny), gV = grid_for(nx * (ny - 1));
    launch(gU, BS, [&] { kernels::LHS1_mid_iter_X(row, col, val, dx, dy, dt, nu, nx, ny, hyb, ghost, ns_rhs,
                                                  interp_rhs, count, i1, i2, i3, i4, xu, yu, alpha, uB, c1, c2, c3,
                                                  c4, q1, q2, q3, q4); });
    launch(gV, BS, [&] { kernels::LHS1_mid_iter_Y(row, col, val, dx, dy, dt, nu, nx, ny, hyb, ghost, ns_rhs,
                                                  interp_rhs, count, i1, i2, i3, i4, xv, yv, alpha, vB, c1, c2, c3,
                                                  c4, q1, q2, q3, q4); });
    launch(gU, BS, [&] { kernels::LHS_BC_X(row, col, val, dx, dy, dt, nu, nx, ny); });
    launch(gV, BS, [&] { kernels::LHS_BC_Y(row, col, val, dx, dy, dt, nu, nx, ny); });
    return need;
}

// intermediate_velocity_update_rhs (both kernels on the u grid)
void ref_iter_update_rhs1(double *rhs1, double *ns_rhs, double *interp_rhs, int nx, int ny)
{
    int gU = grid_for((nx - 1) * ny);
    launch(gU, BS, [&] { kernels::update_rhs1_x(rhs1, ns_rhs, interp_rhs, nx, ny); });
    launch(gU, BS, [&] { kernels::update_rhs1_y(rhs1, ns_rhs, interp_rhs, nx, ny); });
}

// poisson_size_lhs + poisson_calculate_lhs
int ref_iter_lhs2(int *row, int *col, double *val, int nnz, double *dx, double *dy, int nx, int ny, double dt,
                  int *count, double *ns_rhs, double *interp_rhs, int *hyb, int *ghost, double *alpha, double *dpdn,
                  int *i1, int *i2, int *i3, int *i4, double *c1, double *c2, double *c3, double *c4, double *q1,
                  double *q2, double *q3, double *q4, int i_start, int j_start, int width, int height)
{
    for (int k = 0; k < nx * ny; ++k) count[k] = 0;
    launch(1, 1, [&] { kernels::size_LHS2(hyb, count, &i_start, &j_start, width, height, nx, ny); });
    int mx = 0;
    for (int k = 0; k < nx * ny; ++k) mx = count[k] > mx ? count[k] : mx;
    const int need = nx * ny * 5 - 2 * nx - ny * 2 + mx;
    if (need > nnz) return -need;
    for (int k = 0; k < need; ++k) row[k] = col[k] = 0, val[k] = 0;
    int g = grid_for(nx * ny);
    launch(g, BS, [&] { kernels::LHS2_mid_iter(row, col, val, dx, dy, nx, ny, dt, count, ns_rhs, interp_rhs, hyb,
                                               ghost, alpha, dpdn, i1, i2, i3, i4, c1, c2, c3, c4, q1, q2, q3, q4,
                                               1); });
    launch(g, BS, [&] { kernels::LHS2_BC(row, col, val, dx, dy, nx, ny, dt); });
    return need;
}

// poisson_update_rhs
void ref_iter_update_rhs2(double *rhs2, double *ns_rhs, double *interp_rhs, int nx, int ny)
{
    int g = grid_for(nx * ny);
    launch(g, BS, [&] { kernels::update_rhs2(rhs2, ns_rhs, interp_rhs, nx, ny); });
}

}  // extern "C"
