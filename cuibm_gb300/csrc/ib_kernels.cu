// Immersed-boundary kernels of the external (Luo) ghost-node method.
//
// Replaces luo_base/kernels/tagPoints.cu (tag_u_luo, tag_v_luo, tag_p_luo, zero_*_luo),
// luo_base/kernels/biLinearInterpolation.cu (ghost and hybrid interpolation of velocity
// and pressure), luoIBM/kernels/weight.cu, luo_base/kernels/intermediateVelocity.cu
// (setInsideVelocity), FadlunModified/kernels/intermediateVelocity.cu (updateBoundaryX/Y),
// FadlunModified/kernels/calculateForce.cu (control-volume force) and
// luo_base/kernels/structure.cu (prescribed motion).
//
// This translation unit is compiled with -fmad=false: every tag decision uses the
// reference's arithmetic exactly, so tag arrays are bit-identical to the
// reference's.  Intercepts use the closed form of the reference's trigonometric
// expression (intercept_dev), so they and the interpolation weights are exact
// functions of correctly rounded operations.
//
// Determinism.  The reference's tagging threads write into neighbouring nodes
// (ghost tags, body intercepts, image points), so the result depends on thread
// order; its ghost interpolation overwrites the field it reads.  Here:
//  * tagging runs in two passes: each node first records every write it would
//    make (its last write per target and field, in its own segment order), then
//    each target node resolves the records of its five possible writers in
//    global thread order (south, west, self, east, north) - the outcome of the
//    reference's grid run one thread after another;
//  * ghost interpolation stages the new values and applies them in a second
//    launch, so every node reads the field as it was before (what the
//    reference's GPU launch does: all loads precede all stores).
#include <algorithm>
#include <cmath>
#include <vector>

#include "ib_plan.h"
#include "solver.h"

namespace cuibm {

#define IB_EPS 1.e-10

// ---- tagging records ------------------------------------------------------------
// slots: 0 self, 1 west (n-1), 2 east (n+1), 3 south (n-sv), 4 north (n+sv)
struct TagRecords {
    int *flags;      // bits 0-4 ghost written per slot, 8-12 intercept written per slot,
                     // 16 final self block ran, 17 dist slot A written, 18 dist slot B written, 19 hybrid-P self
    int *hyb, *hyb2;
    double *dnode, *dbetween, *uv;
    double *bi;      // [idx][5 slots][4]: bix, biy, ipx, ipy
    double *distA, *distB;
    int nrec;
};

struct TagGeom {
    const double *bx, *by, *vel;
    const double *xc, *yc;
    int i0, j0, width, height, nthreads;
    int nx, ny, total;
    double midX, midY;
    const double *motion;  // moving body: the centre is motion[0], motion[1] (set on the device)
};

// Foot of the perpendicular from (px, py) onto the line through body points k and l.
// The reference (tagPoints.cu, e.g. :107-117) takes the angle th at point k from the
// law of cosines with acos, then moves a / tan(th) along the segment, a = b sin(th).
// That distance is b cos(th) = (p^2 + b^2 - o^2) / (2 p), computed here with +, -, x, /
// and sqrt only: correctly rounded operations, so (with -fmad=false) the intercepts
// and every interpolation weight built from them are the same on the GPU and in a
// host restatement, bit for bit, where the transcendental form differed in the last
// bits between CUDA's and the host library's acos/sin/tan.
__device__ __forceinline__ void intercept_dev(const double *bx, const double *by, int k, int l, double px,
                                              double py, double *ix, double *iy)
{
    const double dxs = bx[l] - bx[k], dys = by[l] - by[k];
    const double dxo = bx[l] - px, dyo = by[l] - py;
    const double dxb = px - bx[k], dyb = py - by[k];
    const double p = sqrt(dxs * dxs + dys * dys);
    const double o = sqrt(dxo * dxo + dyo * dyo);
    const double b = sqrt(dxb * dxb + dyb * dyb);
    const double t = (p * p + b * b - o * o) / (2 * p);
    *iy = by[k] + (by[l] - by[k]) / p * t;
    *ix = bx[k] + (bx[l] - bx[k]) / p * t;
}

struct RecWriter {
    int flags = 0;
    double bi[5][4];
    __device__ void ghost(int slot) { flags |= 1 << slot; }
    __device__ void point(int slot, double bix, double biy, double ipx, double ipy)
    {
        flags |= 1 << (8 + slot);
        bi[slot][0] = bix;
        bi[slot][1] = biy;
        bi[slot][2] = ipx;
        bi[slot][3] = ipy;
    }
};

// one velocity node (KIND 0 = u: tag_u_luo, 1 = v: tag_v_luo)
template <int KIND>
__global__ void k_tag_velocity_records(TagGeom G, TagRecords R)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= G.nthreads) return;
    const int nx = G.nx, ny = G.ny, nU = (nx - 1) * ny;
    const int I = G.i0 + idx % G.width, J = G.j0 + idx / G.width;
    const int sv = KIND == 0 ? nx - 1 : nx;
    const int n = KIND == 0 ? J * (nx - 1) + I : J * nx + I + nU;
    RecWriter w;
    int flags_extra = 0;
    if (KIND == 0 ? (n >= nU) : (n >= nU + nx * (ny - 1))) {
        R.flags[idx] = 0;
        return;
    }
    const double *bx = G.bx, *by = G.by, *vel = G.vel, *xc = G.xc, *yc = G.yc;
    const double midX = G.motion ? G.motion[0] : G.midX, midY = G.motion ? G.motion[1] : G.midY;
    int k = G.total - 1, l = 0;
    bool outsideX = true, outsideY = true, flag = false;
    int fX = -1, fY = -1, f2X = -1, f2Y = -1;
    double uvX = 0.0, uvY = 0.0, Xa = 1.0, Ya = 1.0, Xb = 1.0, Yb = 1.0, x = 0.0, y = 0.0;
    double distA = 0, distB = 0;
    if (KIND == 0) flags_extra |= 1 << 17;  // dist_u_body[ip] = 0 at thread start
    double ix, iy;
    while (l < G.total && (KIND == 1 || !flag)) {
        int bottom, top, left, right;
        if (by[k] > by[l]) { bottom = l; top = k; } else { bottom = k; top = l; }
        if (bx[k] > bx[l]) { left = l; right = k; } else { left = k; right = l; }
        if (by[bottom] - IB_EPS < yc[J] && by[top] - IB_EPS > yc[J] && (KIND == 0 || !flag)) {
            if (fabs(by[l] - by[k]) > IB_EPS) {
                x = bx[k] + (bx[l] - bx[k]) * (yc[J] - by[k]) / (by[l] - by[k]);
                uvX = vel[k] + (vel[l] - vel[k]) * (yc[J] - by[k]) / (by[l] - by[k]);
                if (x > xc[I] + IB_EPS) outsideX = !outsideX;
                if (x > xc[I - 1] + IB_EPS && x < xc[I] - IB_EPS) {
                    fX = n;
                    f2X = n + 1;
                    if (x > midX + IB_EPS) {
                        w.ghost(1);
                        intercept_dev(bx, by, k, l, xc[I - 1], yc[J], &ix, &iy);
                        w.point(1, ix, iy, ix + (ix - xc[I - 1]), iy + (iy - yc[J]));
                        intercept_dev(bx, by, k, l, xc[I], yc[J], &ix, &iy);
                        w.point(0, ix, iy, 2 * xc[I] - ix, 2 * yc[J] - iy);
                    }
                    Xa = xc[I] - x;
                    Xb = xc[I + 1] - xc[I];
                    if (KIND == 0 && x > midX) distA = Xa;
                } else if (x > xc[I] + IB_EPS && x < xc[I + 1] - IB_EPS) {
                    fX = n;
                    f2X = n - 1;
                    if (x < midX - IB_EPS) {
                        w.ghost(2);
                        intercept_dev(bx, by, k, l, xc[I + 1], yc[J], &ix, &iy);
                        w.point(2, ix, iy, ix + (ix - xc[I + 1]), iy + (iy - yc[J]));
                        intercept_dev(bx, by, k, l, xc[I], yc[J], &ix, &iy);
                        w.point(0, ix, iy, 2 * xc[I] - ix, 2 * yc[J] - iy);
                    }
                    Xa = x - xc[I];
                    Xb = xc[I] - xc[I - 1];
                    if (KIND == 0 && x < midX) {
                        distB = Xa;
                        flags_extra |= 1 << 18;
                    }
                } else if (fabs(x - xc[I]) < IB_EPS && fabs(midX - xc[I]) > fabs(midY - yc[J])) {
                    outsideX = true;
                    fX = n;
                    if (x < midX) {
                        w.ghost(2);
                        f2X = n - 1;
                        w.point(2, xc[I], yc[J], xc[I - 1], yc[J]);
                        w.point(0, xc[I], yc[J], xc[I - 1], yc[J]);
                        Xa = 0;
                        Xb = xc[I] - xc[I - 1];
                    }
                    if (x > midX) {
                        w.ghost(1);
                        f2X = n + 1;
                        w.point(1, xc[I], yc[J], xc[I + 1], yc[J]);
                        w.point(0, xc[I], yc[J], xc[I + 1], yc[J]);
                        Xa = 0;
                        Xb = xc[I + 1] - xc[I];
                    }
                    flag = true;
                }
            }
        }
        if (bx[left] - IB_EPS < xc[I] && bx[right] - IB_EPS > xc[I] && (KIND == 0 || !flag)) {
            if (fabs(bx[l] - bx[k]) > IB_EPS) {
                y = by[k] + (by[l] - by[k]) * (xc[I] - bx[k]) / (bx[l] - bx[k]);
                uvY = vel[k] + (vel[l] - vel[k]) * (xc[I] - bx[k]) / (bx[l] - bx[k]);
                if (y > yc[J] + IB_EPS) outsideY = !outsideY;
                if (y > yc[J - 1] + IB_EPS && y < yc[J] - IB_EPS) {
                    fY = n;
                    f2Y = n + sv;
                    if (y > midY + IB_EPS) {
                        w.ghost(3);
                        intercept_dev(bx, by, k, l, xc[I], yc[J - 1], &ix, &iy);
                        w.point(3, ix, iy, ix + (ix - xc[I]), iy + (iy - yc[J - 1]));
                        intercept_dev(bx, by, k, l, xc[I], yc[J], &ix, &iy);
                        w.point(0, ix, iy, 2 * xc[I] - ix, 2 * yc[J] - iy);
                    }
                    Ya = yc[J] - y;
                    Yb = yc[J + 1] - yc[J];
                    if (KIND == 1 && outsideY) {
                        distA = Ya;
                        flags_extra |= 1 << 17;
                    }
                } else if (y > yc[J] + IB_EPS && y < yc[J + 1] - IB_EPS) {
                    fY = n;
                    f2Y = n - sv;
                    if (y < midY - IB_EPS) {
                        w.ghost(4);
                        intercept_dev(bx, by, k, l, xc[I], yc[J + 1], &ix, &iy);
                        w.point(4, ix, iy, ix + (ix - xc[I]), iy + (iy - yc[J + 1]));
                        intercept_dev(bx, by, k, l, xc[I], yc[J], &ix, &iy);
                        w.point(0, ix, iy, 2 * xc[I] - ix, 2 * yc[J] - iy);
                    }
                    Ya = y - yc[J];
                    Yb = yc[J] - yc[J - 1];
                    if (KIND == 1 && outsideY) {
                        distB = Ya;
                        flags_extra |= 1 << 18;
                    }
                } else if (KIND == 0 ? (fabs(y - yc[J]) < IB_EPS && fabs(y - midY) > fabs(x - midX))
                                     : (fabs(y - yc[J]) < IB_EPS && fabs(midY - yc[J]) > fabs(midX - xc[I]))) {
                    outsideY = true;
                    fY = n;
                    if (y < midY) {
                        w.ghost(4);
                        f2X = n - sv;  // the reference sets the x-ray second flag here
                        w.point(4, xc[I], yc[J], xc[I], yc[J - 1]);
                        w.point(0, xc[I], yc[J], xc[I], yc[J - 1]);
                        Ya = 0;
                        Yb = yc[J] - yc[J - 1];
                    }
                    if (y > midY) {
                        w.ghost(3);
                        f2X = n + sv;
                        w.point(3, xc[I], yc[J], xc[I], yc[J + 1]);
                        w.point(0, xc[I], yc[J], xc[I], yc[J + 1]);
                        Ya = 0;
                        Yb = yc[J + 1] - yc[J];
                    }
                    flag = true;
                }
            }
        }
        k = l;
        l = l + 1;
    }
    const bool useX = outsideX && fX >= 0, useY = outsideY && fY >= 0;
    int hy = -1, hy2 = -1;
    double dn = 0, db = 0, uvv = 0;
    bool final_ = false;
    if (KIND == 0 ? useX : (useX && !useY)) {
        final_ = true;
        hy = fX;
        hy2 = f2X;
        dn = Xa;
        db = Xb;
        uvv = uvX;
    } else if (useY) {
        final_ = true;
        hy = fY;
        hy2 = f2Y;
        dn = Ya;
        db = Yb;
        uvv = uvY;
    }
    R.flags[idx] = w.flags | flags_extra | (final_ ? 1 << 16 : 0);
    R.hyb[idx] = hy;
    R.hyb2[idx] = hy2;
    R.dnode[idx] = dn;
    R.dbetween[idx] = db;
    R.uv[idx] = uvv;
    R.distA[idx] = distA;
    R.distB[idx] = distB;
    for (int s = 0; s < 5; ++s)
        if (w.flags & (1 << (8 + s)))
            for (int q = 0; q < 4; ++q) R.bi[(size_t)idx * 20 + s * 4 + q] = w.bi[s][q];
}

// one pressure node of tag_p_luo
__global__ void k_tag_pressure_records(TagGeom G, TagRecords R)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= G.nthreads) return;
    const int nx = G.nx;
    const int I = G.i0 + idx % G.width, J = G.j0 + idx / G.width, ip = J * nx + I;
    RecWriter w;
    int extra = 0;
    if (ip >= nx * G.ny) {
        R.flags[idx] = 0;
        return;
    }
    const double *bx = G.bx, *by = G.by, *xv = G.xc, *yu = G.yc;
    const double midX = G.motion ? G.motion[0] : G.midX, midY = G.motion ? G.motion[1] : G.midY;
    int k = G.total - 1, l = 0;
    bool flag = false;
    double x, y, ix, iy;
    while (l < G.total) {
        int bottom, top, left, right;
        if (by[k] > by[l]) { bottom = l; top = k; } else { bottom = k; top = l; }
        if (bx[k] > bx[l]) { left = l; right = k; } else { left = k; right = l; }
        if (by[bottom] - IB_EPS < yu[J] && by[top] - IB_EPS > yu[J] && !flag) {
            if (fabs(by[l] - by[k]) > IB_EPS) {
                x = bx[k] + (bx[l] - bx[k]) * (yu[J] - by[k]) / (by[l] - by[k]);
                bool g1 = x > midX + IB_EPS && x > xv[I] + IB_EPS + IB_EPS && x < xv[I + 1] - IB_EPS;
                bool g2 = x < midX + IB_EPS && x < xv[I] - IB_EPS && x > xv[I - 1] + IB_EPS;
                if (g1 || g2) {
                    w.ghost(0);
                    intercept_dev(bx, by, k, l, xv[I], yu[J], &ix, &iy);
                    w.point(0, ix, iy, ix + (ix - xv[I]), iy + (iy - yu[J]));
                }
                bool h1 = x > midX + IB_EPS && x < xv[I] - IB_EPS && x > xv[I - 1] + IB_EPS;
                bool h2 = x < midX + IB_EPS && x > xv[I] + IB_EPS && x < xv[I + 1] - IB_EPS;
                if (h1 || h2) {
                    extra |= 1 << 19;
                    intercept_dev(bx, by, k, l, xv[I], yu[J], &ix, &iy);
                    w.point(0, ix, iy, 2 * xv[I] - ix, 2 * yu[J] - iy);
                }
                if (fabs(x - xv[I]) < IB_EPS && fabs(midX - xv[I]) > fabs(midY - yu[J])) {
                    extra |= 1 << 19;
                    if (x < midX) {
                        w.ghost(2);
                        w.point(2, xv[I], yu[J], xv[I - 1], yu[J]);
                        w.point(0, xv[I], yu[J], xv[I - 1], yu[J]);
                    } else if (x > midX) {
                        w.ghost(1);
                        w.point(1, xv[I], yu[J], xv[I + 1], yu[J]);
                        w.point(0, xv[I], yu[J], xv[I + 1], yu[J]);
                    }
                    flag = true;
                }
            }
        }
        if (bx[left] - IB_EPS < xv[I] && bx[right] - IB_EPS > xv[I] && !flag) {
            if (fabs(bx[l] - bx[k]) > IB_EPS) {
                y = by[k] + (by[l] - by[k]) * (xv[I] - bx[k]) / (bx[l] - bx[k]);
                bool g1 = y > midY + IB_EPS && y > yu[J] + IB_EPS && y < yu[J + 1] - IB_EPS;
                bool g2 = y < midY + IB_EPS && y < yu[J] - IB_EPS && y > yu[J - 1] + IB_EPS;
                if (g1 || g2) {
                    w.ghost(0);
                    intercept_dev(bx, by, k, l, xv[I], yu[J], &ix, &iy);
                    w.point(0, ix, iy, ix + (ix - xv[I]), iy + (iy - yu[J]));
                }
                bool h1 = y > midY + IB_EPS && y < yu[J] - IB_EPS && y > yu[J - 1] + IB_EPS;
                bool h2 = y < midY + IB_EPS && y > yu[J] + IB_EPS && y < yu[J + 1] - IB_EPS;
                if (h1 || h2) {
                    extra |= 1 << 19;
                    intercept_dev(bx, by, k, l, xv[I], yu[J], &ix, &iy);
                    w.point(0, ix, iy, 2 * xv[I] - ix, 2 * yu[J] - iy);
                }
                if (fabs(y - yu[J]) < IB_EPS && fabs(midY - yu[J]) > fabs(midX - xv[I])) {
                    extra |= 1 << 19;
                    if (y < midY) {
                        w.ghost(4);
                        w.point(4, xv[I], yu[J], xv[I], yu[J - 1]);
                        w.point(0, xv[I], yu[J], xv[I], yu[J - 1]);
                    }
                    if (y > midY) {
                        w.ghost(3);
                        w.point(3, xv[I], yu[J], xv[I], yu[J + 1]);
                        w.point(0, xv[I], yu[J], xv[I], yu[J + 1]);
                    }
                    flag = true;
                }
            }
        }
        k = l;
        l = l + 1;
    }
    R.flags[idx] = w.flags | extra;
    for (int s = 0; s < 5; ++s)
        if (w.flags & (1 << (8 + s)))
            for (int q = 0; q < 4; ++q) R.bi[(size_t)idx * 20 + s * 4 + q] = w.bi[s][q];
}

struct TagOut {
    int *ghost, *hyb, *hyb2;
    double *dnode, *dbetween, *uv, *bix, *biy, *ipx, *ipy, *dist;
};

// Resolve the writes of the five possible writers of every target node of the box
// (extended by one node on each side) in the reference's serial thread order.
// CLS: 0 u, 1 v, 2 p.
template <int CLS>
__global__ void k_tag_resolve(TagGeom G, TagRecords R, TagOut O)
{
    const int ew = G.width + 2, rows = (G.nthreads + G.width - 1) / G.width;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ew * (rows + 2)) return;
    const int i = t % ew - 1, j = t / ew - 1;  // box coordinates of the target
    const int nx = G.nx, ny = G.ny, nU = (nx - 1) * ny;
    const int I = G.i0 + i, J = G.j0 + j;
    if (I < 0 || J < 0 || I >= nx || J >= ny) return;
    int n, limit;
    if (CLS == 0) { n = J * (nx - 1) + I; limit = nU; if (I >= nx - 1) return; }
    else if (CLS == 1) { n = J * nx + I + nU; limit = nU + nx * (ny - 1); if (J >= ny - 1) return; }
    else { n = J * nx + I; limit = nx * ny; }
    if (n >= limit) return;
    // writers in serial order with the slot through which each reaches this target
    const int wi[5] = {i, i - 1, i, i + 1, i};
    const int wj[5] = {j - 1, j, j, j, j + 1};
    const int ws[5] = {4, 2, 0, 1, 3};
    int ghost = O.ghost[n];
    double b[4];
    bool have_b = false;
    for (int q = 0; q < 5; ++q) {
        if (wi[q] < 0 || wi[q] >= G.width || wj[q] < 0) continue;
        const int idx = wj[q] * G.width + wi[q];
        if (idx >= G.nthreads) continue;
        const int f = R.flags[idx];
        const int s = ws[q];
        if (f & (1 << s)) ghost = n;
        if (CLS != 2 && s == 0 && (f & (1 << 16))) ghost = -1;
        if (f & (1 << (8 + s))) {
            for (int c = 0; c < 4; ++c) b[c] = R.bi[(size_t)idx * 20 + s * 4 + c];
            have_b = true;
        }
    }
    O.ghost[n] = ghost;
    if (have_b) {
        O.bix[n] = b[0];
        O.biy[n] = b[1];
        O.ipx[n] = b[2];
        O.ipy[n] = b[3];
    }
    const bool self_exists = i >= 0 && i < G.width && j >= 0 && j * G.width + i < G.nthreads;
    const int sidx = j * G.width + i;
    if (CLS == 2) {
        if (self_exists && (R.flags[sidx] & (1 << 19))) O.hyb[n] = n;
        return;
    }
    if (self_exists && (R.flags[sidx] & (1 << 16))) {
        O.hyb[n] = R.hyb[sidx];
        O.hyb2[n] = R.hyb2[sidx];
        O.dnode[n] = R.dnode[sidx];
        O.dbetween[n] = R.dbetween[sidx];
        O.uv[n] = R.uv[sidx];
    }
    // dist_u_body / dist_v_body (pressure-indexed): writer before self is the west (u) or south (v) node
    const int ip = J * nx + I;
    const int pi = CLS == 0 ? i - 1 : i, pj = CLS == 0 ? j : j - 1;
    double dv = 0;
    bool have_d = false;
    if (pi >= 0 && pi < G.width && pj >= 0 && pj * G.width + pi < G.nthreads) {
        const int pidx = pj * G.width + pi;
        if (R.flags[pidx] & (1 << 18)) {
            dv = R.distB[pidx];
            have_d = true;
        }
    }
    if (self_exists && (R.flags[sidx] & (1 << 17))) {
        dv = R.distA[sidx];
        have_d = true;
    }
    if (have_d) O.dist[ip] = dv;
}

// zero_pressure_luo / zero_x_luo / zero_y_luo: one thread per row, left to right
__global__ void k_zero_rows(int *tags, int stride, int i0, int i1, int j0, int j1, int rows, int scan_end)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= rows) return;
    const int J = j0 + j;
    if (J > j1) return;
    bool rowIsntDone = true, flag = false;
    for (int i = i0; i < i1; ++i) {
        const int I = J * stride + i;
        if (tags[I - 1] >= 0) {
            if (tags[I] != -1 && tags[I - 1] == 0) rowIsntDone = false;
            if (tags[I] == -1 && rowIsntDone) tags[I] = 0;
            if (tags[I] == 0 && tags[I - 1] != 0) {
                int k = i;
                while (k < scan_end) {
                    k++;
                    if (tags[J * stride + k] != -1) flag = true;
                }
                if (!flag) {
                    tags[I] = -1;
                    rowIsntDone = false;
                }
            }
        }
    }
}

__global__ void k_tag_fill(int nUV, int nP, int *gUV, int *hUV, int *h2UV, double *dn, double *db, double *bix,
                           double *biy, double *ipx, double *ipy, int *gP, int *hP)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nUV) {
        gUV[t] = -1;
        hUV[t] = -1;
        h2UV[t] = -1;
        dn[t] = 1;
        db[t] = 1;
        bix[t] = 0;
        biy[t] = 0;
        ipx[t] = 0;
        ipy[t] = 0;
    }
    if (t < nP) {
        gP[t] = -1;
        hP[t] = -1;
    }
}

// ---- bilinear interpolation --------------------------------------------------------
__device__ __forceinline__ void inverse4_dev(const double a[16], double b[16], double *det)
{
    const double a11 = a[0], a12 = a[1], a13 = a[2], a14 = a[3];
    const double a21 = a[4], a22 = a[5], a23 = a[6], a24 = a[7];
    const double a31 = a[8], a32 = a[9], a33 = a[10], a34 = a[11];
    const double a41 = a[12], a42 = a[13], a43 = a[14], a44 = a[15];
    *det = a11 * a22 * a33 * a44 + a11 * a23 * a34 * a42 + a11 * a24 * a32 * a43 + a12 * a21 * a34 * a43 +
           a12 * a23 * a31 * a44 + a12 * a24 * a33 * a41 + a13 * a21 * a32 * a44 + a13 * a22 * a34 * a41 +
           a13 * a24 * a31 * a42 + a14 * a21 * a33 * a42 + a14 * a22 * a31 * a43 + a14 * a23 * a32 * a41 -
           a11 * a22 * a34 * a43 - a11 * a23 * a32 * a44 - a11 * a24 * a33 * a42 - a12 * a21 * a33 * a44 -
           a12 * a23 * a34 * a41 - a12 * a24 * a31 * a43 - a13 * a21 * a34 * a42 - a13 * a22 * a31 * a44 -
           a13 * a24 * a32 * a41 - a14 * a21 * a32 * a43 - a14 * a22 * a33 * a41 - a14 * a23 * a31 * a42;
    b[0] = a22 * a33 * a44 + a23 * a34 * a42 + a24 * a32 * a43 - a22 * a34 * a43 - a23 * a32 * a44 - a24 * a33 * a42;
    b[1] = a12 * a34 * a43 + a13 * a32 * a44 + a14 * a33 * a42 - a12 * a33 * a44 - a13 * a34 * a42 - a14 * a32 * a43;
    b[2] = a12 * a23 * a44 + a13 * a24 * a42 + a14 * a22 * a43 - a12 * a24 * a43 - a13 * a22 * a44 - a14 * a23 * a42;
    b[3] = a12 * a24 * a33 + a13 * a22 * a34 + a14 * a23 * a32 - a12 * a23 * a34 - a13 * a24 * a32 - a14 * a22 * a33;
    b[4] = a21 * a34 * a43 + a23 * a31 * a44 + a24 * a33 * a41 - a21 * a33 * a44 - a23 * a34 * a41 - a24 * a31 * a43;
    b[5] = a11 * a33 * a44 + a13 * a34 * a41 + a14 * a31 * a43 - a11 * a34 * a43 - a13 * a31 * a44 - a14 * a33 * a41;
    b[6] = a11 * a24 * a43 + a13 * a21 * a44 + a14 * a23 * a41 - a11 * a23 * a44 - a13 * a24 * a41 - a14 * a21 * a43;
    b[7] = a11 * a23 * a34 + a13 * a24 * a31 + a14 * a21 * a33 - a11 * a24 * a33 - a13 * a21 * a34 - a14 * a23 * a31;
    b[8] = a21 * a32 * a44 + a22 * a34 * a41 + a24 * a31 * a42 - a21 * a34 * a42 - a22 * a31 * a44 - a24 * a32 * a41;
    b[9] = a11 * a34 * a42 + a12 * a31 * a44 + a14 * a32 * a41 - a11 * a32 * a44 - a12 * a34 * a41 - a14 * a31 * a42;
    b[10] = a11 * a22 * a44 + a12 * a24 * a41 + a14 * a21 * a42 - a11 * a24 * a42 - a12 * a21 * a44 - a14 * a22 * a41;
    b[11] = a11 * a24 * a32 + a12 * a21 * a34 + a14 * a22 * a31 - a11 * a22 * a34 - a12 * a24 * a31 - a14 * a21 * a32;
    b[12] = a21 * a33 * a42 + a22 * a31 * a43 + a23 * a32 * a41 - a21 * a32 * a43 - a22 * a33 * a41 - a23 * a31 * a42;
    b[13] = a11 * a32 * a43 + a12 * a33 * a41 + a13 * a31 * a42 - a11 * a33 * a42 - a12 * a31 * a43 - a13 * a32 * a41;
    b[14] = a11 * a23 * a42 + a12 * a21 * a43 + a13 * a22 * a41 - a11 * a22 * a43 - a12 * a23 * a41 - a13 * a21 * a42;
    b[15] = a11 * a22 * a33 + a12 * a23 * a31 + a13 * a21 * a32 - a11 * a23 * a32 - a12 * a21 * a33 - a13 * a22 * a31;
}

__device__ __forceinline__ void rows_dev(const double x[4], const double y[4], double a[16])
{
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        a[4 * l] = 1;
        a[4 * l + 1] = x[l];
        a[4 * l + 2] = y[l];
        a[4 * l + 3] = x[l] * y[l];
    }
}

__device__ __forceinline__ void store_dev(int *idx4, double *coef4, int n, const int id[4], const double b[16],
                                          double det, double px, double py)
{
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        idx4[4 * (size_t)n + c] = id[c];
        coef4[4 * (size_t)n + c] = (b[c] + b[4 + c] * px + b[8 + c] * py + b[12 + c] * px * py) / det;
    }
}

struct BoxLaunch {
    int i0, j0, width, nthreads;
};

// Neumann row of the pressure fit at a body-intercept corner: the row of the
// 4x4 system and the unit normal (the corner's value is then -(n . dU/dt))
__device__ __forceinline__ void neumann_row(double px, double py, double bx_, double by_, double *a4, double *n2)
{
    const double nxv = px - bx_, nyv = py - by_;
    const double nl = sqrt(nxv * nxv + nyv * nyv);
    n2[0] = nxv / nl;
    n2[1] = nyv / nl;
    a4[0] = 0;
    a4[1] = nxv / nl;
    a4[2] = nyv / nl;
    a4[3] = nyv / nl * bx_ + nxv / nl * by_;
}

// ---- interpolation plan ---------------------------------------------------------------

// weights of the fit at (px, py): coefficient c of store_dev
__device__ __forceinline__ void fit_weights(const double b[16], double det, double px, double py, double *w)
{
#pragma unroll
    for (int c = 0; c < 4; ++c) w[c] = (b[c] + b[4 + c] * px + b[8 + c] * py + b[12 + c] * px * py) / det;
}

// ---- plan: node lists (the nodes the reference's interpolation threads act on) ----------
// Same launch ranges and index arithmetic as the reference's kernels; list order
// does not matter (every entry writes its own node).
__global__ void k_plan_scan_velocity(BoxLaunch B, int nx, int ny, const int *gtags, const int *htags, IbPlan P)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= B.nthreads) return;
    const int dir = blockIdx.y, nU = (nx - 1) * ny;
    const int I = B.i0 + idx % B.width, J = B.j0 + idx / B.width;
    int n;
    if (dir == 0) {
        n = J * (nx - 1) + I;
        if (n >= nU) return;
    } else {
        if (J * nx + I > nx * (ny - 1)) return;
        n = J * nx + I + nU;
    }
    if (gtags[n] > 0) P.gvNode[atomicAdd(&P.count[0], 1)] = n;
    if (htags[n] > 0) P.hvNode[atomicAdd(&P.count[1], 1)] = n;
}

__global__ void k_plan_scan_pressure(BoxLaunch B, int nx, int ny, const int *gtags, const int *htags, IbPlan P)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= B.nthreads) return;
    const int I = B.i0 + idx % B.width, J = B.j0 + idx / B.width, ip = J * nx + I;
    if (ip >= nx * ny) return;
    if (gtags[ip] > 0) P.gpNode[atomicAdd(&P.count[2], 1)] = ip;
    if (htags[ip] > 0) P.hpNode[atomicAdd(&P.count[3], 1)] = ip;
}

// inside nodes over the reference's u-index map (setInsideVelocity): u node i and
// the v node at the same (I, J)
__global__ void k_plan_scan_inside(int nx, int ny, const int *gtags, IbPlan P)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nU = (nx - 1) * ny, nUV = nU + nx * (ny - 1);
    if (i >= nU) return;
    const int I = i % (nx - 1), J = i / (nx - 1), iv = J * nx + I + nU;
    if (gtags[i] == 0) P.inNode[atomicAdd(&P.count[4], 1)] = i;
    if (iv < nUV && gtags[iv] == 0) P.inNode[atomicAdd(&P.count[4], 1)] = iv;
}

// ---- plan: per-node geometry (the reference's interpolation kernels minus the field) --------
struct PlanGeom {
    int nx, ny;
    const double *xu, *yu, *xv, *yv;
    const int *gUV, *hUV, *gP, *hP;                 // tags
    const double *biX, *biY, *ipX, *ipY;            // velocity intercepts and image points
    const double *bipX, *bipY, *ippX, *ippY;        // pressure intercepts and image points
    int *gIdx, *hIdx, *gpIdx, *hpIdx;               // per-node stencils (the reference's index/coef arrays)
    double *gCoef, *hCoef, *gpCoef, *hpCoef;
};

__device__ __forceinline__ void node_ij(int n, int nx, int nU, int *I, int *J)
{
    if (n < nU) {
        *I = n % (nx - 1);
        *J = n / (nx - 1);
    } else {
        *I = (n - nU) % nx;
        *J = (n - nU) / nx;
    }
}

// corner cell of the image point (the reference's search from I-5, J-5)
__device__ __forceinline__ void image_cell(const double *xc, const double *yc, int I, int J, double px, double py,
                                           int *ii, int *jj)
{
    int a = I - 5, b = J - 5;
    while (xc[a] < px) a++;
    while (yc[b] < py) b++;
    *ii = a;
    *jj = b;
}

// alpha of luoIBM weight (weightX / weightY / weightP) at hybrid node n
__device__ __forceinline__ double blend_alpha(int n, int I, int J, int sv, const double *xc, const double *yc,
                                              const int *gtags, const double *bix, const double *biy)
{
    double d1 = 0, d2 = 0;
    const double dx = xc[I] - xc[I - 1], dy = yc[J] - yc[J - 1];
    double ex, ey;
    if (gtags[n - 1] > 0) {
        ex = bix[n - 1] - xc[I - 1]; ey = biy[n - 1] - yc[J];
        d1 = sqrt(ex * ex + ey * ey);
    } else if (gtags[n + 1] > 0) {
        ex = bix[n + 1] - xc[I + 1]; ey = biy[n + 1] - yc[J];
        d1 = sqrt(ex * ex + ey * ey);
    }
    if (gtags[n - sv] > 0) {
        ex = bix[n - sv] - xc[I]; ey = biy[n - sv] - yc[J - 1];
        d2 = sqrt(ex * ex + ey * ey);
    }
    if (gtags[n + sv] > 0) {
        ex = bix[n + sv] - xc[I]; ey = biy[n + sv] - yc[J + 1];
        d2 = sqrt(ex * ex + ey * ey);
    }
    const double r1 = d1 / dx, r2 = d2 / dy;
    return sqrt(r1 * r1 + r2 * r2);
}

// ghost velocity node (interpolateVelocityToGhostNodeX/Y): value at the image point
__device__ void plan_ghost_velocity(int k, const PlanGeom &G, const IbPlan &P)
{
    const int nx = G.nx, ny = G.ny, nU = (nx - 1) * ny, n = P.gvNode[k];
    const int dir = n >= nU;
    int I, J, ii, jj;
    node_ij(n, nx, nU, &I, &J);
    const double *xc = dir ? G.xv : G.xu, *yc = dir ? G.yv : G.yu;
    image_cell(xc, yc, I, J, G.ipX[n], G.ipY[n], &ii, &jj);
    double x[4] = {xc[ii - 1], xc[ii], xc[ii - 1], xc[ii]};
    double y[4] = {yc[jj - 1], yc[jj - 1], yc[jj], yc[jj]};
    int id[4];
    if (dir == 0) {
        id[0] = (jj - 1) * (nx - 1) + ii - 1; id[1] = id[0] + 1;
        id[2] = jj * (nx - 1) + ii - 1;       id[3] = id[2] + 1;
    } else {
        id[0] = (jj - 1) * nx + ii - 1 + nU; id[1] = id[0] + 1;
        id[2] = jj * nx + ii - 1 + nU;       id[3] = id[2] + 1;
    }
    double mn = 1.0;
    int close = -1, mask = 0;
    bool inflag = false;
    for (int l = 0; l < 4; ++l) {
        double ex = x[l] - G.biX[n], ey = y[l] - G.biY[n];
        double s = sqrt(ex * ex + ey * ey);
        if (s < mn) { mn = s; close = id[l]; }
        if (G.gUV[id[l]] > 0) inflag = true;
    }
    for (int l = 0; l < 4; ++l) {
        if (G.gUV[id[l]] == n) { x[l] = G.biX[id[l]]; y[l] = G.biY[id[l]]; mask |= 1 << l; }
        else if (id[l] == close && !inflag) { x[l] = G.biX[n]; y[l] = G.biY[n]; mask |= 1 << l; }
    }
    double a[16], b[16], det;
    rows_dev(x, y, a);
    inverse4_dev(a, b, &det);
    store_dev(G.gIdx, G.gCoef, n, id, b, det, G.ipX[n], G.ipY[n]);
    fit_weights(b, det, G.ipX[n], G.ipY[n], P.gvW + 4 * (size_t)k);
    for (int l = 0; l < 4; ++l) P.gvIdx[4 * (size_t)k + l] = id[l];
    P.gvMask[k] = mask;
}

// hybrid velocity node (interpolateVelocityToHybridNodeX/Y): value at the node, at
// its image point, and the blend factor of weightX/Y
__device__ void plan_hybrid_velocity(int k, const PlanGeom &G, const IbPlan &P)
{
    const int nx = G.nx, ny = G.ny, nU = (nx - 1) * ny, n = P.hvNode[k];
    const int dir = n >= nU;
    int I, J, ii, jj;
    node_ij(n, nx, nU, &I, &J);
    const double *xc = dir ? G.xv : G.xu, *yc = dir ? G.yv : G.yu;
    image_cell(xc, yc, I, J, G.ipX[n], G.ipY[n], &ii, &jj);
    double x[4] = {xc[ii - 1], xc[ii], xc[ii - 1], xc[ii]};
    double y[4] = {yc[jj - 1], yc[jj - 1], yc[jj], yc[jj]};
    int id[4];
    if (dir == 0) {
        id[0] = (jj - 1) * (nx - 1) + ii - 1; id[1] = id[0] + 1;
        id[2] = jj * (nx - 1) + ii - 1;       id[3] = id[2] + 1;
    } else {
        id[0] = (jj - 1) * nx + ii - 1 + nU; id[1] = id[0] + 1;
        id[2] = jj * nx + ii - 1 + nU;       id[3] = id[2] + 1;
    }
    int mask = 0;
    for (int l = 0; l < 4; ++l)
        if (G.hUV[id[l]] == n) { x[l] = G.biX[n]; y[l] = G.biY[n]; mask |= 1 << l; }
    double a[16], b[16], det;
    rows_dev(x, y, a);
    inverse4_dev(a, b, &det);
    store_dev(G.hIdx, G.hCoef, n, id, b, det, xc[I], yc[J]);
    fit_weights(b, det, xc[I], yc[J], P.hvW + 4 * (size_t)k);
    fit_weights(b, det, G.ipX[n], G.ipY[n], P.hvWi + 4 * (size_t)k);
    for (int l = 0; l < 4; ++l) P.hvIdx[4 * (size_t)k + l] = id[l];
    P.hvMask[k] = mask;
    P.hvAlpha[k] = blend_alpha(n, I, J, dir ? nx : nx - 1, xc, yc, G.gUV, G.biX, G.biY);
}

// hybrid pressure node (interpolatePressureToHybridNode): value at the node, blend of weightP
__device__ void plan_hybrid_pressure(int k, const PlanGeom &G, const IbPlan &P)
{
    const int nx = G.nx, ip = P.hpNode[k];
    const int I = ip % nx, J = ip / nx;
    int ii, jj;
    image_cell(G.xv, G.yu, I, J, G.ippX[ip], G.ippY[ip], &ii, &jj);
    double x[4] = {G.xv[ii - 1], G.xv[ii], G.xv[ii - 1], G.xv[ii]};
    double y[4] = {G.yu[jj - 1], G.yu[jj - 1], G.yu[jj], G.yu[jj]};
    const int id[4] = {(jj - 1) * nx + ii - 1, (jj - 1) * nx + ii, jj * nx + ii - 1, jj * nx + ii};
    double a[16], b[16], det;
    rows_dev(x, y, a);
    int mask = 0;
    for (int l = 0; l < 4; ++l) {
        P.hpN[8 * (size_t)k + 2 * l] = 0;
        P.hpN[8 * (size_t)k + 2 * l + 1] = 0;
        if (G.hP[id[l]] == ip) {
            x[l] = G.bipX[ip];
            y[l] = G.bipY[ip];
            neumann_row(G.ippX[ip], G.ippY[ip], x[l], y[l], a + 4 * l, P.hpN + 8 * (size_t)k + 2 * l);
            mask |= 1 << l;
        }
    }
    inverse4_dev(a, b, &det);
    store_dev(G.hpIdx, G.hpCoef, ip, id, b, det, G.xv[I], G.yu[J]);
    fit_weights(b, det, G.xv[I], G.yu[J], P.hpW + 4 * (size_t)k);
    for (int l = 0; l < 4; ++l) P.hpIdx[4 * (size_t)k + l] = id[l];
    P.hpMask[k] = mask;
    P.hpAlpha[k] = blend_alpha(ip, I, J, nx, G.xv, G.yu, G.gP, G.bipX, G.bipY);
}

// ghost pressure node (interpolatePressureToGhostNode): value at the image point, at the
// body intercept, and the dp/dn correction's normal and distance
__device__ void plan_ghost_pressure(int k, const PlanGeom &G, const IbPlan &P)
{
    const int nx = G.nx, ip = P.gpNode[k];
    const int I = ip % nx, J = ip / nx;
    int ii, jj;
    image_cell(G.xv, G.yu, I, J, G.ippX[ip], G.ippY[ip], &ii, &jj);
    double x[4] = {G.xv[ii - 1], G.xv[ii], G.xv[ii - 1], G.xv[ii]};
    double y[4] = {G.yu[jj - 1], G.yu[jj - 1], G.yu[jj], G.yu[jj]};
    const int id[4] = {(jj - 1) * nx + ii - 1, (jj - 1) * nx + ii, jj * nx + ii - 1, jj * nx + ii};
    double a[16], b[16], det;
    rows_dev(x, y, a);
    double mn = 1.0, cn[2] = {0, 0};
    int close = -1, mask = 0;
    for (int l = 0; l < 4; ++l) {
        double ex = x[l] - G.bipX[ip], ey = y[l] - G.bipY[ip];
        double s = sqrt(ex * ex + ey * ey);
        if (s < mn) { mn = s; close = id[l]; }
    }
    for (int l = 0; l < 4; ++l) {
        P.gpN[8 * (size_t)k + 2 * l] = 0;
        P.gpN[8 * (size_t)k + 2 * l + 1] = 0;
        if (G.gP[id[l]] > 0) {
            x[l] = G.bipX[id[l]];
            y[l] = G.bipY[id[l]];
            neumann_row(G.ippX[id[l]], G.ippY[id[l]], x[l], y[l], a + 4 * l, P.gpN + 8 * (size_t)k + 2 * l);
            mask |= 1 << l;
        }
        if (id[l] == close) {
            x[l] = G.bipX[ip];
            y[l] = G.bipY[ip];
            const double nxv = G.ippX[ip] - x[l], nyv = G.ippY[ip] - y[l];
            const double nl = sqrt(nxv * nxv + nyv * nyv);
            cn[0] = nxv / nl;
            cn[1] = nyv / nl;
        }
    }
    inverse4_dev(a, b, &det);
    store_dev(G.gpIdx, G.gpCoef, ip, id, b, det, G.ippX[ip], G.ippY[ip]);
    fit_weights(b, det, G.ippX[ip], G.ippY[ip], P.gpW + 4 * (size_t)k);
    fit_weights(b, det, G.bipX[ip], G.bipY[ip], P.gpWb + 4 * (size_t)k);
    for (int l = 0; l < 4; ++l) P.gpIdx[4 * (size_t)k + l] = id[l];
    P.gpMask[k] = mask;
    const double ex = G.ippX[ip] - G.xv[I], ey = G.ippY[ip] - G.yu[J];
    P.gpCn[2 * (size_t)k] = cn[0];
    P.gpCn[2 * (size_t)k + 1] = cn[1];
    P.gpDist[k] = sqrt(ex * ex + ey * ey);
}

// blockIdx.y: 0 ghost velocity, 1 hybrid velocity, 2 ghost pressure, 3 hybrid pressure
__global__ void k_plan_build(PlanGeom G, IbPlan P)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int cls = blockIdx.y;
    if (k >= P.count[cls]) return;
    if (cls == 0) plan_ghost_velocity(k, G, P);
    else if (cls == 1) plan_hybrid_velocity(k, G, P);
    else if (cls == 2) plan_ghost_pressure(k, G, P);
    else plan_hybrid_pressure(k, G, P);
}

// ---- per-step immersed-boundary phases -------------------------------------------------
// One block runs a sequence of the reference's IB phases on the plan's node lists
// (a few hundred to a few thousand nodes), with __syncthreads between them.  Ghost
// phases stage their new values and write them after a barrier, so every node
// reads the field as it was before the phase (the reference's launch: all loads
// precede all stores).  Phases run in this order, which contains each of the
// reference's sequences (rhs1: Robin, ghost, inside, hybrid; after the velocity
// solve: weight, ghost; after the Poisson solve: hybrid, weight, ghost pressure;
// after the projection: ghost, inside).
enum IbPhase {
    PH_ROBIN = 1,      // updateRobinBoundary (Uinf = Vinf = 1)
    PH_WEIGHT_U = 2,   // weightX/Y: vel = (1 - alpha) vel + alpha ustar at hybrid nodes
    PH_GHOST_U = 4,    // interpolateVelocityToGhostNodeX/Y on vel
    PH_INSIDE = 8,     // setInsideVelocity on vel
    PH_HYBRID_U = 16,  // interpolateVelocityToHybridNodeX/Y: ustar from vel
    PH_HYBRID_P = 32,  // interpolatePressureToHybridNode: pstar from p
    PH_WEIGHT_P = 64,  // weightP
    PH_GHOST_P = 128   // interpolatePressureToGhostNode on p
};

struct IbStep {
    IbPlan P;
    int nx, ny;
    double *vel, *p;
    const double *uB, *vB, *uBk, *vBk;
    double dt;
    double *ustar, *pstar, *imageValue, *biP, *dpdn, *stage;
    double *xp;
    const double *dx;
};

constexpr int kIbThreads = 512;

__global__ void __launch_bounds__(kIbThreads) k_ib_step(IbStep S, int phases)
{
    const int t = threadIdx.x, T = blockDim.x;
    const int nx = S.nx, ny = S.ny, nU = (nx - 1) * ny;
    const IbPlan &P = S.P;
    double *f = S.vel;
    if (phases & PH_ROBIN) {
        for (int r = t; r < 2 * ny - 1; r += T) {
            if (r < ny) {
                const int J = r, I = nx - 1, i = J * (nx - 1) + I;
                const double beta = 1.0 * S.dt / S.dx[I];
                S.xp[J] = S.xp[J] * (1 - beta) + beta * f[i - 1];
            } else {
                const int J = r - ny, I = nx, i = J * nx + I;
                const double beta = 1.0 * S.dt / S.dx[I - 1];
                S.xp[J + ny] = S.xp[J + ny] * (1 - beta) + beta * f[i + nU - 1];
            }
        }
    }
    if (phases & PH_WEIGHT_U) {
        const int cnt = P.count[1];
        for (int k = t; k < cnt; k += T) {
            const int n = P.hvNode[k];
            const double a = P.hvAlpha[k];
            f[n] = (1 - a) * f[n] + a * S.ustar[n];
        }
        __syncthreads();
    }
    if (phases & PH_GHOST_U) {
        const int cnt = P.count[0];
        const double ub = S.uB[0], vb = S.vB[0];
        for (int k = t; k < cnt; k += T) {
            const int n = P.gvNode[k], m = P.gvMask[k];
            const double qb = n >= nU ? vb : ub;
            double val = 0;
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const double q = (m >> l & 1) ? qb : f[P.gvIdx[4 * k + l]];
                val += P.gvW[4 * k + l] * q;
            }
            S.imageValue[n] = val;
            S.stage[k] = 2 * qb - val;
        }
        __syncthreads();
        for (int k = t; k < cnt; k += T) f[P.gvNode[k]] = S.stage[k];
        __syncthreads();
    }
    if (phases & PH_INSIDE) {
        const int cnt = P.count[4];
        const double ub = S.uB[0], vb = S.vB[0];
        for (int k = t; k < cnt; k += T) {
            const int n = P.inNode[k];
            f[n] = n >= nU ? vb : ub;
        }
        __syncthreads();
    }
    if (phases & PH_HYBRID_U) {
        const int cnt = P.count[1];
        const double ub = S.uB[0], vb = S.vB[0];
        for (int k = t; k < cnt; k += T) {
            const int n = P.hvNode[k], m = P.hvMask[k];
            const double qb = n >= nU ? vb : ub;
            double s = 0, si = 0;
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const double q = (m >> l & 1) ? qb : f[P.hvIdx[4 * k + l]];
                s += P.hvW[4 * k + l] * q;
                si += P.hvWi[4 * k + l] * q;
            }
            S.ustar[n] = s;
            S.imageValue[n] = si;
        }
        __syncthreads();
    }
    const double dudt = (S.uB[0] - S.uBk[0]) / S.dt, dvdt = (S.vB[0] - S.vBk[0]) / S.dt;
    if (phases & PH_HYBRID_P) {
        const int cnt = P.count[3];
        for (int k = t; k < cnt; k += T) {
            const int ip = P.hpNode[k], m = P.hpMask[k];
            double s = 0;
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const double *nn = P.hpN + 8 * k + 2 * l;
                const double q = (m >> l & 1) ? -(nn[0] * dudt + nn[1] * dvdt) : S.p[P.hpIdx[4 * k + l]];
                s += P.hpW[4 * k + l] * q;
            }
            S.pstar[ip] = s;
        }
        __syncthreads();
    }
    if (phases & PH_WEIGHT_P) {
        const int cnt = P.count[3];
        for (int k = t; k < cnt; k += T) {
            const int ip = P.hpNode[k];
            const double a = P.hpAlpha[k];
            S.p[ip] = (1 - a) * S.p[ip] + a * S.pstar[ip];
        }
        __syncthreads();
    }
    if (phases & PH_GHOST_P) {
        const int cnt = P.count[2];
        for (int k = t; k < cnt; k += T) {
            const int ip = P.gpNode[k], m = P.gpMask[k];
            double v = 0, vb = 0;
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const double *nn = P.gpN + 8 * k + 2 * l;
                const double q = (m >> l & 1) ? -(nn[0] * dudt + nn[1] * dvdt) : S.p[P.gpIdx[4 * k + l]];
                v += P.gpW[4 * k + l] * q;
                vb += P.gpWb[4 * k + l] * q;
            }
            S.biP[ip] = vb;
            const double matD = P.gpCn[2 * k] * dudt + P.gpCn[2 * k + 1] * dvdt;
            const double d = P.gpDist[k] * matD;
            S.dpdn[ip] = d;
            S.stage[k] = v + d;
        }
        __syncthreads();
        for (int k = t; k < cnt; k += T) S.p[P.gpNode[k]] = S.stage[k];
    }
}

// control-volume force: the six sums of dragLeftRight, dragBottomTop, dragUnsteady,
// liftLeftRight, liftBottomTop, liftUnsteady in one launch, reduced in a fixed order
__device__ __forceinline__ void force_body(int nx, int ny, int I, int J, int ncx, int ncy, const double *u,
                                           const double *uold, const double *p, const int *gtags, double nu,
                                           const double *dx, const double *dy, double dt, double *part,
                                           unsigned int *arrive, double *out, double *comp)
{
    const int nU = (nx - 1) * ny;
    double s[6] = {0, 0, 0, 0, 0, 0};
    const int stride = gridDim.x * blockDim.x;
    // the six terms' items laid end to end, one item per thread and pass: the four
    // edge sums (a few divisions each) spread over many threads instead of riding on
    // the first few of block 0
    const int o1 = ncy, o3 = o1 + ncx + 1, o4 = o3 + ncy + 1, o2 = o4 + ncx, o5 = o2 + (ncx + 1) * ncy;
    const int total = o5 + ncx * (ncy + 1);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += stride) {
        if (q < o1) {
            const int idx = q;
            const int Ip = (J + idx) * nx + I, Iu = (J + idx) * (nx - 1) + I;
            const double a = u[Iu + ncx] + u[Iu + ncx - 1], b = u[Iu - 1] + u[Iu];
            s[0] += -((p[Ip + ncx] - p[Ip]) * dy[J + idx] + (a * a / 4 - b * b / 4) * dy[J + idx] -
                      nu * ((u[Iu + ncx] - u[Iu + ncx - 1]) / dx[I + ncx] - (u[Iu] - u[Iu - 1]) / dx[I]) * dy[J + idx]);
        } else if (q < o3) {
            const int idx = q - o1;
            const int Iu = J * (nx - 1) + (I - 1 + idx), Iv = nU + (J - 1) * nx + I + idx;
            s[1] += -((0.25 * (u[Iu + ncy * (nx - 1)] + u[Iu + (ncy - 1) * (nx - 1)]) *
                           (u[Iv + ncy * nx] + u[Iv + ncy * nx - 1]) -
                       0.25 * (u[Iu] + u[Iu - (nx - 1)]) * (u[Iv] + u[Iv - 1])) -
                      nu * (((u[Iu + ncy * (nx - 1)] - u[Iu + (ncy - 1) * (nx - 1)]) / 2.0 / (dy[J + ncy] + dy[J + ncy - 1]) +
                             (u[Iv + ncy * nx] - u[Iv + ncy * nx - 1]) / 2.0 / (dx[I + idx] + dx[I + idx - 1])) -
                            ((u[Iu] - u[Iu - (nx - 1)]) / 2.0 / (dy[J] + dy[J - 1]) +
                             (u[Iv] - u[Iv - 1]) / 2.0 / (dx[I + idx] + dx[I + idx - 1])))) *
                    0.5 * (dx[I + idx] + dx[I + idx - 1]);
        } else if (q < o4) {
            const int idx = q - o3;
            const int Iu = (J + idx) * (nx - 1) + (I - 1), Iv = nU + (J - 1 + idx) * nx + I;
            s[3] += -((0.25 * (u[Iu + ncx] + u[Iu + ncx - (nx - 1)]) * (u[Iv + ncx] + u[Iv + ncx - 1]) -
                       0.25 * (u[Iu] + u[Iu - (nx - 1)]) * (u[Iv] + u[Iv - 1])) -
                      nu * (((u[Iu + ncx] - u[Iu + ncx - (nx - 1)]) / 2.0 / (dy[J + idx] + dy[J - 1 + idx]) +
                             (u[Iv + ncx] - u[Iv + ncx - 1]) / 2.0 / (dx[I + ncx] + dx[I + ncx - 1])) -
                            ((u[Iu] - u[Iu - (nx - 1)]) / 2.0 / (dy[J + idx] + dy[J - 1 + idx]) +
                             (u[Iv] - u[Iv - 1]) / 2.0 / (dx[I] + dx[I - 1])))) *
                    0.5 * (dy[J + idx] + dy[J - 1 + idx]);
        } else if (q < o2) {
            const int idx = q - o4;
            const int Ip = J * nx + I + idx, Iv = nU + (J - 1) * nx + I + idx;
            const double a = u[Iv + (ncy + 1) * nx] + u[Iv + ncy * nx], b = u[Iv] + u[Iv - nx];
            s[4] += -((p[Ip + ncy * nx] - p[Ip - nx]) * dx[I + idx] + (0.25 * a * a - 0.25 * b * b) * dx[I + idx] -
                      nu * ((u[Iv + (ncy + 1) * nx] - u[Iv + ncy * nx]) * dx[I + idx] / dy[J + ncy] -
                            (u[Iv] - u[Iv - nx]) * dx[I] / dy[J - 1]));
        } else if (q < o5) {
            const int idx = q - o2;
            const int i = idx % (ncx + 1), j = idx / (ncx + 1), Iu = (J + j) * (nx - 1) + (I - 1 + i);
            s[2] += -(gtags[Iu] == -1) * ((u[Iu] * dy[J + j] - uold[Iu] * dy[J + j]) / dt * 0.5 * (dx[I + i] + dx[I - 1 + i]));
        } else {
            const int idx = q - o5;
            const int i = idx % ncx, j = idx / ncx, Iv = (J - 1 + j) * nx + (I + i) + nU;
            s[5] += -(gtags[Iv] == -1) * ((u[Iv] * dx[I + i] - uold[Iv] * dx[I + i]) / dt * 0.5 * (dy[J + j] + dy[J - 1 + j]));
        }
    }
    // block reduction, then the last block sums the block partials in order
    __shared__ double sh[6][32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < 6; ++k) {
        double a = s[k];
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) sh[k][wid] = a;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double a = 0;
        for (int q = 0; q < nw; ++q) a += sh[threadIdx.x][q];
        part[blockIdx.x * 6 + threadIdx.x] = a;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(arrive, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    // warp k sums term k over the blocks (lanes stride the blocks, then a fixed shuffle
    // tree): the partials are read in parallel, not one dependent load after another
    if (wid < 6) {
        double a = 0;
        for (int b = lane; b < (int)gridDim.x; b += 32) a += __ldcg(part + b * 6 + wid);
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        if (lane == 0) sh[wid][0] = a;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t[6];
        for (int k = 0; k < 6; ++k) t[k] = sh[k][0];
        out[0] = t[0] + t[1] + t[2];
        out[1] = t[3] + t[4] + t[5];
        if (comp)
            for (int k = 0; k < 6; ++k) comp[k] = t[k];
        *arrive = 0;
    }
}

__global__ void k_force(int nx, int ny, const int *bb, const double *u, const double *uold, const double *p,
                        const int *gtags, double nu, const double *dx, const double *dy, double dt, double *part,
                        unsigned int *arrive, double *out)
{
    // the six sums (dragLeftRight, dragBottomTop, dragUnsteady, lift...) follow the force
    force_body(nx, ny, bb[0], bb[1], bb[2], bb[3], u, uold, p, gtags, nu, dx, dy, dt, part, arrive, out, out + 2);
}

// k_force with the box passed by value (caller-owned arrays, no context)
__global__ void k_force_box(int nx, int ny, int I, int J, int ncx, int ncy, const double *u, const double *uold,
                            const double *p, const int *gtags, double nu, const double *dx, const double *dy,
                            double dt, double *part, unsigned int *arrive, double *out)
{
    force_body(nx, ny, I, J, ncx, ncy, u, uold, p, gtags, nu, dx, dy, dt, part, arrive, out, nullptr);
}

// prescribed motion (luo_base/move.cu set_movement): x = xnew + offset, uB = unew with
// xnew, unew taken from a table of the host-evaluated motion indexed by the step
// (plus the per-point velocity offset off[i], zero unless the caller set one)
__global__ void k_body_motion(int total, const int *step, int table_len, const double *table, const double *bdx,
                              const double *off, double *bx, double *uB, double *motion)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int s = *step;
    s = s < 0 ? 0 : (s >= table_len ? table_len - 1 : s);
    const double xnew = table[2 * s], unew = table[2 * s + 1];
    if (i < total) {
        bx[i] = xnew + bdx[i];
        uB[i] = unew + off[i];
    }
    if (i == 0) {
        motion[0] = xnew;
        motion[2] = unew;
    }
}

// flow-induced motion, loose coupling (luo_base/move.cu viv_movement_LC, VIV: 1): the
// body is a spring-mounted cylinder free in y, reduced mass 2, reduced velocity Ured;
// from the lift coefficient Cy = 2 Fy of this step and the pre-step centre and
// velocity (motion[5], motion[7]) an implicit update gives the new velocity and
// centre, then y = midY + offset, vB = vnew.  Every thread evaluates the same
// expression from values no thread of this launch writes.
__global__ void k_body_viv(int total, const double *force, double dt, double Ured, const double *bdy, double *by,
                           double *vB, double *motion)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double Cy = force[1] * 2.0, Mred = 2.0, vold = motion[7], yold = motion[5];
    const double a = dt * M_PI * M_PI * 4 / (Ured * Ured), b = dt * dt * 2 * M_PI * M_PI / (Ured * Ured);
    const double vnew = (vold - a * (yold + dt / 2 * vold) + dt * Cy / 2 / Mred) / (1 + b);
    const double ynew = yold + dt / 2 * (vnew + vold);
    if (i < total) {
        vB[i] = vnew;
        by[i] = ynew + bdy[i];
    }
    if (i == 0) {
        motion[1] = ynew;
        motion[3] = vnew;
    }
}

// flow-induced motion, strong coupling (luo_base/move.cu viv_movement_SC, VIV: 2):
// the same implicit update from the pre-step centre and velocity, with the new centre
// relaxed (factor 0.9) against the one of the previous sub-iteration, motion[1]; the
// relative change of the centre, (previous - new) / previous, goes to motion[8] (the
// reference's SCtol).  One block: every thread reads motion[1] before thread 0
// overwrites it.
__global__ void k_body_viv_sc(int total, const double *force, double dt, double Ured, const double *bdy,
                              double *by, double *vB, double *motion)
{
    const double Cy = force[1] * 2.0, Mred = 2.0, relax = 0.9, vold = motion[7], yold = motion[5];
    const double yprev = motion[1];
    const double a = dt * M_PI * M_PI * 4 / (Ured * Ured), b = dt * dt * 2 * M_PI * M_PI / (Ured * Ured);
    const double vnew = (vold - a * (yold + dt / 2 * vold) + dt * Cy / 2 / Mred) / (1 + b);
    const double ynew = relax * (yold + dt / 2 * (vnew + vold)) + (1 - relax) * yprev;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
        vB[i] = vnew;
        by[i] = ynew + bdy[i];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        motion[1] = ynew;
        motion[3] = vnew;
        motion[8] = (yprev - ynew) / yprev;
    }
}

// The loop test of a strongly coupled step (luo_base.cu:215): another sub-iteration
// while |SCtol| > 0.001 or fewer than two ran.  motion[9] counts the passes done
// (the first included), motion[10] holds the answer for a host-driven loop; in a graph it sets the
// WHILE node's condition.  The reference has no limit: this one stops after
// kCouplingMaxIterations and flags the step.  A NaN SCtol (a centre at exactly 0
// that does not move) fails the test, as it does in the reference.
__global__ void k_coupling_next(double *motion, int *err, int cap, cudaGraphConditionalHandle h, int use_cond)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const double done = motion[9] + 1;
    motion[9] = done;
    int more = fabs(motion[8]) > 0.001 || done < 2;
    if (more && done >= cap) {
        atomicCAS(err, 0, kErrCouplingNotConverged);
        more = 0;
    }
    motion[10] = more;
    if (use_cond) cudaGraphSetConditional(h, more ? 1u : 0u);
}

// A moving body is tagged over a fixed box that holds its travel; the control-volume
// box of its current position must stay inside it.  If it does not, the step's error
// word records it (the tags would be incomplete).
__global__ void k_check_box(const int *bb, int ti0, int tj0, int tncx, int tncy, int *err, int code)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    if (bb[0] < ti0 || bb[1] < tj0 || bb[0] + bb[2] > ti0 + tncx || bb[1] + bb[3] > tj0 + tncy)
        atomicCAS(err, 0, code);
}

// _pre_step copies of the body velocities: uB0 = uBk = uB (and v)
__global__ void k_body_pre_step(int total, const double *uB, const double *vB, double *uBk, double *vBk,
                                double *motion)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < total) {
        uBk[i] = uB[i];
        vBk[i] = vB[i];
    }
    if (i == 0) {
        motion[4] = motion[0];
        motion[5] = motion[1];
        motion[6] = motion[2];
        motion[7] = motion[3];
        motion[8] = 0.0001;  // luo_base.cu:213-214: SCtol, and the passes done by the loop
        motion[9] = 1;       // test: the step's first pass, recorded before the loop
    }
}

__global__ void k_step_counter(int *s) { *s += 1; }

// bodies::calculateBoundingBoxes (bodies.cu:257-293, 303-326): the box of the body
// points scaled by scaleCV about its centre, in cell indices of the centre arrays
// x, y; one thread (the reference's boundingBox kernel), bounded searches
__global__ void k_body_box(int total, const double *bx, const double *by, const double *x, const double *y, int nx,
                           int ny, double scale, int *bb)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double xmax = bx[0], xmin = bx[0], ymax = by[0], ymin = by[0];
    for (int i = 1; i < total; ++i) {
        xmax = bx[i] > xmax ? bx[i] : xmax;
        xmin = bx[i] < xmin ? bx[i] : xmin;
        ymax = by[i] > ymax ? by[i] : ymax;
        ymin = by[i] < ymin ? by[i] : ymin;
    }
    const double ex = xmax - xmin, ey = ymax - ymin;
    xmax += 0.5 * ex * (scale - 1.0);
    xmin -= 0.5 * ex * (scale - 1.0);
    ymax += 0.5 * ey * (scale - 1.0);
    ymin -= 0.5 * ey * (scale - 1.0);
    int i = 0, j = 0;
    while (i + 1 < nx && x[i + 1] < xmin) i++;
    while (j + 1 < ny && y[j + 1] < ymin) j++;
    bb[0] = i;
    bb[1] = j;
    while (i < nx - 1 && x[i] < xmax) i++;
    while (j < ny - 1 && y[j] < ymax) j++;
    bb[2] = i - bb[0];
    bb[3] = j - bb[1];
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static int ref_threads(int w, int h) { return ((int)(((double)w * h - 0.5) / 256) + 1) * 256; }

struct IbHost {
    TagRecords rec{};
    int *bb = nullptr;             // device [i0, j0, ncx, ncy]
    double *motion_table = nullptr;
    int table_len = 0;
    double *staging = nullptr;
    unsigned int *force_arrive = nullptr;
    bool moving = false;
    IbPlan plan{};
};
static std::vector<IbHost> g_ib_host;  // one per context (indexed by Context::ib_slot)

static IbHost &hostside(Context &c) { return g_ib_host[c.ib_slot]; }

IbPlan &ib_plan(Context &c) { return hostside(c).plan; }

void setup_ib(Context &c)
{
    IbArrays &b = c.ib;
    const size_t UV = c.g.nUV, P = c.g.nP;
    const int nb = c.body.total;
    b.ghostUV = c.carve<int>(UV);
    b.hybridUV = c.carve<int>(UV);
    b.hybrid2UV = c.carve<int>(UV);
    b.ghostP = c.carve<int>(P);
    b.hybridP = c.carve<int>(P);
    b.biX = c.carve<double>(UV);
    b.biY = c.carve<double>(UV);
    b.ipX = c.carve<double>(UV);
    b.ipY = c.carve<double>(UV);
    b.bipX = c.carve<double>(P);
    b.bipY = c.carve<double>(P);
    b.ippX = c.carve<double>(P);
    b.ippY = c.carve<double>(P);
    b.distNode = c.carve<double>(UV);
    b.distBetween = c.carve<double>(UV);
    b.distU = c.carve<double>(P);
    b.distV = c.carve<double>(P);
    b.uvBody = c.carve<double>(UV);
    b.ustar = c.carve<double>(UV);
    b.pstar = c.carve<double>(P);
    b.dpdn = c.carve<double>(P);
    b.biP = c.carve<double>(P);
    b.imageValue = c.carve<double>(UV);
    b.gIdx = c.carve<int>(4 * UV);
    b.hIdx = c.carve<int>(4 * UV);
    b.gpIdx = c.carve<int>(4 * P);
    b.hpIdx = c.carve<int>(4 * P);
    b.gCoef = c.carve<double>(4 * UV);
    b.hCoef = c.carve<double>(4 * UV);
    b.gpCoef = c.carve<double>(4 * P);
    b.hpCoef = c.carve<double>(4 * P);
    b.gnValue = c.carve<double>(
        std::max<size_t>(UV > P ? UV : P, 2 * (size_t)ref_threads(c.bb_tag.ncx + 16, c.bb_tag.ncy + 16)));
    b.bx = c.carve<double>(nb);
    b.by = c.carve<double>(nb);
    b.uB = c.carve<double>(nb);
    b.vB = c.carve<double>(nb);
    b.uBk = c.carve<double>(nb);
    b.vBk = c.carve<double>(nb);
    b.bdx = c.carve<double>(nb);
    b.bdy = c.carve<double>(nb);
    b.motion = c.carve<double>(kMotionLen);
    b.velOff = c.carve<double>(2 * (size_t)nb);  // zero (the arena starts zeroed)
    b.forceOut = c.carve<double>(8);  // Fx, Fy, then the six partial sums
    b.surf = c.carve<double>(3 * (size_t)nb + 2);
    const int fblocks = 64;
    b.forcePart = c.carve<double>(6 * fblocks);

    if ((int)g_ib_host.size() <= c.ib_slot || c.ib_slot < 0) {
        c.ib_slot = (int)g_ib_host.size();
        g_ib_host.emplace_back();
    }
    IbHost &H = hostside(c);
    H = IbHost();
    H.bb = c.carve<int>(4);
    H.force_arrive = c.carve<unsigned int>(4);
    CUIBM_TRY(cudaMemsetAsync(H.force_arrive, 0, 4 * sizeof(unsigned int), c.stream));
    // records sized for the box, with room for the box to grow as the body moves
    const int w = c.bb_tag.ncx + 16, h = c.bb_tag.ncy + 16;
    H.rec.nrec = ref_threads(w, h);
    const size_t nr = H.rec.nrec;
    H.rec.flags = c.carve<int>(nr);
    H.rec.hyb = c.carve<int>(nr);
    H.rec.hyb2 = c.carve<int>(nr);
    H.rec.dnode = c.carve<double>(nr);
    H.rec.dbetween = c.carve<double>(nr);
    H.rec.uv = c.carve<double>(nr);
    H.rec.distA = c.carve<double>(nr);
    H.rec.distB = c.carve<double>(nr);
    H.rec.bi = c.carve<double>(nr * 20);
    // interpolation plan: lists sized for every node the box launch can visit
    IbPlan &L = H.plan;
    L.cap_v = 2 * (int)nr;
    L.cap_p = (int)nr;
    L.cap_in = (int)UV;
    const size_t cv = L.cap_v, cp = L.cap_p;
    L.count = c.carve<int>(8);
    L.gvNode = c.carve<int>(cv);
    L.gvIdx = c.carve<int>(4 * cv);
    L.gvMask = c.carve<int>(cv);
    L.gvW = c.carve<double>(4 * cv);
    L.hvNode = c.carve<int>(cv);
    L.hvIdx = c.carve<int>(4 * cv);
    L.hvMask = c.carve<int>(cv);
    L.hvW = c.carve<double>(4 * cv);
    L.hvWi = c.carve<double>(4 * cv);
    L.hvAlpha = c.carve<double>(cv);
    L.gpNode = c.carve<int>(cp);
    L.gpIdx = c.carve<int>(4 * cp);
    L.gpMask = c.carve<int>(cp);
    L.gpN = c.carve<double>(8 * cp);
    L.gpW = c.carve<double>(4 * cp);
    L.gpWb = c.carve<double>(4 * cp);
    L.gpCn = c.carve<double>(2 * cp);
    L.gpDist = c.carve<double>(cp);
    L.hpNode = c.carve<int>(cp);
    L.hpIdx = c.carve<int>(4 * cp);
    L.hpMask = c.carve<int>(cp);
    L.hpN = c.carve<double>(8 * cp);
    L.hpW = c.carve<double>(4 * cp);
    L.hpAlpha = c.carve<double>(cp);
    L.inNode = c.carve<int>(UV);
    CUIBM_TRY(cudaMemsetAsync(L.count, 0, 8 * sizeof(int), c.stream));
    const BodyState &B = c.body;
    H.moving = B.xCoeff != 0 || B.uCoeff != 0 || c.P.VIV == 1 || c.P.VIV == 2;
    // the host-evaluated prescribed motion for every step (luo_base/move.cu:121-146):
    // xnew = xC sin(2 pi f t + xPhase), unew = uC cos(2 pi f t + uPhase), t = dt * step
    H.table_len = c.P.nt + c.P.startStep + 2;
    std::vector<double> tab(2 * (size_t)H.table_len);
    for (int s = 0; s < H.table_len; ++s) {
        const double t = c.P.dt * s;
        tab[2 * s] = B.xCoeff * std::sin(2 * M_PI * B.freq * t + B.xPhase);
        tab[2 * s + 1] = B.uCoeff * std::cos(2 * M_PI * B.freq * t + B.uPhase);
    }
    H.motion_table = c.carve<double>(tab.size());
    CUIBM_TRY(cudaMemcpy(H.motion_table, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice));
}

static BoxLaunch box(Context &c)
{
    return BoxLaunch{c.bb_tag.i0, c.bb_tag.j0, c.bb_tag.ncx, ref_threads(c.bb_tag.ncx, c.bb_tag.ncy)};
}

// luo_base::initialise body part (luo_base.cu:48-86): positions and velocities at
// t = dt*timeStep, then uBk from the velocity at t - dt; the box is the one
// bodies::initialise computed before this move.
void initialise_body(Context &c)
{
    IbHost &H = hostside(c);
    const BodyState &B = c.body;
    const int nb = B.total;
    const double t = c.P.dt * c.timeStep;
    const double xnew = B.xCoeff * std::sin(2 * M_PI * B.freq * t + B.xPhase);
    const double unew = B.uCoeff * std::cos(2 * M_PI * B.freq * t + B.uPhase);
    const double uoldd = B.uCoeff * std::cos(2 * M_PI * B.freq * (t - c.P.dt) + B.uPhase);
    std::vector<double> x(nb), y(B.y), uB(nb, unew), vB(nb, 0.0), uBk(nb, uoldd), vBk(nb, 0.0);
    for (int i = 0; i < nb; ++i) x[i] = xnew + B.dxp[i];
    auto up = [&](double *d, const std::vector<double> &h) {
        CUIBM_TRY(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    };
    up(c.ib.bx, x);
    up(c.ib.by, y);
    up(c.ib.uB, uB);
    up(c.ib.vB, vB);
    up(c.ib.uBk, uBk);
    up(c.ib.vBk, vBk);
    up(c.ib.bdx, B.dxp);
    up(c.ib.bdy, B.dyp);
    double motion[kMotionLen] = {xnew, B.midY, unew, 0, xnew, B.midY, unew, 0, 0.0001, 0, 0, 0};
    CUIBM_TRY(cudaMemcpyAsync(c.ib.motion, motion, sizeof motion, cudaMemcpyHostToDevice, c.stream));
    int bb[4] = {c.bb.i0, c.bb.j0, c.bb.ncx, c.bb.ncy};
    CUIBM_TRY(cudaMemcpyAsync(H.bb, bb, sizeof bb, cudaMemcpyHostToDevice, c.stream));
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
    c.ib_midX = xnew;
    c.ib_midY = B.midY;
}

void launch_tag_points(Context &c)
{
    IbHost &H = hostside(c);
    IbArrays &b = c.ib;
    const int nx = c.g.nx, ny = c.g.ny;
    const int w = c.bb_tag.ncx, h = c.bb_tag.ncy, nthreads = ref_threads(w, h);
    if (nthreads > H.rec.nrec) throw InputError("the body's box outgrew the tagging records");
    const int nfill = c.g.nUV > c.g.nP ? c.g.nUV : c.g.nP;
    k_tag_fill<<<blocks_for(nfill), kBlock, 0, c.stream>>>(c.g.nUV, c.g.nP, b.ghostUV, b.hybridUV, b.hybrid2UV,
                                                          b.distNode, b.distBetween, b.biX, b.biY, b.ipX, b.ipY,
                                                          b.ghostP, b.hybridP);
    // midX is the body's current centre abscissa (the prescribed xnew), midY its centroid
    TagGeom G{b.bx, b.by, b.uB, c.xu, c.yu, c.bb_tag.i0, c.bb_tag.j0, w, h, nthreads, nx, ny, c.body.total, c.ib_midX,
              c.ib_midY, H.moving ? b.motion : nullptr};
    TagOut O{b.ghostUV, b.hybridUV, b.hybrid2UV, b.distNode, b.distBetween, b.uvBody, b.biX, b.biY, b.ipX, b.ipY,
             b.distU};
    const int rows = (nthreads + w - 1) / w;
    const int nres = (w + 2) * (rows + 2);
    k_tag_velocity_records<0><<<blocks_for(nthreads), kBlock, 0, c.stream>>>(G, H.rec);
    k_tag_resolve<0><<<blocks_for(nres), kBlock, 0, c.stream>>>(G, H.rec, O);
    G.vel = b.vB;
    G.xc = c.xv;
    G.yc = c.yv;
    O.dist = b.distV;
    k_tag_velocity_records<1><<<blocks_for(nthreads), kBlock, 0, c.stream>>>(G, H.rec);
    k_tag_resolve<1><<<blocks_for(nres), kBlock, 0, c.stream>>>(G, H.rec, O);
    G.xc = c.xv;
    G.yc = c.yu;
    TagOut OP{b.ghostP, b.hybridP, nullptr, nullptr, nullptr, nullptr, b.bipX, b.bipY, b.ippX, b.ippY, nullptr};
    k_tag_pressure_records<<<blocks_for(nthreads), kBlock, 0, c.stream>>>(G, H.rec);
    k_tag_resolve<2><<<blocks_for(nres), kBlock, 0, c.stream>>>(G, H.rec, OP);
    const int i0 = c.bb_tag.i0, i1 = c.bb_tag.i0 + w, j0 = c.bb_tag.j0, j1 = c.bb_tag.j0 + h;
    const int zrows = ref_threads(i1 - i0, 1);
    k_zero_rows<<<blocks_for(zrows), kBlock, 0, c.stream>>>(b.ghostP, nx, i0, i1, j0, j1, zrows, nx);
    k_zero_rows<<<blocks_for(zrows), kBlock, 0, c.stream>>>(b.ghostUV, nx - 1, i0, i1, j0, j1, zrows, nx - 1);
    k_zero_rows<<<blocks_for(zrows), kBlock, 0, c.stream>>>(b.ghostUV + c.g.nU, nx, i0, i1, j0, j1, zrows, nx - 1);
    // the interpolation plan of these tags
    IbPlan &P = H.plan;
    BoxLaunch B = box(c);
    CUIBM_TRY(cudaMemsetAsync(P.count, 0, 8 * sizeof(int), c.stream));
    k_plan_scan_velocity<<<dim3(blocks_for(B.nthreads), 2), kBlock, 0, c.stream>>>(B, nx, ny, b.ghostUV, b.hybridUV, P);
    k_plan_scan_pressure<<<blocks_for(B.nthreads), kBlock, 0, c.stream>>>(B, nx, ny, b.ghostP, b.hybridP, P);
    k_plan_scan_inside<<<blocks_for(c.g.nU), kBlock, 0, c.stream>>>(nx, ny, b.ghostUV, P);
    PlanGeom G2{nx, ny, c.xu, c.yu, c.xv, c.yv, b.ghostUV, b.hybridUV, b.ghostP, b.hybridP, b.biX, b.biY, b.ipX,
                b.ipY, b.bipX, b.bipY, b.ippX, b.ippY, b.gIdx, b.hIdx, b.gpIdx, b.hpIdx, b.gCoef, b.hCoef,
                b.gpCoef, b.hpCoef};
    k_plan_build<<<dim3(blocks_for(P.cap_v), 4), kBlock, 0, c.stream>>>(G2, P);
    CUIBM_TRY(cudaGetLastError());
    // the embedded method's operator rows follow the tags
    launch_embedded_rows(c);
}

// one block runs the phases in k_ib_step's order on the plan of the current tags
static void launch_ib(Context &c, int phases, double *vel)
{
    IbArrays &b = c.ib;
    IbStep S{hostside(c).plan, c.g.nx, c.g.ny, vel, c.p, b.uB, b.vB, b.uBk, b.vBk, c.P.dt, b.ustar, b.pstar,
             b.imageValue, b.biP, b.dpdn, b.gnValue, c.bc[XPLUS], c.dx};
    k_ib_step<<<1, kIbThreads, 0, c.stream>>>(S, phases);
    CUIBM_TRY(cudaGetLastError());
}

void launch_ghost_velocity(Context &c, double *field, bool) { launch_ib(c, PH_GHOST_U, field); }
void launch_hybrid_velocity(Context &c, const double *field) { launch_ib(c, PH_HYBRID_U, const_cast<double *>(field)); }
void launch_set_inside(Context &c, double *field) { launch_ib(c, PH_INSIDE, field); }
void launch_weight_uhat(Context &c) { launch_ib(c, PH_WEIGHT_U, c.uhat); }
void launch_hybrid_pressure(Context &c) { launch_ib(c, PH_HYBRID_P, c.u); }
void launch_weight_pressure(Context &c) { launch_ib(c, PH_WEIGHT_P, c.u); }
void launch_ghost_pressure(Context &c, bool) { launch_ib(c, PH_GHOST_P, c.u); }
// updateRobinBoundary: Uinf = Vinf = 1 (luo_base/intermediateVelocity.cu:216-217)
void launch_robin(Context &c) { launch_ib(c, PH_ROBIN, c.u); }

// the step's IB sequences, one launch each
void launch_ib_rhs1(Context &c) { launch_ib(c, PH_ROBIN | PH_GHOST_U | PH_INSIDE | PH_HYBRID_U, c.u); }
void launch_ib_after_velocity(Context &c) { launch_ib(c, PH_WEIGHT_U | PH_GHOST_U, c.uhat); }
void launch_ib_after_poisson(Context &c) { launch_ib(c, PH_HYBRID_P | PH_WEIGHT_P | PH_GHOST_P, c.u); }
void launch_ib_after_projection(Context &c) { launch_ib(c, PH_GHOST_U | PH_INSIDE, c.u); }
void launch_ib_robin_inside(Context &c) { launch_ib(c, PH_ROBIN | PH_INSIDE, c.u); }

// ---- surface-integral force (luo_base/calculateForce.cu:76-98 luoForce with
// luo_base/kernels/calculateForce.cu:12-213; dead code in the reference, whose
// moveBody calls the control-volume force instead) -------------------------------
// Per body point: the pressure, interpolated in angle between the two nearest
// body-intercept pressures of the ghost pressure nodes in a 4x4 window; du/dn and
// dv/dn, one-sided from the bilinear velocity at a point sqrt(2) mid_h out along the
// radius; then the traction (viscous tangential stress minus pressure) times the
// segment length |x0 - x1|, summed over the points in index order.
// Mode 1 keeps the reference's two index slips: the pressure search starts its j
// index at the box's i start (luoForce passes startI twice) and dv/dn reads the v
// block with row stride nx-1.  Mode 2 uses the box's j start and stride nx.
// Where the reference reads past an array or an unset index (no intercept on one
// side of the point), the searches stop at the array ends and the point's
// pressure is NaN.
struct SurfaceArgs {
    int n, nx, ny, mode;
    const double *bx, *by, *uB, *vB, *u, *biP, *bipX, *bipY;
    const int *ghostP, *bb;
    const double *xu, *yu, *xv, *yv;
    const double *motion;  // moving body: centre on the device; else midX, midY
    double midX, midY, nu, midH;
    double *surf, *forceOut;
};

__device__ static double surface_pressure(const SurfaceArgs &A, double x, double y, double midX, double midY)
{
    const int nx = A.nx, ny = A.ny;
    int ii = A.bb[0], jj = A.mode == 1 ? A.bb[0] : A.bb[1];
    if (jj > ny - 1) jj = ny - 1;
    while (ii < nx - 1 && A.xv[ii] < x) ii++;
    while (jj < ny - 1 && A.yu[jj] < y) jj++;
    const int I0 = ii - 2, If = ii + 1, J0 = jj - 2, Jf = jj + 1;
    const double dxn = x - midX, dyn = y - midY;
    double thetaNode = asin(dyn / sqrt(dxn * dxn + dyn * dyn));
    if (x < midX) thetaNode = M_PI - thetaNode;
    const bool wrap = thetaNode > M_PI * 5 / 4 || thetaNode < -M_PI / 4;
    if (wrap && x > midX) thetaNode += 2 * M_PI;
    double lo = -10, hi = 10;
    int loID = -1, hiID = -1;
    for (int i = I0; i <= If; i++)
        for (int j = J0; j <= Jf; j++) {
            if (i < 0 || i >= nx || j < 0 || j >= ny) continue;
            const int ip = j * nx + i;
            if (A.ghostP[ip] <= 0) continue;
            const double bxp = A.bipX[ip], byp = A.bipY[ip], ex = bxp - midX, ey = byp - midY;
            double theta = asin(ey / sqrt(ex * ex + ey * ey));
            if (bxp < midX) theta = M_PI - theta;
            if (wrap && bxp > midX) theta += 2 * M_PI;
            if (theta > thetaNode && theta < hi) {
                hi = theta;
                hiID = ip;
            }
            if (theta < thetaNode && theta > lo) {
                lo = theta;
                loID = ip;
            }
        }
    if (loID < 0 || hiID < 0) return nan("");
    return A.biP[loID] + (A.biP[hiID] - A.biP[loID]) * (thetaNode - lo) / (hi - lo);
}

// du/dn (v = 0) or dv/dn (v = 1) at the point
__device__ static double surface_dvel(const SurfaceArgs &A, int v, double x, double y, double midX, double midY)
{
    const int nx = A.nx, ny = A.ny, nU = (nx - 1) * ny;
    const double *xc = v ? A.xv : A.xu, *yc = v ? A.yv : A.yu;
    const int nxc = v ? nx : nx - 1, nyc = v ? ny - 1 : ny;
    int ii = A.bb[0], jj = A.bb[1];
    const double rise = y - midY, run = x - midX, radius = sqrt(rise * rise + run * run);
    const double dn = A.midH * sqrt(2.0), ipx = x + dn / radius * run, ipy = y + dn / radius * rise;
    while (ii < nxc - 1 && xc[ii] < ipx) ii++;
    while (jj < nyc - 1 && yc[jj] < ipy) jj++;
    if (ii < 1) ii = 1;
    if (jj < 1) jj = 1;
    const double x1 = xc[ii - 1], x2 = xc[ii], y3 = yc[jj], y1 = yc[jj - 1];
    int row = nx - 1, base = 0;
    if (v) {
        row = A.mode == 1 ? nx - 1 : nx;  // the reference's v reads use the u row stride
        base = A.mode == 1 ? ny * (nx - 1) : nU;
    }
    const double q3 = A.u[jj * row + (ii - 1) + base], q4 = A.u[jj * row + ii + base];
    const double q1 = A.u[(jj - 1) * row + (ii - 1) + base], q2 = A.u[(jj - 1) * row + ii + base];
    const double topleft = (x2 - ipx) * (y1 - ipy) / (x2 - x1) / (y1 - y3) * q3;
    const double topright = (ipx - x1) * (y1 - ipy) / (x2 - x1) / (y1 - y3) * q4;
    const double botleft = (x2 - ipx) * (ipy - y3) / (x2 - x1) / (y1 - y3) * q1;
    const double botright = (ipx - x1) * (ipy - y3) / (x2 - x1) / (y1 - y3) * q2;
    const double ipu = botleft + botright + topleft + topright;
    return (ipu - (v ? A.vB[0] : A.uB[0])) / dn;
}

__global__ void __launch_bounds__(256) k_surface_force(SurfaceArgs A)
{
    const double midX = A.motion ? A.motion[0] : A.midX, midY = A.motion ? A.motion[1] : A.midY;
    const int n = A.n;
    const double ax = A.bx[0] - A.bx[1], ay = A.by[0] - A.by[1], area = sqrt(ax * ax + ay * ay);
    double *pr = A.surf, *du = A.surf + n, *dv = A.surf + 2 * n;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const double x = A.bx[k], y = A.by[k];
        pr[k] = surface_pressure(A, x, y, midX, midY);
        du[k] = surface_dvel(A, 0, x, y, midX, midY);
        dv[k] = surface_dvel(A, 1, x, y, midX, midY);
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    double fx = 0, fy = 0;
    for (int k = 0; k < n; ++k) {
        const double ey = A.by[k] - midY, ex = A.bx[k] - midX, h = sqrt(ey * ey + ex * ex);
        const double n1 = ex / h, n2 = ey / h, mu = A.nu;
        const double tau_x = mu * ((1 - n1 * n1) * du[k] + (-n1 * n2) * dv[k]);
        const double tau_y = mu * ((-n1 * n2) * du[k] + (1 - n2 * n2) * dv[k]);
        fx += area * tau_x - area * n1 * pr[k];
        fy += area * tau_y - area * n2 * pr[k];
    }
    A.surf[3 * n] = fx;
    A.surf[3 * n + 1] = fy;
    if (A.forceOut) {
        A.forceOut[0] = fx;
        A.forceOut[1] = fy;
    }
}

void launch_surface_force(Context &c, int mode, bool to_step)
{
    if (mode != 1 && mode != 2) throw InputError("surface force mode must be 1 (as the reference) or 2 (corrected)");
    if (c.body.total < 2) throw InputError("the surface force needs at least two body points");
    IbHost &H = hostside(c);
    IbArrays &b = c.ib;
    SurfaceArgs A{c.body.total, c.g.nx, c.g.ny, mode, b.bx, b.by, b.uB, b.vB, c.u, b.biP, b.bipX, b.bipY,
                  b.ghostP, H.bb, c.xu, c.yu, c.xv, c.yv, H.moving ? b.motion : nullptr, c.ib_midX, c.ib_midY,
                  c.P.nu, c.P.midH, b.surf, to_step ? b.forceOut : nullptr};
    k_surface_force<<<1, kBlock, 0, c.stream>>>(A);
    CUIBM_TRY(cudaGetLastError());
}

void launch_force(Context &c)
{
    if (c.force_method) {
        launch_surface_force(c, c.force_method, true);
        return;
    }
    IbHost &H = hostside(c);
    k_force<<<64, kBlock, 0, c.stream>>>(c.g.nx, c.g.ny, H.bb, c.u, c.uold, c.p, c.ib.ghostUV, c.P.nu, c.dx, c.dy,
                                         c.P.dt, c.ib.forcePart, H.force_arrive, c.ib.forceOut);
    CUIBM_TRY(cudaGetLastError());
}

void launch_body_motion(Context &c, double)
{
    IbHost &H = hostside(c);
    if (c.P.VIV == 1) {  // moveBody with VIV: 1 calls viv_movement_LC instead of set_movement
        k_body_viv<<<blocks_for(c.body.total), kBlock, 0, c.stream>>>(c.body.total, c.ib.forceOut, c.P.dt,
                                                                      (double)c.P.Ured, c.ib.bdy, c.ib.by, c.ib.vB,
                                                                      c.ib.motion);
        CUIBM_TRY(cudaGetLastError());
        return;
    }
    if (c.P.VIV == 2) {  // ... and with VIV: 2 viv_movement_SC
        k_body_viv_sc<<<1, kBlock, 0, c.stream>>>(c.body.total, c.ib.forceOut, c.P.dt, (double)c.P.Ured, c.ib.bdy,
                                                  c.ib.by, c.ib.vB, c.ib.motion);
        CUIBM_TRY(cudaGetLastError());
        return;
    }
    k_body_motion<<<blocks_for(c.body.total), kBlock, 0, c.stream>>>(c.body.total, c.step_counter_dev, H.table_len,
                                                                     H.motion_table, c.ib.bdx, c.ib.velOff, c.ib.bx,
                                                                     c.ib.uB, c.ib.motion);
    CUIBM_TRY(cudaGetLastError());
}

// the prescribed body velocity with new per-point offsets: uB = unew + offU, vB = offV
__global__ void k_apply_velocity_offsets(int total, const double *off, const double *motion, double *uB, double *vB)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    uB[i] = motion[2] + off[i];
    vB[i] = off[total + i];
}

void apply_velocity_offsets(Context &c)
{
    if (c.P.VIV) throw InputError("body velocity offsets apply to prescribed motion only (VIV: 0)");
    k_apply_velocity_offsets<<<blocks_for(c.body.total), kBlock, 0, c.stream>>>(c.body.total, c.ib.velOff,
                                                                                c.ib.motion, c.ib.uB, c.ib.vB);
    CUIBM_TRY(cudaGetLastError());
    // the embedded method's hybrid rows hold the body velocity in their right-hand side
    if (c.emb.pid1) launch_embedded_rows(c);
}

const int *force_box_dev(Context &c) { return hostside(c).bb; }

void launch_body_pre_step(Context &c)
{
    k_body_pre_step<<<blocks_for(c.body.total), kBlock, 0, c.stream>>>(c.body.total, c.ib.uB, c.ib.vB, c.ib.uBk,
                                                                       c.ib.vBk, c.ib.motion);
    CUIBM_TRY(cudaGetLastError());
}

void launch_step_counter(Context &c) { k_step_counter<<<1, 1, 0, c.stream>>>(c.step_counter_dev); }

void launch_coupling_next(Context &c, cudaGraphConditionalHandle h, int use_cond)
{
    k_coupling_next<<<1, 32, 0, c.stream>>>(c.ib.motion, c.err_word, kCouplingMaxIterations, h, use_cond);
    CUIBM_TRY(cudaGetLastError());
}

bool body_moves(Context &c) { return c.has_body && hostside(c).moving; }

// updateSolver: the control-volume box of the moved body (the force of the next step uses it)
void launch_body_box(Context &c)
{
    k_body_box<<<1, 32, 0, c.stream>>>(c.body.total, c.ib.bx, c.ib.by, c.x, c.y, c.g.nx, c.g.ny, c.P.scaleCV,
                                        hostside(c).bb);
    CUIBM_TRY(cudaGetLastError());
    k_check_box<<<1, 32, 0, c.stream>>>(hostside(c).bb, c.bb_tag.i0, c.bb_tag.j0, c.bb_tag.ncx, c.bb_tag.ncy,
                                        c.err_word, kErrBodyOutsideTagBox);
    CUIBM_TRY(cudaGetLastError());
}

// ---- control-volume force without allocation -------------------------------------
// The scratch of k_force (6 partial sums per block, then an arrival counter) as a
// fixed array in the library image: up to kCvForceMaxBlocks blocks of 256 threads, one
// per box node ((ncx+1)*(ncy+1) <= 262144), loop over the force's items (about two per
// node).
constexpr int kCvForceMaxBlocks = 1024;
static __device__ __align__(256) double g_cvforce_scratch[6 * kCvForceMaxBlocks + 32];

}  // namespace cuibm

#include <mutex>

namespace {
std::mutex g_cvforce_mutex;
double *g_cvforce_ptr[64] = {};
}  // namespace

extern std::string cuibm_noalloc_error_sink(const std::string &msg);

extern "C" int cuibm_cv_force_noalloc(const double *u, const double *uold, const double *p, const int *ghost_tags_uv,
                                      const double *dx, const double *dy, int nx, int ny, int bb_i, int bb_j,
                                      int bb_ncx, int bb_ncy, double nu, double dt, double *force_out, void *stream)
{
    using namespace cuibm;
    auto fail = [](int code, const std::string &m) {
        cuibm_noalloc_error_sink(m);
        return code;
    };
    if (!u || !uold || !p || !ghost_tags_uv || !dx || !dy || !force_out)
        return fail(1, "cuibm_cv_force_noalloc: null pointer argument");
    // the box's east column reads u at column bb_i + bb_ncx (u has columns 0..nx-2) and its
    // north row reads v at row bb_j + bb_ncy (v has rows 0..ny-2)
    if (nx < 3 || ny < 3 || bb_ncx < 1 || bb_ncy < 1 || bb_i < 1 || bb_j < 1 || bb_i + bb_ncx > nx - 2 ||
        bb_j + bb_ncy > ny - 2 || !(dt > 0))
        return fail(1, "cuibm_cv_force_noalloc: box or grid sizes out of range");
    const long long nodes = (long long)(bb_ncx + 1) * (bb_ncy + 1);
    if (nodes > (long long)kCvForceMaxBlocks * kBlock)
        return fail(1, "cuibm_cv_force_noalloc: box of " + std::to_string(nodes) + " nodes exceeds the limit of " +
                           std::to_string(kCvForceMaxBlocks * kBlock) + " ((ncx+1)*(ncy+1))");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(3, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return fail(3, "cuibm_cv_force_noalloc: device ordinal beyond 63");
    double *scratch;
    {
        std::lock_guard<std::mutex> lk(g_cvforce_mutex);
        if (!g_cvforce_ptr[dev]) {
            void *ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_cvforce_scratch);
            if (e != cudaSuccess || !ptr)
                return fail(3, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_cvforce_ptr[dev] = static_cast<double *>(ptr);
        }
        scratch = g_cvforce_ptr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned int *arrive = reinterpret_cast<unsigned int *>(scratch + 6 * kCvForceMaxBlocks);
    // the arrival counter must start at zero (the previous call's last block resets it, but a
    // call interrupted by an error would not)
    e = cudaMemsetAsync(arrive, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return fail(3, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    const int blocks = (int)((nodes + kBlock - 1) / kBlock);
    k_force_box<<<blocks, kBlock, 0, st>>>(nx, ny, bb_i, bb_j, bb_ncx, bb_ncy, u, uold, p, ghost_tags_uv, nu, dx, dy,
                                          dt, scratch, arrive, force_out);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(3, std::string("k_force launch: ") + cudaGetErrorString(e));
    return 0;
}
