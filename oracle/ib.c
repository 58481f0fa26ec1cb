/*
 * Immersed-boundary kernels of the external (Luo) method (oracle restatement;
 * test infrastructure only).
 *
 * or_tagPoints        luo_base/tagPoints.cu:17-73 (fills), luo_base/kernels/tagPoints.cu
 *                     tag_u_luo :13-427, tag_v_luo :429-826, tag_p_luo :828-1155,
 *                     zero_pressure_luo / zero_x_luo / zero_y_luo :1157-1298
 * or_ghost_velocity   luo_base/kernels/biLinearInterpolation.cu interpolateVelocityToGhostNodeX/Y :13-353
 * or_hybrid_velocity  biLinearInterpolation.cu interpolateVelocityToHybridNodeX/Y :355-668
 * or_hybrid_pressure  biLinearInterpolation.cu interpolatePressureToHybridNode :670-856
 * or_ghost_pressure   biLinearInterpolation.cu interpolatePressureToGhostNode :858-1066
 * or_weight           luoIBM/kernels/weight.cu weightX/weightY/weightP
 * or_setInsideVelocity luo_base/kernels/intermediateVelocity.cu setInsideVelocity
 * or_updateRobinBoundary FadlunModified/kernels/intermediateVelocity.cu updateBoundaryX/Y
 * or_calculateForce   luo_base/calculateForce.cu:21-74 with FadlunModified/kernels/calculateForce.cu
 * or_surfaceForce     luo_base/calculateForce.cu:76-98 (luoForce) with luo_base/kernels/calculateForce.cu
 *                     force_pressure :12-91, force_velocity_x :93-140, force_velocity_y :142-189, force :191-212
 *
 * Race semantics: threads run one after another in global-index order (write
 * conflicts between neighbouring tagged nodes resolve as "last thread wins");
 * the ghost interpolations that overwrite the field they read use snapshot
 * semantics (every node reads the field as it was before the launch).
 * Threads whose bounding-box row index goes past the last row (the last block
 * of the reference's 256-thread grid) are run too, as in the reference.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

#define EPS 1.e-10

/* Which form of the body intercept the tagging uses: 0 the reference's trigonometric
 * form, 1 (the default) its closed form.  Both give the foot of the perpendicular
 * from (px,py) onto the line through body points k and l at distance b cos(th) from
 * point k along the segment.  The reference computes th = acos((p^2 + b^2 - o^2) /
 * (2 p b)), then a = b sin(th) and a / tan(th) (tagPoints.cu, e.g. :107-117): three
 * transcendental calls whose last bits differ between CUDA's and the C library's
 * implementations.  a / tan(th) = b cos(th) = (p^2 + b^2 - o^2) / (2 p) (law of
 * cosines) needs only +, -, x, / and sqrt, which are correctly rounded on both, so
 * with no fused multiply-add the GPU's intercepts (and every interpolation weight
 * built from them) equal this restatement's bit for bit.  Form 0 is kept to pin this
 * restatement against the reference's own kernels (golden fixtures); the two forms
 * differ by a few ulp of the coordinates. */
static int intercept_form = 1;
void or_set_intercept_form(int form) { intercept_form = form; }
int or_get_intercept_form(void) { return intercept_form; }

static void intercept(const double *bx, const double *by, int k, int l, double px, double py, double *ix,
                      double *iy)
{
    if (intercept_form == 0) {
        double p = sqrt(pow((bx[l] - bx[k]), 2) + pow((by[l] - by[k]), 2));
        double o = sqrt(pow((bx[l] - px), 2) + pow((by[l] - py), 2));
        double b = sqrt(pow((px - bx[k]), 2) + pow((py - by[k]), 2));
        double th = acos((p * p + b * b - o * o) / (2 * p * b));
        double a = sin(th) * b;
        *iy = by[k] + (by[l] - by[k]) / p * a / tan(th);
        *ix = bx[k] + (bx[l] - bx[k]) / p * a / tan(th);
        return;
    }
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

/* one velocity node (kind 0 = u, 1 = v) of tag_u_luo / tag_v_luo */
static void tag_velocity_node(or_tags *T, int kind, int idx, const double *bx, const double *by, const double *vel,
                              const double *xc, const double *yc, int i_start, int j_start, int width, int nx,
                              int ny, int total, double midX, double midY)
{
    const int nU = (nx - 1) * ny;
    int i = idx % width, j = idx / width, I = i_start + i, J = j_start + j;
    int sv = kind == 0 ? nx - 1 : nx;
    int n = kind == 0 ? J * (nx - 1) + I : J * nx + I + nU;
    int ip = J * nx + I;
    if (kind == 0 ? (n >= nU) : (n >= nU + nx * (ny - 1))) return;
    int k = total - 1, l = 0;
    int outsideX = 1, outsideY = 1, flag = 0;
    int fX = -1, fY = -1, f2X = -1, f2Y = -1, bottom, top, left, right;
    double uvX = 0.0, uvY = 0.0, Xa = 1.0, Ya = 1.0, Xb = 1.0, Yb = 1.0, x = 0.0, y = 0.0;
    double *bix = T->bi_x, *biy = T->bi_y, *ipx = T->ip_x, *ipy = T->ip_y;
    if (kind == 0) {
        T->dist_u_body[ip] = 0;
    }
    while (l < total && (kind == 1 || !flag)) {
        if (by[k] > by[l]) { bottom = l; top = k; } else { bottom = k; top = l; }
        if (bx[k] > bx[l]) { left = l; right = k; } else { left = k; right = l; }
        /* rays along x */
        if (by[bottom] - EPS < yc[J] && by[top] - EPS > yc[J] && (kind == 0 || !flag)) {
            if (fabs(by[l] - by[k]) > EPS) {
                x = bx[k] + (bx[l] - bx[k]) * (yc[J] - by[k]) / (by[l] - by[k]);
                uvX = vel[k] + (vel[l] - vel[k]) * (yc[J] - by[k]) / (by[l] - by[k]);
                if (x > xc[I] + EPS) outsideX = !outsideX;
                if (x > xc[I - 1] + EPS && x < xc[I] - EPS) {
                    /* crossing in the cell to the left: right of the body */
                    fX = n;
                    f2X = n + 1;
                    if (x > midX + EPS) {
                        T->ghostTagsUV[n - 1] = n - 1;
                        intercept(bx, by, k, l, xc[I - 1], yc[J], &bix[n - 1], &biy[n - 1]);
                        ipy[n - 1] = biy[n - 1] + (biy[n - 1] - yc[J]);
                        ipx[n - 1] = bix[n - 1] + (bix[n - 1] - xc[I - 1]);
                        intercept(bx, by, k, l, xc[I], yc[J], &bix[n], &biy[n]);
                        ipy[n] = 2 * yc[J] - biy[n];
                        ipx[n] = 2 * xc[I] - bix[n];
                    }
                    Xa = xc[I] - x;
                    Xb = xc[I + 1] - xc[I];
                    if (kind == 0 && x > midX) T->dist_u_body[ip] = Xa;
                } else if (x > xc[I] + EPS && x < xc[I + 1] - EPS) {
                    /* crossing in the cell to the right: left of the body */
                    fX = n;
                    f2X = n - 1;
                    if (x < midX - EPS) {
                        T->ghostTagsUV[n + 1] = n + 1;
                        intercept(bx, by, k, l, xc[I + 1], yc[J], &bix[n + 1], &biy[n + 1]);
                        ipy[n + 1] = biy[n + 1] + (biy[n + 1] - yc[J]);
                        ipx[n + 1] = bix[n + 1] + (bix[n + 1] - xc[I + 1]);
                        intercept(bx, by, k, l, xc[I], yc[J], &bix[n], &biy[n]);
                        ipy[n] = 2 * yc[J] - biy[n];
                        ipx[n] = 2 * xc[I] - bix[n];
                    }
                    Xa = x - xc[I];
                    Xb = xc[I] - xc[I - 1];
                    if (kind == 0 && x < midX) T->dist_u_body[ip + 1] = Xa;
                } else if (fabs(x - xc[I]) < EPS && fabs(midX - xc[I]) > fabs(midY - yc[J])) {
                    outsideX = 1;
                    fX = n;
                    if (x < midX) {
                        T->ghostTagsUV[n + 1] = n + 1;
                        f2X = n - 1;
                        bix[n + 1] = xc[I]; biy[n + 1] = yc[J]; ipx[n + 1] = xc[I - 1]; ipy[n + 1] = yc[J];
                        bix[n] = xc[I]; biy[n] = yc[J]; ipx[n] = xc[I - 1]; ipy[n] = yc[J];
                        Xa = 0;
                        Xb = xc[I] - xc[I - 1];
                    }
                    if (x > midX) {
                        T->ghostTagsUV[n - 1] = n - 1;
                        f2X = n + 1;
                        bix[n - 1] = xc[I]; biy[n - 1] = yc[J]; ipx[n - 1] = xc[I + 1]; ipy[n - 1] = yc[J];
                        bix[n] = xc[I]; biy[n] = yc[J]; ipx[n] = xc[I + 1]; ipy[n] = yc[J];
                        Xa = 0;
                        Xb = xc[I + 1] - xc[I];
                    }
                    flag = 1;
                }
            }
        }
        /* rays along y */
        if (bx[left] - EPS < xc[I] && bx[right] - EPS > xc[I] && (kind == 0 || !flag)) {
            if (fabs(bx[l] - bx[k]) > EPS) {
                y = by[k] + (by[l] - by[k]) * (xc[I] - bx[k]) / (bx[l] - bx[k]);
                uvY = vel[k] + (vel[l] - vel[k]) * (xc[I] - bx[k]) / (bx[l] - bx[k]);
                if (y > yc[J] + EPS) outsideY = !outsideY;
                if (y > yc[J - 1] + EPS && y < yc[J] - EPS) {
                    /* crossing just below: above the body */
                    fY = n;
                    f2Y = n + sv;
                    if (y > midY + EPS) {
                        T->ghostTagsUV[n - sv] = n - sv;
                        intercept(bx, by, k, l, xc[I], yc[J - 1], &bix[n - sv], &biy[n - sv]);
                        ipy[n - sv] = biy[n - sv] + (biy[n - sv] - yc[J - 1]);
                        ipx[n - sv] = bix[n - sv] + (bix[n - sv] - xc[I]);
                        intercept(bx, by, k, l, xc[I], yc[J], &bix[n], &biy[n]);
                        ipy[n] = 2 * yc[J] - biy[n];
                        ipx[n] = 2 * xc[I] - bix[n];
                    }
                    Ya = yc[J] - y;
                    Yb = yc[J + 1] - yc[J];
                    if (kind == 1 && outsideY) T->dist_v_body[ip] = Ya;
                } else if (y > yc[J] + EPS && y < yc[J + 1] - EPS) {
                    /* crossing just above: below the body */
                    fY = n;
                    f2Y = n - sv;
                    if (y < midY - EPS) {
                        T->ghostTagsUV[n + sv] = n + sv;
                        intercept(bx, by, k, l, xc[I], yc[J + 1], &bix[n + sv], &biy[n + sv]);
                        ipy[n + sv] = biy[n + sv] + (biy[n + sv] - yc[J + 1]);
                        ipx[n + sv] = bix[n + sv] + (bix[n + sv] - xc[I]);
                        intercept(bx, by, k, l, xc[I], yc[J], &bix[n], &biy[n]);
                        ipy[n] = 2 * yc[J] - biy[n];
                        ipx[n] = 2 * xc[I] - bix[n];
                    }
                    Ya = y - yc[J];
                    Yb = yc[J] - yc[J - 1];
                    if (kind == 1 && outsideY) T->dist_v_body[ip + nx] = Ya;
                } else if (kind == 0 ? (fabs(y - yc[J]) < EPS && fabs(y - midY) > fabs(x - midX))
                                     : (fabs(y - yc[J]) < EPS && fabs(midY - yc[J]) > fabs(midX - xc[I]))) {
                    outsideY = 1;
                    fY = n;
                    if (y < midY) {
                        T->ghostTagsUV[n + sv] = n + sv;
                        f2X = n - sv; /* the reference sets the x-ray flag here */
                        bix[n + sv] = xc[I]; biy[n + sv] = yc[J]; ipx[n + sv] = xc[I]; ipy[n + sv] = yc[J - 1];
                        bix[n] = xc[I]; biy[n] = yc[J]; ipx[n] = xc[I]; ipy[n] = yc[J - 1];
                        Ya = 0;
                        Yb = yc[J] - yc[J - 1];
                    }
                    if (y > midY) {
                        T->ghostTagsUV[n - sv] = n - sv;
                        f2X = n + sv;
                        bix[n - sv] = xc[I]; biy[n - sv] = yc[J]; ipx[n - sv] = xc[I]; ipy[n - sv] = yc[J + 1];
                        bix[n] = xc[I]; biy[n] = yc[J]; ipx[n] = xc[I]; ipy[n] = yc[J + 1];
                        Ya = 0;
                        Yb = yc[J + 1] - yc[J];
                    }
                    flag = 1;
                }
            }
        }
        k = l;
        l = l + 1;
    }
    int useX = outsideX && fX >= 0, useY = outsideY && fY >= 0;
    if (kind == 0 ? useX : (useX && !useY)) {
        T->ghostTagsUV[n] = -1;
        T->hybridTagsUV[n] = fX;
        T->hybridTagsUV2[n] = f2X;
        T->dist_node[n] = Xa;
        T->dist_between[n] = Xb;
        T->uv[n] = uvX;
    } else if (useY) {
        T->ghostTagsUV[n] = -1;
        T->hybridTagsUV[n] = fY;
        T->hybridTagsUV2[n] = f2Y;
        T->dist_node[n] = Ya;
        T->dist_between[n] = Yb;
        T->uv[n] = uvY;
    }
}

/* one pressure node of tag_p_luo */
static void tag_pressure_node(or_tags *T, int idx, const double *bx, const double *by, const double *yu,
                              const double *xv, int i_start, int j_start, int width, int nx, int ny, int total,
                              double midX, double midY)
{
    int i = idx % width, j = idx / width, I = i_start + i, J = j_start + j, ip = J * nx + I;
    if (ip >= nx * ny) return;
    int k = total - 1, l = 0, flag = 0, bottom, top, left, right;
    double x, y;
    double *bx_ = T->bip_x, *by_ = T->bip_y, *px = T->ipp_x, *py = T->ipp_y;
    while (l < total) {
        if (by[k] > by[l]) { bottom = l; top = k; } else { bottom = k; top = l; }
        if (bx[k] > bx[l]) { left = l; right = k; } else { left = k; right = l; }
        if (by[bottom] - EPS < yu[J] && by[top] - EPS > yu[J] && !flag) {
            if (fabs(by[l] - by[k]) > EPS) {
                x = bx[k] + (bx[l] - bx[k]) * (yu[J] - by[k]) / (by[l] - by[k]);
                /* ghost node just inside: right of mid / left of mid */
                if ((x > midX + EPS && x > xv[I] + EPS + EPS && x < xv[I + 1] - EPS) ||
                    (!(x > midX + EPS && x > xv[I] + EPS + EPS && x < xv[I + 1] - EPS) && x < midX + EPS &&
                     x < xv[I] - EPS && x > xv[I - 1] + EPS)) {
                    T->ghostTagsP[ip] = ip;
                    intercept(bx, by, k, l, xv[I], yu[J], &bx_[ip], &by_[ip]);
                    py[ip] = by_[ip] + (by_[ip] - yu[J]);
                    px[ip] = bx_[ip] + (bx_[ip] - xv[I]);
                }
                /* hybrid node just outside */
                if ((x > midX + EPS && x < xv[I] - EPS && x > xv[I - 1] + EPS) ||
                    (!(x > midX + EPS && x < xv[I] - EPS && x > xv[I - 1] + EPS) && x < midX + EPS &&
                     x > xv[I] + EPS && x < xv[I + 1] - EPS)) {
                    T->hybridTagsP[ip] = ip;
                    intercept(bx, by, k, l, xv[I], yu[J], &bx_[ip], &by_[ip]);
                    py[ip] = 2 * yu[J] - by_[ip];
                    px[ip] = 2 * xv[I] - bx_[ip];
                }
                if (fabs(x - xv[I]) < EPS && fabs(midX - xv[I]) > fabs(midY - yu[J])) {
                    T->hybridTagsP[ip] = ip;
                    if (x < midX) {
                        T->ghostTagsP[ip + 1] = ip + 1;
                        bx_[ip + 1] = xv[I]; by_[ip + 1] = yu[J]; px[ip + 1] = xv[I - 1]; py[ip + 1] = yu[J];
                        bx_[ip] = xv[I]; by_[ip] = yu[J]; px[ip] = xv[I - 1]; py[ip] = yu[J];
                    } else if (x > midX) {
                        T->ghostTagsP[ip - 1] = ip - 1;
                        bx_[ip - 1] = xv[I]; by_[ip - 1] = yu[J]; px[ip - 1] = xv[I + 1]; py[ip - 1] = yu[J];
                        bx_[ip] = xv[I]; by_[ip] = yu[J]; px[ip] = xv[I + 1]; py[ip] = yu[J];
                    }
                    flag = 1;
                }
            }
        }
        if (bx[left] - EPS < xv[I] && bx[right] - EPS > xv[I] && !flag) {
            if (fabs(bx[l] - bx[k]) > EPS) {
                y = by[k] + (by[l] - by[k]) * (xv[I] - bx[k]) / (bx[l] - bx[k]);
                if ((y > midY + EPS && y > yu[J] + EPS && y < yu[J + 1] - EPS) ||
                    (!(y > midY + EPS && y > yu[J] + EPS && y < yu[J + 1] - EPS) && y < midY + EPS &&
                     y < yu[J] - EPS && y > yu[J - 1] + EPS)) {
                    T->ghostTagsP[ip] = ip;
                    intercept(bx, by, k, l, xv[I], yu[J], &bx_[ip], &by_[ip]);
                    py[ip] = by_[ip] + (by_[ip] - yu[J]);
                    px[ip] = bx_[ip] + (bx_[ip] - xv[I]);
                }
                if ((y > midY + EPS && y < yu[J] - EPS && y > yu[J - 1] + EPS) ||
                    (!(y > midY + EPS && y < yu[J] - EPS && y > yu[J - 1] + EPS) && y < midY + EPS &&
                     y > yu[J] + EPS && y < yu[J + 1] - EPS)) {
                    T->hybridTagsP[ip] = ip;
                    intercept(bx, by, k, l, xv[I], yu[J], &bx_[ip], &by_[ip]);
                    py[ip] = 2 * yu[J] - by_[ip];
                    px[ip] = 2 * xv[I] - bx_[ip];
                }
                if (fabs(y - yu[J]) < EPS && fabs(midY - yu[J]) > fabs(midX - xv[I])) {
                    T->hybridTagsP[ip] = ip;
                    if (y < midY) {
                        T->ghostTagsP[ip + nx] = ip + nx;
                        bx_[ip + nx] = xv[I]; by_[ip + nx] = yu[J]; px[ip + nx] = xv[I]; py[ip + nx] = yu[J - 1];
                        bx_[ip] = xv[I]; by_[ip] = yu[J]; px[ip] = xv[I]; py[ip] = yu[J - 1];
                    }
                    if (y > midY) {
                        T->ghostTagsP[ip - nx] = ip - nx;
                        bx_[ip - nx] = xv[I]; by_[ip - nx] = yu[J]; px[ip - nx] = xv[I]; py[ip - nx] = yu[J + 1];
                        bx_[ip] = xv[I]; by_[ip] = yu[J]; px[ip] = xv[I]; py[ip] = yu[J + 1];
                    }
                    flag = 1;
                }
            }
        }
        k = l;
        l = l + 1;
    }
}

/* zero_pressure_luo / zero_x_luo / zero_y_luo: one row of the box, left to right;
 * tags[] points at the class block, stride = row length of that class */
static void zero_row(int *tags, int J, int stride, int i_start, int i_end, int scan_end)
{
    int rowIsntDone = 1, flag = 0;
    for (int i = i_start; i < i_end; ++i) {
        int I = J * stride + i;
        if (tags[I - 1] >= 0) {
            if (tags[I] != -1 && tags[I - 1] == 0) rowIsntDone = 0;
            if (tags[I] == -1 && rowIsntDone) tags[I] = 0;
            if (tags[I] == 0 && tags[I - 1] != 0) {
                int k = i;
                while (k < scan_end) {
                    k++;
                    if (tags[J * stride + k] != -1) flag = 1;
                }
                if (!flag) {
                    tags[I] = -1;
                    rowIsntDone = 0;
                }
            }
        }
    }
}

void or_tagPoints(or_tags *T, const double *bx, const double *by, const double *uB, const double *vB,
                  const double *xu, const double *yu, const double *xv, const double *yv, int i_start,
                  int j_start, int width, int height, int nx, int ny, int totalPoints, double midX, double midY)
{
    const int nU = (nx - 1) * ny, nUV = nU + nx * (ny - 1), nP = nx * ny;
    for (int k = 0; k < nUV; ++k) {
        T->ghostTagsUV[k] = -1;
        T->hybridTagsUV[k] = -1;
        T->hybridTagsUV2[k] = -1;
        T->dist_node[k] = 1;
        T->dist_between[k] = 1;
        T->bi_x[k] = 0;
        T->bi_y[k] = 0;
        T->ip_x[k] = 0;
        T->ip_y[k] = 0;
    }
    for (int k = 0; k < nP; ++k) {
        T->ghostTagsP[k] = -1;
        T->hybridTagsP[k] = -1;
    }
    const int threads = ((int)((double)width * height - 0.5) / 256 + 1) * 256;
    for (int idx = 0; idx < threads; ++idx)
        tag_velocity_node(T, 0, idx, bx, by, uB, xu, yu, i_start, j_start, width, nx, ny, totalPoints, midX, midY);
    for (int idx = 0; idx < threads; ++idx)
        tag_velocity_node(T, 1, idx, bx, by, vB, xv, yv, i_start, j_start, width, nx, ny, totalPoints, midX, midY);
    for (int idx = 0; idx < threads; ++idx)
        tag_pressure_node(T, idx, bx, by, yu, xv, i_start, j_start, width, nx, ny, totalPoints, midX, midY);
    const int i_end = i_start + width, j_end = j_start + height;
    const int rows = ((int)((double)(i_end - i_start) - 0.5) / 256 + 1) * 256;
    for (int j = 0; j < rows; ++j) {
        int J = j_start + j;
        if (J > j_end) continue;
        zero_row(T->ghostTagsP, J, nx, i_start, i_end, nx);
    }
    for (int j = 0; j < rows; ++j) {
        int J = j_start + j;
        if (J > j_end) continue;
        zero_row(T->ghostTagsUV, J, nx - 1, i_start, i_end, nx - 1);
    }
    for (int j = 0; j < rows; ++j) {
        int J = j_start + j;
        if (J > j_end) continue;
        zero_row(T->ghostTagsUV + nU, J, nx, i_start, i_end, nx - 1);
    }
}

/* ---- bilinear fit through four points: cofactor inverse (biLinearInterpolation.cu) ---- */
static void inverse4(const double a[16], double b[16], double *det)
{
    double a11 = a[0], a12 = a[1], a13 = a[2], a14 = a[3];
    double a21 = a[4], a22 = a[5], a23 = a[6], a24 = a[7];
    double a31 = a[8], a32 = a[9], a33 = a[10], a34 = a[11];
    double a41 = a[12], a42 = a[13], a43 = a[14], a44 = a[15];
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

static void bilinear_rows(const double x[4], const double y[4], double a[16])
{
    for (int l = 0; l < 4; ++l) {
        a[4 * l] = 1;
        a[4 * l + 1] = x[l];
        a[4 * l + 2] = y[l];
        a[4 * l + 3] = x[l] * y[l];
    }
}

/* weights of q1..q4 at (px,py): (b1k + b2k px + b3k py + b4k px py)/det */
static void weights_at(const double b[16], double det, double px, double py, double w[4])
{
    for (int c = 0; c < 4; ++c) w[c] = (b[c] + b[4 + c] * px + b[8 + c] * py + b[12 + c] * px * py) / det;
}

static void store_stencil(or_interp *R, int n, const int idx[4], const double w[4], const double q[4])
{
    R->index1[n] = idx[0]; R->index2[n] = idx[1]; R->index3[n] = idx[2]; R->index4[n] = idx[3];
    R->q1coef[n] = w[0]; R->q2coef[n] = w[1]; R->q3coef[n] = w[2]; R->q4coef[n] = w[3];
    if (R->q1) { R->q1[n] = q[0]; R->q2[n] = q[1]; R->q3[n] = q[2]; R->q4[n] = q[3]; }
}

static int threads_for(int width, int height) { return ((int)((double)width * height - 0.5) / 256 + 1) * 256; }

void or_ghost_velocity(int dir, double *u, int set, const int *ghostTagsUV, double uB0, const double *yc,
                       const double *xc, const double *bi_x, const double *bi_y, const double *ip_x,
                       const double *ip_y, int i_start, int j_start, int width, int height, int nx, int ny,
                       or_interp *R)
{
    const int nU = (nx - 1) * ny, nUV = nU + nx * (ny - 1);
    double *snap = malloc(sizeof(double) * nUV);
    memcpy(snap, u, sizeof(double) * nUV);
    const int nt = threads_for(width, height);
    for (int idx = 0; idx < nt; ++idx) {
        int I = i_start + idx % width, J = j_start + idx / width;
        int n = dir == 0 ? J * (nx - 1) + I : J * nx + I + nU;
        if (dir == 1 && J * nx + I > nx * (ny - 1)) continue;
        if (n >= nUV || ghostTagsUV[n] <= 0) continue;
        int ii = I - 5, jj = J - 5;
        while (xc[ii] < ip_x[n]) ii++;
        while (yc[jj] < ip_y[n]) jj++;
        double x[4] = {xc[ii - 1], xc[ii], xc[ii - 1], xc[ii]};
        double y[4] = {yc[jj - 1], yc[jj - 1], yc[jj], yc[jj]};
        int id[4];
        if (dir == 0) {
            id[0] = (jj - 1) * (nx - 1) + ii - 1; id[1] = (jj - 1) * (nx - 1) + ii;
            id[2] = jj * (nx - 1) + ii - 1;       id[3] = jj * (nx - 1) + ii;
        } else {
            id[0] = (jj - 1) * nx + ii - 1 + nU; id[1] = (jj - 1) * nx + ii + nU;
            id[2] = jj * nx + ii - 1 + nU;       id[3] = jj * nx + ii + nU;
        }
        double q[4] = {snap[id[0]], snap[id[1]], snap[id[2]], snap[id[3]]};
        double mn = 1.0, s;
        int close = -1, inflag = 0;
        for (int l = 0; l < 4; ++l) {
            s = sqrt(pow(x[l] - bi_x[n], 2) + pow(y[l] - bi_y[n], 2));
            if (s < mn) { mn = s; close = id[l]; }
            if (ghostTagsUV[id[l]] > 0) inflag = 1;
        }
        for (int l = 0; l < 4; ++l) {
            if (ghostTagsUV[id[l]] == n) {
                x[l] = bi_x[id[l]]; y[l] = bi_y[id[l]]; q[l] = uB0;
            } else if (id[l] == close && !inflag) {
                x[l] = bi_x[n]; y[l] = bi_y[n]; q[l] = uB0;
            }
        }
        double a[16], b[16], det, w[4];
        bilinear_rows(x, y, a);
        inverse4(a, b, &det);
        double a0 = b[0] / det * q[0] + b[1] / det * q[1] + b[2] / det * q[2] + b[3] / det * q[3];
        double a1 = b[4] / det * q[0] + b[5] / det * q[1] + b[6] / det * q[2] + b[7] / det * q[3];
        double a2 = b[8] / det * q[0] + b[9] / det * q[1] + b[10] / det * q[2] + b[11] / det * q[3];
        double a3 = b[12] / det * q[0] + b[13] / det * q[1] + b[14] / det * q[2] + b[15] / det * q[3];
        weights_at(b, det, ip_x[n], ip_y[n], w);
        store_stencil(R, n, id, w, q);
        double val = a0 + a1 * ip_x[n] + a2 * ip_y[n] + a3 * ip_x[n] * ip_y[n];
        R->value[n] = val;
        if (set) u[n] = 2 * uB0 - val;
    }
    free(snap);
}

void or_hybrid_velocity(int dir, const double *u, double *ustar, const int *hybridTagsUV, double uB0,
                        const double *yc, const double *xc, const double *bi_x, const double *bi_y,
                        const double *ip_x, const double *ip_y, int i_start, int j_start, int width, int height,
                        int nx, int ny, or_interp *R)
{
    const int nU = (nx - 1) * ny, nUV = nU + nx * (ny - 1);
    const int nt = threads_for(width, height);
    for (int idx = 0; idx < nt; ++idx) {
        int I = i_start + idx % width, J = j_start + idx / width;
        int n = dir == 0 ? J * (nx - 1) + I : J * nx + I + nU;
        if (dir == 1 && J * nx + I > nx * (ny - 1)) continue;
        if (n >= nUV || hybridTagsUV[n] <= 0) continue;
        int ii = I - 5, jj = J - 5;
        while (xc[ii] < ip_x[n]) ii++;
        double x[4] = {xc[ii - 1], xc[ii], xc[ii - 1], xc[ii]};
        while (yc[jj] < ip_y[n]) jj++;
        double y[4] = {yc[jj - 1], yc[jj - 1], yc[jj], yc[jj]};
        int id[4];
        if (dir == 0) {
            id[0] = (jj - 1) * (nx - 1) + ii - 1; id[1] = (jj - 1) * (nx - 1) + ii;
            id[2] = jj * (nx - 1) + ii - 1;       id[3] = jj * (nx - 1) + ii;
        } else {
            id[0] = (jj - 1) * nx + ii - 1 + nU; id[1] = (jj - 1) * nx + ii + nU;
            id[2] = jj * nx + ii - 1 + nU;       id[3] = jj * nx + ii + nU;
        }
        double q[4] = {u[id[0]], u[id[1]], u[id[2]], u[id[3]]};
        for (int l = 0; l < 4; ++l)
            if (hybridTagsUV[id[l]] == n) { x[l] = bi_x[n]; y[l] = bi_y[n]; q[l] = uB0; }
        double a[16], b[16], det, w[4];
        bilinear_rows(x, y, a);
        inverse4(a, b, &det);
        double a0 = (b[0] * q[0] + b[1] * q[1] + b[2] * q[2] + b[3] * q[3]) / det;
        double a1 = (b[4] * q[0] + b[5] * q[1] + b[6] * q[2] + b[7] * q[3]) / det;
        double a2 = (b[8] * q[0] + b[9] * q[1] + b[10] * q[2] + b[11] * q[3]) / det;
        double a3 = (b[12] * q[0] + b[13] * q[1] + b[14] * q[2] + b[15] * q[3]) / det;
        weights_at(b, det, xc[I], yc[J], w);
        store_stencil(R, n, id, w, q);
        ustar[n] = a0 + a1 * xc[I] + a2 * yc[J] + a3 * yc[J] * xc[I];
        R->value[n] = a0 + a1 * ip_x[n] + a2 * ip_y[n] + a3 * ip_x[n] * ip_y[n];
    }
}

void or_hybrid_pressure(const double *p, double *pstar, const int *hybridTagsP, double dudt_u, double dudt_v,
                        const double *yu, const double *xv, const double *bip_x, const double *bip_y,
                        const double *ipp_x, const double *ipp_y, int i_start, int j_start, int width,
                        int height, int nx, int ny, or_interp *R)
{
    const int nt = threads_for(width, height);
    for (int idx = 0; idx < nt; ++idx) {
        int I = i_start + idx % width, J = j_start + idx / width, ip = J * nx + I;
        if (ip >= nx * ny || hybridTagsP[ip] <= 0) continue;
        int ii = I - 5, jj = J - 5;
        while (xv[ii] < ipp_x[ip]) ii++;
        double x[4] = {xv[ii - 1], xv[ii], xv[ii - 1], xv[ii]};
        while (yu[jj] < ipp_y[ip]) jj++;
        double y[4] = {yu[jj - 1], yu[jj - 1], yu[jj], yu[jj]};
        int id[4] = {(jj - 1) * nx + ii - 1, (jj - 1) * nx + ii, jj * nx + ii - 1, jj * nx + ii};
        double q[4] = {p[id[0]], p[id[1]], p[id[2]], p[id[3]]};
        double a[16], b[16], det, w[4];
        bilinear_rows(x, y, a);
        for (int l = 0; l < 4; ++l) {
            if (hybridTagsP[id[l]] == ip) {
                x[l] = bip_x[ip];
                y[l] = bip_y[ip];
                double nxv = ipp_x[ip] - x[l], nyv = ipp_y[ip] - y[l];
                double nl = sqrt(nxv * nxv + nyv * nyv);
                q[l] = -(nxv / nl * dudt_u + nyv / nl * dudt_v);
                a[l * 4] = 0;
                a[l * 4 + 1] = nxv / nl;
                a[l * 4 + 2] = nyv / nl;
                a[l * 4 + 3] = nyv / nl * x[l] + nxv / nl * y[l];
            }
        }
        inverse4(a, b, &det);
        double a0 = b[0] / det * q[0] + b[1] / det * q[1] + b[2] / det * q[2] + b[3] / det * q[3];
        double a1 = b[4] / det * q[0] + b[5] / det * q[1] + b[6] / det * q[2] + b[7] / det * q[3];
        double a2 = b[8] / det * q[0] + b[9] / det * q[1] + b[10] / det * q[2] + b[11] / det * q[3];
        double a3 = b[12] / det * q[0] + b[13] / det * q[1] + b[14] / det * q[2] + b[15] / det * q[3];
        weights_at(b, det, xv[I], yu[J], w);
        store_stencil(R, ip, id, w, q);
        pstar[ip] = a0 + a1 * xv[I] + a2 * yu[J] + a3 * xv[I] * yu[J];
    }
}

void or_ghost_pressure(double *p, int set, const int *ghostTagsP, double dudt_u, double dudt_v,
                       const double *yu, const double *xv, const double *bip_x, const double *bip_y,
                       const double *ipp_x, const double *ipp_y, int i_start, int j_start, int width, int height,
                       int nx, int ny, or_interp *R)
{
    const int nP = nx * ny;
    double *snap = malloc(sizeof(double) * nP);
    memcpy(snap, p, sizeof(double) * nP);
    const int nt = threads_for(width, height);
    for (int idx = 0; idx < nt; ++idx) {
        int I = i_start + idx % width, J = j_start + idx / width, ip = J * nx + I;
        if (ip >= nP || ghostTagsP[ip] <= 0) continue;
        int ii = I - 5, jj = J - 5;
        while (xv[ii] < ipp_x[ip]) ii++;
        while (yu[jj] < ipp_y[ip]) jj++;
        double x[4] = {xv[ii - 1], xv[ii], xv[ii - 1], xv[ii]};
        double y[4] = {yu[jj - 1], yu[jj - 1], yu[jj], yu[jj]};
        int id[4] = {(jj - 1) * nx + ii - 1, (jj - 1) * nx + ii, jj * nx + ii - 1, jj * nx + ii};
        double q[4] = {snap[id[0]], snap[id[1]], snap[id[2]], snap[id[3]]};
        double a[16], b[16], det, w[4];
        bilinear_rows(x, y, a);
        double mn = 1.0, s, matD = 0;
        int close = -1;
        for (int l = 0; l < 4; ++l) {
            s = sqrt(pow(x[l] - bip_x[ip], 2) + pow(y[l] - bip_y[ip], 2));
            if (s < mn) { mn = s; close = id[l]; }
        }
        for (int l = 0; l < 4; ++l) {
            if (ghostTagsP[id[l]] > 0) {
                x[l] = bip_x[id[l]];
                y[l] = bip_y[id[l]];
                double nxv = ipp_x[id[l]] - x[l], nyv = ipp_y[id[l]] - y[l];
                double nl = sqrt(nxv * nxv + nyv * nyv);
                q[l] = -(nxv / nl * dudt_u + nyv / nl * dudt_v);
                a[l * 4] = 0;
                a[l * 4 + 1] = nxv / nl;
                a[l * 4 + 2] = nyv / nl;
                a[l * 4 + 3] = nyv / nl * x[l] + nxv / nl * y[l];
            }
            if (id[l] == close) {
                x[l] = bip_x[ip];
                y[l] = bip_y[ip];
                double nxv = ipp_x[ip] - x[l], nyv = ipp_y[ip] - y[l];
                double nl = sqrt(nxv * nxv + nyv * nyv);
                matD = (nxv / nl * dudt_u + nyv / nl * dudt_v);
            }
        }
        inverse4(a, b, &det);
        double a0 = b[0] / det * q[0] + b[1] / det * q[1] + b[2] / det * q[2] + b[3] / det * q[3];
        double a1 = b[4] / det * q[0] + b[5] / det * q[1] + b[6] / det * q[2] + b[7] / det * q[3];
        double a2 = b[8] / det * q[0] + b[9] / det * q[1] + b[10] / det * q[2] + b[11] / det * q[3];
        double a3 = b[12] / det * q[0] + b[13] / det * q[1] + b[14] / det * q[2] + b[15] / det * q[3];
        weights_at(b, det, ipp_x[ip], ipp_y[ip], w);
        store_stencil(R, ip, id, w, q);
        double ipv = a0 + a1 * ipp_x[ip] + a2 * ipp_y[ip] + a3 * ipp_y[ip] * ipp_x[ip];
        R->value[ip] = a0 + a1 * bip_x[ip] + a2 * bip_y[ip] + a3 * bip_x[ip] * bip_y[ip];
        R->dpdn[ip] = sqrt(pow(ipp_x[ip] - xv[I], 2) + pow(ipp_y[ip] - yu[J], 2)) * matD;
        if (set) p[ip] = ipv + R->dpdn[ip];
    }
    free(snap);
}

void or_weight(int dir, double *f, const double *fstar, const int *ghostTags, const int *hybridTags,
               const double *yc, const double *xc, const double *bi_x, const double *bi_y, int i_start,
               int j_start, int width, int height, int nx, int ny)
{
    const int nU = (nx - 1) * ny;
    const int nt = threads_for(width, height);
    for (int idx = 0; idx < nt; ++idx) {
        int I = i_start + idx % width, J = j_start + idx / width, n, sv;
        if (dir == 0) {
            n = J * (nx - 1) + I;
            sv = nx - 1;
        } else if (dir == 1) {
            if (J * nx + I > nx * (ny - 1)) continue;
            n = J * nx + I + nU;
            sv = nx;
        } else {
            if (J * nx + I > nx * ny) continue;
            n = J * nx + I;
            sv = nx;
        }
        if (hybridTags[n] <= 0) continue;
        double d1 = 0, d2 = 0, alpha, dx = xc[I] - xc[I - 1], dy = yc[J] - yc[J - 1];
        if (ghostTags[n - 1] > 0)
            d1 = sqrt(pow(bi_x[n - 1] - xc[I - 1], 2) + pow(bi_y[n - 1] - yc[J], 2));
        else if (ghostTags[n + 1] > 0)
            d1 = sqrt(pow(bi_x[n + 1] - xc[I + 1], 2) + pow(bi_y[n + 1] - yc[J], 2));
        if (ghostTags[n - sv] > 0) d2 = sqrt(pow(bi_x[n - sv] - xc[I], 2) + pow(bi_y[n - sv] - yc[J - 1], 2));
        if (ghostTags[n + sv] > 0) d2 = sqrt(pow(bi_x[n + sv] - xc[I], 2) + pow(bi_y[n + sv] - yc[J + 1], 2));
        alpha = sqrt(pow(d1 / dx, 2) + pow(d2 / dy, 2));
        f[n] = (1 - alpha) * f[n] + alpha * fstar[n];
    }
}

void or_setInsideVelocity(const int *ghostTags, double *u, double uB0, double vB0, int nx, int ny)
{
    const int nU = (nx - 1) * ny, nUV = nU + nx * (ny - 1);
    for (int i = 0; i < nU; ++i) {
        int I = i % (nx - 1), J = i / (nx - 1), iu = J * (nx - 1) + I, iv = J * nx + I + nU;
        u[iu] = (ghostTags[iu] != 0) * u[iu] + (ghostTags[iu] == 0) * uB0;
        if (iv < nUV) u[iv] = (ghostTags[iv] != 0) * u[iv] + (ghostTags[iv] == 0) * vB0;
    }
}

void or_updateRobinBoundary(const double *u, double *xp, const double *dx, double dt, double Uinf, double Vinf,
                            int nx, int ny)
{
    const int nU = (nx - 1) * ny;
    for (int J = 0; J < ny; ++J) {
        int I = nx - 1, i = J * (nx - 1) + I;
        double beta = Uinf * dt / dx[I];
        xp[J] = xp[J] * (1 - beta) + beta * u[i - 1];
    }
    for (int J = 0; J < ny - 1; ++J) {
        int I = nx, i = J * nx + I;
        double beta = Vinf * dt / dx[I - 1];
        xp[J + ny] = xp[J + ny] * (1 - beta) + beta * u[i + nU - 1];
    }
}

/* control-volume force on the bounding box (Lai & Peskin 2000): per-term
 * arrays summed in index order */
void or_calculateForce(const double *u, const double *uold, const double *p, const int *ghostTagsUV, double nu,
                       const double *dx, const double *dy, double dt, int nx, int ny, int I, int J, int ncx,
                       int ncy, double *fx, double *fy)
{
    const int nU = (nx - 1) * ny;
    double sxx = 0, sxy = 0, sxu = 0, syx = 0, syy = 0, syu = 0;
    for (int idx = 0; idx < ncy; ++idx) { /* dragLeftRight */
        int Ip = (J + idx) * nx + I, Iu = (J + idx) * (nx - 1) + I;
        sxx += -((p[Ip + ncx] - p[Ip]) * dy[J + idx] +
                 ((u[Iu + ncx] + u[Iu + ncx - 1]) * (u[Iu + ncx] + u[Iu + ncx - 1]) / 4 -
                  (u[Iu - 1] + u[Iu]) * (u[Iu - 1] + u[Iu]) / 4) * dy[J + idx] -
                 nu * ((u[Iu + ncx] - u[Iu + ncx - 1]) / dx[I + ncx] - (u[Iu] - u[Iu - 1]) / dx[I]) * dy[J + idx]);
    }
    for (int idx = 0; idx <= ncx; ++idx) { /* dragBottomTop */
        int Iu = J * (nx - 1) + (I - 1 + idx), Iv = nU + (J - 1) * nx + I + idx;
        sxy += -((0.25 * (u[Iu + ncy * (nx - 1)] + u[Iu + (ncy - 1) * (nx - 1)]) *
                      (u[Iv + ncy * nx] + u[Iv + ncy * nx - 1]) -
                  0.25 * (u[Iu] + u[Iu - (nx - 1)]) * (u[Iv] + u[Iv - 1])) -
                 nu * (((u[Iu + ncy * (nx - 1)] - u[Iu + (ncy - 1) * (nx - 1)]) / 2.0 / (dy[J + ncy] + dy[J + ncy - 1]) +
                        (u[Iv + ncy * nx] - u[Iv + ncy * nx - 1]) / 2.0 / (dx[I + idx] + dx[I + idx - 1])) -
                       ((u[Iu] - u[Iu - (nx - 1)]) / 2.0 / (dy[J] + dy[J - 1]) +
                        (u[Iv] - u[Iv - 1]) / 2.0 / (dx[I + idx] + dx[I + idx - 1])))) *
               0.5 * (dx[I + idx] + dx[I + idx - 1]);
    }
    for (int idx = 0; idx < (ncx + 1) * ncy; ++idx) { /* dragUnsteady */
        int i = idx % (ncx + 1), j = idx / (ncx + 1), Iu = (J + j) * (nx - 1) + (I - 1 + i);
        sxu += -(ghostTagsUV[Iu] == -1) *
               ((u[Iu] * dy[J + j] - uold[Iu] * dy[J + j]) / dt * 0.5 * (dx[I + i] + dx[I - 1 + i]));
    }
    *fx = sxx + sxy + sxu;
    for (int idx = 0; idx <= ncy; ++idx) { /* liftLeftRight */
        int Iu = (J + idx) * (nx - 1) + (I - 1), Iv = nU + (J - 1 + idx) * nx + I;
        syx += -((0.25 * (u[Iu + ncx] + u[Iu + ncx - (nx - 1)]) * (u[Iv + ncx] + u[Iv + ncx - 1]) -
                  0.25 * (u[Iu] + u[Iu - (nx - 1)]) * (u[Iv] + u[Iv - 1])) -
                 nu * (((u[Iu + ncx] - u[Iu + ncx - (nx - 1)]) / 2.0 / (dy[J + idx] + dy[J - 1 + idx]) +
                        (u[Iv + ncx] - u[Iv + ncx - 1]) / 2.0 / (dx[I + ncx] + dx[I + ncx - 1])) -
                       ((u[Iu] - u[Iu - (nx - 1)]) / 2.0 / (dy[J + idx] + dy[J - 1 + idx]) +
                        (u[Iv] - u[Iv - 1]) / 2.0 / (dx[I] + dx[I - 1])))) *
               0.5 * (dy[J + idx] + dy[J - 1 + idx]);
    }
    for (int idx = 0; idx < ncx; ++idx) { /* liftBottomTop */
        int Ip = J * nx + I + idx, Iv = nU + (J - 1) * nx + I + idx;
        syy += -((p[Ip + ncy * nx] - p[Ip - nx]) * dx[I + idx] +
                 (0.25 * (u[Iv + (ncy + 1) * nx] + u[Iv + ncy * nx]) * (u[Iv + (ncy + 1) * nx] + u[Iv + ncy * nx]) -
                  0.25 * (u[Iv] + u[Iv - nx]) * (u[Iv] + u[Iv - nx])) * dx[I + idx] -
                 nu * ((u[Iv + (ncy + 1) * nx] - u[Iv + ncy * nx]) * dx[I + idx] / dy[J + ncy] -
                       (u[Iv] - u[Iv - nx]) * dx[I] / dy[J - 1]));
    }
    for (int idx = 0; idx < ncx * (ncy + 1); ++idx) { /* liftUnsteady */
        int i = idx % ncx, j = idx / ncx, Iv = (J - 1 + j) * nx + (I + i) + nU;
        syu += -(ghostTagsUV[Iv] == -1) *
               ((u[Iv] * dx[I + i] - uold[Iv] * dx[I + i]) / dt * 0.5 * (dy[J + j] + dy[J - 1 + j]));
    }
    *fy = syx + syy + syu;
}

/* angle of (px,py) about the centre, continuous over the body as the reference makes
 * it: pi - asin on the left half, +2 pi on the right half when the point the search
 * is about lies outside (-pi/4, 5 pi/4) */
static double surface_angle(double px, double py, double midX, double midY)
{
    double t = asin((py - midY) / sqrt((px - midX) * (px - midX) + (py - midY) * (py - midY)));
    if (px < midX) t = M_PI - t;
    return t;
}

/* The surface-integral force (dead code in the reference's step).  mode 1 follows
 * luoForce as written: the pressure search starts its j index at startI (luoForce
 * passes B.startI_r for both starts) and force_velocity_y reads v with the u row
 * stride nx-1.  mode 2 uses startJ and the v stride nx.  The searches stop at the
 * ends of the coordinate arrays; a point without an intercept on one side gets a
 * NaN pressure (the reference reads an unset index there).  terms: pressure, du/dn,
 * dv/dn per point (3n); forces summed in point order. */
void or_surfaceForce(int mode, const double *bx, const double *by, int n, double uB0, double vB0, const double *u,
                     const double *bip, const double *bip_x, const double *bip_y, const int *ghostTagsP,
                     const double *xu, const double *yu, const double *xv, const double *yv, int startI,
                     int startJ, int nx, int ny, double midX, double midY, double nu, double mid_h, double *terms,
                     double *fx, double *fy)
{
    const int nU = (nx - 1) * ny;
    double *P = terms, *DU = terms + n, *DV = terms + 2 * n;
    for (int k = 0; k < n; k++) {
        /* pressure: nearest intercept angles above and below in the 4x4 window */
        int ii = startI, jj = mode == 1 ? startI : startJ;
        if (jj > ny - 1) jj = ny - 1;
        while (ii < nx - 1 && xv[ii] < bx[k]) ii++;
        while (jj < ny - 1 && yu[jj] < by[k]) jj++;
        double tn = surface_angle(bx[k], by[k], midX, midY);
        int wrap = tn > M_PI * 5 / 4 || tn < -M_PI / 4;
        if (wrap && bx[k] > midX) tn += 2 * M_PI;
        double lo = -10, hi = 10;
        int lo_id = -1, hi_id = -1;
        for (int i = ii - 2; i <= ii + 1; i++)
            for (int j = jj - 2; j <= jj + 1; j++) {
                if (i < 0 || i >= nx || j < 0 || j >= ny) continue;
                int ip = j * nx + i;
                if (ghostTagsP[ip] <= 0) continue;
                double t = surface_angle(bip_x[ip], bip_y[ip], midX, midY);
                if (wrap && bip_x[ip] > midX) t += 2 * M_PI;
                if (t > tn && t < hi) {
                    hi = t;
                    hi_id = ip;
                }
                if (t < tn && t > lo) {
                    lo = t;
                    lo_id = ip;
                }
            }
        P[k] = (lo_id < 0 || hi_id < 0) ? NAN : bip[lo_id] + (bip[hi_id] - bip[lo_id]) * (tn - lo) / (hi - lo);
        /* normal derivatives from the bilinear value sqrt(2) mid_h out along the radius */
        double rise = by[k] - midY, run = bx[k] - midX, radius = sqrt(rise * rise + run * run);
        double dn = mid_h * sqrt(2.0), ex = bx[k] + dn / radius * run, ey = by[k] + dn / radius * rise;
        for (int c = 0; c < 2; c++) {
            const double *xc = c ? xv : xu, *yc = c ? yv : yu;
            int nxc = c ? nx : nx - 1, nyc = c ? ny - 1 : ny;
            int a = startI, b = startJ;
            while (a < nxc - 1 && xc[a] < ex) a++;
            while (b < nyc - 1 && yc[b] < ey) b++;
            if (a < 1) a = 1;
            if (b < 1) b = 1;
            int stride = nx - 1, off = 0;
            if (c) {
                stride = mode == 1 ? nx - 1 : nx;
                off = mode == 1 ? ny * (nx - 1) : nU;
            }
            double x1 = xc[a - 1], x2 = xc[a], y1 = yc[b - 1], y3 = yc[b];
            double q1 = u[(b - 1) * stride + a - 1 + off], q2 = u[(b - 1) * stride + a + off];
            double q3 = u[b * stride + a - 1 + off], q4 = u[b * stride + a + off];
            double tl = (x2 - ex) * (y1 - ey) / (x2 - x1) / (y1 - y3) * q3;
            double tr = (ex - x1) * (y1 - ey) / (x2 - x1) / (y1 - y3) * q4;
            double bl = (x2 - ex) * (ey - y3) / (x2 - x1) / (y1 - y3) * q1;
            double br = (ex - x1) * (ey - y3) / (x2 - x1) / (y1 - y3) * q2;
            double val = bl + br + tl + tr;
            (c ? DV : DU)[k] = (val - (c ? vB0 : uB0)) / dn;
        }
    }
    double area = sqrt((bx[0] - bx[1]) * (bx[0] - bx[1]) + (by[0] - by[1]) * (by[0] - by[1]));
    double sx = 0, sy = 0;
    for (int k = 0; k < n; k++) {
        double h = sqrt((by[k] - midY) * (by[k] - midY) + (bx[k] - midX) * (bx[k] - midX));
        double n1 = (bx[k] - midX) / h, n2 = (by[k] - midY) / h;
        double tx = nu * ((1 - n1 * n1) * DU[k] + (-n1 * n2) * DV[k]);
        double ty = nu * ((-n1 * n2) * DU[k] + (1 - n2 * n2) * DV[k]);
        sx += area * tx - area * n1 * P[k];
        sy += area * ty - area * n2 * P[k];
    }
    *fx = sx;
    *fy = sy;
}
