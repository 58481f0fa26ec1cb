/*
 * Grid and body geometry (oracle restatement; test infrastructure only).
 *
 * or_axis_count / or_axis_fill   io/parseDomainFile.cu:28-222 (operator>> for domain),
 *                                io/parseDomainFile.cu:355-378 (xu, yv)
 * or_circle_count / _points      io/parseBodiesFile.cu:145-178 (type: circle)
 * or_body_place                  src/bodies.cu:20-185 (initialise; update(t=0) with
 *                                no rotation; midX/midY and point offsets)
 * or_bounding_box                src/bodies.cu:256-326 (boundingBox kernel + scaleCV)
 */
#include <math.h>
#include "oracle.h"

/* cells in one sub-domain: geometric stretching count truncated to int,
 * io/parseDomainFile.cu:45-66 */
static int sub_cells(double start, double end, double mid_h, double r)
{
    double a;
    int n;
    if (r < 1) {
        a = mid_h / ((start - end) * (r - 1));
        n = (int)(log(1 / a + 1) / log(r));
    } else if (r == 1) {
        n = (int)((end - start) / mid_h);
    } else {
        a = mid_h / ((end - start) * (r - 1));
        n = (int)(log(1 / a + 1) / log(r));
    }
    return n;
}

int or_axis_count(double start, double mid_h, int nsub, const double *ends, const double *ratios)
{
    double count = 0;
    for (int s = 0; s < nsub; ++s) {
        count += sub_cells(start, ends[s], mid_h, ratios[s]);
        start = ends[s];
    }
    return (int)count;
}

/* c = cell centres, d = cell widths, cs = staggered face coordinate (xu or yv,
 * n-1 entries): io/parseDomainFile.cu:80-222 and :369-377 */
void or_axis_fill(double start, double mid_h, int nsub, const double *ends, const double *ratios, double *c,
                  double *d, double *cs)
{
    int beg = 0, n = or_axis_count(start, mid_h, nsub, ends, ratios);
    for (int s = 0; s < nsub; ++s) {
        double end = ends[s], r = ratios[s];
        int nc = sub_cells(start, end, mid_h, r);
        if (fabs(r - 1.0) < 1.0e-6) {
            double h = (end - start) / nc;
            for (int j = beg; j < beg + nc; ++j) {
                d[j] = h;
                c[j] = (j == beg) ? start + h / 2 : c[j - 1] + 0.5 * d[j] + 0.5 * d[j - 1];
            }
        } else if (end < 0) {
            /* shrinking towards `end`: filled from the right end backwards */
            double h = (end - start) * (r - 1) / (pow(r, nc) - 1);
            int k = 0;
            for (int j = beg + nc - 1; j >= beg; --j, ++k) {
                if (j == beg + nc - 1) {
                    c[j] = end - h / 2.0;
                    d[j] = h;
                } else {
                    d[j] = h * pow(r, k);
                    c[j] = c[j + 1] - 0.5 * d[j] - 0.5 * d[j + 1];
                }
            }
        } else {
            double h = (end - start) * (r - 1) / (pow(r, nc) - 1);
            for (int j = beg; j < beg + nc; ++j) {
                d[j] = h * pow(r, j - beg);
                c[j] = (j == beg) ? start + h * pow(r, j - beg) / 2 : c[j - 1] + 0.5 * d[j] + 0.5 * d[j - 1];
            }
        }
        beg += nc;
        start = end;
    }
    for (int i = 0; i < n - 1; ++i) cs[i] = c[i] + d[i] / 2;
}

int or_circle_count(double R, int numPoints, int selfSize, double mid_h)
{
    if (selfSize) {
        numPoints = (int)(2.0 * R * M_PI / mid_h);
        if (numPoints % 2 != 0) numPoints++;
    }
    return numPoints;
}

void or_circle_points(double cx, double cy, double R, int n, double *X, double *Y)
{
    for (int i = 0; i < n; ++i) {
        X[i] = cx + R * cos(i * 2 * M_PI / n);
        Y[i] = cy + R * sin(i * 2 * M_PI / n);
    }
}

/* Body at t = 0 without rotation: x = X, y = Y; centroid by a serial sum;
 * offsets of each point from the centroid (bodies.cu:159-176). */
void or_body_place(int n, const double *X, const double *Y, double *x, double *y, double *midX, double *midY,
                   double *bdx, double *bdy)
{
    double mx = 0, my = 0;
    for (int i = 0; i < n; ++i) {
        x[i] = X[i];
        y[i] = Y[i];
    }
    for (int i = 0; i < n; ++i) {
        mx += x[i];
        my += y[i];
    }
    mx /= n;
    my /= n;
    for (int i = 0; i < n; ++i) {
        bdx[i] = x[i] - mx;
        bdy[i] = y[i] - my;
    }
    *midX = mx;
    *midY = my;
}

/* Scaled bounding box of the body in cell indices (gx, gy = cell centres). */
void or_bounding_box(int n, const double *x, const double *y, const double *gx, const double *gy, double scale,
                     int *startI, int *startJ, int *ncx, int *ncy)
{
    double xmax = x[0], xmin = x[0], ymax = y[0], ymin = y[0];
    for (int i = 1; i < n; ++i) {
        if (x[i] > xmax) xmax = x[i];
        if (x[i] < xmin) xmin = x[i];
        if (y[i] > ymax) ymax = y[i];
        if (y[i] < ymin) ymin = y[i];
    }
    double dxb = xmax - xmin, dyb = ymax - ymin;
    xmax += 0.5 * dxb * (scale - 1.0);
    xmin -= 0.5 * dxb * (scale - 1.0);
    ymax += 0.5 * dyb * (scale - 1.0);
    ymin -= 0.5 * dyb * (scale - 1.0);
    int i = 0, j = 0;
    while (gx[i + 1] < xmin) i++;
    while (gy[j + 1] < ymin) j++;
    *startI = i;
    *startJ = j;
    while (gx[i] < xmax) i++;
    while (gy[j] < ymax) j++;
    *ncx = i - *startI;
    *ncy = j - *startJ;
}
