// Host-side geometry: the staggered stretched grid and the immersed-body
// points.  Every expression keeps the reference's operation order (this file is
// compiled with -ffp-contract=off): all downstream parity, tags in particular,
// depends on these coordinates being bit-identical to the reference's.
//
//   build_axis     io/parseDomainFile.cu:28-222 (cell count per sub-domain truncated
//                  to int; uniform, shrinking (end < 0) and growing sub-domains) and
//                  io/parseDomainFile.cu:369-377 (face coordinates xu, yv)
//   circle bodies  io/parseBodiesFile.cu:145-178
//   place_bodies   src/bodies.cu:20-185 (t = 0, no rotation: x = X; centroid; offsets)
//   bounding_box   src/bodies.cu:256-326 (scaleCV-scaled box in cell indices)
#include "geometry.h"

#include <cmath>

namespace cuibm {

static int cells_in(double a0, double a1, double h, double r)
{
    if (r < 1) return (int)(std::log(1 / (h / ((a0 - a1) * (r - 1))) + 1) / std::log(r));
    if (r == 1) return (int)((a1 - a0) / h);
    return (int)(std::log(1 / (h / ((a1 - a0) * (r - 1))) + 1) / std::log(r));
}

std::string build_axis(const AxisDesc &A, Axis &out)
{
    const size_t ns = A.ends.size();
    double total = 0, a0 = A.start;
    std::vector<int> counts(ns);
    for (size_t s = 0; s < ns; ++s) {
        counts[s] = cells_in(a0, A.ends[s], A.mid_h, A.ratios[s]);
        if (counts[s] < 0) return "domain.yaml: a sub-domain gives a negative cell count";
        total += counts[s];
        a0 = A.ends[s];
    }
    const int n = (int)total;
    if (n < 3) return "domain.yaml: fewer than 3 cells in a direction";
    out.n = n;
    out.centre.assign(n, 0.0);
    out.width.assign(n, 0.0);
    a0 = A.start;
    int first = 0;
    for (size_t s = 0; s < ns; ++s) {
        const double a1 = A.ends[s], r = A.ratios[s];
        const int m = counts[s];
        double *c = out.centre.data() + first, *w = out.width.data() + first;
        if (std::fabs(r - 1.0) < 1.0e-6) {
            const double h = (a1 - a0) / m;
            for (int j = 0; j < m; ++j) {
                w[j] = h;
                c[j] = j == 0 ? a0 + h / 2 : c[j - 1] + 0.5 * w[j] + 0.5 * w[j - 1];
            }
        } else if (a1 < 0) {
            // cells shrink towards a1: the last cell is the smallest, filled backwards
            const double h = (a1 - a0) * (r - 1) / (std::pow(r, m) - 1);
            for (int k = 0; k < m; ++k) {
                int j = m - 1 - k;
                if (k == 0) {
                    c[j] = a1 - h / 2.0;
                    w[j] = h;
                } else {
                    w[j] = h * std::pow(r, k);
                    c[j] = c[j + 1] - 0.5 * w[j] - 0.5 * w[j + 1];
                }
            }
        } else {
            const double h = (a1 - a0) * (r - 1) / (std::pow(r, m) - 1);
            for (int j = 0; j < m; ++j) {
                w[j] = h * std::pow(r, j);
                c[j] = j == 0 ? a0 + h * std::pow(r, j) / 2 : c[j - 1] + 0.5 * w[j] + 0.5 * w[j - 1];
            }
        }
        first += m;
        a0 = a1;
    }
    out.face.resize(n - 1);
    for (int i = 0; i < n - 1; ++i) out.face[i] = out.centre[i] + out.width[i] / 2;
    return "";
}

std::string build_bodies(const std::vector<BodyDesc> &descs, BodyState &B)
{
    B = BodyState();
    for (const BodyDesc &d : descs) {
        std::vector<double> X, Y;
        if (d.type == "circle") {
            int np = d.numPoints;
            if (d.selfSize) {
                np = (int)(2.0 * d.R * M_PI / d.mid_h);
                if (np % 2 != 0) np++;
            }
            if (np < 3) return "bodies.yaml: a circle needs at least 3 points";
            X.resize(np);
            Y.resize(np);
            for (int i = 0; i < np; ++i) {
                X[i] = d.cx + d.R * std::cos(i * 2 * M_PI / np);
                Y[i] = d.cy + d.R * std::sin(i * 2 * M_PI / np);
            }
        } else {
            X = d.X;
            Y = d.Y;
        }
        B.offsets.push_back((int)B.X.size());
        B.X.insert(B.X.end(), X.begin(), X.end());
        B.Y.insert(B.Y.end(), Y.begin(), Y.end());
    }
    B.total = (int)B.X.size();
    if (B.total == 0) return "";
    const BodyDesc &b0 = descs[0];
    B.xCoeff = b0.xCoefficient;
    B.uCoeff = b0.uCoefficient;
    B.xPhase = b0.xPhase;
    B.uPhase = b0.uPhase;
    B.freq = b0.xfrequency;
    B.yCoeff = b0.yCoefficient;
    B.vCoeff = b0.vCoefficient;
    // positions at t = 0 without rotation, centroid, offsets (bodies.cu:159-176)
    B.x = B.X;
    B.y = B.Y;
    double mx = 0, my = 0;
    for (int i = 0; i < B.total; ++i) {
        mx += B.x[i];
        my += B.y[i];
    }
    mx /= B.total;
    my /= B.total;
    B.midX = mx;
    B.midY = my;
    B.dxp.resize(B.total);
    B.dyp.resize(B.total);
    for (int i = 0; i < B.total; ++i) {
        B.dxp[i] = B.x[i] - mx;
        B.dyp[i] = B.y[i] - my;
    }
    return "";
}

BoundingBox bounding_box(const double *x, const double *y, int n, const Axis &gx, const Axis &gy, double scale)
{
    double xmax = x[0], xmin = x[0], ymax = y[0], ymin = y[0];
    for (int i = 1; i < n; ++i) {
        xmax = x[i] > xmax ? x[i] : xmax;
        xmin = x[i] < xmin ? x[i] : xmin;
        ymax = y[i] > ymax ? y[i] : ymax;
        ymin = y[i] < ymin ? y[i] : ymin;
    }
    const double ex = xmax - xmin, ey = ymax - ymin;
    xmax += 0.5 * ex * (scale - 1.0);
    xmin -= 0.5 * ex * (scale - 1.0);
    ymax += 0.5 * ey * (scale - 1.0);
    ymin -= 0.5 * ey * (scale - 1.0);
    BoundingBox bb;
    int i = 0, j = 0;
    while (i + 1 < gx.n && gx.centre[i + 1] < xmin) i++;
    while (j + 1 < gy.n && gy.centre[j + 1] < ymin) j++;
    bb.i0 = i;
    bb.j0 = j;
    while (i < gx.n - 1 && gx.centre[i] < xmax) i++;
    while (j < gy.n - 1 && gy.centre[j] < ymax) j++;
    bb.ncx = i - bb.i0;
    bb.ncy = j - bb.j0;
    return bb;
}

}  // namespace cuibm
