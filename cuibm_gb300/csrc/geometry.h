// Grid axes and immersed-body state built on the host at set-up.
#pragma once
#include <string>
#include <vector>

#include "config.h"

namespace cuibm {

struct Axis {
    int n = 0;
    std::vector<double> centre;  // x (or y): pressure-cell centres, also xv (yu)
    std::vector<double> width;   // dx (dy)
    std::vector<double> face;    // xu (yv): n-1 staggered face coordinates
};

struct BodyState {
    int total = 0;
    std::vector<int> offsets;
    std::vector<double> X, Y;      // reference coordinates
    std::vector<double> x, y;      // current coordinates
    std::vector<double> dxp, dyp;  // offsets of each point from the centroid at t = 0
    double midX = 0, midY = 0;
    // prescribed motion of body 0 (luo_base/move.cu)
    double xCoeff = 0, uCoeff = 0, xPhase = 0, uPhase = 0, freq = 0, yCoeff = 0, vCoeff = 0;
};

struct BoundingBox {
    int i0 = 0, j0 = 0, ncx = 0, ncy = 0;
};

std::string build_axis(const AxisDesc &A, Axis &out);
std::string build_bodies(const std::vector<BodyDesc> &descs, BodyState &B);
BoundingBox bounding_box(const double *x, const double *y, int n, const Axis &gx, const Axis &gy, double scale);

}  // namespace cuibm
