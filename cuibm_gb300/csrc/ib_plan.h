// The interpolation plan of the ghost-node methods (built in ib_kernels.cu at each
// tagging, read by the external and embedded methods' kernels).
#pragma once
#include "solver.h"

namespace cuibm {

// The ghost and hybrid interpolations are linear in the field: the value at a
// node is sum_l w_l q_l over the four corners of the image point's cell, where
// q_l is the field at the corner or, for corners replaced by the body, the body
// velocity (velocity) or -(n . dU/dt) (pressure Neumann rows).  Which corners
// are replaced, the corner indices and the weights w_l (the rows of the inverse
// 4x4 bilinear fit evaluated at the point) depend only on the tags and the body
// geometry, so they are computed once per tagging (luo_base::tagPoints) into a
// plan of compact node lists; each step then only gathers.  The weights are the
// reference's own q*coef of its biLinearInterpolation kernels, so the values
// agree with its a0 + a1 x + a2 y + a3 x y to rounding.
struct IbPlan {
    int *count;  // [0] ghost velocity, [1] hybrid velocity, [2] ghost pressure, [3] hybrid pressure, [4] inside
    int cap_v, cap_p, cap_in;
    int *gvNode, *gvIdx, *gvMask;  // mask bit l: corner l takes the body value
    double *gvW;
    int *hvNode, *hvIdx, *hvMask;
    double *hvW, *hvWi, *hvAlpha;  // weights at the node and at its image point; blend factor
    int *gpNode, *gpIdx, *gpMask;  // mask bit l: corner l is a Neumann row
    double *gpN, *gpW, *gpWb, *gpCn, *gpDist;  // corner normals; weights at image point and intercept;
                                               // normal and distance of the dp/dn correction
    int *hpNode, *hpIdx, *hpMask;
    double *hpN, *hpW, *hpAlpha;
    int *inNode;  // nodes inside the body (tag 0)
};

// the plan of the context's current tags
IbPlan &ib_plan(Context &c);

}  // namespace cuibm
