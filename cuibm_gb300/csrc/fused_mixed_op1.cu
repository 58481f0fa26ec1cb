// The persistent solves' mixed-precision kernels for the velocity (LHS1) operator (a
// translation unit of their own, so that the kernels' instantiations compile in
// parallel).
#include "fused_kernels.cuh"

namespace cuibm {

void *fused_pick_mixed_op1(const LinearSystem &S) { return pick_mixed_kernel<Op1D<double>, Op1D<float>>(S); }

}  // namespace cuibm
