// The persistent solves' mixed-precision kernels for the pressure (LHS2) operator (a
// translation unit of their own, so that the kernels' instantiations compile in
// parallel).
#include "fused_kernels.cuh"

namespace cuibm {

void *fused_pick_mixed_op2(const LinearSystem &S) { return pick_mixed_kernel<Op2D<double>, Op2D<float>>(S); }

}  // namespace cuibm
