// The persistent solves' FP64 kernels for the velocity (LHS1) operator (a translation
// unit of their own, so that the kernels' instantiations compile in parallel).
#include "fused_kernels.cuh"

namespace cuibm {

void *fused_pick_op1(int precond, int krylov, int pack) { return pick_kernel<Op1D<double>>(precond, krylov, pack); }

}  // namespace cuibm
