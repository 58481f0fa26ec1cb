// The persistent solves' FP64 kernels for the pressure (LHS2) operator (a translation
// unit of their own, so that the kernels' instantiations compile in parallel).
#include "fused_kernels.cuh"

namespace cuibm {

void *fused_pick_op2(int precond, int krylov, int pack) { return pick_kernel<Op2D<double>>(precond, krylov, pack); }

}  // namespace cuibm
