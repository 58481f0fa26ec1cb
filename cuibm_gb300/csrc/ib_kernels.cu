// Immersed-boundary kernels (placeholder until the external method is built).
#include "solver.h"

namespace cuibm {
static void nyi() { throw InputError("immersed-boundary kernels are not built yet"); }
void setup_ib(Context &) { nyi(); }
void launch_tag_points(Context &) { nyi(); }
void launch_ghost_velocity(Context &, double *, bool) { nyi(); }
void launch_hybrid_velocity(Context &, const double *) { nyi(); }
void launch_set_inside(Context &, double *) { nyi(); }
void launch_weight_uhat(Context &) { nyi(); }
void launch_hybrid_pressure(Context &) { nyi(); }
void launch_ghost_pressure(Context &, bool) { nyi(); }
void launch_weight_pressure(Context &) { nyi(); }
void launch_robin(Context &) { nyi(); }
void launch_force(Context &) { nyi(); }
void launch_body_motion(Context &, double) { nyi(); }
void launch_body_pre_step(Context &) { nyi(); }
void initialise_body(Context &) { nyi(); }

__global__ void k_step_counter(int *s) { *s += 1; }
void launch_step_counter(Context &c) { k_step_counter<<<1, 1, 0, c.stream>>>(c.step_counter_dev); }
}  // namespace cuibm
