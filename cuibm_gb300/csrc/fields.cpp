// Field table of the C ABI (cuibm_get_field / cuibm_set_field): device pointer
// and byte size of each named array of the context.
#include "../../include/cuibm.h"
#include "solver.h"

namespace cuibm {

void *field_pointer(Context &c, int f, size_t *bytes)
{
    const size_t D = sizeof(double), I = sizeof(int);
    const size_t UV = c.g.nUV, P = c.g.nP, nx = c.g.nx, ny = c.g.ny, nb = c.body.total;
    auto ret = [&](void *p, size_t b) {
        *bytes = b;
        return p;
    };
    switch (f) {
    case CUIBM_F_U: return ret(c.u, UV * D);
    case CUIBM_F_UHAT: return ret(c.uhat, UV * D);
    case CUIBM_F_UOLD: return ret(c.uold, UV * D);
    case CUIBM_F_P: return ret(c.p, P * D);
    case CUIBM_F_P_OLD: return ret(c.p_old, P * D);
    case CUIBM_F_N: return ret(c.N, UV * D);
    case CUIBM_F_NOLD: return ret(c.Nold, UV * D);
    case CUIBM_F_L: return ret(c.L, UV * D);
    case CUIBM_F_BC1: return ret(c.bc1, UV * D);
    case CUIBM_F_RHS1: return ret(c.rhs1, UV * D);
    case CUIBM_F_RHS2: return ret(c.rhs2, P * D);
    case CUIBM_F_BC_XMINUS: return ret(c.bc[XMINUS], (2 * ny - 1) * D);
    case CUIBM_F_BC_XPLUS: return ret(c.bc[XPLUS], (2 * ny - 1) * D);
    case CUIBM_F_BC_YMINUS: return ret(c.bc[YMINUS], (2 * nx - 1) * D);
    case CUIBM_F_BC_YPLUS: return ret(c.bc[YPLUS], (2 * nx - 1) * D);
    case CUIBM_F_X: return ret(c.x, nx * D);
    case CUIBM_F_DX: return ret(c.dx, nx * D);
    case CUIBM_F_XU: return ret(c.xu, (nx - 1) * D);
    case CUIBM_F_XV: return ret(c.xv, nx * D);
    case CUIBM_F_Y: return ret(c.y, ny * D);
    case CUIBM_F_DY: return ret(c.dy, ny * D);
    case CUIBM_F_YU: return ret(c.yu, ny * D);
    case CUIBM_F_YV: return ret(c.yv, (ny - 1) * D);
    case CUIBM_F_CFL: return ret(c.cfl, P * D);
    case CUIBM_F_WORK_X: return ret(c.work_x, (UV > P ? UV : P) * D);
    case CUIBM_F_WORK_Y: return ret(c.work_y, (UV > P ? UV : P) * D);
    case CUIBM_F_SOLVE_TRACE: return ret(c.solve_trace, 2 * kTraceLen * sizeof(unsigned long long));
    default: break;
    }
    if (!c.has_body) return nullptr;
    IbArrays &b = c.ib;
    switch (f) {
    case CUIBM_F_BODY_X: return ret(b.bx, nb * D);
    case CUIBM_F_BODY_Y: return ret(b.by, nb * D);
    case CUIBM_F_BODY_UB: return ret(b.uB, nb * D);
    case CUIBM_F_BODY_VB: return ret(b.vB, nb * D);
    case CUIBM_F_BODY_MOTION: return ret(b.motion, kMotionLen * D);
    case CUIBM_F_SURFACE_FORCE: return ret(b.surf, (3 * nb + 2) * D);
    case CUIBM_F_FORCES: return ret(b.forceOut, 2 * D);
    case CUIBM_F_BODY_VELOCITY_OFFSET: return ret(b.velOff, 2 * nb * D);
    case CUIBM_F_GHOST_TAGS_UV: return ret(b.ghostUV, UV * I);
    case CUIBM_F_HYBRID_TAGS_UV: return ret(b.hybridUV, UV * I);
    case CUIBM_F_HYBRID_TAGS_UV2: return ret(b.hybrid2UV, UV * I);
    case CUIBM_F_GHOST_TAGS_P: return ret(b.ghostP, P * I);
    case CUIBM_F_HYBRID_TAGS_P: return ret(b.hybridP, P * I);
    case CUIBM_F_BI_X: return ret(b.biX, UV * D);
    case CUIBM_F_BI_Y: return ret(b.biY, UV * D);
    case CUIBM_F_IP_X: return ret(b.ipX, UV * D);
    case CUIBM_F_IP_Y: return ret(b.ipY, UV * D);
    case CUIBM_F_BIP_X: return ret(b.bipX, P * D);
    case CUIBM_F_BIP_Y: return ret(b.bipY, P * D);
    case CUIBM_F_IPP_X: return ret(b.ippX, P * D);
    case CUIBM_F_IPP_Y: return ret(b.ippY, P * D);
    case CUIBM_F_DIST_NODE: return ret(b.distNode, UV * D);
    case CUIBM_F_DIST_BETWEEN: return ret(b.distBetween, UV * D);
    case CUIBM_F_UV_BODY: return ret(b.uvBody, UV * D);
    case CUIBM_F_USTAR: return ret(b.ustar, UV * D);
    case CUIBM_F_PSTAR: return ret(b.pstar, P * D);
    case CUIBM_F_DPDN: return ret(b.dpdn, P * D);
    case CUIBM_F_BI_P: return ret(b.biP, P * D);
    case CUIBM_F_GHOST_UV_INDEX: return ret(b.gIdx, 4 * UV * I);
    case CUIBM_F_GHOST_UV_COEF: return ret(b.gCoef, 4 * UV * D);
    case CUIBM_F_HYBRID_UV_INDEX: return ret(b.hIdx, 4 * UV * I);
    case CUIBM_F_HYBRID_UV_COEF: return ret(b.hCoef, 4 * UV * D);
    case CUIBM_F_GHOST_P_INDEX: return ret(b.gpIdx, 4 * P * I);
    case CUIBM_F_GHOST_P_COEF: return ret(b.gpCoef, 4 * P * D);
    case CUIBM_F_HYBRID_P_INDEX: return ret(b.hpIdx, 4 * P * I);
    case CUIBM_F_HYBRID_P_COEF: return ret(b.hpCoef, 4 * P * D);
    case CUIBM_F_IMAGE_VALUE_UV: return ret(b.imageValue, UV * D);
    default: return nullptr;
    }
}

// A field written from outside can change what the step graph assumed fixed:
// body coordinates force the tags to be recomputed at the next body update.
void field_changed(Context &c, int f)
{
    if (c.has_body && (f == CUIBM_F_BODY_X || f == CUIBM_F_BODY_Y || f == CUIBM_F_BODY_UB || f == CUIBM_F_BODY_VB))
        c.ib_dirty = true;
    if (c.has_body && f == CUIBM_F_BODY_VELOCITY_OFFSET) {
        if (!c.initialised) throw InputError("write body_velocity_offset after cuibm_initialise");
        apply_velocity_offsets(c);
    }
}

}  // namespace cuibm
