// Device view of the smoothed-aggregation hierarchy (built in amg.cu, cycled by
// the V-cycle kernels there and by the persistent solver in fused_solve.cu).
#pragma once
#include "solver.h"

namespace cuibm {

struct DevCsr {
    int n = 0, nnz = 0;
    int *ptr = nullptr, *col = nullptr;
    double *val = nullptr;
};

struct SaLevel {
    int n = 0;
    double omega = 0;
    DevCsr A, P, R;      // A unused on level 0 (structured operator)
    double *dinv = nullptr;
    double *x = nullptr, *b = nullptr, *r = nullptr, *t = nullptr;
    double *coarse_inv = nullptr;  // dense inverse on the coarsest level
    // for the persistent cycle (fused_solve.cu), levels with a coarser one:
    double *wd = nullptr;  // omega * D^-1 (the damped-Jacobi weights)
    DevCsr AP;             // A_l P_l: the upward sweep's residual without neighbour values
    // for the transposed cycle of the discrete adjoint (built on first use): A_l^T on the
    // levels below the finest, the transposed dense inverse on the coarsest
    DevCsr AT;
    double *coarse_inv_t = nullptr;
    // structured hierarchy (structured.cuh): the level's grid (nx = 0: CSR level), its
    // 9-point operator below level 0 and its prolongator's four weights a node
    int nx = 0, ny = 0;
    double *c9 = nullptr;
    double *pw = nullptr;
};

}  // namespace cuibm
