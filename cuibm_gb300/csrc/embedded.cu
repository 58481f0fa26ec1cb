// The embedded ghost-node method (SolverType OSC_CYLINDER, the reference's luo_iter).
//
// Replaces luo_iter/kernels/weight.cu (alpha_u, alpha_v, alpha_p),
// luo_iter/kernels/LHS1.cu (LHS1_mid_iter_X/Y), luo_iter/kernels/LHS2.cu
// (LHS2_mid_iter), luo_iter/kernels/intermediateVelocity.cu and pressure.cu
// (size_LHS1/2, update_rhs1_x/y, update_rhs2) and the per-step rebuild that
// luo_iter/intermediateVelocity.cu:17-80 and luo_iter/poisson.cu:15-58 run.
//
// Design.  The reference resizes, fills and sorts both COO matrices and rebuilds both
// preconditioners every step, although the entries depend only on the tags and the
// body geometry (interpolation corners, their weights, the blend factors alpha): the
// field enters only the right-hand sides.  Here the operators stay matrix-free:
//  * a tagged node's row is a patch (a diagonal and at most five off-diagonal entries)
//    built from the interpolation plan at every tagging (once for a fixed body, each
//    step for a moving one);
//  * the other interior rows of LHS1 are the momentum rows divided by their diagonal
//    (Lhs1Coef::rscale = 1/diagonal, the reference's ns_rhs of those rows); LHS2 keeps
//    its plain rows;
//  * rhs1 = rhs1 ns_rhs + interp_rhs and rhs2 = rhs2 ns_rhs + interp_rhs are fused
//    into the rhs1 and rhs2 kernels.  Only a ghost velocity row's interp_rhs reads the
//    field (the corners that are other ghost nodes keep their field value in the
//    reference's set = false interpolation); the rhs1 kernel computes it.
// Entry per entry the rows are the reference's: hybrid rows (1 - alpha) (momentum or
// pressure row over its diagonal) + alpha (the interpolation at the node), the corners
// at the four neighbours merged into the stencil, one extra entry for a diagonal
// corner (the last one in corner order), corners further away dropped, the node's own
// corner (replaced by the body point) moved to the right-hand side; ghost rows
// node + interpolation at the image point = 2 u_B (velocity) and node - interpolation =
// dp/dn (pressure), the corners that are ghost nodes moved to the right-hand side.
//
// The reference's later steps reuse the previous step's sorted COO arrays without
// clearing the LHS1 values, so entries that a step does not write keep stale values.
// That artefact is not reproduced: the rows here are the ones the reference writes on
// zeroed arrays, which is its first step.
//
// Compiled with -fmad=false: the entry values follow the reference's expressions
// without multiply-add fusion, as the oracle evaluates them.
#include <algorithm>
#include <vector>

#include "ib_plan.h"
#include "solver.h"

namespace cuibm {

struct EmbGeom {
    int nx, ny;
    double dt, nu;
    const double *dx, *dy;
    const int *gUV, *gP;
    const double *uB, *vB;
    const int *hUV, *hP;  // hybrid tags: a node tagged both ways takes the hybrid row
};

// 1/diagonal of the interior LHS1 rows (the ns_rhs of LHS1_mid_iter_X/Y's plain rows),
// 1 on the boundary rows
__global__ void k_emb_rscale(int nx, int ny, double dt, double nu, const double *dx, const double *dy, double *rs)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nU = (nx - 1) * ny;
    if (i >= nU + nx * (ny - 1)) return;
    double v = 1;
    if (i < nU) {
        const int I = i % (nx - 1), J = i / (nx - 1);
        if (I != 0 && I != nx - 2 && J != 0 && J != ny - 1) {
            const double temp = 1 + 0.5 * dt * nu * (1 / (dx[I + 1] * (dx[I + 1] + dx[I]) * 0.5)) +
                                0.5 * dt * nu * (1 / (dx[I] * (dx[I + 1] + dx[I]) * 0.5)) +
                                0.5 * dt * nu * (1 / (dy[J] * (dy[J + 1] + dy[J]) * 0.5)) +
                                0.5 * dt * nu * (1 / (dy[J] * (dy[J - 1] + dy[J]) * 0.5));
            v = 1 / temp;
        }
    } else {
        const int k = i - nU, I = k % nx, J = k / nx;
        if (I != 0 && I != nx - 1 && J != 0 && J != ny - 2) {
            const double temp = 1 + 0.5 * dt * nu * (1 / (dx[I] * (dx[I] + dx[I + 1]) * 0.5)) +
                                0.5 * dt * nu * (1 / (dx[I] * (dx[I] + dx[I - 1]) * 0.5)) +
                                0.5 * dt * nu * (1 / (dy[J + 1] * (dy[J] + dy[J + 1]) * 0.5)) +
                                0.5 * dt * nu * (1 / (dy[J] * (dy[J] + dy[J + 1]) * 0.5));
            v = 1 / temp;
        }
    }
    rs[i] = v;
}

// A hybrid row: stencil coefficients cns (N, E, S, W, already blended by (1 - alpha) and
// divided by the diagonal) merged with the blended interpolation ci at the corners idx.
// Writes the five off-diagonal slots (N, W, E, S, the diagonal-corner extra or -1); the
// node's own corner goes to the right-hand side (the callers).
__device__ void emb_hybrid_row(int i, int s, const double cns[4], const double ci[4], const int idx[4], int *pcol,
                               double *pval)
{
    const int st[9] = {i + s - 1, i + s, i + s + 1, i - 1, i, i + 1, i - s - 1, i - s, i - s + 1};
    double sv[9] = {0, cns[0], 0, cns[3], 1, cns[1], 0, cns[2], 0};
    for (int n = 0; n < 4; ++n)
        for (int m = 0; m < 9; ++m)
            if (st[m] == idx[n] && m != 4) sv[m] -= ci[n];
    const int used[4] = {1, 3, 5, 7};  // N, W, E, S (the centre is the unit diagonal)
    for (int u = 0; u < 4; ++u) {
        pcol[u] = st[used[u]];
        pval[u] = sv[used[u]];
    }
    pcol[4] = -1;
    pval[4] = 0;
    for (int n = 0; n < 4; ++n)
        for (int m = 0; m < 9; m += 2)
            if (m != 4 && st[m] == idx[n]) {  // a diagonal neighbour: the last one wins
                pcol[4] = idx[n];
                pval[4] = -ci[n];
            }
}

// blockIdx.y: 0 ghost velocity, 1 hybrid velocity, 2 ghost pressure, 3 hybrid pressure
__global__ void k_emb_rows(EmbGeom G, IbPlan P, Context::EmbeddedRows E)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int cls = blockIdx.y;
    if (k >= P.count[cls]) return;
    const int nx = G.nx, ny = G.ny, nU = (nx - 1) * ny;
    if (cls == 0) {
        // ghost velocity (LHS1_mid_iter_X/Y ghost branch): 1 at the node, +w at the corners
        // that are neither ghost nodes nor the node; the others go to interp_rhs.  A node
        // tagged hybrid as well takes the hybrid row (LHS1_mid_iter_X/Y test the hybrid tag
        // first), so its ghost slot stays unused.
        const int n = P.gvNode[k];
        if (G.hUV[n] > 0) return;
        int *pc = E.pcol1 + 5 * (size_t)k;
        double *pv = E.pval1 + 5 * (size_t)k;
        int m = 0, in = 0;
        for (int l = 0; l < 4; ++l) {
            const int j = P.gvIdx[4 * k + l];
            const bool ghost = G.gUV[j] > 0;
            if (ghost) in |= 1 << l;
            if (!ghost && j != n) {
                pc[m] = j;
                pv[m] = P.gvW[4 * k + l];
                ++m;
            }
        }
        for (; m < 5; ++m) {
            pc[m] = -1;
            pv[m] = 0;
        }
        E.pdiag1[k] = 1;
        E.pns1[k] = 0;
        E.pint1[k] = 0;  // computed each step by the rhs1 kernel
        E.gin[k] = in;
        E.pid1[n] = k;
    } else if (cls == 1) {
        // hybrid velocity (LHS1_mid_iter_X/Y hybrid branch)
        const int n = P.hvNode[k], slot = E.cap1 + k;
        const bool v = n >= nU;
        const int s = v ? nx : nx - 1, I = v ? (n - nU) % nx : n % (nx - 1), J = v ? (n - nU) / nx : n / (nx - 1);
        const double *dx = G.dx, *dy = G.dy, dt = G.dt, nu = G.nu;
        double cns[5];
        cns[0] = -dt * nu / (dy[J + 1] * (dy[J] + dy[J + 1]));
        cns[1] = -dt * nu / (dx[I] * (dx[I] + dx[I + 1]));
        cns[2] = -dt * nu / (dy[J] * (dy[J] + dy[J + 1]));
        cns[3] = -dt * nu / (dx[I] * (dx[I] + dx[I - 1]));
        cns[4] = 1 - cns[0] - cns[1] - cns[2] - cns[3];
        const double a = P.hvAlpha[k];
        double ci[4];
        int idx[4];
        for (int l = 0; l < 4; ++l) {
            cns[l] = cns[l] * (1 - a) / cns[4];
            ci[l] = P.hvW[4 * k + l] * a;
            idx[l] = P.hvIdx[4 * k + l];
        }
        emb_hybrid_row(n, s, cns, ci, idx, E.pcol1 + 5 * (size_t)slot, E.pval1 + 5 * (size_t)slot);
        E.pdiag1[slot] = 1;
        E.pns1[slot] = (1 - a) / cns[4];
        // the node's own corner holds the body velocity (the interpolation replaced it)
        const double qb = v ? G.vB[0] : G.uB[0];
        double interp = 0;
        for (int l = 0; l < 4; ++l)
            if (idx[l] == n) interp += ci[l] * qb;
        E.pint1[slot] = interp;
        E.pid1[n] = slot;
    } else if (cls == 2) {
        // ghost pressure (LHS2_mid_iter ghost branch): 1 at the node, -w at the corners that
        // are neither ghost nodes nor the node; interp_rhs = dp/dn + sum_l w_l q_l over the
        // ghost corners, q_l = -(n_l . dU/dt), dp/dn = |node - image point| (n . dU/dt)
        const int ip = P.gpNode[k];
        if (G.hP[ip] > 0) return;  // tagged hybrid as well: the hybrid row (LHS2_mid_iter's order)
        int *pc = E.pcol2 + 5 * (size_t)k;
        double *pv = E.pval2 + 5 * (size_t)k;
        int m = 0;
        double au = P.gpDist[k] * P.gpCn[2 * k], av = P.gpDist[k] * P.gpCn[2 * k + 1];
        for (int l = 0; l < 4; ++l) {
            const int j = P.gpIdx[4 * k + l];
            const double w = P.gpW[4 * k + l];
            if (!(G.gP[j] > 0) && j != ip) {
                pc[m] = j;
                pv[m] = -w;
                ++m;
            } else {
                au -= w * P.gpN[8 * k + 2 * l];
                av -= w * P.gpN[8 * k + 2 * l + 1];
            }
        }
        for (; m < 5; ++m) {
            pc[m] = -1;
            pv[m] = 0;
        }
        E.pdiag2[k] = 1;
        E.pns2[k] = 0;
        E.pAu2[k] = au;
        E.pAv2[k] = av;
        E.pid2[ip] = k;
    } else {
        // hybrid pressure (LHS2_mid_iter hybrid branch)
        const int ip = P.hpNode[k], slot = E.cap2 + k;
        const int I = ip % nx, J = ip / nx;
        const double *dx = G.dx, *dy = G.dy, dt = G.dt;
        double cns[5];
        cns[0] = -dt / (dy[J] * (dy[J] + dy[J + 1]) * 0.5);
        cns[1] = -dt / (dx[I] * (dx[I] + dx[I + 1]) * 0.5);
        cns[2] = -dt / (dy[J] * (dy[J] + dy[J - 1]) * 0.5);
        cns[3] = -dt / (dx[I] * (dx[I] + dx[I - 1]) * 0.5);
        cns[4] = -cns[0] - cns[1] - cns[2] - cns[3];
        const double a = P.hpAlpha[k];
        double ci[4];
        int idx[4];
        for (int l = 0; l < 4; ++l) {
            cns[l] = (1 - a) * cns[l] / cns[4];
            ci[l] = a * P.hpW[4 * k + l];
            idx[l] = P.hpIdx[4 * k + l];
        }
        emb_hybrid_row(ip, nx, cns, ci, idx, E.pcol2 + 5 * (size_t)slot, E.pval2 + 5 * (size_t)slot);
        E.pdiag2[slot] = 1;
        E.pns2[slot] = (1 - a) / cns[4];
        // the node's own corner is a Neumann row: q = -(n . dU/dt)
        double au = 0, av = 0;
        for (int l = 0; l < 4; ++l)
            if (idx[l] == ip) {
                au -= ci[l] * P.hpN[8 * k + 2 * l];
                av -= ci[l] * P.hpN[8 * k + 2 * l + 1];
            }
        E.pAu2[slot] = au;
        E.pAv2[slot] = av;
        E.pid2[ip] = slot;
    }
}

void setup_embedded(Context &c)
{
    auto &E = c.emb;
    const IbPlan &P = ib_plan(c);
    E.cap1 = P.cap_v;
    E.cap2 = P.cap_p;
    const size_t s1 = 2 * (size_t)E.cap1, s2 = 2 * (size_t)E.cap2;
    c.rows_key_dev = c.carve<unsigned long long>(1);
    E.pid1 = c.carve<int>(c.g.nUV);
    E.pcol1 = c.carve<int>(5 * s1);
    E.pval1 = c.carve<double>(5 * s1);
    E.pdiag1 = c.carve<double>(s1);
    E.pns1 = c.carve<double>(s1);
    E.pint1 = c.carve<double>(s1);
    E.gin = c.carve<int>(E.cap1);
    E.pid2 = c.carve<int>(c.g.nP);
    E.pcol2 = c.carve<int>(5 * s2);
    E.pval2 = c.carve<double>(5 * s2);
    E.pdiag2 = c.carve<double>(s2);
    E.pns2 = c.carve<double>(s2);
    E.pAu2 = c.carve<double>(s2);
    E.pAv2 = c.carve<double>(s2);
    E.rscale1 = c.carve<double>(c.g.nUV);
    CUIBM_TRY(cudaMemsetAsync(E.pid1, 0xff, c.g.nUV * sizeof(int), c.stream));
    CUIBM_TRY(cudaMemsetAsync(E.pid2, 0xff, c.g.nP * sizeof(int), c.stream));
    k_emb_rscale<<<blocks_for(c.g.nUV), kBlock, 0, c.stream>>>(c.g.nx, c.g.ny, c.P.dt, c.P.nu, c.dx, c.dy,
                                                               E.rscale1);
    CUIBM_TRY(cudaGetLastError());
    c.l1.patch = RowPatch{E.pid1, E.pcol1, E.pval1, E.pdiag1};
    c.l1.rscale = E.rscale1;
    c.l2.patch = RowPatch{E.pid2, E.pcol2, E.pval2, E.pdiag2};
}

// A checksum of which Poisson rows are patched: the sum over patched rows i of
// (i + 1) times an odd constant, modulo 2^64 (order-free, so one block's tree sum
// gives the same word every time).  A moving body changes it when it crosses cells.
__global__ void __launch_bounds__(256) k_rows_key(const int *__restrict__ pid, int n, unsigned long long *key)
{
    __shared__ unsigned long long sh[256];
    unsigned long long s = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        if (pid[i] >= 0) s += (unsigned long long)(i + 1) * 0x9E3779B97F4A7C15ull;
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *key = sh[0];
}

unsigned long long read_rows_key(Context &c)
{
    unsigned long long k = 0;
    if (!c.rows_key_dev) return 0;
    CUIBM_TRY(cudaMemcpyAsync(&k, c.rows_key_dev, sizeof k, cudaMemcpyDeviceToHost, c.stream));
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
    return k;
}

void launch_embedded_rows(Context &c)
{
    auto &E = c.emb;
    if (!E.pid1) return;
    const IbPlan &P = ib_plan(c);
    CUIBM_TRY(cudaMemsetAsync(E.pid1, 0xff, c.g.nUV * sizeof(int), c.stream));
    CUIBM_TRY(cudaMemsetAsync(E.pid2, 0xff, c.g.nP * sizeof(int), c.stream));
    EmbGeom G{c.g.nx,  c.g.ny,  c.P.dt,       c.P.nu,        c.dx, c.dy, c.ib.ghostUV, c.ib.ghostP,
              c.ib.uB, c.ib.vB, c.ib.hybridUV, c.ib.hybridP};
    const int cap = std::max(P.cap_v, P.cap_p);
    k_emb_rows<<<dim3(blocks_for(cap), 4), kBlock, 0, c.stream>>>(G, P, E);
    CUIBM_TRY(cudaGetLastError());
    k_rows_key<<<1, 256, 0, c.stream>>>(E.pid2, c.g.nP, c.rows_key_dev);
    CUIBM_TRY(cudaGetLastError());
    // the rows changed: the solvers' diagonal tables follow (not while the solvers are
    // being set up, which computes them from these rows)
    if (c.sys1.dinv) refresh_system_diagonals(c, c.sys1);
    if (c.sys2.dinv) refresh_system_diagonals(c, c.sys2);
}

int embedded_hybrid_count(Context &c, int system)
{
    if (!c.emb.pid1) return 0;
    int cnt[4] = {0, 0, 0, 0};
    CUIBM_TRY(cudaMemcpyAsync(cnt, ib_plan(c).count, sizeof(cnt), cudaMemcpyDeviceToHost, c.stream));
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
    return system == 1 ? cnt[1] : cnt[3];
}

}  // namespace cuibm
