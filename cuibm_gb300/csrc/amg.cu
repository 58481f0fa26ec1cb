// Smoothed-aggregation algebraic multigrid: the preconditioner the reference
// takes from CUSP (cusp::precond::aggregation::smoothed_aggregation, selected by
// "preconditioner: SMOOTHED_AGGREGATION", src/preconditioner.h:84-113).
//
// Setup (host, once per operator):
//   strength   |a_ij| >= theta sqrt(|a_ii a_jj|), theta from strengthThreshold (default 0,
//              CUSP's: every off-diagonal entry is strong)
//   aggregates standard three-phase greedy aggregation over the matrix graph
//   tentative  T: piecewise-constant prolongator, columns normalised
//   smoothing  P = (I - w D^-1 A) T,  w = 4 / (3 rho(D^-1 A)), rho by power iteration
//   Galerkin   A_c = R A P with R = P^T; repeat until <= kCoarse unknowns
//   coarsest   dense inverse
// V-cycle (device): one damped-Jacobi sweep down (from a zero guess) and one up;
// with R = P^T and Jacobi smoothing the cycle is symmetric, so it also
// preconditions CG.  Level 0 is the matrix-free structured operator; coarse
// levels are CSR.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "amg.h"
#include "operators.cuh"
#include "solver.h"
#include "structured.cuh"

namespace cuibm {

constexpr int kCoarse = 1500;  // dense solve below this size (about 2M FMAs per cycle)

struct HostCsr {
    int n = 0, m = 0;  // rows, cols
    std::vector<int> ptr, col;
    std::vector<double> val;
};

// ---------------------------------------------------------------------------
// host sparse helpers
// ---------------------------------------------------------------------------
static HostCsr transpose(const HostCsr &A)
{
    HostCsr T;
    T.n = A.m;
    T.m = A.n;
    T.ptr.assign(T.n + 1, 0);
    for (int c : A.col) T.ptr[c + 1]++;
    for (int i = 0; i < T.n; ++i) T.ptr[i + 1] += T.ptr[i];
    T.col.resize(A.col.size());
    T.val.resize(A.val.size());
    std::vector<int> pos(T.ptr.begin(), T.ptr.end() - 1);
    for (int i = 0; i < A.n; ++i)
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            int d = pos[A.col[k]]++;
            T.col[d] = i;
            T.val[d] = A.val[k];
        }
    return T;
}

static HostCsr multiply(const HostCsr &A, const HostCsr &B)
{
    HostCsr C;
    C.n = A.n;
    C.m = B.m;
    C.ptr.assign(C.n + 1, 0);
    std::vector<int> mark(B.m, -1);
    std::vector<double> acc(B.m, 0.0);
    std::vector<int> cols;
    for (int i = 0; i < A.n; ++i) {
        cols.clear();
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            int a = A.col[k];
            double av = A.val[k];
            for (int q = B.ptr[a]; q < B.ptr[a + 1]; ++q) {
                int j = B.col[q];
                if (mark[j] != i) {
                    mark[j] = i;
                    acc[j] = 0;
                    cols.push_back(j);
                }
                acc[j] += av * B.val[q];
            }
        }
        std::sort(cols.begin(), cols.end());
        for (int j : cols) {
            C.col.push_back(j);
            C.val.push_back(acc[j]);
        }
        C.ptr[i + 1] = (int)C.col.size();
    }
    return C;
}

static std::vector<double> diagonal(const HostCsr &A)
{
    std::vector<double> d(A.n, 0.0);
    for (int i = 0; i < A.n; ++i)
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
            if (A.col[k] == i) d[i] += A.val[k];
    return d;
}

// spectral radius of D^-1 A by power iteration from a fixed start vector
static double rho_dinv_a(const HostCsr &A, const std::vector<double> &d)
{
    std::vector<double> x(A.n), y(A.n);
    for (int i = 0; i < A.n; ++i) x[i] = 1.0 + 0.25 * std::sin(0.37 * i);
    double lam = 1.0;
    for (int it = 0; it < 20; ++it) {
        double nrm = 0;
        for (int i = 0; i < A.n; ++i) {
            double s = 0;
            for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) s += A.val[k] * x[A.col[k]];
            y[i] = s / d[i];
            nrm += y[i] * y[i];
        }
        nrm = std::sqrt(nrm);
        double xn = 0;
        for (double v : x) xn += v * v;
        lam = nrm / std::sqrt(xn);
        for (int i = 0; i < A.n; ++i) x[i] = y[i] / nrm;
    }
    return lam;
}

// The strength graph for theta > 0: i - j when |a_ij| >= theta sqrt(|a_ii a_jj|) or
// |a_ji| >= theta sqrt(|a_ii a_jj|) (symmetric), off-diagonal; a link carries row i's
// |a_ij| where row i has the entry (phase 2 of the aggregation picks the strongest).
static HostCsr strength_graph(const HostCsr &A, const std::vector<double> &d, double theta)
{
    const int n = A.n;
    auto strong = [&](int i, int k) {
        const int j = A.col[k];
        return j != i && A.val[k] != 0 && std::fabs(A.val[k]) >= theta * std::sqrt(std::fabs(d[i] * d[j]));
    };
    // the links of every row in one flat array (counted first: a rebuilt hierarchy of a
    // moving body repeats this at every step, and a list per row cost most of it)
    std::vector<int> start(n + 1, 0);
    for (int i = 0; i < n; ++i)
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
            if (strong(i, k)) {
                start[i + 1]++;
                start[A.col[k] + 1]++;
            }
    for (int i = 0; i < n; ++i) start[i + 1] += start[i];
    std::vector<std::pair<int, double>> e(start[n]);
    std::vector<int> pos(start.begin(), start.end() - 1);
    for (int i = 0; i < n; ++i)
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
            if (strong(i, k)) {
                const int j = A.col[k];
                const double a = std::fabs(A.val[k]);
                e[pos[i]++] = {j, a};
                e[pos[j]++] = {i, -a};  // the reverse link, used where row j lacks the entry
            }
    HostCsr S;
    S.n = S.m = n;
    S.ptr.assign(n + 1, 0);
    S.col.reserve(e.size());
    S.val.reserve(e.size());
    for (int i = 0; i < n; ++i) {
        std::sort(e.begin() + start[i], e.begin() + start[i + 1],
                  [](const std::pair<int, double> &x, const std::pair<int, double> &y) {
                      return x.first != y.first ? x.first < y.first : x.second > y.second;  // own entry first
                  });
        int last = -1;
        for (int q = start[i]; q < start[i + 1]; ++q) {
            if (e[q].first == last) continue;
            S.col.push_back(e[q].first);
            S.val.push_back(std::fabs(e[q].second));
            last = e[q].first;
        }
        S.ptr[i + 1] = (int)S.col.size();
    }
    return S;
}

// three-phase greedy aggregation over the strength graph A (off-diagonal links);
// returns aggregate id per node and the count
static int aggregate(const HostCsr &A, std::vector<int> &agg)
{
    const int n = A.n;
    agg.assign(n, -1);
    int na = 0;
    // phase 1: a node whose neighbours are all free seeds an aggregate with them
    // (a node without strong links becomes an aggregate of its own)
    for (int i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        bool free_ = true;
        for (int k = A.ptr[i]; k < A.ptr[i + 1] && free_; ++k)
            if (A.col[k] != i && A.val[k] != 0 && agg[A.col[k]] >= 0) free_ = false;
        if (!free_) continue;
        agg[i] = na;
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
            if (A.val[k] != 0) agg[A.col[k]] = na;
        ++na;
    }
    // phase 2: free nodes join a neighbouring aggregate (the strongest link)
    std::vector<int> agg1 = agg;
    for (int i = 0; i < n; ++i) {
        if (agg1[i] >= 0) continue;
        double best = 0;
        int ba = -1;
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            int j = A.col[k];
            if (j != i && agg1[j] >= 0 && std::fabs(A.val[k]) > best) {
                best = std::fabs(A.val[k]);
                ba = agg1[j];
            }
        }
        if (ba >= 0) agg[i] = ba;
    }
    // phase 3: leftovers form aggregates with their free neighbours
    for (int i = 0; i < n; ++i) {
        if (agg[i] >= 0) continue;
        agg[i] = na;
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
            if (agg[A.col[k]] < 0) agg[A.col[k]] = na;
        ++na;
    }
    return na;
}

static void dense_inverse(const HostCsr &A, std::vector<double> &inv)
{
    const int n = A.n;
    std::vector<double> a(n * n, 0.0);
    inv.assign(n * n, 0.0);
    for (int i = 0; i < n; ++i) {
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) a[i * n + A.col[k]] += A.val[k];
        inv[i * n + i] = 1.0;
    }
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(a[r * n + c]) > std::fabs(a[piv * n + c])) piv = r;
        if (piv != c)
            for (int k = 0; k < n; ++k) {
                std::swap(a[c * n + k], a[piv * n + k]);
                std::swap(inv[c * n + k], inv[piv * n + k]);
            }
        double d = a[c * n + c];
        if (d == 0) d = 1e-300;
        for (int k = 0; k < n; ++k) {
            a[c * n + k] /= d;
            inv[c * n + k] /= d;
        }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            double f = a[r * n + c];
            if (f == 0) continue;
            for (int k = 0; k < n; ++k) {
                a[r * n + k] -= f * a[c * n + k];
                inv[r * n + k] -= f * inv[c * n + k];
            }
        }
    }
}


// device memory of the hierarchy: the context's arena, or (a hierarchy that will be
// rebuilt) allocations of its own, freed with it
template <class T>
static T *sa_alloc(Context &c, LinearSystem &S, size_t n)
{
    if (!S.sa_dynamic) return c.carve<T>(n);
    void *p = nullptr;
    CUIBM_TRY(cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(T)));
    S.sa_blocks.push_back(p);
    return static_cast<T *>(p);
}

// the level objects, and the device memory of a hierarchy that has its own (the arena's
// goes with the context)
void free_sa_hierarchy(LinearSystem &S)
{
    for (SaLevel *L : S.amg) delete L;
    S.amg.clear();
    for (void *p : S.sa_blocks) cudaFree(p);
    S.sa_blocks.clear();
}

static DevCsr upload(Context &c, LinearSystem &S, const HostCsr &H)
{
    DevCsr D;
    D.n = H.n;
    D.nnz = (int)H.col.size();
    D.ptr = sa_alloc<int>(c, S, H.ptr.size());
    D.col = sa_alloc<int>(c, S, std::max<size_t>(1, H.col.size()));
    D.val = sa_alloc<double>(c, S, std::max<size_t>(1, H.val.size()));
    CUIBM_TRY(cudaMemcpyAsync(D.ptr, H.ptr.data(), H.ptr.size() * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    if (!H.col.empty()) {
        CUIBM_TRY(cudaMemcpyAsync(D.col, H.col.data(), H.col.size() * sizeof(int), cudaMemcpyHostToDevice, c.stream));
        CUIBM_TRY(cudaMemcpyAsync(D.val, H.val.data(), H.val.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    }
    return D;
}

static bool structured_applies(const Context &c, const LinearSystem &S);
static void build_structured_hierarchy(Context &c, LinearSystem &S);

void build_sa_hierarchy(Context &c, LinearSystem &S)
{
    S.sa_structured = structured_applies(c, S);
    if (S.sa_structured) {
        build_structured_hierarchy(c, S);
        return;
    }
    std::vector<double> wh;
    if (S.w) {
        wh.resize(S.n);
        CUIBM_TRY(cudaMemcpyAsync(wh.data(), S.w, S.n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        CUIBM_TRY(cudaStreamSynchronize(c.stream));
    }
    HostCsr A;
    A.n = A.m = S.n;
    host_operator_csr(c, S.which, S.w ? wh.data() : nullptr, A.ptr, A.col, A.val, S.sa_body_free);
    std::vector<HostCsr> hostA;
    hostA.push_back(A);
    // host buffers are kept alive until the uploads below have been issued and synchronised
    std::vector<HostCsr> keepP, keepR, keepAP;
    std::vector<std::vector<double>> keepD;
    for (int lev = 0; lev < 25; ++lev) {
        const HostCsr &Al = hostA.back();
        SaLevel *L = new SaLevel();
        L->n = Al.n;
        std::vector<double> d = diagonal(Al);
        for (double &v : d)
            if (v == 0) v = 1.0;
        std::vector<double> dinv(d.size());
        for (size_t i = 0; i < d.size(); ++i) dinv[i] = 1.0 / d[i];
        L->dinv = sa_alloc<double>(c, S, L->n);
        keepD.push_back(dinv);
        CUIBM_TRY(cudaMemcpyAsync(L->dinv, keepD.back().data(), L->n * sizeof(double), cudaMemcpyHostToDevice,
                                  c.stream));
        L->x = sa_alloc<double>(c, S, L->n);
        L->b = sa_alloc<double>(c, S, L->n);
        L->r = sa_alloc<double>(c, S, L->n);
        L->t = sa_alloc<double>(c, S, L->n);
        if (lev > 0) L->A = upload(c, S, Al);
        if (Al.n <= kCoarse || lev == 24) {
            std::vector<double> inv;
            dense_inverse(Al, inv);
            L->coarse_inv = sa_alloc<double>(c, S, (size_t)Al.n * Al.n);
            keepD.push_back(inv);
            CUIBM_TRY(cudaMemcpyAsync(L->coarse_inv, keepD.back().data(), inv.size() * sizeof(double),
                                      cudaMemcpyHostToDevice, c.stream));
            S.amg.push_back(L);
            break;
        }
        double rho = rho_dinv_a(Al, d);
        L->omega = 4.0 / (3.0 * rho);
        std::vector<int> agg;
        // theta = 0: every nonzero entry of the level's matrix is a link
        int na = S.strength > 0 ? aggregate(strength_graph(Al, d, S.strength), agg) : aggregate(Al, agg);
        std::vector<int> size(na, 0);
        for (int a : agg) size[a]++;
        HostCsr T;
        T.n = Al.n;
        T.m = na;
        T.ptr.resize(T.n + 1);
        for (int i = 0; i < T.n; ++i) {
            T.ptr[i] = i;
            T.col.push_back(agg[i]);
            T.val.push_back(1.0 / std::sqrt((double)size[agg[i]]));
        }
        T.ptr[T.n] = T.n;
        HostCsr AT = multiply(Al, T);
        HostCsr P = T;  // P = T - w D^-1 A T (same sparsity as A T, which contains T's)
        {
            HostCsr Pn;
            Pn.n = AT.n;
            Pn.m = AT.m;
            Pn.ptr.assign(Pn.n + 1, 0);
            for (int i = 0; i < AT.n; ++i) {
                for (int k = AT.ptr[i]; k < AT.ptr[i + 1]; ++k) {
                    int j = AT.col[k];
                    double v = -L->omega * AT.val[k] / d[i];
                    if (j == agg[i]) v += T.val[i];
                    Pn.col.push_back(j);
                    Pn.val.push_back(v);
                }
                Pn.ptr[i + 1] = (int)Pn.col.size();
            }
            P = Pn;
        }
        HostCsr R = transpose(P);
        HostCsr AP = multiply(Al, P);
        HostCsr Ac = multiply(R, AP);
        keepP.push_back(P);
        keepR.push_back(R);
        keepAP.push_back(AP);
        L->P = upload(c, S, keepP.back());
        L->R = upload(c, S, keepR.back());
        L->AP = upload(c, S, keepAP.back());
        {
            std::vector<double> wd(L->n);
            for (int i = 0; i < L->n; ++i) wd[i] = L->omega * dinv[i];
            L->wd = sa_alloc<double>(c, S, L->n);
            keepD.push_back(wd);
            CUIBM_TRY(cudaMemcpyAsync(L->wd, keepD.back().data(), L->n * sizeof(double), cudaMemcpyHostToDevice,
                                      c.stream));
        }
        S.amg.push_back(L);
        hostA.push_back(Ac);
        CUIBM_TRY(cudaStreamSynchronize(c.stream));  // host vectors may be reallocated
    }
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
}

// Algorithmic bytes of one V-cycle of launch_vcycle, kernel by kernel: per level with
// a coarser one, the downward sweep reads b and the Jacobi weights and writes x and r
// (and reads the level's CSR matrix below level 0, whose operator is matrix-free); the
// restriction reads r and R and writes the coarse b; on the way up the prolongation
// reads the coarse x and P and updates x, and the smoothing sweep reads b, the
// weights and x (and the matrix) and writes its result.  A CSR matrix is 12 bytes per
// entry plus its row pointers.  The coarsest level's dense inverse (8 n_c^2 bytes) is
// an implementation choice, not algorithmic: it is left out, the coarsest level
// counting only its right-hand side and solution.
double sa_vcycle_bytes(const LinearSystem &S)
{
    auto csr = [](const DevCsr &M) { return 12.0 * M.nnz + 4.0 * (M.n + 1); };
    const int nl = (int)S.amg.size();
    double b = 0;
    if (S.sa_structured) {
        // the structured cycle: below level 0 the operator is nine coefficients a node,
        // the prolongator four weights a node (read by the restriction and the prolongation)
        for (int l = 0; l < nl; ++l) {
            const SaLevel *L = S.amg[l];
            const double n = L->n;
            if (l + 1 == nl) {
                b += 16.0 * n;
                break;
            }
            const double nc = S.amg[l + 1]->n, a = l > 0 ? 72.0 * n : 0.0;
            b += 32.0 * n + a;              // down: b, dinv in; x, r out
            b += 8.0 * n + 32.0 * n + 8.0 * nc;  // restriction: r and the weights in, coarse b out
            b += 8.0 * nc + 32.0 * n + 16.0 * n;  // prolongation into x
            b += 32.0 * n + a;              // up
        }
        return b;
    }
    for (int l = 0; l < nl; ++l) {
        const SaLevel *L = S.amg[l];
        const double n = L->n;
        if (l + 1 == nl) {
            b += 16.0 * n;
            break;
        }
        const double nc = S.amg[l + 1]->n;
        const double a = l > 0 ? csr(L->A) : 0.0;
        b += 32.0 * n + a;                   // down: b, dinv in; x, r out
        b += 8.0 * n + csr(L->R) + 8.0 * nc; // restriction
        b += 8.0 * nc + csr(L->P) + 16.0 * n;  // prolongation into x
        b += 32.0 * n + a;                   // up: b, dinv, x in; result out
    }
    return b;
}

int sa_coarsest_size(const LinearSystem &S) { return S.amg.empty() ? 0 : S.amg.back()->n; }

// ---------------------------------------------------------------------------
// V-cycle kernels
// ---------------------------------------------------------------------------
struct Lvl0 {
    int which;
    Lhs1Coef c1;
    Lhs2Coef c2;
    Grid g;
    const double *w;
    template <class X>
    __device__ __forceinline__ double row(int i, const X &x) const
    {
        double y = which == 1 ? lhs1_row_f(c1, g, i, x) : lhs2_row_f(c2, g, i, x);
        return w ? w[i] * y : y;
    }
};

struct CsrRow {
    DevCsr A;
    template <class X>
    __device__ __forceinline__ double row(int i, const X &x) const
    {
        double s = 0;
        for (int k = A.ptr[i]; k < A.ptr[i + 1]; ++k) s += A.val[k] * x(A.col[k]);
        return s;
    }
};

struct JacAccess {
    const double *__restrict__ b, *__restrict__ d;
    double w;
    __device__ __forceinline__ double operator()(int j) const { return w * d[j] * b[j]; }
};

// x = w D^-1 b (first sweep from zero) and r = b - A x, fused
template <class Op>
__global__ void k_sa_down(Op A, int n, const double *__restrict__ b, const double *__restrict__ dinv, double w,
                          double *__restrict__ x, double *__restrict__ r, const int *gate)
{
    if (gate && *gate != KS_RUNNING) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = w * dinv[i] * b[i];
    r[i] = b[i] - A.row(i, JacAccess{b, dinv, w});
}

// y = M v for a CSR matrix (restriction R r, or prolongation added: y += P v)
template <bool ADD>
__global__ void k_csr_mv(DevCsr M, const double *__restrict__ v, double *__restrict__ y, const int *gate)
{
    if (gate && *gate != KS_RUNNING) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M.n) return;
    double s = 0;
    for (int k = M.ptr[i]; k < M.ptr[i + 1]; ++k) s += M.val[k] * v[M.col[k]];
    y[i] = ADD ? y[i] + s : s;
}

// out = x + w D^-1 (b - A x)
template <class Op>
__global__ void k_sa_up(Op A, int n, const double *__restrict__ b, const double *__restrict__ dinv, double w,
                        const double *__restrict__ x, double *__restrict__ out, const int *gate)
{
    if (gate && *gate != KS_RUNNING) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = x[i] + w * dinv[i] * (b[i] - A.row(i, PtrAccess{x}));
}

// coarsest level: x = A^-1 b with the dense inverse (one warp per row)
__global__ void k_dense_mv(int n, const double *__restrict__ inv, const double *__restrict__ b,
                           double *__restrict__ x, const int *gate)
{
    if (gate && *gate != KS_RUNNING) return;
    const int row = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
    if (row >= n) return;
    double s = 0;
    for (int k = lane; k < n; k += 32) s += inv[(size_t)row * n + k] * b[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) x[row] = s;
}

// ---------------------------------------------------------------------------
// structured hierarchy (structured.cuh): set-up on the device
// ---------------------------------------------------------------------------
// A coarse level's 9-point operator
struct Row9 {
    int nx, ny;
    const double *c9;
    template <class X>
    __device__ __forceinline__ double row(int i, const X &x) const
    {
        return st_row9(nx, ny, c9, i, x);
    }
};

// The Poisson system of the plain and external methods: its operator is the 5-point
// QTBNQ on the pressure grid at every row (pins change diagonals only), and it is
// fixed.  By default from kStructuredMin unknowns: below, the graph aggregation's
// smaller aggregates take fewer iterations (the Re 40 cylinder's steady state: 4
// against 9) and the solve is bound by its phase count, not by the cycle's loads.
constexpr int kStructuredMin = 200000;

static bool structured_applies(const Context &c, const LinearSystem &S)
{
    const bool want = c.P.saStructured == 1 || (c.P.saStructured == -1 && S.n >= kStructuredMin);
    // the persistent solves built for two blocks per SM (-solverPack 2, batches) leave the
    // structured cycle out to keep their registers
    return want && c.P.solverPack != 2 && S.which == 2 && S.precond == PC_SMOOTHED_AGGREGATION && !S.sa_dynamic &&
           (c.P.solverType == ST_NAVIERSTOKES || c.P.solverType == ST_LUO) && !c.l2.patch.pid &&
           S.n == c.g.nx * c.g.ny && S.n > kCoarse;
}

// diagonal of a level operator (row i against the unit vector e_i) and its inverse
template <class Op>
__global__ void k_st_diag(Op A, int n, double *__restrict__ dinv)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double d = A.row(i, [i](int j) { return j == i ? 1.0 : 0.0; });
    if (d == 0) d = 1.0;
    dinv[i] = 1.0 / d;
}

// power iteration for rho(D^-1 A): y = D^-1 A x and the block sums of y^2 (summed in a
// fixed order by k_st_sum, so the estimate is the same on every run)
template <class Op>
__global__ void k_st_rho_apply(Op A, int n, const double *__restrict__ dinv, const double *__restrict__ x,
                               double *__restrict__ y, double *__restrict__ part)
{
    __shared__ double sh[kBlock / 32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0;
    if (i < n) {
        v = dinv[i] * A.row(i, PtrAccess{x});
        y[i] = v;
    }
    v *= v;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int k = 0; k < (int)blockDim.x / 32; ++k) t += sh[k];
        part[blockIdx.x] = t;
    }
}

__global__ void k_st_sum(int nb, const double *__restrict__ part, double *__restrict__ out)
{
    __shared__ double sh[kBlock];
    double t = 0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) t += part[k];
    sh[threadIdx.x] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int k = 0; k < (int)blockDim.x; ++k) s += sh[k];
        *out = s;
    }
}

__global__ void k_st_normalise(int n, const double *__restrict__ y, const double *__restrict__ sq,
                               double *__restrict__ x)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = y[i] / sqrt(*sq);
}

__global__ void k_st_scale(int n, const double *__restrict__ a, double s, double *__restrict__ y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = s * a[i];
}

// the prolongator's weights: P_iJ = [i in J] - w D^-1_i (A 1_J)_i for J the aggregates
// around node i, (A 1_J)_i being row i against the indicator of aggregate J
template <class Op>
__global__ void k_st_weights(Op A, int nx, int ny, int cnx, int cny, const double *__restrict__ dinv, double omega,
                             double *__restrict__ pw)
{
    const int n = nx * ny;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int iy = i / nx, ix = i - iy * nx;
    const StAxis ax = st_axis(ix, nx, cnx), ay = st_axis(iy, ny, cny);
    const double wdi = omega * dinv[i];
    auto weight = [&](int jx, int jy) {
        const double a = A.row(i, [&](int k) {
            const int ky = k / nx, kx = k - ky * nx;
            return st_axis(kx, nx, cnx).a == jx && st_axis(ky, ny, cny).a == jy ? 1.0 : 0.0;
        });
        return (ax.a == jx && ay.a == jy ? 1.0 : 0.0) - wdi * a;
    };
    pw[i] = weight(ax.a, ay.a);
    pw[n + i] = ax.s ? weight(ax.a + ax.s, ay.a) : 0.0;
    pw[2 * n + i] = ay.s ? weight(ax.a, ay.a + ay.s) : 0.0;
    pw[3 * n + i] = ax.s && ay.s ? weight(ax.a + ax.s, ay.a + ay.s) : 0.0;
}

// Galerkin product by probing: with the coarse nodes coloured (Jx mod 3, Jy mod 3),
// (P^T A P e_c)_J for the indicator e_c of one colour is the one entry of row J of the
// 9-point coarse operator whose neighbour has that colour
__global__ void k_st_probe_prolong(int nx, int ny, int cnx, int cny, const double *__restrict__ pw, int cx, int cy,
                                   double *__restrict__ y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx * ny) return;
    y[i] = st_prolong(nx, ny, cnx, cny, pw, i, [&](int J) {
        const int Jy = J / cnx, Jx = J - Jy * cnx;
        return Jx % 3 == cx && Jy % 3 == cy ? 1.0 : 0.0;
    });
}

template <class Op>
__global__ void k_st_apply(Op A, int n, const double *__restrict__ x, double *__restrict__ y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = A.row(i, PtrAccess{x});
}

__global__ void k_st_probe_restrict(int nx, int ny, int cnx, int cny, const double *__restrict__ pw, int cx, int cy,
                                    const double *__restrict__ w, double *__restrict__ c9)
{
    const int nc = cnx * cny;
    const int J = blockIdx.x * blockDim.x + threadIdx.x;
    if (J >= nc) return;
    const double v = st_restrict(nx, ny, cnx, cny, pw, J, PtrAccess{w});
    const int Jy = J / cnx, Jx = J - Jy * cnx;
    int dx = (cx - Jx % 3 + 3) % 3, dy = (cy - Jy % 3 + 3) % 3;
    if (dx == 2) dx = -1;
    if (dy == 2) dy = -1;
    const bool inside = Jx + dx >= 0 && Jx + dx < cnx && Jy + dy >= 0 && Jy + dy < cny;
    c9[(3 * (dy + 1) + dx + 1) * nc + J] = inside ? v : 0.0;
}

// prolongation added to the level's iterate: x += P xc
__global__ void k_st_prolong_add(int nx, int ny, int cnx, int cny, const double *__restrict__ pw,
                                 const double *__restrict__ xc, double *__restrict__ x, const int *gate)
{
    if (gate && *gate != KS_RUNNING) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nx * ny) x[i] += st_prolong(nx, ny, cnx, cny, pw, i, PtrAccess{xc});
}

// restriction: bc = P^T r
__global__ void k_st_restrict(int nx, int ny, int cnx, int cny, const double *__restrict__ pw,
                              const double *__restrict__ r, double *__restrict__ bc, const int *gate)
{
    if (gate && *gate != KS_RUNNING) return;
    const int J = blockIdx.x * blockDim.x + threadIdx.x;
    if (J < cnx * cny) bc[J] = st_restrict(nx, ny, cnx, cny, pw, J, PtrAccess{r});
}

// One level of the structured set-up: Jacobi tables, rho(D^-1 A) by 20 power
// iterations (from the graph set-up's start vector), the prolongator's weights and the
// next level's 9-point operator (nine probes).  Returns the next level's coefficients.
template <class Op>
static double *st_level(Context &c, LinearSystem &S, const Op &A, SaLevel *L, double *scratch)
{
    const int n = L->n, nx = L->nx, ny = L->ny, nb = blocks_for(n);
    k_st_diag<<<nb, kBlock, 0, c.stream>>>(A, n, L->dinv);
    double *xv = scratch, *yv = scratch + n, *wv = scratch + 2 * (size_t)n, *part = scratch + 3 * (size_t)n;
    double *acc = part + nb;
    std::vector<double> x0(n);
    double nrm = 0;
    for (int i = 0; i < n; ++i) {
        x0[i] = 1.0 + 0.25 * std::sin(0.37 * i);
        nrm += x0[i] * x0[i];
    }
    nrm = std::sqrt(nrm);
    for (double &v : x0) v /= nrm;
    CUIBM_TRY(cudaMemcpyAsync(xv, x0.data(), n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    constexpr int kIts = 20;
    for (int it = 0; it < kIts; ++it) {
        k_st_rho_apply<<<nb, kBlock, 0, c.stream>>>(A, n, L->dinv, xv, yv, part);
        k_st_sum<<<1, kBlock, 0, c.stream>>>(nb, part, acc + it);
        k_st_normalise<<<nb, kBlock, 0, c.stream>>>(n, yv, acc + it, xv);
    }
    double sq = 0;
    CUIBM_TRY(cudaMemcpyAsync(&sq, acc + kIts - 1, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    CUIBM_TRY(cudaStreamSynchronize(c.stream));  // x0 and sq
    const double rho = std::sqrt(sq);
    if (!(rho > 0) || !std::isfinite(rho)) throw CudaError("structured smoothed aggregation: no spectral radius");
    L->omega = 4.0 / (3.0 * rho);
    L->wd = sa_alloc<double>(c, S, n);
    k_st_scale<<<nb, kBlock, 0, c.stream>>>(n, L->dinv, L->omega, L->wd);
    const int cnx = st_coarse(nx), cny = st_coarse(ny), nc = cnx * cny;
    L->pw = sa_alloc<double>(c, S, 4 * (size_t)n);
    k_st_weights<<<nb, kBlock, 0, c.stream>>>(A, nx, ny, cnx, cny, L->dinv, L->omega, L->pw);
    double *c9 = sa_alloc<double>(c, S, 9 * (size_t)nc);
    for (int cy = 0; cy < 3; ++cy)
        for (int cx = 0; cx < 3; ++cx) {
            k_st_probe_prolong<<<nb, kBlock, 0, c.stream>>>(nx, ny, cnx, cny, L->pw, cx, cy, yv);
            k_st_apply<<<nb, kBlock, 0, c.stream>>>(A, n, yv, wv);
            k_st_probe_restrict<<<blocks_for(nc), kBlock, 0, c.stream>>>(nx, ny, cnx, cny, L->pw, cx, cy, wv, c9);
        }
    CUIBM_TRY(cudaGetLastError());
    return c9;
}

static void build_structured_hierarchy(Context &c, LinearSystem &S)
{
    Lvl0 A0{S.which, c.l1, c.l2, c.g, S.w};
    const int n0 = S.n;
    double *scratch = c.carve<double>(4 * (size_t)n0 + blocks_for(n0) + 64);
    int nx = c.g.nx, ny = c.g.ny;
    const double *c9 = nullptr;  // the current level's operator (levels below 0)
    for (int lev = 0; lev < 25; ++lev) {
        SaLevel *L = new SaLevel();
        L->n = nx * ny;
        L->nx = nx;
        L->ny = ny;
        L->c9 = const_cast<double *>(c9);
        L->dinv = sa_alloc<double>(c, S, L->n);
        L->x = sa_alloc<double>(c, S, L->n);
        L->b = sa_alloc<double>(c, S, L->n);
        L->r = sa_alloc<double>(c, S, L->n);
        L->t = sa_alloc<double>(c, S, L->n);
        const bool coarsest = lev > 0 && (L->n <= kCoarse || lev == 24);
        if (coarsest) {
            // the 9-point operator to the host, its dense inverse back
            std::vector<double> h(9 * (size_t)L->n);
            CUIBM_TRY(cudaMemcpyAsync(h.data(), c9, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            CUIBM_TRY(cudaStreamSynchronize(c.stream));
            HostCsr H;
            H.n = H.m = L->n;
            H.ptr.assign(L->n + 1, 0);
            for (int i = 0; i < L->n; ++i) {
                const int iy = i / nx, ix = i - iy * nx;
                for (int k = 0; k < 9; ++k) {
                    const int dy = k / 3 - 1, dx = k % 3 - 1;
                    const double v = h[(size_t)k * L->n + i];
                    if (v == 0 || ix + dx < 0 || ix + dx >= nx || iy + dy < 0 || iy + dy >= ny) continue;
                    H.col.push_back(i + dy * nx + dx);
                    H.val.push_back(v);
                }
                H.ptr[i + 1] = (int)H.col.size();
            }
            k_st_diag<<<blocks_for(L->n), kBlock, 0, c.stream>>>(Row9{nx, ny, c9}, L->n, L->dinv);
            std::vector<double> inv;
            dense_inverse(H, inv);
            L->coarse_inv = sa_alloc<double>(c, S, inv.size());
            CUIBM_TRY(cudaMemcpyAsync(L->coarse_inv, inv.data(), inv.size() * sizeof(double), cudaMemcpyHostToDevice,
                                      c.stream));
            CUIBM_TRY(cudaStreamSynchronize(c.stream));
            S.amg.push_back(L);
            break;
        }
        c9 = lev == 0 ? st_level(c, S, A0, L, scratch) : st_level(c, S, Row9{nx, ny, c9}, L, scratch);
        S.amg.push_back(L);
        nx = st_coarse(nx);
        ny = st_coarse(ny);
    }
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
}

// z = V(r): r on level 0 is the Krylov residual, z the preconditioned vector
void launch_vcycle(Context &c, LinearSystem &S, const double *r, double *z)
{
    const int nl = (int)S.amg.size();
    const int *gate = &S.ks->status;
    Lvl0 A0{S.which, c.l1, c.l2, c.g, S.w};
    if (S.sa_structured) {
        const double *bl = r;
        for (int l = 0; l < nl - 1; ++l) {
            SaLevel *L = S.amg[l], *C = S.amg[l + 1];
            if (l == 0)
                k_sa_down<<<blocks_for(L->n), kBlock, 0, c.stream>>>(A0, L->n, bl, L->dinv, L->omega, L->x, L->r,
                                                                     gate);
            else
                k_sa_down<<<blocks_for(L->n), kBlock, 0, c.stream>>>(Row9{L->nx, L->ny, L->c9}, L->n, bl, L->dinv,
                                                                     L->omega, L->x, L->r, gate);
            k_st_restrict<<<blocks_for(C->n), kBlock, 0, c.stream>>>(L->nx, L->ny, C->nx, C->ny, L->pw, L->r, C->b,
                                                                      gate);
            bl = C->b;
        }
        SaLevel *C = S.amg[nl - 1];
        k_dense_mv<<<(C->n + 7) / 8, 256, 0, c.stream>>>(C->n, C->coarse_inv, C->b, C->x, gate);
        const double *xup = C->x;
        for (int l = nl - 2; l >= 0; --l) {
            SaLevel *L = S.amg[l], *Cl = S.amg[l + 1];
            k_st_prolong_add<<<blocks_for(L->n), kBlock, 0, c.stream>>>(L->nx, L->ny, Cl->nx, Cl->ny, L->pw, xup,
                                                                         L->x, gate);
            double *out = (l == 0) ? z : L->t;
            const double *bb = (l == 0) ? r : L->b;
            if (l == 0)
                k_sa_up<<<blocks_for(L->n), kBlock, 0, c.stream>>>(A0, L->n, bb, L->dinv, L->omega, L->x, out, gate);
            else
                k_sa_up<<<blocks_for(L->n), kBlock, 0, c.stream>>>(Row9{L->nx, L->ny, L->c9}, L->n, bb, L->dinv,
                                                                   L->omega, L->x, out, gate);
            xup = out;
        }
        CUIBM_TRY(cudaGetLastError());
        return;
    }
    // downward
    const double *bl = r;
    for (int l = 0; l < nl - 1; ++l) {
        SaLevel *L = S.amg[l];
        if (l == 0)
            k_sa_down<<<blocks_for(L->n), kBlock, 0, c.stream>>>(A0, L->n, bl, L->dinv, L->omega, L->x, L->r, gate);
        else
            k_sa_down<<<blocks_for(L->n), kBlock, 0, c.stream>>>(CsrRow{L->A}, L->n, bl, L->dinv, L->omega, L->x,
                                                                 L->r, gate);
        k_csr_mv<false><<<blocks_for(L->R.n), kBlock, 0, c.stream>>>(L->R, L->r, S.amg[l + 1]->b, gate);
        bl = S.amg[l + 1]->b;
    }
    SaLevel *C = S.amg[nl - 1];
    double *xc = (nl == 1) ? z : C->x;
    k_dense_mv<<<(C->n + 7) / 8, 256, 0, c.stream>>>(C->n, C->coarse_inv, nl == 1 ? r : C->b, xc, gate);
    // upward: level l result goes to t_l (l > 0) or z (l = 0)
    const double *xup = xc;
    for (int l = nl - 2; l >= 0; --l) {
        SaLevel *L = S.amg[l];
        k_csr_mv<true><<<blocks_for(L->P.n), kBlock, 0, c.stream>>>(L->P, xup, L->x, gate);
        double *out = (l == 0) ? z : L->t;
        const double *bb = (l == 0) ? r : L->b;
        if (l == 0)
            k_sa_up<<<blocks_for(L->n), kBlock, 0, c.stream>>>(A0, L->n, bb, L->dinv, L->omega, L->x, out, gate);
        else
            k_sa_up<<<blocks_for(L->n), kBlock, 0, c.stream>>>(CsrRow{L->A}, L->n, bb, L->dinv, L->omega, L->x, out,
                                                               gate);
        xup = out;
    }
    CUIBM_TRY(cudaGetLastError());
}

// ---- the transposed cycle (discrete adjoint) ----------------------------------------
// The Galerkin hierarchy of A^T with the same prolongators is the transposed one:
// P^T A^T P = (P^T A P)^T, so a V-cycle for A^T needs only the transposed level
// matrices and the transposed coarsest inverse.  They are made from the forward
// hierarchy the first time the adjoint asks (and again after a rebuild), in blocks that
// go with the hierarchy.
static void *sa_block(LinearSystem &S, size_t bytes)
{
    void *p = nullptr;
    CUIBM_TRY(cudaMalloc(&p, std::max<size_t>(1, bytes)));
    S.sa_blocks.push_back(p);
    return p;
}

void ensure_transposed_levels(Context &c, LinearSystem &S)
{
    if (S.sa_structured)
        throw InputError("the transposed cycle takes the graph-aggregated hierarchy (-saStructured 0)");
    for (size_t l = 0; l < S.amg.size(); ++l) {
        SaLevel *L = S.amg[l];
        if (l > 0 && !L->AT.ptr) {
            HostCsr H;
            H.n = H.m = L->A.n;
            H.ptr.resize(H.n + 1);
            H.col.resize(L->A.nnz);
            H.val.resize(L->A.nnz);
            CUIBM_TRY(cudaMemcpyAsync(H.ptr.data(), L->A.ptr, H.ptr.size() * sizeof(int), cudaMemcpyDeviceToHost,
                                      c.stream));
            if (L->A.nnz) {
                CUIBM_TRY(cudaMemcpyAsync(H.col.data(), L->A.col, H.col.size() * sizeof(int), cudaMemcpyDeviceToHost,
                                          c.stream));
                CUIBM_TRY(cudaMemcpyAsync(H.val.data(), L->A.val, H.val.size() * sizeof(double),
                                          cudaMemcpyDeviceToHost, c.stream));
            }
            CUIBM_TRY(cudaStreamSynchronize(c.stream));
            const HostCsr T = transpose(H);
            DevCsr D;
            D.n = T.n;
            D.nnz = (int)T.col.size();
            D.ptr = static_cast<int *>(sa_block(S, T.ptr.size() * sizeof(int)));
            D.col = static_cast<int *>(sa_block(S, T.col.size() * sizeof(int)));
            D.val = static_cast<double *>(sa_block(S, T.val.size() * sizeof(double)));
            CUIBM_TRY(cudaMemcpyAsync(D.ptr, T.ptr.data(), T.ptr.size() * sizeof(int), cudaMemcpyHostToDevice,
                                      c.stream));
            if (D.nnz) {
                CUIBM_TRY(cudaMemcpyAsync(D.col, T.col.data(), T.col.size() * sizeof(int), cudaMemcpyHostToDevice,
                                          c.stream));
                CUIBM_TRY(cudaMemcpyAsync(D.val, T.val.data(), T.val.size() * sizeof(double),
                                          cudaMemcpyHostToDevice, c.stream));
            }
            CUIBM_TRY(cudaStreamSynchronize(c.stream));
            L->AT = D;
        }
        if (L->coarse_inv && !L->coarse_inv_t) {
            const size_t n = L->n;
            std::vector<double> a(n * n), t(n * n);
            CUIBM_TRY(cudaMemcpyAsync(a.data(), L->coarse_inv, a.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                      c.stream));
            CUIBM_TRY(cudaStreamSynchronize(c.stream));
            for (size_t i = 0; i < n; ++i)
                for (size_t j = 0; j < n; ++j) t[j * n + i] = a[i * n + j];
            L->coarse_inv_t = static_cast<double *>(sa_block(S, t.size() * sizeof(double)));
            CUIBM_TRY(cudaMemcpyAsync(L->coarse_inv_t, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice,
                                      c.stream));
            CUIBM_TRY(cudaStreamSynchronize(c.stream));
        }
    }
}

struct Lvl0T {
    int which;
    Op1T a1;
    Op2T a2;
    template <class X>
    __device__ __forceinline__ double row(int i, const X &x) const
    {
        return which == 1 ? a1.row(i, x) : a2.row(i, x);
    }
};

// z = the V-cycle of launch_vcycle for A^T: every level operator transposed (level 0: the
// matrix-free A^T of the transposed lists T).  S holds the forward hierarchy and the
// gate (the status of the solve it serves).
void launch_vcycle_transposed(Context &c, LinearSystem &S, const TransposeList &T, const double *r, double *z)
{
    const int nl = (int)S.amg.size();
    const int *gate = &S.ks->status;
    Lvl0T A0{S.which, Op1T{c.l1, c.g, T}, Op2T{c.l2, c.g, T}};
    const double *bl = r;
    for (int l = 0; l < nl - 1; ++l) {
        SaLevel *L = S.amg[l];
        if (l == 0)
            k_sa_down<<<blocks_for(L->n), kBlock, 0, c.stream>>>(A0, L->n, bl, L->dinv, L->omega, L->x, L->r, gate);
        else
            k_sa_down<<<blocks_for(L->n), kBlock, 0, c.stream>>>(CsrRow{L->AT}, L->n, bl, L->dinv, L->omega, L->x,
                                                                 L->r, gate);
        k_csr_mv<false><<<blocks_for(L->R.n), kBlock, 0, c.stream>>>(L->R, L->r, S.amg[l + 1]->b, gate);
        bl = S.amg[l + 1]->b;
    }
    SaLevel *C = S.amg[nl - 1];
    double *xc = (nl == 1) ? z : C->x;
    k_dense_mv<<<(C->n + 7) / 8, 256, 0, c.stream>>>(C->n, C->coarse_inv_t, nl == 1 ? r : C->b, xc, gate);
    const double *xup = xc;
    for (int l = nl - 2; l >= 0; --l) {
        SaLevel *L = S.amg[l];
        k_csr_mv<true><<<blocks_for(L->P.n), kBlock, 0, c.stream>>>(L->P, xup, L->x, gate);
        double *out = (l == 0) ? z : L->t;
        const double *bb = (l == 0) ? r : L->b;
        if (l == 0)
            k_sa_up<<<blocks_for(L->n), kBlock, 0, c.stream>>>(A0, L->n, bb, L->dinv, L->omega, L->x, out, gate);
        else
            k_sa_up<<<blocks_for(L->n), kBlock, 0, c.stream>>>(CsrRow{L->AT}, L->n, bb, L->dinv, L->omega, L->x, out,
                                                               gate);
        xup = out;
    }
    CUIBM_TRY(cudaGetLastError());
}

}  // namespace cuibm
