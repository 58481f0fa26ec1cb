// Persistent linear solves, host side: set-up, tables, launches (the kernels are in
// fused_kernels.cuh, instantiated by fused_op1.cu, fused_op2.cu, fused_mixed_op1.cu and
// fused_mixed_op2.cu).
#include "fused_kernels.cuh"

namespace cuibm {

// unscaled operator diagonal, summed as the stepwise row functions sum it
template <class Op>
__global__ void k_fused_diag(Op A, int n, double *diag)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    diag[i] = A.row(i, [&](int j) { return j == i ? 1.0 : 0.0; });
}

__global__ void k_to_float(const double *__restrict__ src, float *__restrict__ dst, long n)
{
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (float)src[i];
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct Op1Plain {
    Lhs1Coef c;
    Grid g;
    template <class X>
    __device__ __forceinline__ double row(int i, const X &x) const
    {
        return lhs1_row_f(c, g, i, x);
    }
};
struct Op2Plain {
    Lhs2Coef c;
    Grid g;
    template <class X>
    __device__ __forceinline__ double row(int i, const X &x) const
    {
        return lhs2_row_f(c, g, i, x);
    }
};

// Float copies of a system's tables for the mixed-precision solve (device memory in
// the context arena; this host record points at them).
struct MixedState {
    Lhs1T<float> l1{};
    Lhs2T<float> l2{};
    float *diag = nullptr, *dinv = nullptr, *w = nullptr, *winv = nullptr;
    float *wd0 = nullptr;  // level 0's omega D^-1 (refreshed with the diagonal)
    FArgs<float> *dev = nullptr;
};

static float *to_float(Context &c, const double *src, size_t n)
{
    float *dst = c.carve<float>(std::max<size_t>(n, 1));
    if (n) {
        k_to_float<<<blocks_for((long)n), kBlock, 0, c.stream>>>(src, dst, (long)n);
        CUIBM_TRY(cudaGetLastError());
    }
    return dst;
}

static void convert_into(Context &c, const double *src, float *dst, size_t n)
{
    if (!src || !dst || !n) return;
    k_to_float<<<blocks_for((long)n), kBlock, 0, c.stream>>>(src, dst, (long)n);
    CUIBM_TRY(cudaGetLastError());
}

// the operator diagonal the persistent solver's rows use (rows may change when a body
// moves), and its float copies
void refresh_fused_diag(Context &c, LinearSystem &S)
{
    if (!S.diag) return;
    if (S.which == 1)
        k_fused_diag<<<blocks_for(S.n), kBlock, 0, c.stream>>>(Op1Plain{c.l1, c.g}, S.n, S.diag);
    else
        k_fused_diag<<<blocks_for(S.n), kBlock, 0, c.stream>>>(Op2Plain{c.l2, c.g}, S.n, S.diag);
    CUIBM_TRY(cudaGetLastError());
    if (MixedState *m = static_cast<MixedState *>(S.mixed)) {
        convert_into(c, S.diag, m->diag, S.n);
        convert_into(c, S.dinv, m->dinv, S.n);
    }
}

void refresh_fused_level0(Context &c, LinearSystem &S)
{
    MixedState *m = static_cast<MixedState *>(S.mixed);
    if (m && m->wd0 && !S.amg.empty()) convert_into(c, S.amg[0]->wd, m->wd0, S.n);
}

static cudaLaunchConfig_t coop_config(Context &c, LinearSystem &S, cudaLaunchAttribute *attr)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(S.fused_grid);
    cfg.blockDim = dim3(S.fused_threads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = c.stream;
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

template <class Op>
static void launch_fused_op(Context &c, LinearSystem &S, Op A, const double *b, double *x)
{
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = coop_config(c, S, attr);
    using Fn = void (*)(Op, const FArgs<double> *, const double *, double *);
    const FArgs<double> *args = static_cast<const FArgs<double> *>(S.fargs);
    CUIBM_TRY(cudaLaunchKernelEx(&cfg, reinterpret_cast<Fn>(S.fused_fn), A, args, b, x));
}

template <class Op64, class Op32>
static void launch_fused_mixed(Context &c, LinearSystem &S, Op64 A, Op32 A32, const double *b, double *x)
{
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t cfg = coop_config(c, S, attr);
    using Fn = void (*)(Op64, Op32, const FArgs<double> *, const FArgs<float> *, const double *, double *);
    const FArgs<double> *args = static_cast<const FArgs<double> *>(S.fargs);
    const FArgs<float> *fargs = static_cast<MixedState *>(S.mixed)->dev;
    CUIBM_TRY(cudaLaunchKernelEx(&cfg, reinterpret_cast<Fn>(S.fused_fn), A, A32, args, fargs, b, x));
}

// Below this many unknowns the FP64 Jacobi BiCGSTAB folds its direction and half step
// into the phases that apply A (FArgs::fold1; CUIBM_FOLD1=0 or 1 overrides).  None by
// default: at the Re 40 cylinder's 145k velocity unknowns the folded solve took 153 us
// in 14 phases against 149 us in 22 (the recomputation's FP64 issue costs what the
// barriers save); the FP32 inner solves of iterative refinement always fold.
constexpr int kFoldMax = 0;

// Structured restrictions into coarse levels up to this size take 8 lanes a coarse node
constexpr int kRestrictGroupMax = 20000;

// From this many unknowns on, the FP64 BiCGSTAB cycles' first sweep is a phase of its
// own (FArgs::split0; CUIBM_SPLIT0=0 keeps it folded)
constexpr int kSplitMin = 200000;

// Upload the solver's arguments (after the SA hierarchy exists).
static void upload_fargs(Context &c, LinearSystem &S)
{
    FArgs<double> a = {};
    a.n = S.n;
    a.r = S.r;
    a.rs = S.rs;
    a.p = S.p;
    a.p2 = S.p2;
    a.Mp = S.Mp;
    a.AMp = S.AMp;
    a.AMp2 = S.AMp2;
    a.s = S.s;
    a.Ms = S.Ms;
    a.AMs = S.AMs;
    a.z = S.z;
    a.q = S.q;
    a.dinv = S.dinv;
    a.w = S.w;
    a.winv = S.winv;
    a.diag = S.diag;
    a.partials = S.fpartials;
    a.sync = S.fsync;
    a.trace = c.trace_solve ? c.solve_trace + (S.which - 1) * kTraceLen : nullptr;
    a.ks = S.ks;
    a.err = c.err_word;
    a.which = S.which;
    a.nlev = (int)S.amg.size();
    for (int l = 0; l < a.nlev; ++l) {
        const SaLevel *L = S.amg[l];
        FLevel<double> &F = a.lev[l];
        auto view = [](const DevCsr &M) { return CsrV<double>{M.n, M.nnz, M.ptr, M.col, M.val}; };
        F.n = L->n;
        F.A = view(L->A);
        F.P = view(L->P);
        F.R = view(L->R);
        F.AP = view(L->AP);
        F.wd = L->wd;
        F.x = L->x;
        F.b = L->b;
        F.r = L->r;
        F.t = L->t;
        F.inv = L->coarse_inv;
        F.nx = L->nx;
        F.ny = L->ny;
        F.c9 = L->c9;
        F.pw = L->pw;
        F.fz = l > 0 && L->nx > 0;
        F.rg = L->nx > 0 && l + 1 < a.nlev && S.amg[l + 1]->n <= kRestrictGroupMax;
    }
    a.st = S.sa_structured;
    a.split0 = S.n >= kSplitMin && !(getenv("CUIBM_SPLIT0") && getenv("CUIBM_SPLIT0")[0] == '0');
    {
        const char *e = getenv("CUIBM_FOLD1");
        a.fold1 = e && (e[0] == '0' || e[0] == '1') ? e[0] == '1' : S.n < kFoldMax;
    }
    a.ym = S.ym;
    a.wdef = S.wdef;
    a.aedef = S.aedef;
    a.Edef = S.Edef;
    MixedState *m = static_cast<MixedState *>(S.mixed);
    FArgs<double> *d = S.fargs ? static_cast<FArgs<double> *>(S.fargs) : c.carve<FArgs<double>>(1);
    CUIBM_TRY(cudaMemcpyAsync(d, &a, sizeof(a), cudaMemcpyHostToDevice, c.stream));
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
    S.fargs = d;
    if (m) {
        // the float solver shares the reduction buffers, the barrier and the trace
        FArgs<float> fa = {};
        CUIBM_TRY(cudaMemcpy(&fa, m->dev, sizeof(fa), cudaMemcpyDeviceToHost));
        fa.partials = S.fpartials;
        fa.sync = S.fsync;
        fa.trace = a.trace;
        fa.ks = S.ks;
        fa.err = c.err_word;
        CUIBM_TRY(cudaMemcpy(m->dev, &fa, sizeof(fa), cudaMemcpyHostToDevice));
    }
}

// The float side of a mixed-precision system: vectors, operator tables, Jacobi and
// symmetrisation tables and the SA hierarchy's matrices and smoother weights (index
// arrays and the coarsest dense inverse are shared with the FP64 copies); for the
// Poisson system with SA also A^T e and e^T A e for the constant-mode correction.
static void setup_mixed(Context &c, LinearSystem &S)
{
    MixedState *m = new MixedState();
    S.mixed = m;
    const int n = S.n, nx = c.g.nx, ny = c.g.ny;
    if (S.which == 1) {
        const Lhs1Coef &t = c.l1;
        m->l1 = Lhs1T<float>{to_float(c, t.uE, nx - 1), to_float(c, t.uW, nx - 1), to_float(c, t.uN, ny),
                             to_float(c, t.uS, ny),     to_float(c, t.vE, nx),     to_float(c, t.vW, nx),
                             to_float(c, t.vN, ny - 1), to_float(c, t.vS, ny - 1), t.patch,
                             t.rscale ? to_float(c, t.rscale, c.g.nUV) : nullptr};
    } else {
        const Lhs2Coef &t = c.l2;
        m->l2 = Lhs2T<float>{to_float(c, t.E, nx), to_float(c, t.W, nx), to_float(c, t.N, ny), to_float(c, t.S, ny),
                             t.pin0, t.pinc, t.patch};
    }
    m->diag = to_float(c, S.diag, n);
    m->dinv = to_float(c, S.dinv, n);
    if (S.w) {
        m->w = to_float(c, S.w, n);
        m->winv = to_float(c, S.winv, n);
    }
    FArgs<float> f = {};
    f.n = n;
    float **vecs[] = {&f.r, &f.rs, &f.p, &f.p2, &f.Mp, &f.AMp, &f.AMp2, &f.s, &f.Ms, &f.AMs, &f.bin, &f.xin};
    for (float **v : vecs) *v = c.carve<float>(n);
    f.z = f.Ms;  // as in the FP64 layout: CG's z and q reuse BiCGSTAB's Ms and AMs
    f.q = f.AMs;
    f.dinv = m->dinv;
    f.w = m->w;
    f.winv = m->winv;
    f.diag = m->diag;
    f.which = S.which;
    f.nlev = (int)S.amg.size();
    for (int l = 0; l < f.nlev; ++l) {
        const SaLevel *L = S.amg[l];
        FLevel<float> &F = f.lev[l];
        auto view = [&](const DevCsr &M) {
            return CsrV<float>{M.n, M.nnz, M.ptr, M.col, M.val ? to_float(c, M.val, M.nnz) : nullptr};
        };
        F.n = L->n;
        F.A = view(L->A);
        F.P = view(L->P);
        F.R = view(L->R);
        F.AP = view(L->AP);
        F.wd = L->wd ? to_float(c, L->wd, L->n) : nullptr;
        if (l == 0) m->wd0 = const_cast<float *>(F.wd);
        F.x = c.carve<float>(L->n);
        F.b = c.carve<float>(L->n);
        F.r = c.carve<float>(L->n);
        F.t = c.carve<float>(L->n);
        F.inv = L->coarse_inv;  // shared: the coarse solve runs in FP64
        F.nx = L->nx;
        F.ny = L->ny;
        F.c9 = L->c9 ? to_float(c, L->c9, 9 * (size_t)L->n) : nullptr;
        F.pw = L->pw ? to_float(c, L->pw, 4 * (size_t)L->n) : nullptr;
        F.fz = l > 0;
        F.rg = L->nx > 0 && l + 1 < f.nlev && S.amg[l + 1]->n <= kRestrictGroupMax;
    }
    f.st = S.sa_structured;
    f.fold1 = 1;
    m->dev = c.carve<FArgs<float>>(1);
    CUIBM_TRY(cudaMemcpyAsync(m->dev, &f, sizeof(f), cudaMemcpyHostToDevice, c.stream));
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
}

// The constant-mode correction of the SA-preconditioned BiCGSTAB on the Poisson system
// (both precisions): w = A^T e (column sums) and E = e^T A e of the operator the solver
// iterates on, and the buffer for the cycle's output.  The pressure operator's
// near-null space is the constant (pinned at one cell); the cycle resolves it poorly,
// and re-solving it exactly - z = y + e (e.r - w.y) / E, so that e^T (A z - r) = 0 - is
// a one-vector coarse correction.  The FP32 cycle always gets it.  In FP64 the
// constant mode's eigenvalue shrinks like 1/n, and the correction pays from about
// 2e5 unknowns on (the Re 550 cylinder's Poisson solve: 30 iterations instead of 55;
// at the Re 40 cylinder's 73k it costs a fifth iteration at the steady state); it is
// used from kDeflateMin unknowns, CUIBM_DEFLATE=1 or 0 overrides that.
constexpr int kDeflateMin = 200000;

static void setup_deflation(Context &c, LinearSystem &S)
{
    S.ym = nullptr;
    S.wdef = nullptr;
    S.Edef = 0;
    if (!(S.which == 2 && mixed_vcycle(S))) return;
    const char *e = getenv("CUIBM_DEFLATE");
    const bool mixed = S.precision == PRECISION_MIXED;
    S.ym = c.carve<double>(S.n);
    bool on = S.n >= kDeflateMin;
    if (e && (e[0] == '0' || e[0] == '1')) on = e[0] == '1';
    if (!mixed && !on) return;
    std::vector<int> ptr, col;
    std::vector<double> val, w(S.n, 0.0), ae(S.n, 0.0);
    host_operator_csr(c, 2, nullptr, ptr, col, val);
    for (size_t k = 0; k < col.size(); ++k) w[col[k]] += val[k];
    for (int i = 0; i < S.n; ++i)
        for (int k = ptr[i]; k < ptr[i + 1]; ++k) ae[i] += val[k];
    double E = 0;
    for (double v : w) E += v;
    if (!(E != 0)) return;  // no pinned cell: the operator is singular, leave the cycle alone
    S.wdef = c.carve<double>(S.n);
    S.aedef = c.carve<double>(S.n);
    S.Edef = E;
    CUIBM_TRY(cudaMemcpyAsync(S.wdef, w.data(), S.n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    CUIBM_TRY(cudaMemcpyAsync(S.aedef, ae.data(), S.n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    CUIBM_TRY(cudaStreamSynchronize(c.stream));
}

void free_fused(LinearSystem &S)
{
    delete static_cast<MixedState *>(S.mixed);
    S.mixed = nullptr;
}

void launch_fused_solve(Context &c, LinearSystem &S, const double *b, double *x)
{
    CUIBM_TRY(cudaMemsetAsync(S.fsync, 0, sizeof(FusedSyncState), c.stream));
    if (MixedState *m = static_cast<MixedState *>(S.mixed)) {
        // the refinement's outer residual is that of the original system (no
        // symmetrisation weights); the FP32 operator carries them for CG
        if (S.which == 1)
            launch_fused_mixed(c, S, Op1D<double>{tab64(c.l1), c.g, S.diag, mixed_vcycle(S) ? S.w : nullptr},
                               Op1D<float>{m->l1, c.g, m->diag, m->w}, b, x);
        else
            launch_fused_mixed(c, S, Op2D<double>{tab64(c.l2), c.g, S.diag, mixed_vcycle(S) ? S.w : nullptr},
                               Op2D<float>{m->l2, c.g, m->diag, m->w}, b, x);
        return;
    }
    if (S.which == 1)
        launch_fused_op(c, S, Op1D<double>{tab64(c.l1), c.g, S.diag, S.w}, b, x);
    else
        launch_fused_op(c, S, Op2D<double>{tab64(c.l2), c.g, S.diag, S.w}, b, x);
}

void set_fused_trace(Context &c, LinearSystem &S, bool on)
{
    (void)on;  // read from c.trace_solve
    if (S.fused_fn) upload_fargs(c, S);
}

// Algorithmic bytes of one solve of `it` iterations as the persistent kernel
// does it: 8 bytes per vector value each phase reads or writes (every vector
// once per phase), 12 per matrix entry (value and column) and 4 per row pointer.
// Used to report achieved bandwidth; the phases are latency- and FP64-issue-
// bound, so this is a floor on traffic, not the bound.
double solve_bytes(const LinearSystem &S, int it)
{
    // mixed precision: the multigrid levels' vectors and matrix values are float (and,
    // for refinement, the Krylov vectors too; its FP64 residual phases are left out)
    const bool mixed = S.precision == PRECISION_MIXED && S.mixed;
    const bool ir = mixed && !mixed_vcycle(S);
    const double n = S.n, D = ir ? 4 : 8, DL = mixed ? 4 : 8, E = mixed ? 8 : 12;
    auto csr = [E](const DevCsr &M) { return E * M.nnz + 4.0 * (M.n + 1); };
    double vc = 0;  // one V-cycle without its first sweep's vector reads
    const int L = (int)S.amg.size();
    // the coarsest level's dense inverse (8 n_c^2 bytes a cycle) is an implementation
    // choice, not algorithmic: solve_dense_bytes reports it apart
    if (L == 1) {
        vc = 2 * DL * S.amg[0]->n;
    } else if (L > 1 && S.sa_structured) {
        // the structured cycle: the prolongator is four weights a node (read by the
        // restriction and the prolongation), a coarse operator nine coefficients a node;
        // the level-0 operator is the matrix-free one (its diagonal a value a node)
        vc += 2 * DL * n;
        for (int l = 0; l < L - 1; ++l) {
            const double m = S.amg[l]->n, mc = S.amg[l + 1]->n, a9 = l > 0 ? 9 * DL * m : DL * m;
            if (l > 0) vc += 3 * DL * m + a9;          // residual
            vc += DL * m + 4 * DL * m + DL * mc;        // restriction
            vc += 7 * DL * m + DL * mc;                 // x_l = w D^-1 b_l + P x_l+1
            vc += 4 * DL * m + a9;                      // out_l = x_l + w D^-1 (b_l - A_l x_l)
        }
        vc += 2 * DL * S.amg[L - 1]->n;
    } else if (L > 1) {
        vc += 2 * DL * n;  // first sweep: omega D^-1 and r_0 (its input is counted by the caller)
        for (int l = 0; l < L - 1; ++l) {
            const SaLevel *V = S.amg[l], *C = S.amg[l + 1];
            if (l > 0) vc += 3 * DL * V->n + csr(V->A);
            vc += DL * V->n + csr(V->R) + DL * C->n;                           // restriction
            vc += 4 * DL * V->n + csr(V->P) + csr(V->AP) + DL * C->n;          // prolongation and sweep
        }
        const double nc = S.amg[L - 1]->n;
        vc += 2 * DL * nc;
    }
    double per_it, init;
    if (S.krylov == KRYLOV_CG) {
        init = 6 * D * n + (S.precond == PC_SMOOTHED_AGGREGATION ? vc + D * n : 0);
        per_it = 6 * D * n + 7 * D * n + (S.precond == PC_SMOOTHED_AGGREGATION ? vc : 2 * D * n);
    } else {
        init = 6 * D * n;
        if (S.precond == PC_SMOOTHED_AGGREGATION)
            per_it = 7 * D * n + 4 * D * n + 6 * D * n + 4 * D * n + 8 * D * n + 2 * vc;
        else
            per_it = 9 * D * n + 7 * D * n + 8 * D * n;
    }
    return init + it * per_it;
}

// Bytes of the coarsest level's dense inverse read by the solve's V-cycles (two per
// BiCGSTAB iteration, one per CG iteration and one before it), apart from solve_bytes
double solve_dense_bytes(const LinearSystem &S, int it)
{
    if (S.precond != PC_SMOOTHED_AGGREGATION || S.amg.empty()) return 0;
    const double nc = S.amg.back()->n;
    const double cycles = S.krylov == KRYLOV_CG ? it + 1.0 : 2.0 * it;
    return cycles * 8.0 * nc * nc;
}

// Decide whether the system can use the persistent solver, size its grid (one
// block per SM unless CUIBM_FUSED_BLOCKS_PER_SM asks for more and the kernel's
// registers allow it) and build its tables.  A mixed-precision system gets its
// mixed kernel and the float tables.
// the SA hierarchy was rebuilt (new levels, same vectors): the solver's arguments follow
void refresh_fused_hierarchy(Context &c, LinearSystem &S)
{
    if (!S.fused_fn) return;
    if (S.amg.empty() || (int)S.amg.size() > kMaxLevels || sa_coarsest_size(S) > kDenseMax)
        throw InputError("the rebuilt smoothed-aggregation hierarchy does not fit the persistent solver");
    upload_fargs(c, S);
}

void set_fused_grid(LinearSystem &S, int blocks)
{
    if (!S.fused_fn) return;
    S.fused_grid = blocks > 0 ? std::min(S.fused_grid_max, blocks) : S.fused_grid_default;
}

void setup_fused(Context &c, LinearSystem &S)
{
    S.fused_fn = nullptr;
    S.fused_grid = 0;
    if (S.precond == PC_SMOOTHED_AGGREGATION &&
        (S.amg.empty() || (int)S.amg.size() > kMaxLevels || sa_coarsest_size(S) > kDenseMax))
        return;
    const bool mixed = S.precision == PRECISION_MIXED;
    void *fn;
    if (S.which == 1)
        fn = mixed ? fused_pick_mixed_op1(S) : fused_pick_op1(S.precond, S.krylov, c.P.solverPack);
    else
        fn = mixed ? fused_pick_mixed_op2(S) : fused_pick_op2(S.precond, S.krylov, c.P.solverPack);
    int dev = 0, sms = 0, coop = 0, per_sm = 0;
    CUIBM_TRY(cudaGetDevice(&dev));
    CUIBM_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CUIBM_TRY(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    S.fused_threads = c.P.solverThreads > 0 ? c.P.solverThreads : kFT;
    CUIBM_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, S.fused_threads, 0));
    if (!coop || per_sm < 1) return;
    int want = 1;
    if (const char *e = getenv("CUIBM_FUSED_BLOCKS_PER_SM")) want = std::max(1, atoi(e));
    S.fused_grid_default = sms * std::min(per_sm, want);
    S.fused_grid_max = sms * per_sm;
    S.fused_fn = fn;
    set_fused_grid(S, c.P.solverBlocks);
    const int n = S.n;
    S.p2 = c.carve<double>(n);
    S.AMp2 = c.carve<double>(n);
    S.fpartials = c.carve<double>((size_t)2 * 4 * S.fused_grid_max);  // room for any grid
    S.fsync = c.carve<FusedSyncState>(1);
    S.diag = c.carve<double>(n);
    CUIBM_TRY(cudaMemsetAsync(S.fsync, 0, sizeof(FusedSyncState), c.stream));
    refresh_fused_diag(c, S);
    S.winv = nullptr;
    if (S.w) {
        std::vector<double> w(n), wi(n);
        CUIBM_TRY(cudaMemcpyAsync(w.data(), S.w, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        CUIBM_TRY(cudaStreamSynchronize(c.stream));
        for (int i = 0; i < n; ++i) wi[i] = 1.0 / w[i];
        S.winv = c.carve<double>(n);
        CUIBM_TRY(cudaMemcpyAsync(S.winv, wi.data(), n * sizeof(double), cudaMemcpyHostToDevice, c.stream));
        CUIBM_TRY(cudaStreamSynchronize(c.stream));
    }
    setup_deflation(c, S);
    if (mixed) setup_mixed(c, S);
    upload_fargs(c, S);
}

}  // namespace cuibm
