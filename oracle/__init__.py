"""CPU oracle of the fractional-step path (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
legs use this package, as the test oracle or the CPU baseline.  The product
(cuibm_gb300) never imports it.

liboracle.so (oracle/*.c) is a plain-C restatement of the reference's kernels
and of the CUSP Krylov solvers it calls; this module wraps it with numpy and
restates the host orchestration of a time step (NavierStokesSolver::stepTime,
NavierStokesSolver.cu:163-188).  The restatement is pinned bit-for-bit against
the reference's own kernel code by the golden fixtures in tests/golden.
"""
import ctypes
import json
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_KERNELS = os.path.join(HERE, "_ref", "libcuibm_refkernels.so")
REF_IO = os.path.join(HERE, "_ref", "libcuibm_refio.so")

_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build(ref=False):
    """Compile liboracle.so (and, with ref=True, the reference-derived _ref libraries)."""
    subprocess.run(["make", "-s", "-C", HERE] + (["all", "ref"] if ref else ["all"]), check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = ctypes.CDLL(LIB)
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


# ---------------------------------------------------------------------------
# case files (the JSON twins that cuibm_gb300.cases writes next to the YAML)
# ---------------------------------------------------------------------------
def load_case(folder):
    def rd(n):
        with open(os.path.join(folder, n + ".json")) as f:
            return json.load(f)
    return rd("simParams"), rd("flow"), rd("domain"), rd("bodies")


def axis_arrays(ax):
    """(centres, widths, faces) of one domain axis (io/parseDomainFile.cu)."""
    L = lib()
    ends = f64([s["end"] for s in ax["subDomains"]])
    ratios = f64([s["stretchRatio"] for s in ax["subDomains"]])
    L.or_axis_count.restype = ctypes.c_int
    L.or_axis_count.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp, _dp]
    n = L.or_axis_count(float(ax["start"]), float(ax["mid_h"]), len(ends), _d(ends), _d(ratios))
    c, w, face = np.zeros(n), np.zeros(n), np.zeros(n - 1)
    L.or_axis_fill.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp, _dp, _dp, _dp, _dp]
    L.or_axis_fill(float(ax["start"]), float(ax["mid_h"]), len(ends), _d(ends), _d(ratios), _d(c), _d(w), _d(face))
    return c, w, face


class Grid:
    def __init__(self, domain):
        xs = [a for a in domain if a["direction"] == "x"][0]
        ys = [a for a in domain if a["direction"] == "y"][0]
        self.x, self.dx, self.xu = axis_arrays(xs)
        self.y, self.dy, self.yv = axis_arrays(ys)
        self.xv, self.yu = self.x.copy(), self.y.copy()
        self.nx, self.ny = len(self.x), len(self.y)
        self.nU = (self.nx - 1) * self.ny
        self.nV = self.nx * (self.ny - 1)
        self.nUV = self.nU + self.nV
        self.nP = self.nx * self.ny

    @classmethod
    def from_arrays(cls, x, dx, xu, y, dy, yv):
        g = cls.__new__(cls)
        g.x, g.dx, g.xu, g.y, g.dy, g.yv = map(f64, (x, dx, xu, y, dy, yv))
        g.xv, g.yu = g.x.copy(), g.y.copy()
        g.nx, g.ny = len(g.x), len(g.y)
        g.nU = (g.nx - 1) * g.ny
        g.nV = g.nx * (g.ny - 1)
        g.nUV = g.nU + g.nV
        g.nP = g.nx * g.ny
        return g


def boundary_arrays(flow, nx, ny):
    """bc[XMINUS..YPLUS] (NavierStokesSolver.cu:104-128)."""
    val = {}
    for b in flow[0]["boundaryConditions"]:
        val[b["location"]] = (float(b["u"][1]), float(b["v"][1]))
    xm, xp = np.zeros(2 * ny - 1), np.zeros(2 * ny - 1)
    ym, yp = np.zeros(2 * nx - 1), np.zeros(2 * nx - 1)
    ym[:nx - 1], yp[:nx - 1] = val["yMinus"][0], val["yPlus"][0]
    ym[nx - 1:], yp[nx - 1:] = val["yMinus"][1], val["yPlus"][1]
    xm[:ny], xp[:ny] = val["xMinus"][0], val["xPlus"][0]
    xm[ny:], xp[ny:] = val["xMinus"][1], val["xPlus"][1]
    return xm, xp, ym, yp


# ---------------------------------------------------------------------------
# kernels
# ---------------------------------------------------------------------------
def _sig(name, *args, restype=None):
    fn = getattr(lib(), name)
    fn.argtypes = list(args)
    fn.restype = restype
    return fn


D, I_, INT = ctypes.c_double, ctypes.c_int, ctypes.c_int


def generate_N(u, g, bc):
    N = np.zeros(g.nUV)
    xm, xp, ym, yp = bc
    _sig("or_generateN", _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, INT, INT)(
        _d(N), _d(u), _d(g.dx), _d(g.dy), _d(ym), _d(yp), _d(xm), _d(xp), g.nx, g.ny)
    return N


def generate_L(u, g, bc, nu):
    L = np.zeros(g.nUV)
    xm, xp, ym, yp = bc
    _sig("or_generateL", _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, INT, INT, D)(
        _d(L), _d(u), _d(g.dx), _d(g.dy), _d(ym), _d(yp), _d(xm), _d(xp), g.nx, g.ny, nu)
    return L


def generate_bc1(u, g, bc, nu, dt):
    b1 = np.zeros(g.nUV)
    xm, xp, ym, yp = bc
    _sig("or_generateBC1", _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, D, D, INT, INT)(
        _d(u), _d(b1), _d(ym), _d(yp), _d(xm), _d(xp), _d(g.dx), _d(g.dy), nu, dt, g.nx, g.ny)
    return b1


def generate_rhs(L, Nold, N, u, bc1, dt):
    r = np.zeros(len(u))
    _sig("or_generateRHS", _dp, _dp, _dp, _dp, _dp, _dp, D, INT)(
        _d(r), _d(L), _d(Nold), _d(N), _d(u), _d(bc1), dt, len(u))
    return r


def lhs1_coo(g, dt, nu):
    nnz = (g.nx - 1) * g.ny * 5 - 2 * g.ny - 2 * (g.nx - 1) + (g.ny - 1) * g.nx * 5 - 2 * (g.ny - 1) - 2 * g.nx
    row, col, val = np.zeros(nnz, np.int32), np.zeros(nnz, np.int32), np.zeros(nnz)
    _sig("or_lhs1_coo", _ip, _ip, _dp, _dp, _dp, D, D, INT, INT)(
        _i(row), _i(col), _d(val), _d(g.dx), _d(g.dy), dt, nu, g.nx, g.ny)
    return row, col, val


def lhs2_coo(g, dt, centre_pin=True):
    nnz = 5 * g.nx * g.ny - 2 * g.ny - 2 * g.nx
    row, col, val = np.zeros(nnz, np.int32), np.zeros(nnz, np.int32), np.zeros(nnz)
    _sig("or_lhs2_coo", INT, _ip, _ip, _dp, _dp, _dp, INT, INT, D)(
        int(centre_pin), _i(row), _i(col), _d(val), _d(g.dx), _d(g.dy), g.nx, g.ny, dt)
    return row, col, val


def generate_rhs2(uhat, g, bc):
    r = np.zeros(g.nP)
    xm, xp, ym, yp = bc
    _sig("or_generateRHS2", _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, INT, INT)(
        _d(r), _d(uhat), _d(ym), _d(yp), _d(xm), _d(xp), _d(g.dx), _d(g.dy), g.nx, g.ny)
    return r


def project(u, uhat, p, g, dt):
    u = u.copy()
    uold = np.zeros(g.nUV)
    _sig("or_project", _dp, _dp, _dp, _dp, _dp, _dp, D, INT, INT)(
        _d(u), _d(uhat), _d(uold), _d(p), _d(g.dx), _d(g.dy), dt, g.nx, g.ny)
    return u, uold


def initial_velocity(g, uI, vI, uP=0.0, vP=0.0):
    u = np.zeros(g.nUV)
    _sig("or_initialiseVelocity", _dp, _dp, _dp, _dp, _dp, D, D, D, D, D, D, D, D, INT, INT)(
        _d(u), _d(g.xu), _d(g.yu), _d(g.xv), _d(g.yv), uI, vI, uP, vP, g.x[-1], g.x[0], g.y[-1], g.y[0], g.nx, g.ny)
    return u


def cfl(u, g, dt):
    c = np.zeros(g.nP)
    _sig("or_calculateCFL", _dp, _dp, _dp, _dp, INT, INT, D)(_d(c), _d(u), _d(g.dx), _d(g.dy), g.nx, g.ny, dt)
    return c


# ---------------------------------------------------------------------------
# sparse solves
# ---------------------------------------------------------------------------
class Csr:
    def __init__(self, n, row, col, val):
        self.n = n
        self.ptr = np.zeros(n + 1, np.int32)
        self.col = np.zeros(len(row), np.int32)
        self.val = np.zeros(len(row))
        _sig("or_coo_to_csr", INT, INT, _ip, _ip, _dp, _ip, _ip, _dp)(
            n, len(row), _i(np.ascontiguousarray(row, np.int32)), _i(np.ascontiguousarray(col, np.int32)),
            _d(f64(val)), _i(self.ptr), _i(self.col), _d(self.val))

    def scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.val, self.col, self.ptr), shape=(self.n, self.n))

    def matvec(self, x):
        y = np.zeros(self.n)
        _sig("or_csr_spmv", INT, _ip, _ip, _dp, _dp, _dp)(self.n, _i(self.ptr), _i(self.col), _d(self.val),
                                                          _d(f64(x)), _d(y))
        return y


def bicgstab(A, b, x, rtol, maxit, precond=1):
    """Right-preconditioned BiCGSTAB under cusp::monitor semantics; returns (x, iters, converged)."""
    x = f64(x).copy()
    res = ctypes.c_double()
    it = _sig("or_bicgstab", INT, _ip, _ip, _dp, _dp, _dp, D, INT, INT, ctypes.c_void_p, _dp, restype=INT)(
        A.n, _i(A.ptr), _i(A.col), _d(A.val), _d(f64(b)), _d(x), rtol, maxit, precond, None, ctypes.byref(res))
    return x, abs(it) - (1 if it < 0 else 0), it >= 0


def direct_solve(A, b):
    import scipy.sparse.linalg as spla
    return spla.spsolve(A.scipy().tocsc(), f64(b))


# ---------------------------------------------------------------------------
# step orchestration of the plain solver (NavierStokesSolver::stepTime)
# ---------------------------------------------------------------------------
class PlainSolver:
    """NAVIER_STOKES_SOLVER on the CPU.  solve='direct' solves both systems
    exactly (sparse LU) so that fields can be compared with any converged
    solver; solve='krylov' uses the case's BiCGSTAB tolerances."""

    def __init__(self, folder=None, grid=None, flow=None, nu=None, dt=None, sim=None, solve="direct"):
        if folder is not None:
            sim_, flow_, dom, _ = load_case(folder)
            sim = sim or sim_[0]
            flow = flow or flow_
            grid = grid or Grid(dom)
            nu = nu if nu is not None else float(flow_[0]["nu"])
            dt = dt if dt is not None else float(sim_[0]["dt"])
        self.g, self.nu, self.dt, self.sim = grid, nu, dt, sim
        self.bc = boundary_arrays(flow, grid.nx, grid.ny)
        f0 = flow[0]
        ip = f0.get("initialPerturbation", [0.0, 0.0])
        self.u = initial_velocity(grid, float(f0["initialVelocity"][0]), float(f0["initialVelocity"][1]),
                                  float(ip[0]), float(ip[1]))
        self.uhat = self.u.copy()
        self.uold = np.zeros(grid.nUV)
        self.N = np.zeros(grid.nUV)
        self.Nold = np.zeros(grid.nUV)
        self.p = np.zeros(grid.nP)
        self.A1 = Csr(grid.nUV, *lhs1_coo(grid, dt, nu))
        self.A2 = Csr(grid.nP, *lhs2_coo(grid, dt, centre_pin=True))
        self.solve = solve
        self.timeStep = 0
        self.iters = (0, 0)
        if solve == "direct":
            import scipy.sparse.linalg as spla
            self._lu1 = spla.splu(self.A1.scipy().tocsc())
            self._lu2 = spla.splu(self.A2.scipy().tocsc())

    def _tol(self, system):
        for s in self.sim.get("linearSolvers", []):
            if s["system"] == system:
                return float(s.get("tolerance", 1e-5)), int(s.get("maxIterations", 10000))
        return 1e-5, 10000

    def step(self):
        g, bc = self.g, self.bc
        self.Nold = self.N
        self.N = generate_N(self.u, g, bc)
        L = generate_L(self.u, g, bc, self.nu)
        b1 = generate_bc1(self.u, g, bc, self.nu, self.dt)
        rhs1 = generate_rhs(L, self.Nold, self.N, self.u, b1, self.dt)
        if self.solve == "direct":
            self.uhat = self._lu1.solve(rhs1)
        else:
            tol, mx = self._tol("velocity")
            self.uhat, it1, ok = bicgstab(self.A1, rhs1, self.uhat, tol, mx, 1)
        rhs2 = generate_rhs2(self.uhat, g, bc)
        if self.solve == "direct":
            self.p = self._lu2.solve(rhs2)
        else:
            tol, mx = self._tol("Poisson")
            self.p, it2, ok = bicgstab(self.A2, rhs2, self.p, tol, mx, 1)
        self.u, self.uold = project(self.u, self.uhat, self.p, g, self.dt)
        self.timeStep += 1


def circle_points(cx, cy, R, n):
    X, Y = np.zeros(n), np.zeros(n)
    _sig("or_circle_points", D, D, D, INT, _dp, _dp)(cx, cy, R, n, _d(X), _d(Y))
    return X, Y


# ---------------------------------------------------------------------------
# immersed boundary (external method)
# ---------------------------------------------------------------------------
class _Tags(ctypes.Structure):
    _fields_ = [(n, _ip) for n in ("ghostTagsUV", "ghostTagsP", "hybridTagsUV", "hybridTagsP", "hybridTagsUV2")] + \
               [(n, _dp) for n in ("dist_node", "dist_between", "dist_u_body", "dist_v_body", "uv",
                                   "bi_x", "bi_y", "ip_x", "ip_y", "bip_x", "bip_y", "ipp_x", "ipp_y")]


class _Interp(ctypes.Structure):
    _fields_ = [(n, _ip) for n in ("index1", "index2", "index3", "index4")] + \
               [(n, _dp) for n in ("q1coef", "q2coef", "q3coef", "q4coef", "value", "dpdn", "q1", "q2", "q3", "q4")]


class Tags:
    """Tag arrays and body intercepts of luo_base (tagPoints)."""

    def __init__(self, g):
        self.ghostTagsUV = -np.ones(g.nUV, np.int32)
        self.hybridTagsUV = -np.ones(g.nUV, np.int32)
        self.hybridTagsUV2 = -np.ones(g.nUV, np.int32)
        self.ghostTagsP = -np.ones(g.nP, np.int32)
        self.hybridTagsP = -np.ones(g.nP, np.int32)
        for k in ("dist_node", "dist_between", "uv", "bi_x", "bi_y", "ip_x", "ip_y"):
            setattr(self, k, np.zeros(g.nUV))
        for k in ("dist_u_body", "dist_v_body", "bip_x", "bip_y", "ipp_x", "ipp_y"):
            setattr(self, k, np.zeros(g.nP))

    def c(self):
        return _Tags(**{f: (_i(getattr(self, f)) if "Tags" in f else _d(getattr(self, f))) for f, _ in _Tags._fields_})


class Stencils:
    """Per-node interpolation stencil (4 indices, 4 weights) and interpolated value."""

    def __init__(self, n):
        self.index = np.zeros((4, n), np.int32)
        self.coef = np.zeros((4, n))
        self.value = np.zeros(n)
        self.dpdn = np.zeros(n)
        self.q = np.zeros((4, n))

    def c(self):
        return _Interp(index1=_i(self.index[0]), index2=_i(self.index[1]), index3=_i(self.index[2]),
                       index4=_i(self.index[3]), q1coef=_d(self.coef[0]), q2coef=_d(self.coef[1]),
                       q3coef=_d(self.coef[2]), q4coef=_d(self.coef[3]), value=_d(self.value), dpdn=_d(self.dpdn),
                       q1=_d(self.q[0]), q2=_d(self.q[1]), q3=_d(self.q[2]), q4=_d(self.q[3]))


def set_intercept_form(form):
    """Body intercepts of the tagging: 0 the reference's trigonometric form (acos, sin,
    tan), 1 its closed form (the default, what the GPU computes).  Returns the previous
    form."""
    prev = _sig("or_get_intercept_form", restype=INT)()
    _sig("or_set_intercept_form", INT)(int(form))
    return prev


class intercept_form:
    """Context manager: tag with the given intercept form inside the block."""

    def __init__(self, form):
        self.form = form

    def __enter__(self):
        self.prev = set_intercept_form(self.form)
        return self

    def __exit__(self, *exc):
        set_intercept_form(self.prev)
        return False


# arrays luo_base::tagPoints does not refill (luo_base/tagPoints.cu:26-40): a re-tagging
# keeps their values where the kernels do not write
_TAG_CARRIED = ("dist_u_body", "dist_v_body", "uv", "bip_x", "bip_y", "ipp_x", "ipp_y")


def tag_points(g, bx, by, uB, vB, bb, midX, midY, prev=None):
    T = Tags(g)
    if prev is not None:
        for k in _TAG_CARRIED:
            setattr(T, k, getattr(prev, k).copy())
    ct = T.c()
    i0, j0, ncx, ncy = (int(v) for v in bb)
    _sig("or_tagPoints", ctypes.POINTER(_Tags), _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, INT, INT, INT, INT, INT, INT,
         INT, D, D)(ctypes.byref(ct), _d(f64(bx)), _d(f64(by)), _d(f64(uB)), _d(f64(vB)), _d(g.xu), _d(g.yu), _d(g.xv),
                    _d(g.yv), i0, j0, ncx, ncy, g.nx, g.ny, len(bx), midX, midY)
    return T


# ---- modified Fadlun (oracle/fadlun.c) ------------------------------------------------
def fadlun_lhs1_coo(g, dt, nu, T):
    """fadlunModified::generateLHS1 before the reference's sort (unsorted COO)."""
    row, col, val = lhs1_coo(g, dt, nu)
    _sig("or_fadlun_lhs1_coo", _ip, _ip, _dp, INT, _ip, _ip, _ip, _dp, _dp, _dp, _dp, D, D, INT, INT)(
        _i(row), _i(col), _d(val), len(row), _i(T.hybridTagsUV), _i(T.hybridTagsUV2), _i(T.ghostTagsUV),
        _d(T.dist_node), _d(T.dist_between), _d(g.dx), _d(g.dy), dt, nu, g.nx, g.ny)
    return row, col, val


def fadlun_lhs2_coo(g, dt, T):
    """fadlunModified::generateLHS2 before the reference's sort (unsorted COO)."""
    row, col, val = lhs2_coo(g, dt, centre_pin=False)
    _sig("or_fadlun_lhs2_coo", _ip, _ip, _dp, _dp, _dp, _ip, _ip, _dp, _dp, INT, INT, D)(
        _i(row), _i(col), _d(val), _d(T.dist_u_body), _d(T.dist_v_body), _i(T.ghostTagsP), _i(T.hybridTagsP),
        _d(g.dx), _d(g.dy), g.nx, g.ny, dt)
    return row, col, val


def fadlun_update_rhs1(rhs, T, g):
    r = f64(rhs).copy()
    _sig("or_fadlun_update_rhs1", _ip, _ip, _dp, _dp, _dp, _dp, INT, INT)(
        _i(T.hybridTagsUV), _i(T.ghostTagsUV), _d(r), _d(T.dist_node), _d(T.dist_between), _d(T.uv), g.nx, g.ny)
    return r


def fadlun_rhs2(uhat, T, g, bc):
    r = np.zeros(g.nP)
    xm, xp, ym, yp = bc
    _sig("or_fadlun_rhs2", _dp, _dp, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, INT, INT)(
        _d(r), _d(f64(uhat)), _i(T.ghostTagsP), _i(T.hybridTagsP), _d(T.dist_u_body), _d(T.dist_v_body), _d(ym),
        _d(yp), _d(xm), _d(xp), _d(g.dx), _d(g.dy), g.nx, g.ny)
    return r


def fadlun_project(uhat, p, T, g, dt):
    u = np.zeros(g.nUV)
    _sig("or_fadlun_project", _dp, _dp, _dp, _ip, _dp, _dp, D, INT, INT)(
        _d(u), _d(f64(uhat)), _d(f64(p)), _i(T.ghostTagsP), _d(g.dx), _d(g.dy), dt, g.nx, g.ny)
    return u


# ---- embedded method (oracle/embedded.c) ----------------------------------------------
def _plain_nnz(g, system):
    nx, ny = g.nx, g.ny
    if system == 1:
        return (nx - 1) * ny * 5 - 2 * ny - 2 * (nx - 1) + nx * (ny - 1) * 5 - 2 * nx - 2 * (ny - 1)
    return nx * ny * 5 - 2 * nx - 2 * ny


def iter_alpha(kind, T, g, bb, alpha=None):
    """alpha_u (kind 0), alpha_v (1), alpha_p (2) of luo_iter/kernels/weight.cu into alpha."""
    n = g.nP if kind == 2 else g.nUV
    alpha = np.zeros(n) if alpha is None else alpha
    i0, j0, ncx, _ = (int(v) for v in bb)
    if kind == 2:
        gt, ht, xc, yc, bix, biy = T.ghostTagsP, T.hybridTagsP, g.xv, g.yu, T.bip_x, T.bip_y
    else:
        gt, ht, bix, biy = T.ghostTagsUV, T.hybridTagsUV, T.bi_x, T.bi_y
        xc, yc = (g.xu, g.yu) if kind == 0 else (g.xv, g.yv)
    _sig("or_iter_alpha", INT, _dp, _ip, _ip, _dp, _dp, _dp, _dp, INT, INT, INT, INT, INT)(
        kind, _d(alpha), _i(gt), _i(ht), _d(yc), _d(xc), _d(bix), _d(biy), i0, j0, ncx, g.nx, g.ny)
    return alpha


def iter_lhs1(g, dt, nu, T, S, alpha, uB0, vB0, bb):
    """The embedded LHS1 (luo_iter::intermediate_velocity_size_lhs/_calculate_lhs) on zeroed
    arrays: unsorted COO, ns_rhs and interp_rhs.  S: the velocity stencils of the step."""
    nh = int((T.hybridTagsUV > 0).sum())
    nnz = _plain_nnz(g, 1) + nh
    row, col, val = np.zeros(nnz, np.int32), np.zeros(nnz, np.int32), np.zeros(nnz)
    ns, interp, count = np.zeros(g.nUV), np.zeros(g.nUV), np.zeros(g.nUV, np.int32)
    i0, j0, ncx, ncy = (int(v) for v in bb)
    ix = [np.ascontiguousarray(S.index[k]) for k in range(4)]
    cf = [np.ascontiguousarray(S.coef[k]) for k in range(4)]
    qs = [np.ascontiguousarray(S.q[k]) for k in range(4)]
    got = _sig("or_iter_lhs1", _ip, _ip, _dp, INT, _dp, _dp, D, D, INT, INT, _ip, _ip, _dp, _dp, _ip, _ip, _ip, _ip,
               _ip, _dp, D, D, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, INT, INT, INT, INT, restype=INT)(
        _i(row), _i(col), _d(val), nnz, _d(g.dx), _d(g.dy), dt, nu, g.nx, g.ny, _i(T.hybridTagsUV),
        _i(T.ghostTagsUV), _d(ns), _d(interp), _i(count), *(_i(a) for a in ix), _d(f64(alpha)), uB0, vB0,
        *(_d(a) for a in cf), *(_d(a) for a in qs), i0, j0, ncx, ncy)
    if got != nnz:
        raise RuntimeError("or_iter_lhs1: %d entries, expected %d" % (got, nnz))
    return row, col, val, ns, interp


def iter_update_rhs1(rhs1, ns, interp, g):
    r = f64(rhs1).copy()
    _sig("or_iter_update_rhs1", _dp, _dp, _dp, INT, INT)(_d(r), _d(f64(ns)), _d(f64(interp)), g.nx, g.ny)
    return r


def iter_lhs2(g, dt, T, S, alpha, bb):
    """The embedded LHS2 (luo_iter::poisson_size_lhs/_calculate_lhs) on zeroed arrays:
    unsorted COO, ns_rhs and interp_rhs.  S: the pressure stencils of the step (dpdn too)."""
    nh = int((T.hybridTagsP > 0).sum())
    nnz = _plain_nnz(g, 2) + nh
    row, col, val = np.zeros(nnz, np.int32), np.zeros(nnz, np.int32), np.zeros(nnz)
    ns, interp, count = np.zeros(g.nP), np.zeros(g.nP), np.zeros(g.nP, np.int32)
    i0, j0, ncx, ncy = (int(v) for v in bb)
    ix = [np.ascontiguousarray(S.index[k]) for k in range(4)]
    cf = [np.ascontiguousarray(S.coef[k]) for k in range(4)]
    qs = [np.ascontiguousarray(S.q[k]) for k in range(4)]
    got = _sig("or_iter_lhs2", _ip, _ip, _dp, INT, _dp, _dp, INT, INT, D, _ip, _dp, _dp, _ip, _ip, _dp, _dp, _ip, _ip,
               _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, INT, INT, INT, INT, restype=INT)(
        _i(row), _i(col), _d(val), nnz, _d(g.dx), _d(g.dy), g.nx, g.ny, dt, _i(count), _d(ns), _d(interp),
        _i(T.hybridTagsP), _i(T.ghostTagsP), _d(f64(alpha)), _d(S.dpdn), *(_i(a) for a in ix),
        *(_d(a) for a in cf), *(_d(a) for a in qs), i0, j0, ncx, ncy)
    if got != nnz:
        raise RuntimeError("or_iter_lhs2: %d entries, expected %d" % (got, nnz))
    return row, col, val, ns, interp


def iter_update_rhs2(rhs2, ns, interp, g):
    r = f64(rhs2).copy()
    _sig("or_iter_update_rhs2", _dp, _dp, _dp, INT, INT)(_d(r), _d(f64(ns)), _d(f64(interp)), g.nx, g.ny)
    return r


def ghost_velocity(direc, u, T, uB0, g, bb, set_=True, S=None):
    u = f64(u).copy()
    S = Stencils(g.nUV) if S is None else S
    cs = S.c()
    xc, yc = (g.xu, g.yu) if direc == 0 else (g.xv, g.yv)
    i0, j0, ncx, ncy = (int(v) for v in bb)
    _sig("or_ghost_velocity", INT, _dp, INT, _ip, D, _dp, _dp, _dp, _dp, _dp, _dp, INT, INT, INT, INT, INT, INT,
         ctypes.POINTER(_Interp))(direc, _d(u), int(set_), _i(T.ghostTagsUV), uB0, _d(yc), _d(xc), _d(T.bi_x),
                                  _d(T.bi_y), _d(T.ip_x), _d(T.ip_y), i0, j0, ncx, ncy, g.nx, g.ny, ctypes.byref(cs))
    return u, S


def hybrid_velocity(direc, u, ustar, T, uB0, g, bb, S=None):
    ustar = f64(ustar).copy()
    S = Stencils(g.nUV) if S is None else S
    cs = S.c()
    xc, yc = (g.xu, g.yu) if direc == 0 else (g.xv, g.yv)
    i0, j0, ncx, ncy = (int(v) for v in bb)
    _sig("or_hybrid_velocity", INT, _dp, _dp, _ip, D, _dp, _dp, _dp, _dp, _dp, _dp, INT, INT, INT, INT, INT, INT,
         ctypes.POINTER(_Interp))(direc, _d(f64(u)), _d(ustar), _i(T.hybridTagsUV), uB0, _d(yc), _d(xc),
                                  _d(T.bi_x), _d(T.bi_y), _d(T.ip_x), _d(T.ip_y), i0, j0, ncx, ncy, g.nx, g.ny,
                                  ctypes.byref(cs))
    return ustar, S


def hybrid_pressure(p, T, dudt, dvdt, g, bb, S=None):
    pstar = np.zeros(g.nP)
    S = Stencils(g.nP) if S is None else S
    cs = S.c()
    i0, j0, ncx, ncy = (int(v) for v in bb)
    _sig("or_hybrid_pressure", _dp, _dp, _ip, D, D, _dp, _dp, _dp, _dp, _dp, _dp, INT, INT, INT, INT, INT, INT,
         ctypes.POINTER(_Interp))(_d(f64(p)), _d(pstar), _i(T.hybridTagsP), dudt, dvdt, _d(g.yu), _d(g.xv),
                                  _d(T.bip_x), _d(T.bip_y), _d(T.ipp_x), _d(T.ipp_y), i0, j0, ncx, ncy, g.nx, g.ny,
                                  ctypes.byref(cs))
    return pstar, S


def ghost_pressure(p, T, dudt, dvdt, g, bb, set_=True, S=None):
    p = f64(p).copy()
    S = Stencils(g.nP) if S is None else S
    cs = S.c()
    i0, j0, ncx, ncy = (int(v) for v in bb)
    _sig("or_ghost_pressure", _dp, INT, _ip, D, D, _dp, _dp, _dp, _dp, _dp, _dp, INT, INT, INT, INT, INT, INT,
         ctypes.POINTER(_Interp))(_d(p), int(set_), _i(T.ghostTagsP), dudt, dvdt, _d(g.yu), _d(g.xv), _d(T.bip_x),
                                  _d(T.bip_y), _d(T.ipp_x), _d(T.ipp_y), i0, j0, ncx, ncy, g.nx, g.ny,
                                  ctypes.byref(cs))
    return p, S


def weight(direc, f, fstar, T, g, bb):
    f = f64(f).copy()
    i0, j0, ncx, ncy = (int(v) for v in bb)
    if direc == 2:
        gt, ht, xc, yc, bix, biy = T.ghostTagsP, T.hybridTagsP, g.xv, g.yu, T.bip_x, T.bip_y
    else:
        gt, ht, bix, biy = T.ghostTagsUV, T.hybridTagsUV, T.bi_x, T.bi_y
        xc, yc = (g.xu, g.yu) if direc == 0 else (g.xv, g.yv)
    _sig("or_weight", INT, _dp, _dp, _ip, _ip, _dp, _dp, _dp, _dp, INT, INT, INT, INT, INT, INT)(
        direc, _d(f), _d(f64(fstar)), _i(gt), _i(ht), _d(yc), _d(xc), _d(bix), _d(biy), i0, j0, ncx, ncy, g.nx, g.ny)
    return f


def set_inside(u, T, uB0, vB0, g):
    u = f64(u).copy()
    _sig("or_setInsideVelocity", _ip, _dp, D, D, INT, INT)(_i(T.ghostTagsUV), _d(u), uB0, vB0, g.nx, g.ny)
    return u


def robin(u, xp, g, dt, Uinf=1.0, Vinf=1.0):
    xp = f64(xp).copy()
    _sig("or_updateRobinBoundary", _dp, _dp, _dp, D, D, D, INT, INT)(_d(f64(u)), _d(xp), _d(g.dx), dt, Uinf, Vinf,
                                                                      g.nx, g.ny)
    return xp


def force(u, uold, p, T, nu, g, dt, bb):
    fx, fy = ctypes.c_double(), ctypes.c_double()
    i0, j0, ncx, ncy = (int(v) for v in bb)
    _sig("or_calculateForce", _dp, _dp, _dp, _ip, D, _dp, _dp, D, INT, INT, INT, INT, INT, INT, _dp, _dp)(
        _d(f64(u)), _d(f64(uold)), _d(f64(p)), _i(T.ghostTagsUV), nu, _d(g.dx), _d(g.dy), dt, g.nx, g.ny, i0, j0, ncx,
        ncy, ctypes.byref(fx), ctypes.byref(fy))
    return fx.value, fy.value


def surface_force(mode, bx, by, uB0, vB0, u, bip, bip_x, bip_y, ghostTagsP, xu, yu, xv, yv, bb, nx, ny, midX,
                  midY, nu, mid_h):
    """The surface-integral force (or_surfaceForce): (terms [pressure, du/dn, dv/dn per
    point], Fx, Fy); mode 1 as luo_base::luoForce is written, 2 corrected."""
    n = len(bx)
    terms = np.zeros(3 * n)
    fx, fy = ctypes.c_double(), ctypes.c_double()
    i0, j0 = int(bb[0]), int(bb[1])
    _sig("or_surfaceForce", INT, _dp, _dp, INT, D, D, _dp, _dp, _dp, _dp, _ip, _dp, _dp, _dp, _dp, INT, INT, INT,
         INT, D, D, D, D, _dp, _dp, _dp)(
        int(mode), _d(f64(bx)), _d(f64(by)), n, float(uB0), float(vB0), _d(f64(u)), _d(f64(bip)), _d(f64(bip_x)),
        _d(f64(bip_y)), _i(np.ascontiguousarray(ghostTagsP, np.int32)), _d(f64(xu)), _d(f64(yu)), _d(f64(xv)),
        _d(f64(yv)), i0, j0, int(nx), int(ny), float(midX), float(midY), float(nu), float(mid_h), _d(terms),
        ctypes.byref(fx), ctypes.byref(fy))
    return terms, fx.value, fy.value


def bounding_box(x, y, g, scale):
    a = [ctypes.c_int() for _ in range(4)]
    _sig("or_bounding_box", INT, _dp, _dp, _dp, _dp, D, _ip, _ip, _ip, _ip)(
        len(x), _d(f64(x)), _d(f64(y)), _d(g.x), _d(g.y), scale, *(ctypes.byref(v) for v in a))
    return tuple(v.value for v in a)


class Amg:
    """Smoothed-aggregation hierarchy of the oracle (oracle/amg.c)."""

    def __init__(self, A, coarse=256):
        self.A = A
        fn = _sig("or_sa_build", INT, _ip, _ip, _dp, D, INT, restype=ctypes.c_void_p)
        self.h = fn(A.n, _i(A.ptr), _i(A.col), _d(A.val), 0.0, coarse)

    def __del__(self):
        try:
            _sig("or_sa_free", ctypes.c_void_p)(self.h)
        except Exception:
            pass


def bicgstab_pc(A, b, x, rtol, maxit, pc, amg=None):
    """BiCGSTAB with preconditioner kind pc (0 none, 1 diagonal, 2 smoothed aggregation)."""
    x = f64(x).copy()
    res = ctypes.c_double()
    it = _sig("or_bicgstab", INT, _ip, _ip, _dp, _dp, _dp, D, INT, INT, ctypes.c_void_p, _dp, restype=INT)(
        A.n, _i(A.ptr), _i(A.col), _d(A.val), _d(f64(b)), _d(x), rtol, maxit, pc, amg.h if amg else None,
        ctypes.byref(res))
    return x, (it if it >= 0 else -it - 1), it >= 0


_PC = {"NONE": 0, "DIAGONAL": 1, "SMOOTHED_AGGREGATION": 2}
COUPLING_MAX_PASSES = 50  # passes of a strongly coupled step before it is reported unconverged


class LuoSolver:
    """The external (Luo) ghost-node method on the CPU: luo_base::stepTime
    (luo_base.cu:208-233) with luoIBM's phases - generateRHS1
    (luoIBM/intermediateVelocity.cu:128-167), weightUhat, generateRHS2 and
    weightPressure (luoIBM/intermediatePressure.cu:280-342), the projection of
    luo_base/projectVelocity.cu:237-279 and the body update (force, motion) of
    luo_base.cu:255-264.  solve='direct' solves both systems exactly;
    solve='krylov' uses BiCGSTAB with the case's preconditioners and tolerances."""

    def __init__(self, folder, solve="direct", vel_offset=None):
        sim, flow, dom, bodies = load_case(folder)
        self.sim = sim[0]
        g = self.g = Grid(dom)
        self.nu = float(flow[0]["nu"])
        self.dt = float(self.sim["dt"])
        self.bc = [a.copy() for a in boundary_arrays(flow, g.nx, g.ny)]
        f0 = flow[0]
        ip = f0.get("initialPerturbation", [0.0, 0.0])
        self.u = initial_velocity(g, float(f0["initialVelocity"][0]), float(f0["initialVelocity"][1]),
                                  float(ip[0]), float(ip[1]))
        self.uhat = self.u.copy()
        self.uold = np.zeros(g.nUV)
        self.N = np.zeros(g.nUV)
        self.p = np.zeros(g.nP)
        b0 = bodies[0]
        o = b0["circleOptions"]
        n = int(o[3])
        if len(o) > 5 and o[4] in (True, "true"):
            n = int(2.0 * float(o[2]) * np.pi / float(o[5]))
            n += n % 2
        X, Y = circle_points(float(o[0]), float(o[1]), float(o[2]), n)
        mx = 0.0
        for v in X:
            mx += v
        my = 0.0
        for v in Y:
            my += v
        mx /= n
        my /= n
        self.bdx = np.array([v - mx for v in X])
        self.scale = float(self.sim.get("scaleCV", 2.0))
        self.bb = bounding_box(X, Y, g, self.scale)
        self.coef = {k: float(b0.get(k, 0.0)) for k in ("xCoefficient", "uCoefficient", "xPhase", "uPhase",
                                                         "xfrequency")}
        self.timeStep = 0
        xnew, unew = self.motion(0)
        self.bx = np.array([xnew + v for v in self.bdx])
        self.by = Y.copy()
        # per-point offsets of the body velocity (u, v), added wherever the prescribed motion
        # sets it (a perturbation for derivative checks; zero in the reference's model)
        ou, ov = (np.zeros(n), np.zeros(n)) if vel_offset is None else (f64(vel_offset[0]), f64(vel_offset[1]))
        self.vel_offset = (ou.copy(), ov.copy())
        self.uB = np.full(n, unew) + ou
        self.vB = np.zeros(n) + ov
        self.uBk = np.full(n, self.coef["uCoefficient"] * np.cos(
            2 * np.pi * self.coef["xfrequency"] * (0 - self.dt) + self.coef["uPhase"]))
        self.midX, self.midY = xnew, my
        self.bdy = np.array([v - my for v in Y])
        self.viv = int(self.sim.get("VIV", 0))
        self.ured = float(int(self.sim.get("Ured", 3)))
        self.vbody = 0.0
        self.vBk = self.vB.copy()
        self.Nold = np.zeros(g.nUV)
        self.midY0, self.vbody0 = self.midY, self.vbody
        self.sctol, self.sub_iterations = 1e-4, 0
        self.T = tag_points(g, self.bx, self.by, self.uB, self.vB, self.bb, self.midX, self.midY)
        self.u = set_inside(self.u, self.T, self.uB[0], self.vB[0], g)
        self.A1 = Csr(g.nUV, *lhs1_coo(g, self.dt, self.nu))
        self.A2 = Csr(g.nP, *lhs2_coo(g, self.dt, centre_pin=False))
        self.solve = solve
        self.fx = self.fy = 0.0
        if solve == "none":  # a subclass assembles its own operators
            pass
        elif solve == "direct":
            import scipy.sparse.linalg as spla
            self._lu1 = spla.splu(self.A1.scipy().tocsc())
            self._lu2 = spla.splu(self.A2.scipy().tocsc())
        else:
            ls = {s["system"]: s for s in self.sim.get("linearSolvers", [])}
            self.cfg = {k: (float(ls[k].get("tolerance", 1e-5)), int(ls[k].get("maxIterations", 10000)),
                            _PC.get(ls[k].get("preconditioner", "DIAGONAL"), 1)) for k in ("velocity", "Poisson")}
            self.amg1 = Amg(self.A1) if self.cfg["velocity"][2] == 2 else None
            self.amg2 = Amg(self.A2) if self.cfg["Poisson"][2] == 2 else None
        self.iters = (0, 0)

    @property
    def moving(self):
        return self.coef["xCoefficient"] != 0 or self.coef["uCoefficient"] != 0 or self.viv in (1, 2)

    def _move_body(self):
        """luo_base::moveBody after the force (luo_base.cu:154-178): the prescribed motion
        at t = dt * timeStep (set_movement, luo_base/move.cu:11-36) or, with VIV: 1, the
        loosely coupled spring-mounted cylinder (viv_movement_LC, luo_base/move.cu:38-62),
        or with VIV: 2 the strongly coupled one (viv_movement_SC, luo_base/move.cu:64-94):
        the same update with the new centre relaxed (0.9) against the previous
        sub-iteration's, and SCtol = (previous - new) / previous."""
        if self.viv in (1, 2):
            Cy, Mred, Ured, dt = self.fy * 2.0, 2.0, self.ured, self.dt
            vold, yold = self.vbody0, self.midY0  # the _pre_step copies centerVelocityV0, midY0
            a = dt * np.pi * np.pi * 4 / (Ured * Ured)
            b = dt * dt * 2 * np.pi * np.pi / (Ured * Ured)
            vnew = (vold - a * (yold + dt / 2 * vold) + dt * Cy / 2 / Mred) / (1 + b)
            if self.viv == 1:
                ynew = yold + dt / 2 * (vnew + vold)
            else:
                relax, yprev = 0.9, self.midY
                ynew = relax * (yold + dt / 2 * (vnew + vold)) + (1 - relax) * yprev
                with np.errstate(divide="ignore", invalid="ignore"):
                    self.sctol = float(np.float64(yprev - ynew) / np.float64(yprev))
            self.vbody, self.midY = vnew, ynew
            self.vB = np.full(len(self.by), vnew)
            self.by = np.array([ynew + v for v in self.bdy])
            return
        xnew, unew = self.motion(self.timeStep)
        self.bx = np.array([xnew + v for v in self.bdx])
        self.uB = np.full(len(self.bx), unew) + self.vel_offset[0]
        self.midX = xnew

    def _update_solver(self):
        """luo_base::updateSolver (luo_base.cu:137-146): the box of the moved body, its tags."""
        if not self.moving:
            return
        self.bb = bounding_box(self.bx, self.by, self.g, self.scale)
        self.T = tag_points(self.g, self.bx, self.by, self.uB, self.vB, self.bb, self.midX, self.midY, prev=self.T)

    def motion(self, step):
        c = self.coef
        t = self.dt * step
        return (c["xCoefficient"] * np.sin(2 * np.pi * c["xfrequency"] * t + c["xPhase"]),
                c["uCoefficient"] * np.cos(2 * np.pi * c["xfrequency"] * t + c["uPhase"]))

    def _solve(self, which, b, x0):
        if self.solve == "direct":
            return (self._lu1 if which == 1 else self._lu2).solve(b), 0
        key = "velocity" if which == 1 else "Poisson"
        tol, mx, pc = self.cfg[key]
        A, amg = (self.A1, self.amg1) if which == 1 else (self.A2, self.amg2)
        x, it, ok = bicgstab_pc(A, b, x0, tol, mx, pc, amg)
        if not ok:
            raise RuntimeError("oracle %s solve did not converge" % key)
        return x, it

    def _pre_step(self):
        """luo_base::_pre_step (luo_base.cu:235-248) and the loop state of luo_base.cu:213-214."""
        self.uold = self.u.copy()
        self.uBk = self.uB.copy()
        self.vBk = self.vB.copy()
        self.Nold = self.N
        self.midY0, self.vbody0 = self.midY, self.vbody
        self.sctol = 1e-4

    def step(self):
        """luo_base::stepTime (luo_base.cu:208-233): one pass of the phases, or with VIV: 2
        passes while |SCtol| > 0.001 or fewer than two ran (this restatement stops with an
        error after COUPLING_MAX_PASSES; the reference has no limit)."""
        self._pre_step()
        self._pass(True)
        done = 1
        if self.viv == 2:
            while True:
                self._pass(False)
                done += 1
                more = abs(self.sctol) > 0.001 or done < 2
                if not more:
                    break
                if done >= COUPLING_MAX_PASSES:
                    raise RuntimeError("strong coupling did not converge")
        self.sub_iterations = done
        self.timeStep += 1

    def _pass(self, first):
        g, T, bb, dt = self.g, self.T, self.bb, self.dt
        xm, xp, ym, yp = self.bc
        if not first:
            self.u = self.uold.copy()  # generateRHS1: u = uold (luoIBM/intermediateVelocity.cu:33)
        ub, vb = float(self.uB[0]), float(self.vB[0])
        # generateRHS1: Robin outflow, ghost nodes, inside, hybrid nodes, explicit terms
        xp[:] = robin(self.u, xp, g, dt)
        u, _ = ghost_velocity(0, self.u, T, ub, g, bb)
        u, _ = ghost_velocity(1, u, T, vb, g, bb)
        u = set_inside(u, T, ub, vb, g)
        ustar = np.zeros(g.nUV)
        ustar, _ = hybrid_velocity(0, u, ustar, T, ub, g, bb)
        ustar, _ = hybrid_velocity(1, u, ustar, T, vb, g, bb)
        bc = (xm, xp, ym, yp)
        self.N = generate_N(u, g, bc)
        L = generate_L(u, g, bc, self.nu)
        b1 = generate_bc1(u, g, bc, self.nu, dt)
        rhs1 = generate_rhs(L, self.Nold, self.N, u, b1, dt)
        self.uhat, it1 = self._solve(1, rhs1, self.uhat)
        uh = weight(0, self.uhat, ustar, T, g, bb)
        uh = weight(1, uh, ustar, T, g, bb)
        # generateRHS2 and the Poisson solve
        uh, _ = ghost_velocity(0, uh, T, ub, g, bb)
        uh, _ = ghost_velocity(1, uh, T, vb, g, bb)
        self.uhat = uh
        rhs2 = generate_rhs2(uh, g, bc)
        self.p, it2 = self._solve(2, rhs2, self.p)
        dudt = (float(self.uB[0]) - float(self.uBk[0])) / dt
        dvdt = (float(self.vB[0]) - float(self.vBk[0])) / dt  # nonzero in a later coupled pass
        pstar, _ = hybrid_pressure(self.p, T, dudt, dvdt, g, bb)
        p = weight(2, self.p, pstar, T, g, bb)
        p, _ = ghost_pressure(p, T, dudt, dvdt, g, bb)
        self.p = p
        # projection, ghost nodes and inside velocity of the new field
        u, self.uold = project(u, self.uhat, self.p, g, dt)
        u, _ = ghost_velocity(0, u, T, ub, g, bb)
        u, _ = ghost_velocity(1, u, T, vb, g, bb)
        self.u = set_inside(u, T, ub, vb, g)
        # body update: control-volume force, then the prescribed motion at t = dt * timeStep
        self.fx, self.fy = force(self.u, self.uold, self.p, T, self.nu, g, dt, bb)
        self._move_body()
        self._update_solver()
        self.iters = (it1, it2)


def csr_from_coo_summed(n, row, col, val):
    """CSR with duplicate COO entries summed and explicit zeros dropped (the matrix the
    reference's COO SpMV applies)."""
    import scipy.sparse as sp
    keep = f64(val) != 0  # zero entries, some with columns outside the matrix (LHS_mid_Y's 1 - nx)
    A = sp.coo_matrix((f64(val)[keep], (np.asarray(row)[keep], np.asarray(col)[keep])), shape=(n, n)).tocsr()
    A.sum_duplicates()
    A.eliminate_zeros()
    A.sort_indices()
    C = Csr.__new__(Csr)
    C.n = n
    C.ptr = np.ascontiguousarray(A.indptr, np.int32)
    C.col = np.ascontiguousarray(A.indices, np.int32)
    C.val = np.ascontiguousarray(A.data, np.float64)
    return C


class FadlunSolver(LuoSolver):
    """The modified Fadlun method on the CPU: luo_base::stepTime (luo_base.cu:208-233)
    with fadlunModified's phases - generateRHS1 (FadlunModified/intermediateVelocity.cu:
    15-38: Robin outflow, explicit terms, updateRHS1forIB), generateRHS2 and the solves
    on the Fadlun LHS1/LHS2 assembled once from the initial tags (fadlunModified.cu:
    48-62; updateSolver does not rebuild them), the masked projection
    (fadlunModified.cu:109-127) and the body update (force, motion)."""

    def __init__(self, folder, solve="direct"):
        super().__init__(folder, solve="none")
        g = self.g
        # luo_base::initialise does not set the inside velocity for this method
        f0 = load_case(folder)[1][0]
        ip = f0.get("initialPerturbation", [0.0, 0.0])
        self.u = initial_velocity(g, float(f0["initialVelocity"][0]), float(f0["initialVelocity"][1]),
                                  float(ip[0]), float(ip[1]))
        self.uhat = self.u.copy()
        self.A1 = csr_from_coo_summed(g.nUV, *fadlun_lhs1_coo(g, self.dt, self.nu, self.T))
        self.A2 = csr_from_coo_summed(g.nP, *fadlun_lhs2_coo(g, self.dt, self.T))
        self.solve = solve
        if solve == "direct":
            import scipy.sparse.linalg as spla
            self._lu1 = spla.splu(self.A1.scipy().tocsc())
            self._lu2 = spla.splu(self.A2.scipy().tocsc())
        else:
            ls = {s["system"]: s for s in self.sim.get("linearSolvers", [])}
            self.cfg = {k: (float(ls[k].get("tolerance", 1e-5)), int(ls[k].get("maxIterations", 10000)),
                            _PC.get(ls[k].get("preconditioner", "DIAGONAL"), 1)) for k in ("velocity", "Poisson")}
            self.amg1 = Amg(self.A1) if self.cfg["velocity"][2] == 2 else None
            self.amg2 = Amg(self.A2) if self.cfg["Poisson"][2] == 2 else None

    def _pass(self, first):
        # a later coupled pass continues from the current u: generateRHS1 has no u = uold
        g, T, bb, dt = self.g, self.T, self.bb, self.dt
        xm, xp, ym, yp = self.bc
        # generateRHS1
        xp[:] = robin(self.u, xp, g, dt)
        bc = (xm, xp, ym, yp)
        self.N = generate_N(self.u, g, bc)
        L = generate_L(self.u, g, bc, self.nu)
        b1 = generate_bc1(self.u, g, bc, self.nu, dt)
        rhs1 = generate_rhs(L, self.Nold, self.N, self.u, b1, dt)
        rhs1 = fadlun_update_rhs1(rhs1, T, g)
        self.uhat, it1 = self._solve(1, rhs1, self.uhat)
        # generateRHS2, Poisson
        rhs2 = fadlun_rhs2(self.uhat, T, g, bc)
        self.p, it2 = self._solve(2, rhs2, self.p)
        # masked projection
        self.u = fadlun_project(self.uhat, self.p, T, g, dt)
        # body update: control-volume force, then the prescribed motion at t = dt * timeStep
        self.fx, self.fy = force(self.u, self.uold, self.p, T, self.nu, g, dt, bb)
        self._move_body()
        self._update_solver()
        self.iters = (it1, it2)


class EmbeddedSolver(LuoSolver):
    """The embedded method (SolverType OSC_CYLINDER) on the CPU: luo_base::stepTime
    (luo_base.cu:208-233) with luo_iter's phases - intermediate_velocity_setup
    (luo_iter/intermediateVelocity.cu:17-80: Robin outflow, inside velocity, explicit
    terms, alpha, the set = false stencils, LHS1 rebuilt, rhs1 updated), the velocity
    solve, poisson_setup (luo_iter/poisson.cu:15-58: rhs2, alpha, pressure stencils,
    LHS2 rebuilt, rhs2 updated), the Poisson solve, luo_base::_project_velocity
    (luo_base/projectVelocity.cu:11-53) and the body update (force, motion, tags).

    The operators are rebuilt every step on zeroed arrays (the reference's first step;
    later steps of the reference reuse its previous sorted COO arrays without clearing
    the LHS1 values, which this restatement does not reproduce)."""

    def __init__(self, folder, solve="direct", vel_offset=None):
        super().__init__(folder, solve="none", vel_offset=vel_offset)
        g = self.g
        # luo_iter::initialise (luo_base::initialise) does not set the inside velocity
        f0 = load_case(folder)[1][0]
        ip = f0.get("initialPerturbation", [0.0, 0.0])
        self.u = initial_velocity(g, float(f0["initialVelocity"][0]), float(f0["initialVelocity"][1]),
                                  float(ip[0]), float(ip[1]))
        self.uhat = self.u.copy()
        self.solve = solve
        self._fact = {1: (None, None), 2: (None, None)}
        if solve != "direct":
            ls = {s["system"]: s for s in self.sim.get("linearSolvers", [])}
            self.cfg = {k: (float(ls[k].get("tolerance", 1e-5)), int(ls[k].get("maxIterations", 10000)),
                            _PC.get(ls[k].get("preconditioner", "DIAGONAL"), 1)) for k in ("velocity", "Poisson")}

    def _solve(self, which, b, x0):
        A = self.A1 if which == 1 else self.A2
        key, fact = self._fact[which]
        same = key is not None and all(np.array_equal(a, k) for a, k in zip((A.ptr, A.col, A.val), key))
        if self.solve == "direct":
            if not same:
                import scipy.sparse.linalg as spla
                fact = spla.splu(A.scipy().tocsc())
                self._fact[which] = ((A.ptr.copy(), A.col.copy(), A.val.copy()), fact)
            return fact.solve(b), 0
        tol, mx, pc = self.cfg["velocity" if which == 1 else "Poisson"]
        if pc == 2 and not same:
            fact = Amg(A)
            self._fact[which] = ((A.ptr.copy(), A.col.copy(), A.val.copy()), fact)
        x, it, ok = bicgstab_pc(A, b, x0, tol, mx, pc, fact if pc == 2 else None)
        if not ok:
            raise RuntimeError("oracle %s solve did not converge" % ("velocity" if which == 1 else "Poisson"))
        return x, it

    def _pass(self, first):
        g, T, bb, dt = self.g, self.T, self.bb, self.dt
        xm, xp, ym, yp = self.bc
        ub, vb = float(self.uB[0]), float(self.vB[0])
        # intermediate_velocity_setup: u = uold, Robin outflow, inside velocity, explicit terms
        if not first:
            self.u = self.uold.copy()
        xp[:] = robin(self.u, xp, g, dt)
        u = set_inside(self.u, T, ub, vb, g)
        bc = (xm, xp, ym, yp)
        self.N = generate_N(u, g, bc)
        L = generate_L(u, g, bc, self.nu)
        b1 = generate_bc1(u, g, bc, self.nu, dt)
        rhs1 = generate_rhs(L, self.Nold, self.N, u, b1, dt)
        alpha = iter_alpha(0, T, g, bb)
        iter_alpha(1, T, g, bb, alpha)
        S = Stencils(g.nUV)
        ghost_velocity(0, u, T, ub, g, bb, set_=False, S=S)
        ghost_velocity(1, u, T, vb, g, bb, set_=False, S=S)
        ustar, _ = hybrid_velocity(0, u, np.zeros(g.nUV), T, ub, g, bb, S=S)
        hybrid_velocity(1, u, ustar, T, vb, g, bb, S=S)
        row, col, val, ns, interp = iter_lhs1(g, dt, self.nu, T, S, alpha, ub, vb, bb)
        self.A1 = csr_from_coo_summed(g.nUV, row, col, val)
        rhs1 = iter_update_rhs1(rhs1, ns, interp, g)
        self.uhat, it1 = self._solve(1, rhs1, self.uhat)
        # poisson_setup
        rhs2 = generate_rhs2(self.uhat, g, bc)
        # zero in a step's first pass (_pre_step set uBk = uB), not in a later coupled pass
        dudt = (float(self.uB[0]) - float(self.uBk[0])) / dt
        dvdt = (float(self.vB[0]) - float(self.vBk[0])) / dt
        Sp = Stencils(g.nP)
        ghost_pressure(self.p, T, dudt, dvdt, g, bb, set_=False, S=Sp)
        hybrid_pressure(self.p, T, dudt, dvdt, g, bb, S=Sp)
        row, col, val, ns, interp = iter_lhs2(g, dt, T, Sp, iter_alpha(2, T, g, bb), bb)
        self.A2 = csr_from_coo_summed(g.nP, row, col, val)
        rhs2 = iter_update_rhs2(rhs2, ns, interp, g)
        self.p, it2 = self._solve(2, rhs2, self.p)
        # luo_base::_project_velocity: projection, ghost nodes (set), inside velocity
        u, self.uold = project(u, self.uhat, self.p, g, dt)
        u, _ = ghost_velocity(0, u, T, ub, g, bb)
        u, _ = ghost_velocity(1, u, T, vb, g, bb)
        self.u = set_inside(u, T, ub, vb, g)
        # body update: control-volume force, then the prescribed motion at t = dt * timeStep
        self.fx, self.fy = force(self.u, self.uold, self.p, T, self.nu, g, dt, bb)
        self._move_body()
        self._update_solver()
        self.iters = (it1, it2)
