"""Tangent-linear model of the embedded method's time step (TEST INFRASTRUCTURE ONLY).

Only tests/ use this module, as the FP64 tangent-linear reference of the GPU's
discrete adjoint.  It runs the oracle's restated step (EmbeddedSolver._pass, the
reference's luo_iter step) on dual numbers: liboracle_dual.so is ns.c, ib.c and
embedded.c compiled with every double a (value, derivative) pair (oracle/dual.h),
so each kernel propagates the derivative along one direction of the parameters
exactly, operation by operation.  The linear systems are solved by sparse LU:
A x = b with A = Av + e Ad, b = bv + e bd gives xv = Av^-1 bv and
xd = Av^-1 (bd - Ad xv).

Parameters (the derivative's direction is a combination of them):
  nu          the kinematic viscosity;
  uCoefficient the amplitude of the prescribed body velocity u_B(t) = uCoefficient
              cos(2 pi f t + uPhase) (luo_base/move.cu set_movement); the prescribed
              path xCoefficient sin(2 pi f t + xPhase) is a separate input of the
              reference's bodies.yaml and is held fixed, so the body's positions, tags
              and interpolation weights do not depend on any parameter;
  offsets     per-point offsets of the body velocity (u and v of each point), added
              wherever the motion sets it.  The reference's kernels read only the first
              point's velocity (biLinearInterpolation.cu, setInsideVelocity use uB[0]), so
              only point 0's offsets act on the flow.

The objective is J = sum over steps n of wx[n] Fx^n + wy[n] Fy^n, the control-volume
force of each step (period-averaged drag: wx = 2 / nt, wy = 0).
"""
import ctypes
import os

import numpy as np

from . import (EmbeddedSolver, Stencils, _plain_nnz, f64, iter_alpha, lib)

HERE = os.path.dirname(os.path.abspath(__file__))
LIBD = os.path.join(HERE, "_build", "liboracle_dual.so")
_libd = None


class Dual(ctypes.Structure):
    _fields_ = [("v", ctypes.c_double), ("d", ctypes.c_double)]


def libd():
    global _libd
    if _libd is None:
        lib()  # builds both libraries if needed
        _libd = ctypes.CDLL(LIBD)
    return _libd


def _arg(a):
    if isinstance(a, np.ndarray):
        if a.dtype == np.complex128 or a.dtype == np.int32:
            if not a.flags.c_contiguous:
                raise ValueError("dual kernels need contiguous arrays")
            return ctypes.c_void_p, ctypes.c_void_p(a.ctypes.data)
        raise TypeError("array of %s passed to a dual kernel" % a.dtype)
    if isinstance(a, (complex, np.complexfloating)):
        return Dual, Dual(float(a.real), float(a.imag))
    if isinstance(a, (float, np.floating)):
        return Dual, Dual(float(a), 0.0)
    if isinstance(a, (bool, int, np.integer)):
        return ctypes.c_int, ctypes.c_int(int(a))
    if isinstance(a, ctypes._Pointer) or isinstance(a, ctypes.c_void_p) or a is None:
        return ctypes.c_void_p, a
    if hasattr(a, "_obj"):  # ctypes.byref
        return ctypes.c_void_p, a
    raise TypeError("cannot pass %r to a dual kernel" % (a,))


def dcall(name, *args, restype=None):
    fn = getattr(libd(), name)
    conv = [_arg(a) for a in args]
    fn.argtypes = [t for t, _ in conv]
    fn.restype = restype
    return fn(*[v for _, v in conv])


def cx(a):
    """A dual array: value a, derivative 0 (complex128 layout)."""
    return np.ascontiguousarray(a, dtype=np.complex128)


class _DTags(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("ghostTagsUV", "ghostTagsP", "hybridTagsUV", "hybridTagsP",
                                               "hybridTagsUV2", "dist_node", "dist_between", "dist_u_body",
                                               "dist_v_body", "uv", "bi_x", "bi_y", "ip_x", "ip_y", "bip_x",
                                               "bip_y", "ipp_x", "ipp_y")]


class _DInterp(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("index1", "index2", "index3", "index4", "q1coef", "q2coef",
                                               "q3coef", "q4coef", "value", "dpdn", "q1", "q2", "q3", "q4")]


class DStencils:
    def __init__(self, n):
        self.index = np.zeros((4, n), np.int32)
        self.coef = np.zeros((4, n), np.complex128)
        self.value = np.zeros(n, np.complex128)
        self.dpdn = np.zeros(n, np.complex128)
        self.q = np.zeros((4, n), np.complex128)

    def c(self):
        p = lambda a: ctypes.c_void_p(a.ctypes.data)
        st = _DInterp(*[p(self.index[k]) for k in range(4)], *[p(self.coef[k]) for k in range(4)], p(self.value),
                      p(self.dpdn), *[p(self.q[k]) for k in range(4)])
        st._owner = self  # the arrays must outlive the call that writes through these pointers
        return st


class DualSolver(EmbeddedSolver):
    """EmbeddedSolver whose fields carry the derivative along one direction of the
    parameters: seed with direction(d_nu, d_ucoef, d_offu, d_offv) before stepping; the
    geometry (positions, tags, boxes) is the plain solver's, the fields are duals."""

    def __init__(self, folder, vel_offset=None):
        super().__init__(folder, solve="direct", vel_offset=vel_offset)
        if self.viv:
            raise ValueError("the tangent model covers prescribed motion only")
        self.direction(0.0, 0.0, None, None)

    def direction(self, d_nu=0.0, d_ucoef=0.0, d_offu=None, d_offv=None):
        n = len(self.bx)
        self.d_nu, self.d_ucoef = float(d_nu), float(d_ucoef)
        self.d_off = (np.zeros(n) if d_offu is None else f64(d_offu), np.zeros(n) if d_offv is None else f64(d_offv))
        g = self.g
        self.ud = cx(self.u)
        self.Nd = cx(self.N)
        self.pd = cx(self.p)
        self.bcd = [cx(a) for a in self.bc]
        self.dub = self.d_ucoef * self._cosine(0) + self.d_off[0][0]  # the body velocity of the first step
        self.dvb = self.d_off[1][0]
        self.dJ = 0.0
        self.J = 0.0
        self.fxd = []
        self.fyd = []
        assert g.nUV == len(self.ud)

    def _cosine(self, step):
        c = self.coef
        return np.cos(2 * np.pi * c["xfrequency"] * (self.dt * step) + c["uPhase"])

    def _dsolve(self, n, row, col, val, b):
        import scipy.sparse as sp
        import scipy.sparse.linalg as spla
        val = np.asarray(val)
        keep = val.real != 0
        r, c_ = np.asarray(row)[keep], np.asarray(col)[keep]
        Av = sp.coo_matrix((val.real[keep], (r, c_)), shape=(n, n)).tocsc()
        Ad = sp.coo_matrix((val.imag[keep], (r, c_)), shape=(n, n)).tocsr()
        lu = spla.splu(Av)
        xv = lu.solve(np.ascontiguousarray(b.real))
        xd = lu.solve(np.ascontiguousarray(b.imag) - Ad @ xv)
        return xv + 1j * xd

    def step_dual(self, wx=0.0, wy=0.0):
        """One step of the plain solver and its tangent; J += wx Fx + wy Fy."""
        g, T, bb, dt = self.g, self.T, self.bb, self.dt
        nu = complex(self.nu, self.d_nu)
        xm, xp, ym, yp = self.bcd
        i0, j0, ncx, ncy = (int(v) for v in bb)
        ub = complex(float(self.uB[0]), self.dub)
        vb = complex(float(self.vB[0]), self.dvb)
        # the plain step first (the geometry of the next step, the values to check against)
        self._pre_step()
        Nold_d = self.Nd
        # intermediate_velocity_setup: Robin outflow, inside velocity, explicit terms
        xp = xp.copy()
        dcall("or_updateRobinBoundary", self.ud, xp, cx(g.dx), complex(dt), 1.0, 1.0, g.nx, g.ny)
        u = self.ud.copy()
        gt = np.ascontiguousarray(T.ghostTagsUV, np.int32)
        dcall("or_setInsideVelocity", gt, u, ub, vb, g.nx, g.ny)
        uold_d = u.copy()
        args_bc = (cx(g.dx), cx(g.dy), ym, yp, xm, xp)
        N = np.zeros(g.nUV, np.complex128)
        dcall("or_generateN", N, u, *args_bc, g.nx, g.ny)
        L = np.zeros(g.nUV, np.complex128)
        dcall("or_generateL", L, u, *args_bc, g.nx, g.ny, nu)
        b1 = np.zeros(g.nUV, np.complex128)
        dcall("or_generateBC1", u, b1, ym, yp, xm, xp, cx(g.dx), cx(g.dy), nu, complex(dt), g.nx, g.ny)
        rhs1 = np.zeros(g.nUV, np.complex128)
        dcall("or_generateRHS", rhs1, L, Nold_d, N, u, b1, complex(dt), g.nUV)
        alpha = iter_alpha(0, T, g, bb)
        iter_alpha(1, T, g, bb, alpha)
        S = DStencils(g.nUV)
        Td = self._dtags()
        for direc, q in ((0, ub), (1, vb)):
            xc, yc = (g.xu, g.yu) if direc == 0 else (g.xv, g.yv)
            dcall("or_ghost_velocity", direc, u.copy(), 0, gt, q, cx(yc), cx(xc), Td["bi_x"], Td["bi_y"],
                  Td["ip_x"], Td["ip_y"], i0, j0, ncx, ncy, g.nx, g.ny, ctypes.byref(S.c()))
        ustar = np.zeros(g.nUV, np.complex128)
        ht = np.ascontiguousarray(T.hybridTagsUV, np.int32)
        for direc, q in ((0, ub), (1, vb)):
            xc, yc = (g.xu, g.yu) if direc == 0 else (g.xv, g.yv)
            dcall("or_hybrid_velocity", direc, u, ustar, ht, q, cx(yc), cx(xc), Td["bi_x"], Td["bi_y"], Td["ip_x"],
                  Td["ip_y"], i0, j0, ncx, ncy, g.nx, g.ny, ctypes.byref(S.c()))
        nh = int((T.hybridTagsUV > 0).sum())
        nnz = _plain_nnz(g, 1) + nh
        row, col = np.zeros(nnz, np.int32), np.zeros(nnz, np.int32)
        val = np.zeros(nnz, np.complex128)
        ns, interp = np.zeros(g.nUV, np.complex128), np.zeros(g.nUV, np.complex128)
        count = np.zeros(g.nUV, np.int32)
        ix = [np.ascontiguousarray(S.index[k]) for k in range(4)]
        cf = [np.ascontiguousarray(S.coef[k]) for k in range(4)]
        qs = [np.ascontiguousarray(S.q[k]) for k in range(4)]
        got = dcall("or_iter_lhs1", row, col, val, nnz, cx(g.dx), cx(g.dy), complex(dt), nu, g.nx, g.ny, ht, gt, ns,
                    interp, count, *ix, cx(alpha), ub, vb, *cf, *qs, i0, j0, ncx, ncy, restype=ctypes.c_int)
        if got != nnz:
            raise RuntimeError("dual or_iter_lhs1: %d entries, expected %d" % (got, nnz))
        dcall("or_iter_update_rhs1", rhs1, ns, interp, g.nx, g.ny)
        uhat = self._dsolve(g.nUV, row, col, val, rhs1)
        # poisson_setup
        rhs2 = np.zeros(g.nP, np.complex128)
        dcall("or_generateRHS2", rhs2, uhat, ym, yp, xm, xp, cx(g.dx), cx(g.dy), g.nx, g.ny)
        zero = complex(0.0)  # the body acceleration (uB - uBk) / dt is 0 in a step's first pass
        Sp = DStencils(g.nP)
        gtp = np.ascontiguousarray(T.ghostTagsP, np.int32)
        htp = np.ascontiguousarray(T.hybridTagsP, np.int32)
        dcall("or_ghost_pressure", self.pd.copy(), 0, gtp, zero, zero, cx(g.yu), cx(g.xv), Td["bip_x"], Td["bip_y"],
              Td["ipp_x"], Td["ipp_y"], i0, j0, ncx, ncy, g.nx, g.ny, ctypes.byref(Sp.c()))
        pstar = np.zeros(g.nP, np.complex128)
        dcall("or_hybrid_pressure", self.pd, pstar, htp, zero, zero, cx(g.yu), cx(g.xv), Td["bip_x"], Td["bip_y"],
              Td["ipp_x"], Td["ipp_y"], i0, j0, ncx, ncy, g.nx, g.ny, ctypes.byref(Sp.c()))
        alpha_p = iter_alpha(2, T, g, bb)
        nh = int((T.hybridTagsP > 0).sum())
        nnz = _plain_nnz(g, 2) + nh
        row, col = np.zeros(nnz, np.int32), np.zeros(nnz, np.int32)
        val = np.zeros(nnz, np.complex128)
        ns, interp = np.zeros(g.nP, np.complex128), np.zeros(g.nP, np.complex128)
        count = np.zeros(g.nP, np.int32)
        ix = [np.ascontiguousarray(Sp.index[k]) for k in range(4)]
        cf = [np.ascontiguousarray(Sp.coef[k]) for k in range(4)]
        qs = [np.ascontiguousarray(Sp.q[k]) for k in range(4)]
        got = dcall("or_iter_lhs2", row, col, val, nnz, cx(g.dx), cx(g.dy), g.nx, g.ny, complex(dt), count, ns, interp,
                    htp, gtp, cx(alpha_p), Sp.dpdn, *ix, *cf, *qs, i0, j0, ncx, ncy, restype=ctypes.c_int)
        if got != nnz:
            raise RuntimeError("dual or_iter_lhs2: %d entries, expected %d" % (got, nnz))
        dcall("or_iter_update_rhs2", rhs2, ns, interp, g.nx, g.ny)
        p = self._dsolve(g.nP, row, col, val, rhs2)
        # projection, ghost nodes (set), inside velocity
        unew = u.copy()
        uold = np.zeros(g.nUV, np.complex128)
        dcall("or_project", unew, uhat, uold, p, cx(g.dx), cx(g.dy), complex(dt), g.nx, g.ny)
        for direc, q in ((0, ub), (1, vb)):
            xc, yc = (g.xu, g.yu) if direc == 0 else (g.xv, g.yv)
            dcall("or_ghost_velocity", direc, unew, 1, gt, q, cx(yc), cx(xc), Td["bi_x"], Td["bi_y"], Td["ip_x"],
                  Td["ip_y"], i0, j0, ncx, ncy, g.nx, g.ny, ctypes.byref(DStencils(g.nUV).c()))
        dcall("or_setInsideVelocity", gt, unew, ub, vb, g.nx, g.ny)
        fx, fy = Dual(), Dual()
        dcall("or_calculateForce", unew, uold, p, gt, nu, cx(g.dx), cx(g.dy), complex(dt), g.nx, g.ny, i0, j0, ncx,
              ncy, ctypes.byref(fx), ctypes.byref(fy))
        self.fxd.append(complex(fx.v, fx.d))
        self.fyd.append(complex(fy.v, fy.d))
        self.J += wx * fx.v + wy * fy.v
        self.dJ += wx * fx.d + wy * fy.d
        # the plain values of this step (the body update below uses them: force, motion, tags)
        self.u, self.uhat, self.p, self.N, self.uold = unew.real.copy(), uhat.real.copy(), p.real.copy(), \
            N.real.copy(), uold.real.copy()
        self.bc[1][:] = xp.real
        self.fx, self.fy = fx.v, fy.v
        self.ud, self.Nd, self.pd = unew, N, p
        self.bcd[1] = xp
        self._move_body()
        self._update_solver()
        self.dub = self.d_ucoef * self._cosine(self.timeStep) + self.d_off[0][0]
        self.dvb = self.d_off[1][0]
        self.timeStep += 1

    def _dtags(self):
        T = self.T
        return {k: cx(getattr(T, k)) for k in ("bi_x", "bi_y", "ip_x", "ip_y", "bip_x", "bip_y", "ipp_x", "ipp_y")}
