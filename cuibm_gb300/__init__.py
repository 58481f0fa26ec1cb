"""GB300-native fractional-step solver with cuIBM's interface.

The compute path is libcuibm_gb300.so (hand-written sm_103a CUDA behind the C
ABI of include/cuibm.h).  This module is the host-side mirror of the
reference's solver classes: ``NavierStokesSolver`` has the reference's life
cycle (``initialise``, ``stepTime``, ``writeData``, ``finished``,
``shutDown``; src/cuIBM.cu:61-74, NavierStokesSolver.h:152-181) and is built
from a case folder with the reference's four YAML files and command-line
overrides.  There is no CPU fallback: importing the package without the built
library raises.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libcuibm_gb300.so")

# status codes (cuibm_status)
OK, ERR_BAD_INPUT, ERR_IO, ERR_CUDA, ERR_NOT_CONVERGED, ERR_NAN, ERR_STATE, ERR_UNSUPPORTED = range(8)
ASYNC = 2  # CUIBM_COPY_ASYNC: field copies enqueued on the solver's stream
STATUS_NAMES = {0: "OK", 1: "BAD_INPUT", 2: "IO", 3: "CUDA", 4: "NOT_CONVERGED", 5: "NAN", 6: "STATE",
                7: "UNSUPPORTED"}

# solver types (src/types.h order)
NAVIER_STOKES, FADLUN, OSC_CYLINDER, FSI, LUO = range(5)

# fields (enum order of include/cuibm.h)
_FIELD_NAMES = [
    "u", "uhat", "uold", "p", "p_old", "N", "Nold", "L", "bc1", "rhs1", "rhs2",
    "bc_xminus", "bc_xplus", "bc_yminus", "bc_yplus",
    "x", "dx", "xu", "xv", "y", "dy", "yu", "yv",
    "body_x", "body_y", "body_uB", "body_vB",
    "ghost_tags_uv", "hybrid_tags_uv", "hybrid_tags_uv2", "ghost_tags_p", "hybrid_tags_p",
    "bi_x", "bi_y", "ip_x", "ip_y", "bip_x", "bip_y", "ipp_x", "ipp_y",
    "dist_node", "dist_between", "uv_body", "ustar", "pstar", "dpdn", "bi_p",
    "ghost_uv_index", "ghost_uv_coef", "hybrid_uv_index", "hybrid_uv_coef",
    "ghost_p_index", "ghost_p_coef", "hybrid_p_index", "hybrid_p_coef",
    "image_value_uv", "cfl", "work_x", "work_y", "solve_trace", "body_motion",
    "surface_force", "forces", "body_velocity_offset",
]
FIELDS = {n: i for i, n in enumerate(_FIELD_NAMES)}
_INT_FIELDS = {"ghost_tags_uv", "hybrid_tags_uv", "hybrid_tags_uv2", "ghost_tags_p", "hybrid_tags_p",
               "ghost_uv_index", "hybrid_uv_index", "ghost_p_index", "hybrid_p_index"}

_OP_NAMES = [
    "rhs1_terms", "generate_rhs1", "solve_velocity", "weight_uhat", "generate_rhs2", "rhs2", "solve_poisson",
    "weight_pressure", "project", "project_velocity", "update_body", "apply_lhs1", "apply_lhs2", "tag_points",
    "ghost_velocity_u", "ghost_velocity_uhat", "hybrid_velocity", "hybrid_pressure", "ghost_pressure",
    "set_inside", "robin_boundary", "force", "cfl", "surface_force", "surface_force_corrected",
    "apply_lhs1_t", "apply_lhs2_t", "precondition_poisson",
]
OPS = {n: i for i, n in enumerate(_OP_NAMES)}


def _field_dtype(name):
    if name in _INT_FIELDS:
        return np.int32
    return np.uint64 if name == "solve_trace" else np.float64


class CuibmError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS_NAMES.get(status, status), message))
        self.status = status


class Info(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("nx", "ny", "numU", "numV", "numUV", "numP", "solver_type",
                                            "time_step", "nt", "nsave")] + \
               [("dt", ctypes.c_double), ("nu", ctypes.c_double)] + \
               [(n, ctypes.c_int) for n in ("total_points", "bb_start_i", "bb_start_j", "bb_ncx", "bb_ncy",
                                            "nnz_lhs1", "nnz_lhs2", "velocity_precond", "poisson_precond",
                                            "velocity_krylov", "poisson_krylov", "amg_levels",
                                            "velocity_precision", "poisson_precision", "sa_rebuilds",
                                            "sa_structured")]


class AdjointStats(ctypes.Structure):
    _fields_ = [("ms", ctypes.c_double)] + [(n, ctypes.c_longlong) for n in (
        "forward_steps", "tape_steps", "velocity_iterations", "poisson_iterations", "solves_reused")]


_lib = None


def library():
    """The loaded C-ABI library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libcuibm_gb300.so is not built (run `python -m cuibm_gb300.build` "
                              "or __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        vp, ip, cp, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)
        L.cuibm_create.argtypes = [cp, ip, ctypes.POINTER(cp), ctypes.POINTER(vp)]
        L.cuibm_initialise.argtypes = [vp]
        L.cuibm_step.argtypes = [vp, ip]
        L.cuibm_finished.argtypes = [vp]
        L.cuibm_write_data.argtypes = [vp]
        L.cuibm_shutdown.argtypes = [vp]
        L.cuibm_destroy.argtypes = [vp]
        L.cuibm_destroy.restype = None
        L.cuibm_last_error.argtypes = [vp]
        L.cuibm_last_error.restype = cp
        L.cuibm_get_info.argtypes = [vp, ctypes.POINTER(Info)]
        L.cuibm_get_field.argtypes = [vp, ip, vp, ctypes.c_size_t, ip]
        L.cuibm_set_field.argtypes = [vp, ip, vp, ctypes.c_size_t, ip]
        L.cuibm_get_forces.argtypes = [vp, dp, dp]
        L.cuibm_get_iterations.argtypes = [vp, ctypes.POINTER(ip), ctypes.POINTER(ip)]
        L.cuibm_get_matrix.argtypes = [vp, ip, vp, vp, vp, ctypes.c_size_t]
        L.cuibm_run.argtypes = [vp, ip]
        L.cuibm_get_stream.argtypes = [vp, ctypes.POINTER(vp)]
        L.cuibm_get_timer.argtypes = [vp, cp, dp, ctypes.POINTER(ip)]
        L.cuibm_set_option.argtypes = [vp, cp, ctypes.c_double]
        L.cuibm_case_info.argtypes = [cp, ip, ctypes.POINTER(cp), ctypes.POINTER(Info)]
        L.cuibm_case_array.argtypes = [cp, ip, ctypes.POINTER(cp), ip, dp, ctypes.c_size_t]
        L.cuibm_case_error.restype = cp
        L.cuibm_profile_kernel.argtypes = [vp, cp, ip, dp, dp]
        L.cuibm_launch_count.argtypes = [vp, ctypes.POINTER(ctypes.c_longlong)]
        L.cuibm_cv_force_noalloc.argtypes = [vp, vp, vp, vp, vp, vp, ip, ip, ip, ip, ip, ip, ctypes.c_double,
                                             ctypes.c_double, vp, vp]
        L.cuibm_adjoint.argtypes = [vp, ip, ip, dp, dp, dp, dp, ctypes.c_size_t, ctypes.POINTER(AdjointStats)]
        L.cuibm_batch_create.argtypes = [ip, ctypes.POINTER(cp), ip, ctypes.POINTER(cp), ip, ctypes.POINTER(vp)]
        L.cuibm_batch_initialise.argtypes = [vp]
        L.cuibm_batch_step.argtypes = [vp, ip]
        L.cuibm_batch_autotune.argtypes = [vp, ip, ctypes.POINTER(ip)]
        L.cuibm_batch_size.argtypes = [vp]
        L.cuibm_batch_instance.argtypes = [vp, ip]
        L.cuibm_batch_instance.restype = vp
        L.cuibm_batch_error.argtypes = [vp]
        L.cuibm_batch_error.restype = cp
        L.cuibm_batch_destroy.argtypes = [vp]
        L.cuibm_batch_destroy.restype = None
        _lib = L
    return _lib


class NavierStokesSolver:
    """A simulation on one GPU, created from a cuIBM case folder.

    ``args`` are the reference's command-line overrides, e.g. ``["-nt", "10"]``.
    The solver type (NAVIER_STOKES_SOLVER, LUO, ...) comes from simParams.yaml
    exactly as in the reference's main (src/cuIBM.cu:42-60).
    """

    def __init__(self, case_folder, args=()):
        L = library()
        argv = [a.encode() if isinstance(a, str) else a for a in args]
        arr = (ctypes.c_char_p * max(1, len(argv)))(*argv)
        h = ctypes.c_void_p()
        st = L.cuibm_create(str(case_folder).encode(), len(argv), arr, ctypes.byref(h))
        if st != OK:
            raise CuibmError(st, L.cuibm_last_error(None).decode())
        self._h = h
        self._L = L
        self.info = self.get_info()

    # ---- life cycle (reference method names) -------------------------------
    def _check(self, st):
        if st != OK:
            raise CuibmError(st, self._L.cuibm_last_error(self._h).decode())

    def initialise(self):
        self._check(self._L.cuibm_initialise(self._h))

    def stepTime(self, nsteps=1):
        self._check(self._L.cuibm_step(self._h, int(nsteps)))

    def writeData(self):
        self._check(self._L.cuibm_write_data(self._h))

    def finished(self):
        return bool(self._L.cuibm_finished(self._h))

    def shutDown(self):
        self._check(self._L.cuibm_shutdown(self._h))

    @classmethod
    def _view(cls, L, h):
        """A solver object over a context that something else owns (a batch instance)."""
        s = cls.__new__(cls)
        s._h, s._L, s._owner = ctypes.c_void_p(h), L, False
        s.info = s.get_info()
        return s

    def close(self):
        if getattr(self, "_h", None):
            if getattr(self, "_owner", True):
                self._L.cuibm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- discrete adjoint (embedded method, prescribed motion) ---------------
    def adjoint(self, nsteps, wx, wy=None, snapshots=64):
        """Gradients of J = sum_n wx[n] Fx^n + wy[n] Fy^n over steps 1..nsteps from the
        initial condition (cuibm_adjoint): returns (J, grad, stats) with grad =
        [dJ/dnu, dJ/duCoefficient, dJ/d(u offsets of the points)..., dJ/d(v offsets)...]."""
        nb = self.info.total_points
        wx = np.ascontiguousarray(np.broadcast_to(np.asarray(wx, np.float64), (nsteps,)))
        wy = np.ascontiguousarray(np.zeros(nsteps) if wy is None else np.broadcast_to(np.asarray(wy, np.float64),
                                                                                      (nsteps,)))
        grad = np.zeros(2 + 2 * nb)
        J = ctypes.c_double()
        st = AdjointStats()
        dp = ctypes.POINTER(ctypes.c_double)
        self._check(self._L.cuibm_adjoint(self._h, int(nsteps), int(snapshots), wx.ctypes.data_as(dp),
                                          wy.ctypes.data_as(dp), ctypes.byref(J), grad.ctypes.data_as(dp),
                                          grad.size, ctypes.byref(st)))
        return J.value, grad, {k: getattr(st, k) for k, _ in AdjointStats._fields_}

    # ---- data access ---------------------------------------------------------
    def get_info(self):
        info = Info()
        self._check(self._L.cuibm_get_info(self._h, ctypes.byref(info)))
        return info

    def field_size(self, name):
        i = self.info
        UV, P, nx, ny, nb = i.numUV, i.numP, i.nx, i.ny, i.total_points
        sizes = {"bc_xminus": 2 * ny - 1, "bc_xplus": 2 * ny - 1, "bc_yminus": 2 * nx - 1, "bc_yplus": 2 * nx - 1,
                 "x": nx, "dx": nx, "xu": nx - 1, "xv": nx, "y": ny, "dy": ny, "yu": ny, "yv": ny - 1,
                 "body_x": nb, "body_y": nb, "body_uB": nb, "body_vB": nb,
                 "work_x": max(UV, P), "work_y": max(UV, P), "solve_trace": 2 * 4096,
                 "body_motion": 12, "surface_force": 3 * nb + 2, "forces": 2, "body_velocity_offset": 2 * nb}
        if name in sizes:
            return sizes[name]
        if name in ("p", "p_old", "rhs2", "ghost_tags_p", "hybrid_tags_p", "bip_x", "bip_y", "ipp_x", "ipp_y",
                    "pstar", "dpdn", "bi_p", "cfl"):
            return P
        if name in ("ghost_uv_index", "ghost_uv_coef", "hybrid_uv_index", "hybrid_uv_coef"):
            return 4 * UV
        if name in ("ghost_p_index", "ghost_p_coef", "hybrid_p_index", "hybrid_p_coef"):
            return 4 * P
        return UV

    def get(self, name):
        dtype = _field_dtype(name)
        out = np.empty(self.field_size(name), dtype=dtype)
        self._check(self._L.cuibm_get_field(self._h, FIELDS[name], out.ctypes.data, out.nbytes, 0))
        return out

    def set(self, name, values):
        dtype = _field_dtype(name)
        a = np.ascontiguousarray(values, dtype=dtype)
        if a.size != self.field_size(name):
            raise ValueError("%s needs %d values, got %d" % (name, self.field_size(name), a.size))
        self._check(self._L.cuibm_set_field(self._h, FIELDS[name], a.ctypes.data, a.nbytes, 0))

    def get_into(self, name, ptr, nbytes, on_device=False, asynchronous=False):
        """Copy a field into caller memory (host pointer, or device pointer when on_device);
        asynchronous: enqueue on the solver's stream and return (pinned host memory)."""
        flags = int(bool(on_device)) | (ASYNC if asynchronous else 0)
        self._check(self._L.cuibm_get_field(self._h, FIELDS[name], ctypes.c_void_p(ptr), nbytes, flags))

    def set_from(self, name, ptr, nbytes, on_device=False, asynchronous=False):
        """Copy caller memory into a field (the counterpart of get_into)."""
        flags = int(bool(on_device)) | (ASYNC if asynchronous else 0)
        self._check(self._L.cuibm_set_field(self._h, FIELDS[name], ctypes.c_void_p(ptr), nbytes, flags))

    def forces(self):
        fx, fy = ctypes.c_double(), ctypes.c_double()
        self._check(self._L.cuibm_get_forces(self._h, ctypes.byref(fx), ctypes.byref(fy)))
        return fx.value, fy.value

    def surface_force(self, corrected=False):
        """The surface-integral force on the body (luo_base::luoForce, which the
        reference's step leaves unused): (Fx, Fy, pressure, du/dn, dv/dn per body
        point) from the current fields; corrected=True fixes the reference's two
        index slips (its pressure search's j start, its v row stride)."""
        self.run("surface_force_corrected" if corrected else "surface_force")
        a = self.get("surface_force")
        n = (a.size - 2) // 3
        return a[3 * n], a[3 * n + 1], a[:n], a[n:2 * n], a[2 * n:3 * n]

    def iterations(self):
        a, b = ctypes.c_int(), ctypes.c_int()
        self._check(self._L.cuibm_get_iterations(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def matrix(self, system):
        nnz = self.info.nnz_lhs1 if system == 1 else self.info.nnz_lhs2
        row = np.empty(nnz, np.int32)
        col = np.empty(nnz, np.int32)
        val = np.empty(nnz, np.float64)
        self._check(self._L.cuibm_get_matrix(self._h, system, row.ctypes.data, col.ctypes.data, val.ctypes.data,
                                             nnz))
        return row, col, val

    def run(self, op):
        self._check(self._L.cuibm_run(self._h, OPS[op] if isinstance(op, str) else int(op)))

    def stream(self):
        s = ctypes.c_void_p()
        self._check(self._L.cuibm_get_stream(self._h, ctypes.byref(s)))
        return s.value or 0

    def timer(self, name):
        ms, n = ctypes.c_double(), ctypes.c_int()
        self._check(self._L.cuibm_get_timer(self._h, name.encode(), ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def set_option(self, key, value):
        self._check(self._L.cuibm_set_option(self._h, key.encode(), float(value)))

    def profile_kernel(self, name, reps=20):
        """(mean ms per launch, algorithmic bytes per launch) of one kernel, CUDA-event timed."""
        ms, b = ctypes.c_double(), ctypes.c_double()
        self._check(self._L.cuibm_profile_kernel(self._h, name.encode(), int(reps), ctypes.byref(ms),
                                                 ctypes.byref(b)))
        return ms.value, b.value

    def launch_count(self):
        """Kernels of this library launched by the last step (graph nodes x loop trips)."""
        n = ctypes.c_longlong()
        self._check(self._L.cuibm_launch_count(self._h, ctypes.byref(n)))
        return n.value

    @property
    def timeStep(self):
        return self.get_info().time_step


def _argv(args):
    argv = [a.encode() if isinstance(a, str) else a for a in args]
    return len(argv), (ctypes.c_char_p * max(1, len(argv)))(*argv)


def case_info(case_folder, args=()):
    """Parse a case folder on the host only (no GPU): the same Info a solver would report."""
    L = library()
    n, arr = _argv(args)
    info = Info()
    st = L.cuibm_case_info(str(case_folder).encode(), n, arr, ctypes.byref(info))
    if st != OK:
        raise CuibmError(st, L.cuibm_case_error().decode())
    return info


def case_array(case_folder, name, args=()):
    """Grid or body array of a case, built on the host exactly as the solver builds it."""
    L = library()
    info = case_info(case_folder, args)
    size = {"x": info.nx, "dx": info.nx, "xu": info.nx - 1, "xv": info.nx, "y": info.ny, "dy": info.ny,
            "yu": info.ny, "yv": info.ny - 1, "body_x": info.total_points, "body_y": info.total_points}[name]
    out = np.empty(size)
    n, arr = _argv(args)
    st = L.cuibm_case_array(str(case_folder).encode(), n, arr, FIELDS[name],
                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), size)
    if st != OK:
        raise CuibmError(st, L.cuibm_case_error().decode())
    return out


class Batch:
    """Many independent cases advanced together on one GPU (cuibm_batch_*).

    Each instance is a full solver with its own stream; its persistent solves use
    ``solver_blocks`` blocks (None: a quarter of the SMs, two blocks per SM) so that several instances'
    solves run at once.  ``instances`` are solver objects for fields, forces and
    output; the batch owns them.
    """

    def __init__(self, case_folders, args=(), solver_blocks=None):
        L = library()
        folders = [str(f).encode() for f in case_folders]
        farr = (ctypes.c_char_p * len(folders))(*folders)
        argv = [a.encode() if isinstance(a, str) else a for a in args]
        aarr = (ctypes.c_char_p * max(1, len(argv)))(*argv)
        h = ctypes.c_void_p()
        st = L.cuibm_batch_create(len(folders), farr, len(argv), aarr, int(solver_blocks or 0), ctypes.byref(h))
        if st != OK:
            raise CuibmError(st, L.cuibm_batch_error(None).decode())
        self._h, self._L = h, L
        self.instances = [NavierStokesSolver._view(L, L.cuibm_batch_instance(h, k)) for k in range(len(folders))]

    def _check(self, st):
        if st != OK:
            raise CuibmError(st, self._L.cuibm_batch_error(self._h).decode())

    def initialise(self):
        self._check(self._L.cuibm_batch_initialise(self._h))

    def stepTime(self, nsteps=1):
        self._check(self._L.cuibm_batch_step(self._h, int(nsteps)))

    def autotune(self, steps=2):
        """Pick the persistent solves' block counts by timing the batch (cuibm_batch_autotune;
        every instance advances 16 x steps); returns the choice: one block count for all
        instances, or minus the rows a thread of counts sized per instance."""
        nb = ctypes.c_int()
        self._check(self._L.cuibm_batch_autotune(self._h, int(steps), ctypes.byref(nb)))
        return nb.value

    def close(self):
        if getattr(self, "_h", None):
            for s in self.instances:
                s._h = None
            self._L.cuibm_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
