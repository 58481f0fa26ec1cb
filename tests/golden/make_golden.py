"""Generate the golden fixtures of tests/golden from the reference's own code.

Run in a checkout where the cuIBM source tree is available (it is read in
place, never copied):

    python tests/golden/make_golden.py [--ref /path/to/cuIBM/src]

It builds oracle/_ref (the reference's kernel files and its grid/body parsers
compiled for the CPU through oracle/ref_shim.h and oracle/ref_include) and runs
them on small seeded cases.  Each case's inputs and the reference's outputs are
saved as an .npz next to this script; tests/test_oracle_golden.py checks the
oracle against them bit for bit.
"""
import argparse
import ctypes
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cuibm_gb300 import cases  # noqa: E402

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def d(a):
    return a.ctypes.data_as(_dp)


def i(a):
    return a.ctypes.data_as(_ip)


def ref_libs(ref_src):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "REF=" + ref_src], check=True)
    K = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libcuibm_refkernels.so"))
    IO = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libcuibm_refio.so"))
    return K, IO


def ref_grid(IO, folder):
    nx, ny, h = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
    IO.ref_parse_domain(os.path.join(folder, "domain.json").encode(), ctypes.byref(nx), ctypes.byref(ny),
                        ctypes.byref(h))
    nx, ny = nx.value, ny.value
    arr = {k: np.zeros(n) for k, n in (("x", nx), ("dx", nx), ("xu", nx - 1), ("xv", nx), ("y", ny), ("dy", ny),
                                         ("yu", ny), ("yv", ny - 1))}
    IO.ref_domain_arrays(*(d(arr[k]) for k in ("x", "dx", "xu", "xv", "y", "dy", "yu", "yv")))
    return nx, ny, arr


def ref_body(IO, folder):
    n = ctypes.c_int()
    IO.ref_parse_bodies(os.path.join(folder, "bodies.json").encode(), ctypes.byref(n))
    if n.value == 0:
        return None
    npts = IO.ref_body_numpoints(0)
    X, Y, coef = np.zeros(npts), np.zeros(npts), np.zeros(10)
    IO.ref_body_points(0, d(X), d(Y), d(coef))
    return X, Y, coef


def grid_case(IO, name, folder):
    """Grid and body arrays only (large benchmark grids)."""
    nx, ny, G = ref_grid(IO, folder)
    out = {"nx": np.int32(nx), "ny": np.int32(ny)}
    out.update({"grid_" + k: v for k, v in G.items()})
    body = ref_body(IO, folder)
    if body is not None:
        out["body_X"], out["body_Y"], out["body_coef"] = body
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name, "nx=%d ny=%d" % (nx, ny))


def ns_case(K, IO, name, folder, rng, nu, dt):
    """Inputs and reference outputs of the plain-solver kernels on one grid."""
    nx, ny, G = ref_grid(IO, folder)
    nU, nV = (nx - 1) * ny, nx * (ny - 1)
    nUV, nP = nU + nV, nx * ny
    out = {"nx": np.int32(nx), "ny": np.int32(ny), "nu": np.float64(nu), "dt": np.float64(dt)}
    out.update({"grid_" + k: v for k, v in G.items()})
    u = rng.standard_normal(nUV)
    uhat = rng.standard_normal(nUV)
    Nold = rng.standard_normal(nUV)
    p = rng.standard_normal(nP)
    xm, xp = rng.standard_normal(2 * ny - 1), rng.standard_normal(2 * ny - 1)
    ym, yp = rng.standard_normal(2 * nx - 1), rng.standard_normal(2 * nx - 1)
    out.update(u=u, uhat=uhat, Nold=Nold, p=p, xm=xm, xp=xp, ym=ym, yp=yp)
    dx, dy = G["dx"], G["dy"]
    N = np.zeros(nUV)
    K.ref_generateN(d(N), d(u), d(dx), d(dy), d(ym), d(yp), d(xm), d(xp), nx, ny)
    L = np.zeros(nUV)
    K.ref_generateL.argtypes = [_dp] * 8 + [ctypes.c_int, ctypes.c_int, ctypes.c_double]
    K.ref_generateL(d(L), d(u), d(dx), d(dy), d(ym), d(yp), d(xm), d(xp), nx, ny, nu)
    bc1 = np.zeros(nUV)
    K.ref_generateBC1.argtypes = [_dp] * 8 + [ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int]
    K.ref_generateBC1(d(u), d(bc1), d(ym), d(yp), d(xm), d(xp), d(dx), d(dy), nu, dt, nx, ny)
    rhs1 = np.zeros(nUV)
    K.ref_generateRHS.argtypes = [_dp] * 6 + [ctypes.c_double, ctypes.c_int, ctypes.c_int]
    K.ref_generateRHS(d(rhs1), d(L), d(Nold), d(N), d(u), d(bc1), dt, nx, ny)
    out.update(N=N, L=L, bc1=bc1, rhs1=rhs1)
    nnz1 = nU * 5 - 2 * ny - 2 * (nx - 1) + nV * 5 - 2 * (ny - 1) - 2 * nx
    for luo in (0, 1):
        r1, c1, v1 = np.zeros(nnz1, np.int32), np.zeros(nnz1, np.int32), np.zeros(nnz1)
        gt = -np.ones(nUV, np.int32)
        K.ref_generateLHS1.argtypes = [ctypes.c_int, _ip, _ip, _dp, _ip, _dp, _dp, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_int, ctypes.c_int]
        K.ref_generateLHS1(luo, i(r1), i(c1), d(v1), i(gt), d(dx), d(dy), dt, nu, nx, ny)
        out["lhs1_%s_row" % ("luo" if luo else "ns")] = r1
        out["lhs1_%s_col" % ("luo" if luo else "ns")] = c1
        out["lhs1_%s_val" % ("luo" if luo else "ns")] = v1
        nnz2 = 5 * nP - 2 * ny - 2 * nx
        r2, c2, v2 = np.zeros(nnz2, np.int32), np.zeros(nnz2, np.int32), np.zeros(nnz2)
        K.ref_generateLHS2.argtypes = [ctypes.c_int, _ip, _ip, _dp, ctypes.c_int, _dp, _dp, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_double]
        K.ref_generateLHS2(luo, i(r2), i(c2), d(v2), nnz2, d(dx), d(dy), nx, ny, dt)
        out["lhs2_%s_row" % ("luo" if luo else "ns")] = r2
        out["lhs2_%s_col" % ("luo" if luo else "ns")] = c2
        out["lhs2_%s_val" % ("luo" if luo else "ns")] = v2
    rhs2 = np.zeros(nP)
    K.ref_generateRHS2.argtypes = [ctypes.c_int] + [_dp] * 8 + [ctypes.c_int, ctypes.c_int]
    K.ref_generateRHS2(0, d(rhs2), d(uhat), d(ym), d(yp), d(xm), d(xp), d(dx), d(dy), nx, ny)
    out["rhs2"] = rhs2
    up, uold = u.copy(), np.zeros(nUV)
    K.ref_project.argtypes = [ctypes.c_int] + [_dp] * 6 + [ctypes.c_double, ctypes.c_int, ctypes.c_int]
    K.ref_project(0, d(up), d(uhat), d(uold), d(p), d(dx), d(dy), dt, nx, ny)
    out.update(u_projected=up, uold_projected=uold)
    uic = np.zeros(nUV)
    K.ref_initialiseVelocity.argtypes = [_dp] * 5 + [ctypes.c_double] * 8 + [ctypes.c_int, ctypes.c_int]
    K.ref_initialiseVelocity(d(uic), d(G["xu"]), d(G["yu"]), d(G["xv"]), d(G["yv"]), 0.7, -0.3, 0.2, 0.1,
                             G["x"][-1], G["x"][0], G["y"][-1], G["y"][0], nx, ny)
    out["u_initial"] = uic
    c = np.zeros(nP)
    K.ref_calculateCFL.argtypes = [_dp, _dp, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_double]
    K.ref_calculateCFL(d(c), d(u), d(dx), d(dy), nx, ny, dt)
    out["cfl"] = c
    body = ref_body(IO, folder)
    if body is not None:
        out["body_X"], out["body_Y"], out["body_coef"] = body
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name, "nx=%d ny=%d" % (nx, ny))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference/src")
    a = ap.parse_args()
    K, IO = ref_libs(a.ref)
    rng = np.random.default_rng(20261203)
    with tempfile.TemporaryDirectory() as tmp:
        # stretched grid with all three sub-domain kinds in both directions
        f = os.path.join(tmp, "stretched")
        cases.write_case(f, [{"type": "simulation", "dt": 0.01, "nt": 1, "nsave": 1}],
                         [{"type": "flow", "nu": 0.02, "initialVelocity": [1.0, 0.0],
                           "boundaryConditions": cases.bcs((1, 0), (1, 0), (1, 0), (1, 0))}],
                         [cases.axis("x", -2.0, 0.1, [(-0.5, 1.1), (0.5, 1.0), (2.5, 1.08)]),
                          cases.axis("y", -1.5, 0.1, [(-0.4, 1.12), (0.4, 1.0), (1.6, 1.1)])],
                         [{"type": "circle", "circleOptions": [0.0, 0.0, 0.25, 24, False, 0.1]}])
        ns_case(K, IO, "ns_stretched", f, rng, nu=0.02, dt=0.01)
        f = os.path.join(tmp, "cavity")
        cases.cavity(f, n=16, nu=0.01, dt=0.01, nt=1)
        ns_case(K, IO, "ns_cavity16", f, rng, nu=0.01, dt=0.01)
        # grids and bodies of the benchmark cylinders (Re 40 and Re 550)
        f = os.path.join(tmp, "cyl40")
        cases.cylinder(f, h=0.02, ratio=1.03, points=157, nt=1)
        grid_case(IO, "grid_cylinder_re40", f)
        f = os.path.join(tmp, "cyl550")
        cases.cylinder(f, h=0.005, ratio=1.01, points=629, nt=1)
        grid_case(IO, "grid_cylinder_re550", f)


if __name__ == "__main__":
    main()
