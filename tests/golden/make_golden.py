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


class RefTagArrays(ctypes.Structure):
    _fields_ = [(n, _ip) for n in ("ghostTagsUV", "ghostTagsP", "hybridTagsUV", "hybridTagsP", "hybridTagsUV2")] + \
               [(n, _dp) for n in ("distance_from_intersection_to_node", "distance_between_nodes_at_IB",
                                   "distance_from_u_to_body", "distance_from_v_to_body", "uv",
                                   "body_intercept_x", "body_intercept_y", "image_point_x", "image_point_y",
                                   "body_intercept_p_x", "body_intercept_p_y", "image_point_p_x", "image_point_p_y",
                                   "x1", "y1", "x2", "y2", "x1_p", "y1_p", "x2_p", "y2_p",
                                   "x1_ip", "y1_ip", "x2_ip", "y2_ip")]


class RefInterpArrays(ctypes.Structure):
    _fields_ = [(n, _ip) for n in ("index1", "index2", "index3", "index4")] + \
               [(n, _dp) for n in ("q1coef", "q2coef", "q3coef", "q4coef", "x1", "x2", "x3", "x4", "y1", "y2",
                                   "y3", "y4", "q1", "q2", "q3", "q4", "image_point_u", "a0", "a1", "a2", "a3")]


def bounding_box(x, y, gx, gy, scale):
    """src/bodies.cu:256-326 (scaled box in cell indices), as in the oracle."""
    xmax, xmin, ymax, ymin = x.max(), x.min(), y.max(), y.min()
    ex, ey = xmax - xmin, ymax - ymin
    xmax += 0.5 * ex * (scale - 1.0)
    xmin -= 0.5 * ex * (scale - 1.0)
    ymax += 0.5 * ey * (scale - 1.0)
    ymin -= 0.5 * ey * (scale - 1.0)
    i = j = 0
    while gx[i + 1] < xmin:
        i += 1
    while gy[j + 1] < ymin:
        j += 1
    i0, j0 = i, j
    while gx[i] < xmax:
        i += 1
    while gy[j] < ymax:
        j += 1
    return i0, j0, i - i0, j - j0


def ib_case(K, IO, name, folder, rng, nu, dt, uB0=0.25, vB0=-0.15, uBk=0.2, vBk=-0.1, scale=2.0):
    """Tagging, interpolation, blending, inside velocity, Robin outflow and force
    of the external method on a small stretched grid around a circle."""
    nx, ny, G = ref_grid(IO, folder)
    nU, nV = (nx - 1) * ny, nx * (ny - 1)
    nUV, nP = nU + nV, nx * ny
    X, Y, _ = ref_body(IO, folder)
    n = len(X)
    # bodies::initialise (no rotation: x = X), centroid by a serial sum, then the t = 0
    # motion of luo_base::initialise with zero coefficients: x = 0 + (x - midX)
    mx = 0.0
    my = 0.0
    for v in X:
        mx += v
    for v in Y:
        my += v
    mx /= n
    my /= n
    i0, j0, ncx, ncy = bounding_box(X, Y, G["x"], G["y"], scale)
    bx = np.array([0.0 + (v - mx) for v in X])
    by = Y.copy()
    midX, midY = 0.0, my
    uB = np.full(n, uB0)
    vB = np.full(n, vB0)
    out = {"nx": np.int32(nx), "ny": np.int32(ny), "nu": np.float64(nu), "dt": np.float64(dt),
           "bb": np.array([i0, j0, ncx, ncy], np.int32), "bx": bx, "by": by, "uB": uB, "vB": vB,
           "midX": np.float64(midX), "midY": np.float64(midY), "uBk": np.float64(uBk), "vBk": np.float64(vBk),
           "body_X": X, "body_Y": Y}
    out.update({"grid_" + k: v for k, v in G.items()})
    p_sized = {"ghostTagsP", "hybridTagsP", "distance_from_u_to_body", "distance_from_v_to_body",
               "body_intercept_p_x", "body_intercept_p_y", "image_point_p_x", "image_point_p_y",
               "x1_p", "y1_p", "x2_p", "y2_p"}
    arr = {}
    for f, _ in RefTagArrays._fields_:
        size = nP if f in p_sized else nUV
        arr[f] = np.zeros(size + 2 * max(nx, ny), np.int32 if "Tags" in f else np.float64)[:size].copy()
    ta = RefTagArrays(**{f: (i(arr[f]) if "Tags" in f else d(arr[f])) for f, _ in RefTagArrays._fields_})
    K.ref_tagPoints.argtypes = [ctypes.POINTER(RefTagArrays)] + [_dp] * 8 + [ctypes.c_int] * 7 + \
        [ctypes.c_double, ctypes.c_double]
    K.ref_tagPoints(ctypes.byref(ta), d(bx), d(by), d(uB), d(vB), d(G["xu"]), d(G["yu"]), d(G["xv"]), d(G["yv"]),
                    i0, j0, ncx, ncy, nx, ny, n, midX, midY)
    for f in ("ghostTagsUV", "ghostTagsP", "hybridTagsUV", "hybridTagsP", "hybridTagsUV2",
              "distance_from_intersection_to_node", "distance_between_nodes_at_IB", "uv",
              "body_intercept_x", "body_intercept_y", "image_point_x", "image_point_y",
              "body_intercept_p_x", "body_intercept_p_y", "image_point_p_x", "image_point_p_y",
              "distance_from_u_to_body", "distance_from_v_to_body"):
        out["tag_" + f] = arr[f].copy()

    def interp_arrays(size):
        a = {f: np.zeros(size, np.int32 if f.startswith("index") else np.float64) for f, _ in RefInterpArrays._fields_}
        r = RefInterpArrays(**{f: (i(a[f]) if f.startswith("index") else d(a[f])) for f, _ in RefInterpArrays._fields_})
        return a, r

    gU, gP = arr["ghostTagsUV"], arr["ghostTagsP"]
    hU, hP = arr["hybridTagsUV"], arr["hybridTagsP"]
    bix, biy, ipx, ipy = (arr[k] for k in ("body_intercept_x", "body_intercept_y", "image_point_x", "image_point_y"))
    bpx, bpy, ppx, ppy = (arr[k] for k in ("body_intercept_p_x", "body_intercept_p_y", "image_point_p_x",
                                           "image_point_p_y"))
    u = 1.0 + 0.2 * rng.standard_normal(nUV)
    p = 0.1 * rng.standard_normal(nP)
    out.update(u_in=u.copy(), p_in=p.copy())
    # ghost-node velocity, u then v, set = true (luoIBM::rhs1GNInterpolation)
    K.ref_interpolateVelocityToGhostNode.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _ip] + [_dp] * 9 + \
        [ctypes.c_int] * 6 + [ctypes.POINTER(RefInterpArrays)]
    ug = u.copy()
    for direc, (xc, yc, vel) in enumerate(((G["xu"], G["yu"], uB), (G["xv"], G["yv"], vB))):
        a, r = interp_arrays(nUV)
        K.ref_interpolateVelocityToGhostNode(direc, d(ug), 1, i(gU), d(bx), d(by), d(vel), d(yc), d(xc), d(bix),
                                             d(biy), d(ipx), d(ipy), i0, j0, ncx, ncy, nx, ny, ctypes.byref(r))
        for f in ("index1", "index2", "index3", "index4", "q1coef", "q2coef", "q3coef", "q4coef", "image_point_u"):
            out["ghost%d_%s" % (direc, f)] = a[f]
    out["u_ghost"] = ug
    # hybrid-node velocity from the ghost-filled field (luoIBM::rhs1HNInterpolation)
    K.ref_interpolateVelocityToHybridNode.argtypes = [ctypes.c_int, _dp, _dp, _ip] + [_dp] * 9 + \
        [ctypes.c_int] * 6 + [ctypes.POINTER(RefInterpArrays)]
    ustar = np.zeros(nUV)
    for direc, (xc, yc, vel) in enumerate(((G["xu"], G["yu"], uB), (G["xv"], G["yv"], vB))):
        a, r = interp_arrays(nUV)
        K.ref_interpolateVelocityToHybridNode(direc, d(ug), d(ustar), i(hU), d(bx), d(by), d(vel), d(yc), d(xc),
                                              d(bix), d(biy), d(ipx), d(ipy), i0, j0, ncx, ncy, nx, ny,
                                              ctypes.byref(r))
        for f in ("index1", "index2", "index3", "index4", "q1coef", "q2coef", "q3coef", "q4coef", "image_point_u"):
            out["hybrid%d_%s" % (direc, f)] = a[f]
    out["ustar"] = ustar
    # pressure: hybrid (pstar), weightP, ghost (set = true) - luoIBM::weightPressure
    uBk_a, vBk_a = np.full(n, uBk), np.full(n, vBk)
    K.ref_interpolatePressureToHybridNode.argtypes = [_dp, _dp, _dp, _ip] + [_dp] * 14 + [ctypes.c_int] * 6 + \
        [ctypes.c_double, ctypes.POINTER(RefInterpArrays)]
    pstar = np.zeros(nP)
    a, r = interp_arrays(nP)
    K.ref_interpolatePressureToHybridNode(d(p), d(pstar), d(ug), i(hP), d(bx), d(by), d(uB), d(uBk_a), d(vB),
                                          d(vBk_a), d(G["yu"]), d(G["yv"]), d(G["xu"]), d(G["xv"]), d(bpx), d(bpy),
                                          d(ppx), d(ppy), i0, j0, ncx, ncy, nx, ny, dt, ctypes.byref(r))
    for f in ("index1", "index2", "index3", "index4", "q1coef", "q2coef", "q3coef", "q4coef"):
        out["phybrid_" + f] = a[f]
    out["pstar"] = pstar
    K.ref_weight.argtypes = [ctypes.c_int, _dp, _dp, _ip, _ip] + [_dp] * 6 + [ctypes.c_int] * 6
    pw = p.copy()
    K.ref_weight(2, d(pw), d(pstar), i(gP), i(hP), d(G["yu"]), d(G["xv"]), d(bpx), d(bpy), d(ppx), d(ppy), i0, j0,
                 ncx, ncy, nx, ny)
    out["p_weighted"] = pw.copy()
    K.ref_interpolatePressureToGhostNode.argtypes = [_dp, ctypes.c_int, _dp, _ip, _dp, _dp, _dp] + [_dp] * 12 + \
        [_dp] + [ctypes.c_int] * 6 + [ctypes.c_double, ctypes.POINTER(RefInterpArrays)]
    dpdn, bip = np.zeros(nP), np.zeros(nP)
    a, r = interp_arrays(nP)
    K.ref_interpolatePressureToGhostNode(d(pw), 1, d(ug), i(gP), d(bx), d(by), d(dpdn), d(uB), d(uBk_a), d(vB),
                                         d(vBk_a), d(G["yu"]), d(G["yv"]), d(G["xu"]), d(G["xv"]), d(bpx), d(bpy),
                                         d(ppx), d(ppy), d(bip), i0, j0, ncx, ncy, nx, ny, dt, ctypes.byref(r))
    for f in ("index1", "index2", "index3", "index4", "q1coef", "q2coef", "q3coef", "q4coef"):
        out["pghost_" + f] = a[f]
    out.update(p_ghost=pw, dpdn=dpdn, body_intercept_p=bip)
    # velocity blending (weightUhat) on a random uhat
    uhat = 1.0 + 0.2 * rng.standard_normal(nUV)
    out["uhat_in"] = uhat.copy()
    K.ref_weight(0, d(uhat), d(ustar), i(gU), i(hU), d(G["yu"]), d(G["xu"]), d(bix), d(biy), d(ipx), d(ipy), i0,
                 j0, ncx, ncy, nx, ny)
    K.ref_weight(1, d(uhat), d(ustar), i(gU), i(hU), d(G["yv"]), d(G["xv"]), d(bix), d(biy), d(ipx), d(ipy), i0,
                 j0, ncx, ncy, nx, ny)
    out["uhat_weighted"] = uhat
    # inside velocity := body velocity (grid over numUV threads, luoIBM::zeroVelocity)
    ui = ug.copy()
    K.ref_setInsideVelocity.argtypes = [_ip, _dp, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    K.ref_setInsideVelocity(i(gU), d(ui), d(uB), d(vB), nx, ny, nUV)
    out["u_inside"] = ui
    # convective outflow update of the x+ boundary array
    xp = 1.0 + 0.1 * rng.standard_normal(2 * ny - 1)
    out["xp_in"] = xp.copy()
    K.ref_updateRobinBoundary.argtypes = [_dp, _dp, _dp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_int, ctypes.c_int]
    K.ref_updateRobinBoundary(d(ug), d(xp), d(G["dx"]), dt, 1.0, 1.0, nx, ny)
    out["xp_robin"] = xp
    # control-volume force
    uold = ug + 0.01 * rng.standard_normal(nUV)
    out["uold_in"] = uold
    fx, fy = ctypes.c_double(), ctypes.c_double()
    K.ref_calculateForce.argtypes = [_dp, _dp, _dp, _ip, ctypes.c_double, _dp, _dp, ctypes.c_double] + \
        [ctypes.c_int] * 6 + [_dp, _dp]
    K.ref_calculateForce(d(ug), d(uold), d(p), i(gU), nu, d(G["dx"]), d(G["dy"]), dt, nx, ny, i0, j0, ncx, ncy,
                         ctypes.byref(fx), ctypes.byref(fy))
    out["force"] = np.array([fx.value, fy.value])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name, "nx=%d ny=%d bb=%s ghostUV=%d hybridUV=%d ghostP=%d hybridP=%d" % (
        nx, ny, (i0, j0, ncx, ncy), (gU > 0).sum(), (hU > 0).sum(), (gP > 0).sum(), (hP > 0).sum()))


def fadlun_case(K, IO, name, folder, rng, nu, dt, scale=2.0):
    """The modified-Fadlun kernels (fadlunModified.cu) on the tags of a circle: LHS1 and
    LHS2 as the reference leaves them before its sort, the IB update of rhs1, rhs2
    and the masked projection."""
    nx, ny, G = ref_grid(IO, folder)
    nU, nV = (nx - 1) * ny, nx * (ny - 1)
    nUV, nP = nU + nV, nx * ny
    X, Y, _ = ref_body(IO, folder)
    n = len(X)
    mx = 0.0
    my = 0.0
    for v in X:
        mx += v
    for v in Y:
        my += v
    mx /= n
    my /= n
    i0, j0, ncx, ncy = bounding_box(X, Y, G["x"], G["y"], scale)
    bx = np.array([0.0 + (v - mx) for v in X])
    by = Y.copy()
    uB = np.zeros(n)
    vB = np.zeros(n)
    p_sized = {"ghostTagsP", "hybridTagsP", "distance_from_u_to_body", "distance_from_v_to_body",
               "body_intercept_p_x", "body_intercept_p_y", "image_point_p_x", "image_point_p_y",
               "x1_p", "y1_p", "x2_p", "y2_p"}
    arr = {}
    for f, _ in RefTagArrays._fields_:
        size = nP if f in p_sized else nUV
        arr[f] = np.zeros(size + 2 * max(nx, ny), np.int32 if "Tags" in f else np.float64)[:size].copy()
    ta = RefTagArrays(**{f: (i(arr[f]) if "Tags" in f else d(arr[f])) for f, _ in RefTagArrays._fields_})
    K.ref_tagPoints.argtypes = [ctypes.POINTER(RefTagArrays)] + [_dp] * 8 + [ctypes.c_int] * 7 + \
        [ctypes.c_double, ctypes.c_double]
    K.ref_tagPoints(ctypes.byref(ta), d(bx), d(by), d(uB), d(vB), d(G["xu"]), d(G["yu"]), d(G["xv"]), d(G["yv"]),
                    i0, j0, ncx, ncy, nx, ny, n, 0.0, my)
    out = {"nx": np.int32(nx), "ny": np.int32(ny), "nu": np.float64(nu), "dt": np.float64(dt),
           "bb": np.array([i0, j0, ncx, ncy], np.int32), "bx": bx, "by": by, "midY": np.float64(my)}
    out.update({"grid_" + k: v for k, v in G.items()})
    for f in ("ghostTagsUV", "ghostTagsP", "hybridTagsUV", "hybridTagsP", "hybridTagsUV2",
              "distance_from_intersection_to_node", "distance_between_nodes_at_IB", "uv",
              "distance_from_u_to_body", "distance_from_v_to_body"):
        out["tag_" + f] = arr[f].copy()
    gU, hU, h2U, gP, hP = (arr[k] for k in ("ghostTagsUV", "hybridTagsUV", "hybridTagsUV2", "ghostTagsP",
                                              "hybridTagsP"))
    dn, db, uv = (arr[k] for k in ("distance_from_intersection_to_node", "distance_between_nodes_at_IB", "uv"))
    du, dv = arr["distance_from_u_to_body"], arr["distance_from_v_to_body"]
    nnz1 = (nx - 1) * ny * 5 - 2 * ny - 2 * (nx - 1) + (ny - 1) * nx * 5 - 2 * (ny - 1) - 2 * nx
    r1, c1, v1 = np.zeros(nnz1, np.int32), np.zeros(nnz1, np.int32), np.zeros(nnz1)
    K.ref_fadlun_lhs1.argtypes = [_ip, _ip, _dp, ctypes.c_int, _ip, _ip, _ip, _dp, _dp, _dp, _dp, ctypes.c_double,
                                  ctypes.c_double, ctypes.c_int, ctypes.c_int]
    K.ref_fadlun_lhs1(i(r1), i(c1), d(v1), nnz1, i(hU), i(h2U), i(gU), d(dn), d(db), d(G["dx"]), d(G["dy"]), dt, nu,
                      nx, ny)
    out.update({"lhs1_row": r1, "lhs1_col": c1, "lhs1_val": v1})
    nnz2 = 5 * nx * ny - 2 * ny - 2 * nx
    r2, c2, v2 = np.zeros(nnz2, np.int32), np.zeros(nnz2, np.int32), np.zeros(nnz2)
    K.ref_fadlun_lhs2.argtypes = [_ip, _ip, _dp, ctypes.c_int, _dp, _dp, _ip, _ip, _dp, _dp, ctypes.c_int,
                                  ctypes.c_int, ctypes.c_double]
    K.ref_fadlun_lhs2(i(r2), i(c2), d(v2), nnz2, d(du), d(dv), i(gP), i(hP), d(G["dx"]), d(G["dy"]), nx, ny, dt)
    out.update({"lhs2_row": r2, "lhs2_col": c2, "lhs2_val": v2})
    rhs1 = rng.standard_normal(nUV)
    out["rhs1_in"] = rhs1.copy()
    K.ref_fadlun_update_rhs1.argtypes = [_ip, _ip, _dp, _dp, _dp, _dp, ctypes.c_int, ctypes.c_int]
    K.ref_fadlun_update_rhs1(i(hU), i(gU), d(rhs1), d(dn), d(db), d(uv), nx, ny)
    out["rhs1_out"] = rhs1
    uhat = 1.0 + 0.2 * rng.standard_normal(nUV)
    bcs = {k: 1.0 + 0.1 * rng.standard_normal(2 * ny - 1 if k in ("xm", "xp") else 2 * nx - 1)
           for k in ("xm", "xp", "ym", "yp")}
    out["uhat_in"] = uhat
    out.update({"bc_" + k: v for k, v in bcs.items()})
    rhs2 = np.zeros(nP)
    K.ref_fadlun_rhs2.argtypes = [_dp, _dp, _ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, ctypes.c_int,
                                  ctypes.c_int]
    K.ref_fadlun_rhs2(d(rhs2), d(uhat), i(gP), i(hP), i(gU), d(du), d(dv), d(bcs["ym"]), d(bcs["yp"]),
                      d(bcs["xm"]), d(bcs["xp"]), d(G["dx"]), d(G["dy"]), nx, ny)
    out["rhs2"] = rhs2
    p = 0.1 * rng.standard_normal(nP)
    out["p_in"] = p
    u = np.zeros(nUV)
    uold = np.zeros(nUV)
    K.ref_fadlun_project.argtypes = [_dp, _dp, _dp, _dp, _ip, _dp, _dp, ctypes.c_double, ctypes.c_int, ctypes.c_int]
    K.ref_fadlun_project(d(u), d(uhat), d(uold), d(p), i(gP), d(G["dx"]), d(G["dy"]), dt, nx, ny)
    out["u_projected"] = u
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name, "nx=%d ny=%d ghostUV=%d hybridUV=%d ghostP=%d hybridP=%d" % (
        nx, ny, (gU > 0).sum(), (hU > 0).sum(), (gP > 0).sum(), (hP > 0).sum()))


def iter_case(K, IO, name, folder, rng, nu, dt, uB0=0.25, vB0=-0.15, uBk=0.2, vBk=-0.1, scale=2.0):
    """The embedded method's per-step kernels (luo_iter/*.cu) on the tags of a circle:
    alpha, the velocity and pressure stencils of the set = false interpolations, LHS1
    and LHS2 on zeroed arrays (unsorted), ns_rhs, interp_rhs and the rhs updates.  The
    body velocity differs from its previous value so that the dp/dn terms are pinned."""
    nx, ny, G = ref_grid(IO, folder)
    nU, nV = (nx - 1) * ny, nx * (ny - 1)
    nUV, nP = nU + nV, nx * ny
    X, Y, _ = ref_body(IO, folder)
    n = len(X)
    mx = 0.0
    my = 0.0
    for v in X:
        mx += v
    for v in Y:
        my += v
    mx /= n
    my /= n
    i0, j0, ncx, ncy = bounding_box(X, Y, G["x"], G["y"], scale)
    bx = np.array([0.0 + (v - mx) for v in X])
    by = Y.copy()
    uB, vB = np.full(n, uB0), np.full(n, vB0)
    p_sized = {"ghostTagsP", "hybridTagsP", "distance_from_u_to_body", "distance_from_v_to_body",
               "body_intercept_p_x", "body_intercept_p_y", "image_point_p_x", "image_point_p_y",
               "x1_p", "y1_p", "x2_p", "y2_p"}
    arr = {}
    for f, _ in RefTagArrays._fields_:
        size = nP if f in p_sized else nUV
        arr[f] = np.zeros(size + 2 * max(nx, ny), np.int32 if "Tags" in f else np.float64)[:size].copy()
    ta = RefTagArrays(**{f: (i(arr[f]) if "Tags" in f else d(arr[f])) for f, _ in RefTagArrays._fields_})
    K.ref_tagPoints.argtypes = [ctypes.POINTER(RefTagArrays)] + [_dp] * 8 + [ctypes.c_int] * 7 + \
        [ctypes.c_double, ctypes.c_double]
    K.ref_tagPoints(ctypes.byref(ta), d(bx), d(by), d(uB), d(vB), d(G["xu"]), d(G["yu"]), d(G["xv"]), d(G["yv"]),
                    i0, j0, ncx, ncy, nx, ny, n, 0.0, my)
    out = {"nx": np.int32(nx), "ny": np.int32(ny), "nu": np.float64(nu), "dt": np.float64(dt),
           "bb": np.array([i0, j0, ncx, ncy], np.int32), "bx": bx, "by": by, "uB": uB, "vB": vB,
           "uBk": np.float64(uBk), "vBk": np.float64(vBk), "midY": np.float64(my)}
    out.update({"grid_" + k: v for k, v in G.items()})
    gU, hU, gP, hP = (arr[k] for k in ("ghostTagsUV", "hybridTagsUV", "ghostTagsP", "hybridTagsP"))
    bix, biy, ipx, ipy = (arr[k] for k in ("body_intercept_x", "body_intercept_y", "image_point_x", "image_point_y"))
    bpx, bpy, ppx, ppy = (arr[k] for k in ("body_intercept_p_x", "body_intercept_p_y", "image_point_p_x",
                                           "image_point_p_y"))
    for f in ("ghostTagsUV", "ghostTagsP", "hybridTagsUV", "hybridTagsP"):
        out["tag_" + f] = arr[f].copy()

    def interp_arrays(size):
        a = {f: np.zeros(size, np.int32 if f.startswith("index") else np.float64) for f, _ in RefInterpArrays._fields_}
        r = RefInterpArrays(**{f: (i(a[f]) if f.startswith("index") else d(a[f])) for f, _ in RefInterpArrays._fields_})
        return a, r

    stencil = ("index1", "index2", "index3", "index4", "q1coef", "q2coef", "q3coef", "q4coef", "q1", "q2", "q3", "q4")
    u = 1.0 + 0.2 * rng.standard_normal(nUV)
    out["u_in"] = u.copy()
    # luo_iter::intermediate_velocity_interpolation_setup: four set = false launches
    # into one set of stencil arrays
    a, r = interp_arrays(nUV)
    K.ref_interpolateVelocityToGhostNode.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _ip] + [_dp] * 9 + \
        [ctypes.c_int] * 6 + [ctypes.POINTER(RefInterpArrays)]
    K.ref_interpolateVelocityToHybridNode.argtypes = [ctypes.c_int, _dp, _dp, _ip] + [_dp] * 9 + \
        [ctypes.c_int] * 6 + [ctypes.POINTER(RefInterpArrays)]
    for direc, (xc, yc, vel) in enumerate(((G["xu"], G["yu"], uB), (G["xv"], G["yv"], vB))):
        K.ref_interpolateVelocityToGhostNode(direc, d(u), 0, i(gU), d(bx), d(by), d(vel), d(yc), d(xc), d(bix),
                                             d(biy), d(ipx), d(ipy), i0, j0, ncx, ncy, nx, ny, ctypes.byref(r))
    ustar = np.zeros(nUV)
    for direc, (xc, yc, vel) in enumerate(((G["xu"], G["yu"], uB), (G["xv"], G["yv"], vB))):
        K.ref_interpolateVelocityToHybridNode(direc, d(u), d(ustar), i(hU), d(bx), d(by), d(vel), d(yc), d(xc),
                                              d(bix), d(biy), d(ipx), d(ipy), i0, j0, ncx, ncy, nx, ny,
                                              ctypes.byref(r))
    for f in stencil:
        out["vel_" + f] = a[f].copy()
    K.ref_iter_alpha.argtypes = [ctypes.c_int, _dp, _ip, _ip] + [_dp] * 6 + [ctypes.c_int] * 5
    alpha = np.zeros(nUV)
    K.ref_iter_alpha(0, d(alpha), i(gU), i(hU), d(G["yu"]), d(G["xu"]), d(bix), d(biy), d(ipx), d(ipy), i0, j0, ncx,
                     nx, ny)
    K.ref_iter_alpha(1, d(alpha), i(gU), i(hU), d(G["yv"]), d(G["xv"]), d(bix), d(biy), d(ipx), d(ipy), i0, j0, ncx,
                     nx, ny)
    out["alpha_uv"] = alpha.copy()
    nnz1 = (nx - 1) * ny * 5 - 2 * ny - 2 * (nx - 1) + nx * (ny - 1) * 5 - 2 * nx - 2 * (ny - 1) + int((hU > 0).sum())
    r1, c1, v1 = np.zeros(nnz1, np.int32), np.zeros(nnz1, np.int32), np.zeros(nnz1)
    ns1, in1, cnt1 = np.zeros(nUV), np.zeros(nUV), np.zeros(nUV, np.int32)
    K.ref_iter_lhs1.argtypes = [_ip, _ip, _dp, ctypes.c_int, _dp, _dp, ctypes.c_double, ctypes.c_double,
                                ctypes.c_int, ctypes.c_int, _ip, _ip, _dp, _dp, _ip, _ip, _ip, _ip, _ip] + \
        [_dp] * 15 + [ctypes.c_int] * 4
    K.ref_iter_lhs1.restype = ctypes.c_int
    got = K.ref_iter_lhs1(i(r1), i(c1), d(v1), nnz1, d(G["dx"]), d(G["dy"]), dt, nu, nx, ny, i(hU), i(gU), d(ns1),
                          d(in1), i(cnt1), i(a["index1"]), i(a["index2"]), i(a["index3"]), i(a["index4"]),
                          d(G["xu"]), d(G["yu"]), d(G["xv"]), d(G["yv"]), d(alpha), d(uB), d(vB), d(a["q1coef"]),
                          d(a["q2coef"]), d(a["q3coef"]), d(a["q4coef"]), d(a["q1"]), d(a["q2"]), d(a["q3"]),
                          d(a["q4"]), i0, j0, ncx, ncy)
    assert got == nnz1, (got, nnz1)
    out.update({"lhs1_row": r1, "lhs1_col": c1, "lhs1_val": v1, "ns_rhs1": ns1, "interp_rhs1": in1})
    rhs1 = rng.standard_normal(nUV)
    out["rhs1_in"] = rhs1.copy()
    K.ref_iter_update_rhs1.argtypes = [_dp, _dp, _dp, ctypes.c_int, ctypes.c_int]
    K.ref_iter_update_rhs1(d(rhs1), d(ns1), d(in1), nx, ny)
    out["rhs1_out"] = rhs1
    # luo_iter::poisson_interpolation_setup: stencil arrays zeroed, then the ghost
    # (set = false, dp/dn) and hybrid pressure launches
    p = 0.1 * rng.standard_normal(nP)
    out["p_in"] = p.copy()
    uBk_a, vBk_a = np.full(n, uBk), np.full(n, vBk)
    a, r = interp_arrays(nUV)
    dpdn, bip = np.zeros(nP), np.zeros(nP)
    K.ref_interpolatePressureToGhostNode.argtypes = [_dp, ctypes.c_int, _dp, _ip, _dp, _dp, _dp] + [_dp] * 12 + \
        [_dp] + [ctypes.c_int] * 6 + [ctypes.c_double, ctypes.POINTER(RefInterpArrays)]
    K.ref_interpolatePressureToGhostNode(d(p), 0, d(u), i(gP), d(bx), d(by), d(dpdn), d(uB), d(uBk_a), d(vB),
                                         d(vBk_a), d(G["yu"]), d(G["yv"]), d(G["xu"]), d(G["xv"]), d(bpx), d(bpy),
                                         d(ppx), d(ppy), d(bip), i0, j0, ncx, ncy, nx, ny, dt, ctypes.byref(r))
    K.ref_interpolatePressureToHybridNode.argtypes = [_dp, _dp, _dp, _ip] + [_dp] * 14 + [ctypes.c_int] * 6 + \
        [ctypes.c_double, ctypes.POINTER(RefInterpArrays)]
    pstar = np.zeros(nP)
    K.ref_interpolatePressureToHybridNode(d(p), d(pstar), d(u), i(hP), d(bx), d(by), d(uB), d(uBk_a), d(vB),
                                          d(vBk_a), d(G["yu"]), d(G["yv"]), d(G["xu"]), d(G["xv"]), d(bpx), d(bpy),
                                          d(ppx), d(ppy), i0, j0, ncx, ncy, nx, ny, dt, ctypes.byref(r))
    for f in stencil:
        out["p_" + f] = a[f][:nP].copy()
    out["dpdn"] = dpdn.copy()
    alpha_p = np.zeros(nP)
    K.ref_iter_alpha(2, d(alpha_p), i(gP), i(hP), d(G["yu"]), d(G["xv"]), d(bpx), d(bpy), d(ppx), d(ppy), i0, j0,
                     ncx, nx, ny)
    out["alpha_p"] = alpha_p.copy()
    nnz2 = nx * ny * 5 - 2 * nx - 2 * ny + int((hP > 0).sum())
    r2, c2, v2 = np.zeros(nnz2, np.int32), np.zeros(nnz2, np.int32), np.zeros(nnz2)
    ns2, in2, cnt2 = np.zeros(nP), np.zeros(nP), np.zeros(nP, np.int32)
    K.ref_iter_lhs2.argtypes = [_ip, _ip, _dp, ctypes.c_int, _dp, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                _ip, _dp, _dp, _ip, _ip, _dp, _dp, _ip, _ip, _ip, _ip] + [_dp] * 8 + \
        [ctypes.c_int] * 4
    K.ref_iter_lhs2.restype = ctypes.c_int
    got = K.ref_iter_lhs2(i(r2), i(c2), d(v2), nnz2, d(G["dx"]), d(G["dy"]), nx, ny, dt, i(cnt2), d(ns2), d(in2),
                          i(hP), i(gP), d(alpha_p), d(dpdn), i(a["index1"]), i(a["index2"]), i(a["index3"]),
                          i(a["index4"]), d(a["q1coef"]), d(a["q2coef"]), d(a["q3coef"]), d(a["q4coef"]), d(a["q1"]),
                          d(a["q2"]), d(a["q3"]), d(a["q4"]), i0, j0, ncx, ncy)
    assert got == nnz2, (got, nnz2)
    out.update({"lhs2_row": r2, "lhs2_col": c2, "lhs2_val": v2, "ns_rhs2": ns2, "interp_rhs2": in2})
    rhs2 = rng.standard_normal(nP)
    out["rhs2_in"] = rhs2.copy()
    K.ref_iter_update_rhs2.argtypes = [_dp, _dp, _dp, ctypes.c_int, ctypes.c_int]
    K.ref_iter_update_rhs2(d(rhs2), d(ns2), d(in2), nx, ny)
    out["rhs2_out"] = rhs2
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name, "nx=%d ny=%d ghostUV=%d hybridUV=%d ghostP=%d hybridP=%d" % (
        nx, ny, (gU > 0).sum(), (hU > 0).sum(), (gP > 0).sum(), (hP > 0).sum()))


def surface_case(K, IO, name, folder, ib_name, nu):
    """luo_base::luoForce, the surface-integral force the reference's step leaves
    unused, on the state of an external-method fixture: its tags, body-intercept
    pressures and ghost-filled velocity, with the domain's mid_h."""
    nx, ny, h = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
    IO.ref_parse_domain(os.path.join(folder, "domain.json").encode(), ctypes.byref(nx), ctypes.byref(ny),
                        ctypes.byref(h))
    z = dict(np.load(os.path.join(HERE, ib_name + ".npz")))
    assert (nx.value, ny.value) == (int(z["nx"]), int(z["ny"]))
    n = len(z["bx"])
    i0, j0, ncx, ncy = (int(v) for v in z["bb"])
    args = [z["body_intercept_p"], z["tag_body_intercept_p_x"], z["tag_body_intercept_p_y"], z["bx"], z["by"],
            z["grid_xu"], z["grid_yu"], z["grid_xv"], z["grid_yv"]]
    args = [np.ascontiguousarray(a, np.float64) for a in args]
    gP = np.ascontiguousarray(z["tag_ghostTagsP"], np.int32)
    u = np.ascontiguousarray(z["u_ghost"], np.float64)
    uB, vB = np.ascontiguousarray(z["uB"]), np.ascontiguousarray(z["vB"])
    # the reference reads an unset index where a point has no intercept on one side:
    # only cases where every point has both are run through it
    sys.path.insert(0, ROOT)
    import oracle
    t0, _, _ = oracle.surface_force(1, z["bx"], z["by"], float(uB[0]), float(vB[0]), u, z["body_intercept_p"],
                                    z["tag_body_intercept_p_x"], z["tag_body_intercept_p_y"], gP, z["grid_xu"],
                                    z["grid_yu"], z["grid_xv"], z["grid_yv"], (i0, j0, ncx, ncy), nx.value, ny.value,
                                    float(z["midX"]), float(z["midY"]), nu, h.value)
    assert np.all(np.isfinite(t0[:n])), "a body point without intercepts on both sides"
    terms = np.zeros(3 * n)
    fx, fy = ctypes.c_double(), ctypes.c_double()
    K.ref_luoForce.argtypes = [_dp] * 9 + [_ip, _dp, _dp, _dp] + [ctypes.c_int] * 7 + [ctypes.c_double] * 4 + \
        [_dp, _dp, _dp]
    K.ref_luoForce(*(d(a) for a in args), i(gP), d(u), d(uB), d(vB), i0, j0, ncx, ncy, n, nx.value, ny.value,
                   float(z["midX"]), float(z["midY"]), nu, h.value, d(terms), ctypes.byref(fx), ctypes.byref(fy))
    out = {"ib_fixture": np.array(ib_name), "mid_h": np.float64(h.value), "nu": np.float64(nu), "terms": terms,
           "force": np.array([fx.value, fy.value])}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name, "F = (%.6e, %.6e)" % (fx.value, fy.value))


def recorded_run(ref_root, name, case_dir):
    """Outputs the reference's authors recorded for one of its validation cases
    (validation/<case_dir>: forces_init = time, Fx, Fy for the first 1000 steps;
    midPosition_init = step, X, Y, U, V; iterations_init = velocity and Poisson
    iterations per step, which holds two lines per step).  The case's parameters are
    restated in the test that uses the fixture."""
    d = os.path.join(ref_root, "validation", case_dir)

    def table(fname, skip):
        rows = []
        with open(os.path.join(d, fname)) as f:
            for k, line in enumerate(f):
                if k < skip or not line.strip():
                    continue
                rows.append([float(v) for v in line.replace(",", " ").split()])
        return np.array(rows)

    out = {"forces": table("forces_init", 1), "mid_position": table("midPosition_init", 1),
           "iterations": table("iterations_init", 0)}
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name, {k: v.shape for k, v in out.items()})


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CUIBM_REF_SRC"),
                    help="src folder of a cuIBM source tree (default: $CUIBM_REF_SRC)")
    ap.add_argument("--only", default=None, help="generate one group: fadlun, iter, surface, recorded")
    a = ap.parse_args()
    if not a.ref:
        ap.error("give --ref <cuIBM>/src or set CUIBM_REF_SRC")
    if a.only == "recorded":  # data files of the reference tree, no build needed
        recorded_run(os.path.dirname(os.path.abspath(a.ref)), "recorded_osc_static_external",
                     "osc/static/external")
        return
    K, IO = ref_libs(a.ref)
    if a.only == "surface":
        with tempfile.TemporaryDirectory() as tmp:
            # the case folders of ib_circle48 and ib_circle101
            f = os.path.join(tmp, "ib1")
            cases.cylinder(f, h=0.05, ratio=1.1, extent=2.0, core=0.6, points=48, nu=0.02, dt=0.01, nt=1)
            surface_case(K, IO, "surface_circle48", f, "ib_circle48", nu=0.02)
            f = os.path.join(tmp, "ib2")
            cases.cylinder(f, h=0.025, ratio=1.08, extent=2.5, core=0.7, points=101, nu=0.02, dt=0.005, nt=1,
                           radius=0.43)
            surface_case(K, IO, "surface_circle101", f, "ib_circle101", nu=0.02)
        return
    if a.only == "fadlun":
        with tempfile.TemporaryDirectory() as tmp:
            rng = np.random.default_rng(20261204)
            f = os.path.join(tmp, "fad1")
            cases.cylinder(f, h=0.05, ratio=1.1, extent=2.0, core=0.6, points=48, nu=0.02, dt=0.01, nt=1)
            fadlun_case(K, IO, "fadlun_circle48", f, rng, nu=0.02, dt=0.01)
            f = os.path.join(tmp, "fad2")
            cases.cylinder(f, h=0.025, ratio=1.08, extent=2.5, core=0.7, points=101, nu=0.02, dt=0.005, nt=1,
                           radius=0.43)
            fadlun_case(K, IO, "fadlun_circle101", f, rng, nu=0.02, dt=0.005)
        return
    if a.only == "iter":
        with tempfile.TemporaryDirectory() as tmp:
            rng = np.random.default_rng(20261205)
            f = os.path.join(tmp, "it1")
            cases.cylinder(f, h=0.05, ratio=1.1, extent=2.0, core=0.6, points=48, nu=0.02, dt=0.01, nt=1)
            iter_case(K, IO, "iter_circle48", f, rng, nu=0.02, dt=0.01)
            f = os.path.join(tmp, "it2")
            cases.cylinder(f, h=0.025, ratio=1.08, extent=2.5, core=0.7, points=101, nu=0.02, dt=0.005, nt=1,
                           radius=0.43)
            iter_case(K, IO, "iter_circle101", f, rng, nu=0.02, dt=0.005, uB0=0.1, vB0=0.05, uBk=0.1, vBk=0.05)
        return
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
        # external-method kernels around a circle (two resolutions / point counts)
        f = os.path.join(tmp, "ib1")
        cases.cylinder(f, h=0.05, ratio=1.1, extent=2.0, core=0.6, points=48, nu=0.02, dt=0.01, nt=1)
        ib_case(K, IO, "ib_circle48", f, rng, nu=0.02, dt=0.01)
        f = os.path.join(tmp, "ib2")
        cases.cylinder(f, h=0.025, ratio=1.08, extent=2.5, core=0.7, points=101, nu=0.02, dt=0.005, nt=1,
                       radius=0.43)
        ib_case(K, IO, "ib_circle101", f, rng, nu=0.02, dt=0.005, uB0=0.0, vB0=0.0, uBk=0.0, vBk=0.0)
        # grids and bodies of the benchmark cylinders (Re 40 and Re 550)
        f = os.path.join(tmp, "cyl40")
        cases.cylinder(f, h=0.02, ratio=1.03, points=157, nt=1)
        grid_case(IO, "grid_cylinder_re40", f)
        f = os.path.join(tmp, "cyl550")
        cases.cylinder(f, h=0.005, ratio=1.01, points=629, nt=1)
        grid_case(IO, "grid_cylinder_re550", f)


if __name__ == "__main__":
    main()
