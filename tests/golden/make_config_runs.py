"""Writes the whole-run fixtures of the benchmark configurations (tests/golden/config_*.npz)
with the CPU oracle (oracle/: the restated kernels, FP64, both linear systems solved
by sparse LU, so that any converged solver can be compared with them).

  config_cavity64.npz       lid-driven cavity 64 x 64, Re 100, dt 0.01, plain method:
                            u and p after 1000 steps (and after 100)
  config_cylinder_re40.npz  impulsively started cylinder Re 40, 270 x 270 (h 0.02,
                            stretched 1.03 to [-15, 15]^2), 157 points, external method,
                            dt 0.01: C_D and C_L of every step, u and p after 2000 steps
  config_cylinder_re550.npz cylinder Re 550, 922 x 922 (h 0.005, stretched 1.01), 629
                            points, external method, dt 0.002: C_D and C_L of steps
                            1-40, u and p after 40 steps on every 8th node in each
                            direction, and the fields' L2 norms

C_D = 2 Fx and C_L = 2 Fy (unit diameter and free-stream speed).  Run from the
repository root:  python tests/golden/make_config_runs.py [--only cavity64|re40|re550]
(about 1, 3 and 5 minutes on 8 cores).
"""
import argparse
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from cuibm_gb300 import cases  # noqa: E402

STRIDE_RE550 = 8  # subsampling of the Re 550 fields


def cavity64(tmp):
    f = cases.cavity(os.path.join(tmp, "cavity64"), n=64, nu=0.01, dt=0.01, nt=1000)
    s = oracle.PlainSolver(f, solve="direct")
    out = {}
    for k in range(1, 1001):
        s.step()
        if k in (100, 1000):
            out["u_%d" % k], out["p_%d" % k] = s.u.copy(), s.p.copy()
    return out


def cylinder_re40(tmp):
    f = cases.cylinder(os.path.join(tmp, "re40"), h=0.02, ratio=1.03, points=157, nu=1.0 / 40, dt=0.01, nt=2000)
    s = oracle.LuoSolver(f, solve="direct")
    cd, cl, out = [], [], {}
    for k in range(1, 2001):
        s.step()
        cd.append(2 * s.fx)
        cl.append(2 * s.fy)
        if k == 2000:
            out["u_%d" % k], out["p_%d" % k] = s.u.copy(), s.p.copy()
    out["cd"], out["cl"] = np.array(cd), np.array(cl)
    return out


def subsample(g, u, p, stride):
    """u, v and p on every stride-th node of their own grids (row-major, u block first)."""
    uu = u[:g.nU].reshape(g.ny, g.nx - 1)[::stride, ::stride].ravel()
    vv = u[g.nU:].reshape(g.ny - 1, g.nx)[::stride, ::stride].ravel()
    pp = p.reshape(g.ny, g.nx)[::stride, ::stride].ravel()
    return np.concatenate([uu, vv]), pp


def cylinder_re550(tmp):
    f = cases.cylinder(os.path.join(tmp, "re550"), h=0.005, ratio=1.01, points=629, nu=1.0 / 550, dt=0.002,
                       nt=40)
    s = oracle.LuoSolver(f, solve="direct")
    cd, cl = [], []
    for _ in range(40):
        s.step()
        cd.append(2 * s.fx)
        cl.append(2 * s.fy)
    us, ps = subsample(s.g, s.u, s.p, STRIDE_RE550)
    return {"cd": np.array(cd), "cl": np.array(cl), "u_sub": us, "p_sub": ps, "stride": STRIDE_RE550,
            "u_norm": np.linalg.norm(s.u), "p_norm": np.linalg.norm(s.p)}


RUNS = {"cavity64": cavity64, "re40": cylinder_re40, "re550": cylinder_re550}
NAMES = {"cavity64": "config_cavity64", "re40": "config_cylinder_re40", "re550": "config_cylinder_re550"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=sorted(RUNS), default=None)
    a = ap.parse_args()
    with tempfile.TemporaryDirectory() as tmp:
        for key in ([a.only] if a.only else list(RUNS)):
            t = time.time()
            out = RUNS[key](tmp)
            path = os.path.join(HERE, NAMES[key] + ".npz")
            np.savez_compressed(path, **out)
            print("wrote %s in %.0f s (%d KB)" % (path, time.time() - t, os.path.getsize(path) // 1024))


if __name__ == "__main__":
    main()
