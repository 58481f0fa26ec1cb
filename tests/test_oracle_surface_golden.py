"""The oracle's surface-integral force (luo_base::luoForce, left unused by the
reference's step) against the reference's own kernels run on the CPU
(tests/golden/surface_*.npz, made by tests/golden/make_golden.py --only surface
from the state of the ib_* fixtures).  The pressures and normal derivatives agree
bit for bit; the forces, summed in point order on both sides, too.  The corrected
form (mode 2) has no reference counterpart: it is checked here to reduce to mode
1 where the two index slips do not matter, and on the GPU against this oracle."""
import os

import numpy as np
import pytest

import oracle


def state(golden_dir, name):
    s = dict(np.load(os.path.join(golden_dir, name + ".npz")))
    z = dict(np.load(os.path.join(golden_dir, str(s["ib_fixture"]) + ".npz")))
    return s, z


def run(mode, s, z, **over):
    a = dict(bx=z["bx"], by=z["by"], uB0=float(z["uB"][0]), vB0=float(z["vB"][0]), u=z["u_ghost"],
             bip=z["body_intercept_p"], bip_x=z["tag_body_intercept_p_x"], bip_y=z["tag_body_intercept_p_y"],
             ghostTagsP=z["tag_ghostTagsP"], xu=z["grid_xu"], yu=z["grid_yu"], xv=z["grid_xv"], yv=z["grid_yv"],
             bb=z["bb"], nx=int(z["nx"]), ny=int(z["ny"]), midX=float(z["midX"]), midY=float(z["midY"]),
             nu=float(s["nu"]), mid_h=float(s["mid_h"]))
    a.update(over)
    return oracle.surface_force(mode, **a)


@pytest.mark.parametrize("name", ["surface_circle48", "surface_circle101"])
def test_surface_force_matches_reference(golden_dir, name):
    s, z = state(golden_dir, name)
    terms, fx, fy = run(1, s, z)
    assert np.array_equal(terms, s["terms"])
    assert (fx, fy) == tuple(s["force"])


@pytest.mark.parametrize("name", ["surface_circle48", "surface_circle101"])
def test_corrected_surface_force(golden_dir, name):
    s, z = state(golden_dir, name)
    n = len(z["bx"])
    t1, _, _ = run(1, s, z)
    t2, fx2, fy2 = run(2, s, z)
    # du/dn reads the u block the same way in both forms
    assert np.array_equal(t1[n:2 * n], t2[n:2 * n])
    # with the box's j start equal to its i start, the pressure search is the same
    bb = np.array(z["bb"]).copy()
    bb[1] = bb[0]
    t1s, _, _ = run(1, s, z, bb=bb)
    t2s, _, _ = run(2, s, z, bb=bb)
    assert np.array_equal(t1s[:n], t2s[:n])
    # dv/dn of the corrected form is the bilinear v at the extended point: a uniform
    # v field gives a derivative of (v - vB) / dn exactly
    nU = (int(z["nx"]) - 1) * int(z["ny"])
    u = np.array(z["u_ghost"]).copy()
    u[nU:] = 0.75
    t2u, _, _ = run(2, s, z, u=u)
    dn = float(s["mid_h"]) * np.sqrt(2.0)
    assert np.allclose(t2u[2 * n:], (0.75 - float(z["vB"][0])) / dn, rtol=1e-12, atol=1e-12)
    assert np.isfinite(fx2) and np.isfinite(fy2)
