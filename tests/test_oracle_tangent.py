"""The oracle's tangent-linear model of the embedded method's step (oracle/tangent.py,
the restated step run on dual numbers) against central finite differences of the
plain oracle, on a small oscillating cylinder in fluid at rest: the derivative of the
period-averaged drag J = (2 / nt) sum_n Fx^n with respect to the viscosity, the
amplitude of the prescribed body velocity (uCoefficient, the path held fixed) and the
per-point body-velocity offsets.  This pins the FP64 tangent-linear reference that
the GPU adjoint is checked against."""
import os

import numpy as np
import pytest

import oracle
from cuibm_gb300 import cases
from oracle import tangent

NT = 12
REL_STEP = 1e-6  # central differences: J(p (1 + h)) - J(p (1 - h)) over 2 h p
RTOL = 1e-6      # tangent vs finite differences (truncation ~h^2, rounding ~1e-16 / h)
POINTS = 48


def osc_case(folder, um=0.5, period=1.0):
    w = 2 * np.pi / period
    motion = {"xCoefficient": um / w, "uCoefficient": um, "xfrequency": 1.0 / period, "xPhase": -np.pi / 2,
              "uPhase": -np.pi / 2}
    return cases.cylinder(folder, h=0.05, ratio=1.1, extent=3.0, core=0.6, points=POINTS, nu=0.02, dt=0.01, nt=NT,
                          method="OSC_CYLINDER", quiescent=True, motion=motion)


def drag(folder, nu=None, ucoef=None, off=None):
    s = oracle.EmbeddedSolver(folder, solve="direct", vel_offset=off)
    if nu is not None:
        s.nu = nu
    if ucoef is not None:
        s.coef["uCoefficient"] = ucoef
        s.uB = np.full(POINTS, s.motion(0)[1]) + s.vel_offset[0]
    J = 0.0
    for _ in range(NT):
        s.step()
        J += 2.0 / NT * s.fx
    return J


def tangent_of(folder, **direction):
    d = tangent.DualSolver(folder)
    d.direction(**direction)
    for _ in range(NT):
        d.step_dual(wx=2.0 / NT)
    return d


@pytest.fixture(scope="module")
def case(tmp_path_factory):
    return osc_case(str(tmp_path_factory.mktemp("osc") / "c"))


def test_dual_step_values_are_the_plain_step(case):
    s = oracle.EmbeddedSolver(case, solve="direct")
    d = tangent_of(case, d_nu=1.0)
    for _ in range(NT):
        s.step()
    assert np.array_equal(d.u, s.u) and np.array_equal(d.p, s.p) and d.fx == s.fx


@pytest.mark.parametrize("param", ["nu", "ucoef", "offu0", "offv0"])
def test_tangent_matches_central_differences(case, param):
    s = oracle.EmbeddedSolver(case, solve="direct")
    nu0, uc0 = s.nu, s.coef["uCoefficient"]
    unit = np.eye(POINTS)[0]
    zero = np.zeros(POINTS)
    if param == "nu":
        d = tangent_of(case, d_nu=1.0)
        h = REL_STEP * nu0
        fd = (drag(case, nu=nu0 + h) - drag(case, nu=nu0 - h)) / (2 * h)
    elif param == "ucoef":
        d = tangent_of(case, d_ucoef=1.0)
        h = REL_STEP * uc0
        fd = (drag(case, ucoef=uc0 + h) - drag(case, ucoef=uc0 - h)) / (2 * h)
    elif param == "offu0":
        d = tangent_of(case, d_offu=unit)
        h = REL_STEP
        fd = (drag(case, off=(h * unit, zero)) - drag(case, off=(-h * unit, zero))) / (2 * h)
    else:
        d = tangent_of(case, d_offv=unit)
        h = REL_STEP
        fd = (drag(case, off=(zero, h * unit)) - drag(case, off=(zero, -h * unit))) / (2 * h)
    assert abs(d.dJ - fd) <= RTOL * abs(fd) + 1e-12, (param, d.dJ, fd)


def test_offsets_of_other_points_do_not_act(case):
    """The reference's kernels read the body velocity of point 0 only (uB[0]): an offset
    of any other point changes nothing, and its derivative is exactly zero."""
    unit = np.eye(POINTS)[7]
    d = tangent_of(case, d_offu=unit, d_offv=unit)
    assert d.dJ == 0.0
    assert drag(case, off=(1e-3 * unit, 1e-3 * unit)) == drag(case)
