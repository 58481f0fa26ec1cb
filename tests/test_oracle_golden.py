"""The oracle restatement against the reference's own code (golden fixtures).

tests/golden/*.npz were produced by tests/golden/make_golden.py, which runs the
reference's kernel files and grid/body parsers compiled for the CPU.  Every
comparison here is bit-exact: the oracle keeps the reference's operation
order and is compiled without fused multiply-add.
"""
import os

import numpy as np
import pytest

import oracle


def bits_equal(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


def load(golden_dir, name):
    path = os.path.join(golden_dir, name + ".npz")
    return dict(np.load(path))


def grid_of(z):
    return oracle.Grid.from_arrays(z["grid_x"], z["grid_dx"], z["grid_xu"], z["grid_y"], z["grid_dy"], z["grid_yv"])


NS_CASES = ["ns_stretched", "ns_cavity16"]


@pytest.mark.parametrize("name", NS_CASES)
def test_convection_diffusion_rhs(golden_dir, name):
    z = load(golden_dir, name)
    g = grid_of(z)
    bc = (z["xm"], z["xp"], z["ym"], z["yp"])
    nu, dt = float(z["nu"]), float(z["dt"])
    N = oracle.generate_N(z["u"], g, bc)
    assert bits_equal(N, z["N"])
    L = oracle.generate_L(z["u"], g, bc, nu)
    assert bits_equal(L, z["L"])
    b1 = oracle.generate_bc1(z["u"], g, bc, nu, dt)
    assert bits_equal(b1, z["bc1"])
    r = oracle.generate_rhs(z["L"], z["Nold"], z["N"], z["u"], z["bc1"], dt)
    assert bits_equal(r, z["rhs1"])


@pytest.mark.parametrize("name", NS_CASES)
def test_operators_coo(golden_dir, name):
    z = load(golden_dir, name)
    g = grid_of(z)
    nu, dt = float(z["nu"]), float(z["dt"])
    r, c, v = oracle.lhs1_coo(g, dt, nu)
    for tag in ("ns", "luo"):  # luoIBM's LHS1 rows equal the plain ones
        assert np.array_equal(r, z["lhs1_%s_row" % tag]) and np.array_equal(c, z["lhs1_%s_col" % tag])
        assert bits_equal(v, z["lhs1_%s_val" % tag])
    for tag, pin in (("ns", True), ("luo", False)):
        r, c, v = oracle.lhs2_coo(g, dt, centre_pin=pin)
        assert np.array_equal(r, z["lhs2_%s_row" % tag]) and np.array_equal(c, z["lhs2_%s_col" % tag])
        assert bits_equal(v, z["lhs2_%s_val" % tag])


@pytest.mark.parametrize("name", NS_CASES)
def test_rhs2_projection_ic_cfl(golden_dir, name):
    z = load(golden_dir, name)
    g = grid_of(z)
    bc = (z["xm"], z["xp"], z["ym"], z["yp"])
    dt = float(z["dt"])
    assert bits_equal(oracle.generate_rhs2(z["uhat"], g, bc), z["rhs2"])
    u, uold = oracle.project(z["u"], z["uhat"], z["p"], g, dt)
    assert bits_equal(u, z["u_projected"]) and bits_equal(uold, z["uold_projected"])
    assert bits_equal(oracle.initial_velocity(g, 0.7, -0.3, 0.2, 0.1), z["u_initial"])
    c = oracle.cfl(z["u"], g, dt)
    assert bits_equal(c, z["cfl"])


def _domain_from_golden(name):
    # the case descriptions the golden grids were made from (make_golden.py)
    from cuibm_gb300 import cases
    if name == "ns_stretched":
        return [cases.axis("x", -2.0, 0.1, [(-0.5, 1.1), (0.5, 1.0), (2.5, 1.08)]),
                cases.axis("y", -1.5, 0.1, [(-0.4, 1.12), (0.4, 1.0), (1.6, 1.1)])]
    if name == "ns_cavity16":
        return [cases.axis("x", 0.0, 1 / 16, [(1.0, 1.0)]), cases.axis("y", 0.0, 1 / 16, [(1.0, 1.0)])]
    if name == "grid_cylinder_re40":
        s = [(-0.6, 1.03), (0.6, 1.0), (15.0, 1.03)]
        return [cases.axis("x", -15.0, 0.02, s), cases.axis("y", -15.0, 0.02, s)]
    if name == "grid_cylinder_re550":
        s = [(-0.6, 1.01), (0.6, 1.0), (15.0, 1.01)]
        return [cases.axis("x", -15.0, 0.005, s), cases.axis("y", -15.0, 0.005, s)]
    raise KeyError(name)


@pytest.mark.parametrize("name", NS_CASES + ["grid_cylinder_re40", "grid_cylinder_re550"])
def test_grid_generation(golden_dir, name):
    z = load(golden_dir, name)
    g = oracle.Grid(_domain_from_golden(name))
    assert (g.nx, g.ny) == (int(z["nx"]), int(z["ny"]))
    for k in ("x", "dx", "xu", "xv", "y", "dy", "yu", "yv"):
        assert bits_equal(getattr(g, k), z["grid_" + k]), k


@pytest.mark.parametrize("name,points", [("grid_cylinder_re40", 157), ("grid_cylinder_re550", 629)])
def test_circle_points(golden_dir, name, points):
    z = load(golden_dir, name)
    X, Y = oracle.circle_points(0.0, 0.0, 0.5, points)
    assert bits_equal(X, z["body_X"]) and bits_equal(Y, z["body_Y"])
