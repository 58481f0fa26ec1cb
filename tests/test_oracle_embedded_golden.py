"""The oracle's embedded-method restatement (oracle/embedded.c) against the
reference's own luo_iter kernels run on the CPU (tests/golden/iter_*.npz, written
by tests/golden/make_golden.py --only iter): alpha, the set = false stencils
(index, coefficient, corner value), LHS1 and LHS2 on zeroed arrays in the
reference's entry order, ns_rhs, interp_rhs and both right-hand-side updates, bit
for bit."""
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["iter_circle48", "iter_circle101"]


@pytest.fixture(autouse=True)
def reference_intercepts():
    """These fixtures come from the reference's own kernels, which compute the body
    intercepts in trigonometric form: the oracle tags in that form here."""
    with oracle.intercept_form(0):
        yield


def bits_equal(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype == np.float64:
        return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))
    return np.array_equal(a, b)


def setup(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    g = oracle.Grid.from_arrays(*(z["grid_" + k] for k in ("x", "dx", "xu", "y", "dy", "yv")))
    bb = tuple(int(v) for v in z["bb"])
    T = oracle.tag_points(g, z["bx"], z["by"], z["uB"], z["vB"], bb, 0.0, float(z["midY"]))
    return z, g, bb, T


def velocity_stencils(z, g, bb, T):
    ub, vb = float(z["uB"][0]), float(z["vB"][0])
    S = oracle.Stencils(g.nUV)
    u = z["u_in"]
    oracle.ghost_velocity(0, u, T, ub, g, bb, set_=False, S=S)
    oracle.ghost_velocity(1, u, T, vb, g, bb, set_=False, S=S)
    ustar = np.zeros(g.nUV)
    ustar, _ = oracle.hybrid_velocity(0, u, ustar, T, ub, g, bb, S=S)
    oracle.hybrid_velocity(1, u, ustar, T, vb, g, bb, S=S)
    return S


def pressure_stencils(z, g, bb, T):
    dt = float(z["dt"])
    dudt = (float(z["uB"][0]) - float(z["uBk"])) / dt
    dvdt = (float(z["vB"][0]) - float(z["vBk"])) / dt
    S = oracle.Stencils(g.nP)
    oracle.ghost_pressure(z["p_in"], T, dudt, dvdt, g, bb, set_=False, S=S)
    oracle.hybrid_pressure(z["p_in"], T, dudt, dvdt, g, bb, S=S)
    return S


@pytest.mark.parametrize("name", CASES)
def test_tags_and_counts(name):
    z, g, bb, T = setup(name)
    for f in ("ghostTagsUV", "hybridTagsUV", "ghostTagsP", "hybridTagsP"):
        assert np.array_equal(getattr(T, f), z["tag_" + f]), f
    assert (T.hybridTagsUV > 0).sum() > 50 and (T.hybridTagsP > 0).sum() > 20


@pytest.mark.parametrize("name", CASES)
def test_alpha_bit_exact(name):
    z, g, bb, T = setup(name)
    a = oracle.iter_alpha(0, T, g, bb)
    oracle.iter_alpha(1, T, g, bb, a)
    assert bits_equal(a, z["alpha_uv"])
    assert bits_equal(oracle.iter_alpha(2, T, g, bb), z["alpha_p"])


@pytest.mark.parametrize("name", CASES)
def test_stencils_bit_exact(name):
    z, g, bb, T = setup(name)
    for pre, S, n in (("vel_", velocity_stencils(z, g, bb, T), g.nUV), ("p_", pressure_stencils(z, g, bb, T), g.nP)):
        for k in range(4):
            assert np.array_equal(S.index[k][:n], z[pre + "index%d" % (k + 1)][:n]), (pre, k)
            assert bits_equal(S.coef[k][:n], z[pre + "q%dcoef" % (k + 1)][:n]), (pre, k)
            assert bits_equal(S.q[k][:n], z[pre + "q%d" % (k + 1)][:n]), (pre, k)


@pytest.mark.parametrize("name", CASES)
def test_lhs1_and_rhs1_bit_exact(name):
    z, g, bb, T = setup(name)
    S = velocity_stencils(z, g, bb, T)
    a = oracle.iter_alpha(0, T, g, bb)
    oracle.iter_alpha(1, T, g, bb, a)
    row, col, val, ns, interp = oracle.iter_lhs1(g, float(z["dt"]), float(z["nu"]), T, S, a, float(z["uB"][0]),
                                                 float(z["vB"][0]), bb)
    assert np.array_equal(row, z["lhs1_row"]) and np.array_equal(col, z["lhs1_col"])
    assert bits_equal(val, z["lhs1_val"])
    assert bits_equal(ns, z["ns_rhs1"]) and bits_equal(interp, z["interp_rhs1"])
    assert bits_equal(oracle.iter_update_rhs1(z["rhs1_in"], ns, interp, g), z["rhs1_out"])


@pytest.mark.parametrize("name", CASES)
def test_lhs2_and_rhs2_bit_exact(name):
    z, g, bb, T = setup(name)
    S = pressure_stencils(z, g, bb, T)
    assert bits_equal(S.dpdn, z["dpdn"])
    row, col, val, ns, interp = oracle.iter_lhs2(g, float(z["dt"]), T, S, oracle.iter_alpha(2, T, g, bb), bb)
    assert np.array_equal(row, z["lhs2_row"]) and np.array_equal(col, z["lhs2_col"])
    assert bits_equal(val, z["lhs2_val"])
    assert bits_equal(ns, z["ns_rhs2"]) and bits_equal(interp, z["interp_rhs2"])
    assert bits_equal(oracle.iter_update_rhs2(z["rhs2_in"], ns, interp, g), z["rhs2_out"])


def test_dpdn_terms_exercised():
    z = np.load(os.path.join(GOLDEN, "iter_circle48.npz"))
    assert (z["dpdn"] != 0).sum() > 10 and (z["interp_rhs2"] != 0).sum() > 10
