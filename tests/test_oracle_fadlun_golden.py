"""The oracle's modified-Fadlun restatement (oracle/fadlun.c) against the
reference's own FadlunModified kernels run on the CPU (tests/golden/fadlun_*.npz,
written by tests/golden/make_golden.py --only fadlun): bit for bit."""
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["fadlun_circle48", "fadlun_circle101"]


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    g = oracle.Grid.from_arrays(*(z["grid_" + k] for k in ("x", "dx", "xu", "y", "dy", "yv")))
    T = oracle.Tags(g)
    names = {"ghostTagsUV": "ghostTagsUV", "ghostTagsP": "ghostTagsP", "hybridTagsUV": "hybridTagsUV",
             "hybridTagsP": "hybridTagsP", "hybridTagsUV2": "hybridTagsUV2",
             "dist_node": "distance_from_intersection_to_node", "dist_between": "distance_between_nodes_at_IB",
             "uv": "uv", "dist_u_body": "distance_from_u_to_body", "dist_v_body": "distance_from_v_to_body"}
    for mine, ref in names.items():
        setattr(T, mine, np.ascontiguousarray(z["tag_" + ref]))
    return z, g, T


def bits_equal(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64) if np.asarray(a).dtype == np.float64 else a,
                          np.asarray(b).view(np.uint64) if np.asarray(b).dtype == np.float64 else b)


@pytest.mark.parametrize("name", CASES)
def test_tags_present(name):
    z, g, T = load(name)
    assert (T.hybridTagsUV > 0).sum() > 10 and (T.ghostTagsUV > 0).sum() > 10 and (T.ghostTagsP > 0).sum() > 5


@pytest.mark.parametrize("name", CASES)
def test_lhs1_bit_exact(name):
    z, g, T = load(name)
    r, c, v = oracle.fadlun_lhs1_coo(g, float(z["dt"]), float(z["nu"]), T)
    assert np.array_equal(r, z["lhs1_row"]) and np.array_equal(c, z["lhs1_col"])
    assert bits_equal(v, z["lhs1_val"])


@pytest.mark.parametrize("name", CASES)
def test_lhs2_bit_exact(name):
    z, g, T = load(name)
    r, c, v = oracle.fadlun_lhs2_coo(g, float(z["dt"]), T)
    assert np.array_equal(r, z["lhs2_row"]) and np.array_equal(c, z["lhs2_col"])
    assert bits_equal(v, z["lhs2_val"])


@pytest.mark.parametrize("name", CASES)
def test_rhs_and_projection_bit_exact(name):
    z, g, T = load(name)
    assert bits_equal(oracle.fadlun_update_rhs1(z["rhs1_in"], T, g), z["rhs1_out"])
    bc = (z["bc_xm"], z["bc_xp"], z["bc_ym"], z["bc_yp"])
    assert bits_equal(oracle.fadlun_rhs2(z["uhat_in"], T, g, bc), z["rhs2"])
    assert bits_equal(oracle.fadlun_project(z["uhat_in"], z["p_in"], T, g, float(z["dt"])), z["u_projected"])
