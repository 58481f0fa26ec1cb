"""The structured smoothed-aggregation design on the CPU (tests/structured_sa_ref.py,
the statement the GPU hierarchy is checked against): on the pressure operators of the
lid-driven cavity (plain method, centre pin) and the Re 40 cylinder (external method,
stretched 270 x 270 grid) the Galerkin operators of every coarse level couple only
neighbouring aggregates (9-point stencils: what lets the GPU store them as nine
coefficient arrays and build them by nine probes), the level sizes follow the 3 x 3
rule, and the cycle preconditions BiCGSTAB on the cylinder's operator."""
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import oracle
import structured_sa_ref as ref
from cuibm_gb300 import cases

NINE = {(dx, dy) for dx in (-1, 0, 1) for dy in (-1, 0, 1)}


def pressure_operator(tmp, kind):
    if kind == "cavity":
        f = cases.cavity(os.path.join(tmp, "cav"), n=64, nu=0.01, dt=0.01, nt=10)
        g = oracle.PlainSolver(f, solve="none").g
        r, c, v = oracle.lhs2_coo(g, 0.01, centre_pin=True)[:3]
    else:
        f = cases.cylinder(os.path.join(tmp, "cyl"), h=0.02, ratio=1.03, points=157, nu=1.0 / 40, dt=0.01, nt=10)
        g = oracle.LuoSolver(f, solve="none").g
        r, c, v = oracle.lhs2_coo(g, 0.01, centre_pin=False)[:3]
    return sp.coo_matrix((v, (r, c)), shape=(g.nP, g.nP)).tocsr(), g.nx, g.ny


@pytest.mark.parametrize("kind,sizes", [("cavity", [4096, 441]), ("cylinder", [72900, 8100, 900])])
def test_coarse_operators_are_nine_point(tmp_path, kind, sizes):
    A, nx, ny = pressure_operator(str(tmp_path), kind)
    assert ref.stencil_offsets(A, nx, ny) <= NINE
    levels = ref.hierarchy(A, nx, ny)
    assert [L["A"].shape[0] for L in levels] == sizes
    for L in levels[1:]:
        offs = ref.stencil_offsets(L["A"], L["nx"], L["ny"])
        assert offs <= NINE, offs - NINE
        assert (1, 1) in offs and (-1, 1) in offs  # the corners are really there
    # the tentative prolongator keeps the constant: P's rows sum to 1 - w D^-1 (A 1)
    for L in levels[:-1]:
        rs = np.asarray(L["P"].sum(axis=1)).ravel()
        A1 = np.asarray(L["A"].sum(axis=1)).ravel()
        assert np.allclose(rs, 1.0 - L["omega"] * L["dinv"] * A1, rtol=0, atol=1e-12)


def test_cycle_preconditions_bicgstab(tmp_path):
    A, nx, ny = pressure_operator(str(tmp_path), "cylinder")
    levels = ref.hierarchy(A, nx, ny)
    n = A.shape[0]
    M = spla.LinearOperator((n, n), matvec=lambda b: ref.vcycle(levels, b))
    rng = np.random.default_rng(0)
    b = rng.standard_normal(n)
    its = [0]

    def count(_):
        its[0] += 1

    x, info = spla.bicgstab(A, b, M=M, rtol=1e-8, maxiter=200, callback=count)
    assert info == 0
    assert np.linalg.norm(b - A @ x) <= 1e-8 * np.linalg.norm(b)
    # a random right-hand side (the worst case: the time loop's solves start from the last
    # pressure); diagonal scaling alone does not reach 1e-8 in 2000 iterations
    assert its[0] < 200, its[0]


@pytest.mark.parametrize("nx,ny,sizes", [(600, 5, [3000, 200]), (5, 600, [3000, 200]), (97, 47, [4559, 480]),
                                         (1000, 13, [13000, 1332])])
def test_narrow_and_odd_grids(tmp_path, nx, ny, sizes):
    """Aggregates at the remainder rules' corners (a coarse direction of one node,
    aggregates 4 or 5 wide): the coarse operators stay 9-point and the cycle still
    preconditions BiCGSTAB on a plain channel's pressure operator."""
    h = 0.01
    sim = {"type": "simulation", "dt": 0.001, "nt": 10, "nsave": 10, "SolverType": "NAVIER_STOKES_SOLVER",
           "linearSolvers": cases.solvers("DIAGONAL", 1e-8, "SMOOTHED_AGGREGATION", 1e-8, pois_krylov="BICGSTAB")}
    flow = [{"type": "flow", "nu": 0.01, "initialVelocity": [0.0, 0.0], "initialPerturbation": [0.0, 0.0],
             "boundaryConditions": cases.bcs((0, 0), (0, 0), (0, 0), (1.0, 0))}]
    dom = [cases.axis("x", 0.0, h, [(nx * h, 1.0)]), cases.axis("y", 0.0, h, [(ny * h, 1.0)])]
    f = cases.write_case(os.path.join(str(tmp_path), "c"), [sim], flow, dom, [])
    g = oracle.PlainSolver(f, solve="none").g
    r, c, v = oracle.lhs2_coo(g, 0.001, centre_pin=True)[:3]
    A = sp.coo_matrix((v, (r, c)), shape=(g.nP, g.nP)).tocsr()
    levels = ref.hierarchy(A, g.nx, g.ny)
    assert [L["A"].shape[0] for L in levels] == sizes
    for L in levels[1:]:
        assert ref.stencil_offsets(L["A"], L["nx"], L["ny"]) <= NINE
    n = A.shape[0]
    M = spla.LinearOperator((n, n), matvec=lambda b: ref.vcycle(levels, b))
    b = A @ np.random.default_rng(1).standard_normal(n)
    x, info = spla.bicgstab(A, b, M=M, rtol=1e-8, maxiter=300)
    assert info == 0 and np.linalg.norm(b - A @ x) <= 1e-8 * np.linalg.norm(b)
