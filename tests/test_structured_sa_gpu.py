"""The structured smoothed-aggregation hierarchy on the GPU (set up on the device:
Jacobi tables, power iteration, prolongator weights, Galerkin operators by probing)
against tests/structured_sa_ref.py, the same construction in scipy: one V-cycle of
the Poisson preconditioner (CUIBM_OP_PRECONDITION_POISSON, stepwise kernels) on the
Re 40 cylinder's pressure operator (270 x 270, external method; -saStructured 1, as
the default takes it from 200k unknowns) and on the Re 550 cylinder's (922 x 922, four
levels, the default), from the GPU's own matrix.  Whole runs with the structured
hierarchy (in the persistent solver) are checked against the FP64 oracle by the Re 550
configuration tests; here a tightly solved run with it and one with the graph
aggregation (-saStructured 0) give the same fields."""
import numpy as np
import pytest
import scipy.sparse as sp

import structured_sa_ref as ref

cb = pytest.importorskip("cuibm_gb300")
from cuibm_gb300 import cases  # noqa: E402

pytestmark = pytest.mark.gpu

RTOL_CYCLE = 1e-9  # the coarsest level's inverse (nearly singular operator) amplifies rounding


def cylinder(folder, fine, **kw):
    if fine:
        return cases.cylinder(folder, h=0.005, ratio=1.01, points=629, nu=1.0 / 550, dt=0.002, nt=40, **kw)
    return cases.cylinder(folder, h=0.02, ratio=1.03, points=157, nu=1.0 / 40, dt=0.01, nt=40, **kw)


@pytest.mark.parametrize("fine,levels", [(False, [72900, 8100, 900]), (True, [850084, 94249, 10404, 1156])])
def test_vcycle_matches_scipy_statement(tmp_path, fine, levels):
    f = cylinder(str(tmp_path / "c"), fine, pois_pc="SMOOTHED_AGGREGATION")
    with cb.NavierStokesSolver(f, [] if fine else ["-saStructured", "1"]) as s:
        s.set_option("write_output", 0)
        s.initialise()
        i = s.info
        assert i.sa_structured == 1 and i.amg_levels == len(levels)
        r, c, v = s.matrix(2)
        A = sp.coo_matrix((v, (r, c)), shape=(i.numP, i.numP)).tocsr()
        H = ref.hierarchy(A, i.nx, i.ny)
        assert [L["A"].shape[0] for L in H] == levels
        rng = np.random.default_rng(3)
        for b in (rng.standard_normal(i.numP), A @ rng.standard_normal(i.numP)):
            s.set("work_x", np.concatenate([b, np.zeros(max(i.numUV, i.numP) - i.numP)]))
            s.run("precondition_poisson")
            z = s.get("work_y")[:i.numP]
            zr = ref.vcycle(H, b)
            err = np.max(np.abs(z - zr)) / np.max(np.abs(zr))
            print("levels %s: cycle vs scipy statement %.2e" % (levels, err))
            assert err < RTOL_CYCLE


def test_structured_and_graph_hierarchies_give_the_same_run(tmp_path):
    out = []
    for flag in ("1", "0"):
        f = cylinder(str(tmp_path / ("c" + flag)), False, pois_pc="SMOOTHED_AGGREGATION", vel_tol=1e-12,
                     pois_tol=1e-12)
        with cb.NavierStokesSolver(f, ["-saStructured", flag]) as s:
            s.set_option("write_output", 0)
            s.initialise()
            assert s.info.sa_structured == int(flag)
            s.stepTime(20)
            out.append((s.get("u"), s.get("p"), s.forces(), s.iterations()))
    (u1, p1, f1, it1), (u0, p0, f0, it0) = out
    print("iterations of the last step: structured %s, graph %s" % (it1, it0))
    assert np.linalg.norm(u1 - u0) <= 1e-10 * np.linalg.norm(u0)
    assert np.linalg.norm((p1 - p1.mean()) - (p0 - p0.mean())) <= 1e-9 * np.linalg.norm(p0 - p0.mean())
    assert abs(f1[0] - f0[0]) < 1e-9 and abs(f1[1] - f0[1]) < 1e-9


@pytest.mark.parametrize("nx,ny", [(600, 5), (5, 600), (97, 47)])
def test_narrow_and_odd_grids(tmp_path, nx, ny):
    """The structured hierarchy on grids whose aggregates reach the remainder rules'
    corners (a coarse direction of one node, aggregates 4 or 5 wide, odd sizes): one
    V-cycle against the scipy statement, and tightly solved steps converging in the
    persistent solver."""
    h = 0.01
    sim = {"type": "simulation", "dt": 0.001, "nt": 10, "nsave": 10, "SolverType": "NAVIER_STOKES_SOLVER",
           "linearSolvers": cases.solvers("DIAGONAL", 1e-12, "SMOOTHED_AGGREGATION", 1e-12,
                                          pois_krylov="BICGSTAB")}  # CG's hierarchy is of the symmetrised operator
    flow = [{"type": "flow", "nu": 0.01, "initialVelocity": [0.0, 0.0], "initialPerturbation": [0.0, 0.0],
             "boundaryConditions": cases.bcs((0, 0), (0, 0), (0, 0), (1.0, 0))}]
    dom = [cases.axis("x", 0.0, h, [(nx * h, 1.0)]), cases.axis("y", 0.0, h, [(ny * h, 1.0)])]
    f = cases.write_case(str(tmp_path / "c"), [sim], flow, dom, [])
    with cb.NavierStokesSolver(f, ["-saStructured", "1"]) as s:
        s.set_option("write_output", 0)
        s.initialise()
        i = s.info
        assert (i.nx, i.ny) == (nx, ny) and i.sa_structured == 1
        r, c, v = s.matrix(2)
        A = sp.coo_matrix((v, (r, c)), shape=(i.numP, i.numP)).tocsr()
        H = ref.hierarchy(A, nx, ny)
        assert i.amg_levels == len(H)
        b = np.random.default_rng(4).standard_normal(i.numP)
        s.set("work_x", np.concatenate([b, np.zeros(max(i.numUV, i.numP) - i.numP)]))
        s.run("precondition_poisson")
        z, zr = s.get("work_y")[:i.numP], ref.vcycle(H, b)
        assert np.max(np.abs(z - zr)) / np.max(np.abs(zr)) < RTOL_CYCLE
        s.stepTime(5)
        assert s.iterations()[1] > 0
        assert np.all(np.isfinite(s.get("p")))
