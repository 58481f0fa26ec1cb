"""Mixed precision (`precision: MIXED`): an SA-preconditioned BiCGSTAB keeps its
Krylov vectors, residuals and stopping rule in FP64 and runs its V-cycles in FP32
(the constant pressure mode re-solved in FP64); the other solves run FP32 Krylov
iterations under FP64 iterative refinement.  The FP64 residual decides
convergence, so with tight tolerances the fields match the FP64 oracle as the
plain FP64 solves do: velocity within 1e-9 relative L2, pressure 1e-8, drag and
lift within 1e-6."""
import numpy as np
import pytest

import oracle

cb = pytest.importorskip("cuibm_gb300")
from cuibm_gb300 import cases  # noqa: E402

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def cyl(path, method, **kw):
    args = dict(h=0.05, ratio=1.1, extent=3.0, core=0.6, points=48, nu=0.025, dt=0.01, nt=30, vel_tol=1e-12,
                pois_tol=1e-12, pois_pc="SMOOTHED_AGGREGATION", method=method, precision="MIXED")
    args.update(kw)
    return cases.cylinder(path, **args)


SOLVERS = {"LUO": oracle.LuoSolver, "FADLUN": oracle.FadlunSolver, "OSC_CYLINDER": oracle.EmbeddedSolver}


@pytest.mark.parametrize("method", ["LUO", "FADLUN", "OSC_CYLINDER"])
@pytest.mark.parametrize("graph", [1, 0])
def test_cylinder_mixed_matches_oracle(tmp_path, method, graph):
    f = cyl(str(tmp_path / "c"), method)
    ref = SOLVERS[method](f, solve="direct")
    with cb.NavierStokesSolver(f) as s:
        assert s.info.poisson_precision == 1
        s.set_option("write_output", 0)
        s.set_option("use_graph", graph)
        s.initialise()
        for k in range(20):
            s.stepTime(1)
            ref.step()
            fx, fy = s.forces()
            assert abs(2 * fx - 2 * ref.fx) < 1e-6 and abs(2 * fy - 2 * ref.fy) < 1e-6, k
        assert rel_l2(s.get("u"), ref.u) < 1e-9
        assert rel_l2(s.get("p"), ref.p) < 1e-8
        it1, it2 = s.iterations()
        assert 0 < it1 < 200 and 0 < it2 < 400


def test_cavity_mixed_cg_matches_oracle(tmp_path):
    """CG on the symmetrised Poisson operator: refinement around FP32 CG with the FP32 cycle."""
    f = cases.cavity(str(tmp_path / "c"), n=32, nu=0.01, dt=0.01, nt=40, vel_tol=1e-12, pois_tol=1e-12,
                     precision="MIXED")
    ref = oracle.PlainSolver(f, solve="direct")
    with cb.NavierStokesSolver(f) as s:
        s.set_option("write_output", 0)
        s.initialise()
        for k in range(40):
            s.stepTime(1)
            ref.step()
        assert rel_l2(s.get("u"), ref.u) < 1e-9
        assert rel_l2(s.get("p"), ref.p) < 1e-8


def test_oscillating_embedded_mixed(tmp_path):
    """The embedded method's rows move with the body: the float tables follow them."""
    motion = {"xCoefficient": 0.05, "uCoefficient": 0.05 * 2 * np.pi, "xfrequency": 1.0, "xPhase": 0.0,
              "uPhase": 0.0}
    f = cyl(str(tmp_path / "c"), "OSC_CYLINDER", motion=motion)
    ref = oracle.EmbeddedSolver(f, solve="direct")
    with cb.NavierStokesSolver(f) as s:
        s.set_option("write_output", 0)
        s.initialise()
        for k in range(15):
            s.stepTime(1)
            ref.step()
        assert rel_l2(s.get("u"), ref.u) < 1e-9
        assert abs(2 * s.forces()[0] - 2 * ref.fx) < 1e-6


def test_mixed_at_benchmark_tolerance(tmp_path):
    """At the benchmark's 1e-5 both runs stop on the FP64 residual: the mixed run's
    solution stays as close to the FP64 run's as the tolerance allows."""
    f1 = cyl(str(tmp_path / "a"), "LUO", vel_tol=1e-5, pois_tol=1e-5, precision=None)
    f2 = cyl(str(tmp_path / "b"), "LUO", vel_tol=1e-5, pois_tol=1e-5)
    with cb.NavierStokesSolver(f1) as a, cb.NavierStokesSolver(f2) as b:
        for s in (a, b):
            s.set_option("write_output", 0)
            s.initialise()
            s.stepTime(20)
        assert rel_l2(b.get("u"), a.get("u")) < 1e-4
        assert abs(2 * a.forces()[0] - 2 * b.forces()[0]) < 1e-3
