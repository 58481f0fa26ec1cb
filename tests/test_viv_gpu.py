"""Flow-induced motion (simulation VIV), the reference's viv_movement_LC and
viv_movement_SC.  Loose coupling (VIV: 1): after each step's control-volume force
the spring-mounted cylinder's vertical velocity and centre are advanced on the
device from the lift, the body points follow and the tags, the interpolation plan
(and the embedded method's rows) are rebuilt.  Strong coupling (VIV: 2): the step's
phases repeat from u = uold, with a relaxed centre update, until the centre's
relative change is below 1e-3 (at least two passes); the loop runs on the device
as a WHILE graph node, or host-driven without the graph.  A cross-flow makes the
lift, and the body moves; fields, forces, the body's position and velocity and the
passes of every step match the oracle (fields to 1e-9 relative L2, drag and lift
to 1e-6)."""
import numpy as np
import pytest

import oracle

cb = pytest.importorskip("cuibm_gb300")
from cuibm_gb300 import cases  # noqa: E402

pytestmark = pytest.mark.gpu

SOLVERS = {"LUO": oracle.LuoSolver, "OSC_CYLINDER": oracle.EmbeddedSolver}


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def viv_case(path, method, viv=1, **kw):
    args = dict(h=0.05, ratio=1.1, extent=4.0, core=0.6, points=48, nu=0.025, dt=0.01, nt=100, vel_tol=1e-12,
                pois_tol=1e-12, pois_pc="SMOOTHED_AGGREGATION", method=method, vinf=0.3,
                extra={"VIV": viv, "Ured": 4})
    args.update(kw)
    return cases.cylinder(path, **args)


@pytest.mark.parametrize("method", ["LUO", "OSC_CYLINDER"])
@pytest.mark.parametrize("graph", [1, 0])
def test_viv_matches_oracle(tmp_path, method, graph):
    f = viv_case(str(tmp_path / "c"), method)
    ref = SOLVERS[method](f, solve="direct")
    with cb.NavierStokesSolver(f) as s:
        s.set_option("write_output", 0)
        s.set_option("use_graph", graph)
        s.initialise()
        y0 = s.get("body_y").mean()
        for k in range(25):
            s.stepTime(1)
            ref.step()
            fx, fy = s.forces()
            assert abs(2 * fx - 2 * ref.fx) < 1e-6 and abs(2 * fy - 2 * ref.fy) < 1e-6, k
        by, vB = s.get("body_y"), s.get("body_vB")
        assert np.max(np.abs(by - ref.by)) < 1e-10 and np.max(np.abs(vB - ref.vB)) < 1e-9
        assert abs(by.mean() - y0) > 1e-5  # the body moved
        assert np.array_equal(s.get("ghost_tags_uv"), ref.T.ghostTagsUV)
        assert rel_l2(s.get("u"), ref.u) < 1e-9
        assert rel_l2(s.get("p"), ref.p) < 1e-8


@pytest.mark.parametrize("method", ["LUO", "OSC_CYLINDER"])
@pytest.mark.parametrize("graph", [1, 0])
def test_strong_coupling_matches_oracle(tmp_path, method, graph):
    f = viv_case(str(tmp_path / "c"), method, viv=2)
    ref = SOLVERS[method](f, solve="direct")
    with cb.NavierStokesSolver(f) as s:
        s.set_option("write_output", 0)
        s.set_option("use_graph", graph)
        s.initialise()
        y0 = s.get("body_y").mean()
        passes = []
        for k in range(20):
            s.stepTime(1)
            ref.step()
            m = s.get("body_motion")
            passes.append(ref.sub_iterations)
            assert int(m[9]) == ref.sub_iterations, (k, m[9], ref.sub_iterations)
            assert abs(m[8] - ref.sctol) <= 1e-6 * max(1.0, abs(ref.sctol)), k
            fx, fy = s.forces()
            assert abs(2 * fx - 2 * ref.fx) < 1e-6 and abs(2 * fy - 2 * ref.fy) < 1e-6, k
        assert max(passes) > 2  # the coupling test, not the two-pass minimum, ended some steps
        by, vB = s.get("body_y"), s.get("body_vB")
        assert np.max(np.abs(by - ref.by)) < 1e-10 and np.max(np.abs(vB - ref.vB)) < 1e-9
        assert abs(by.mean() - y0) > 1e-5
        assert np.array_equal(s.get("ghost_tags_uv"), ref.T.ghostTagsUV)
        assert rel_l2(s.get("u"), ref.u) < 1e-9
        assert rel_l2(s.get("uold"), ref.uold) < 1e-9
        assert rel_l2(s.get("p"), ref.p) < 1e-8
        assert rel_l2(s.get("bc_xplus"), ref.bc[1]) < 1e-12  # the outflow advanced once per pass


def test_strong_coupling_needs_a_restarting_method(tmp_path):
    with pytest.raises(cb.CuibmError) as e:
        cb.NavierStokesSolver(viv_case(str(tmp_path / "c"), "FADLUN", viv=2))
    assert "VIV: 2" in str(e.value)
