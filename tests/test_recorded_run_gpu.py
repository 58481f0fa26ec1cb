"""Against outputs the reference's authors recorded for one of its validation cases
(validation/osc/static/external: a cylinder of diameter 0.2 oscillating in fluid at
rest, Re 100, external method, dt 0.001; tests/golden/recorded_osc_static_external.npz,
extracted by tests/golden/make_golden.py --only recorded).  The case is restated
here from its simParams/flow/domain/bodies files.

The body's prescribed position and velocity (midPosition_init, 6 significant
figures) are reproduced step for step.  The recorded forces are not: the library and
the oracle restatement (direct solves) agree with each other to 1e-5 but sit 8-11 %
above the recording in the first steps and about 11 % off (median over the first
300 steps where |Fx| > 0.05; up to 80 % next to sign changes) later; the restatement's
kernels are bit-exact against the reference's own kernel code, so the gap lies in
what the recording ran (its CUSP solves, whose iterates are not reproducible here,
or the code version it was made with).  The recording itself shows that it came
from a different build: iterations_init has 2000 rows for 1000 steps, every time
step written twice (rows "1 2 7", "1 2 7", "2 2 15", "2 2 15", ...), where the
shipped code writes one row per step - NavierStokesSolver::writeCommon
(NavierStokesSolver.cu:350) is the only writer, reached once per step through
luoIBM::writeData -> luoIBM::writeCommon -> luo_base::writeCommon
(luoIBM.cu:69-89, luo_base.cu:180-182).  The forces are checked for their sign
pattern and size only; the body motion exactly."""
import os

import numpy as np
import pytest

cb = pytest.importorskip("cuibm_gb300")
from cuibm_gb300 import cases  # noqa: E402

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def osc_static_external(folder):
    sim = {"type": "simulation", "dt": 0.001, "scaleCV": 5.0, "nt": 4000, "nsave": 10000, "startStep": 0,
           "SolverType": "LUO",
           "linearSolvers": cases.solvers("DIAGONAL", 1e-5, "SMOOTHED_AGGREGATION", 1e-5, pois_maxit=100000)}
    flow = [{"type": "flow", "nu": 0.002, "initialVelocity": [0.0, 0.0], "initialPerturbation": [0.0, 0.0],
             "boundaryConditions": cases.bcs((0, 0), (0, 0), (0, 0), (0, 0), xp_type="CONVECTIVE")}]
    dom = [cases.axis("x", -5.5, 0.005, [(-0.4, 1.05), (0.4, 1.0), (5.5, 1.05)]),
           cases.axis("y", -3.5, 0.005, [(-0.2, 1.05), (0.2, 1.0), (3.5, 1.05)])]
    body = [{"type": "circle", "circleOptions": [0.0, 0.0, 0.1, 158, True, 0.005], "xCoefficient": -0.1591549431,
             "xPhase": 0.0, "uCoefficient": -1.0, "uPhase": 0.0, "xfrequency": 1.0}]
    return cases.write_case(folder, [sim], flow, dom, body)


def test_recorded_oscillating_cylinder(tmp_path):
    z = np.load(os.path.join(HERE, "golden", "recorded_osc_static_external.npz"))
    F, M = z["forces"], z["mid_position"]
    steps = 300
    with cb.NavierStokesSolver(osc_static_external(str(tmp_path / "osc"))) as s:
        s.set_option("write_output", 0)
        s.initialise()
        assert s.info.total_points == 126  # selfSize: int(2 pi R / h), made even
        fx = np.zeros(steps)
        for k in range(steps):
            # row k is written after step k+1, whose body update moved the body to t = dt * k
            s.stepTime(1)
            fx[k] = s.forces()[0]
            m = s.get("body_motion")
            assert abs(m[0] - M[k, 1]) <= 5e-6 * abs(M[k, 1]) + 1e-9, (k, m[0], M[k, 1])
            assert abs(m[2] - M[k, 3]) <= 5e-6 * abs(M[k, 3]) + 1e-9, (k, m[2], M[k, 3])
        # forces: the same impulsive start and sign changes, within the gap described above
        ref = F[:steps, 1]
        assert np.all(np.sign(fx[:50]) == np.sign(ref[:50]))
        big = np.abs(ref) > 0.05
        gap = np.abs(fx[big] - ref[big]) / np.abs(ref[big])
        print("relative gap to the recorded Fx where |Fx| > 0.05: median %.3f, max %.3f" % (np.median(gap), gap.max()))
        assert np.median(gap) < 0.15  # 0.108 measured
