"""C ABI and host-side logic (no GPU): the library loads, exports every entry
point include/cuibm.h declares, and builds grids and bodies bit-identically to
the reference's own parsers (golden fixtures)."""
import ctypes
import os
import re

import numpy as np
import pytest

import cuibm_gb300 as cb
from cuibm_gb300 import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "cuibm.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cuibm_[a-z_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    lib = cb.library()
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n


def bits_equal(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("name,h,ratio,points", [("grid_cylinder_re40", 0.02, 1.03, 157),
                                                  ("grid_cylinder_re550", 0.005, 1.01, 629)])
def test_host_grid_and_body_match_reference(tmp_path, golden_dir, name, h, ratio, points):
    f = cases.cylinder(str(tmp_path / name), h=h, ratio=ratio, points=points, nt=1)
    z = np.load(os.path.join(golden_dir, name + ".npz"))
    info = cb.case_info(f)
    assert (info.nx, info.ny) == (int(z["nx"]), int(z["ny"]))
    for k in ("x", "dx", "xu", "xv", "y", "dy", "yu", "yv"):
        assert bits_equal(cb.case_array(f, k), z["grid_" + k]), k
    assert bits_equal(cb.case_array(f, "body_x"), z["body_X"])
    assert bits_equal(cb.case_array(f, "body_y"), z["body_Y"])
    assert info.total_points == points and info.solver_type == cb.LUO


def test_stretched_grid_matches_reference(tmp_path, golden_dir):
    f = str(tmp_path / "s")
    cases.write_case(f, [{"type": "simulation", "dt": 0.01, "nt": 1, "nsave": 1}],
                     [{"type": "flow", "nu": 0.02, "initialVelocity": [1.0, 0.0],
                       "boundaryConditions": cases.bcs((1, 0), (1, 0), (1, 0), (1, 0))}],
                     [cases.axis("x", -2.0, 0.1, [(-0.5, 1.1), (0.5, 1.0), (2.5, 1.08)]),
                      cases.axis("y", -1.5, 0.1, [(-0.4, 1.12), (0.4, 1.0), (1.6, 1.1)])], [])
    z = np.load(os.path.join(golden_dir, "ns_stretched.npz"))
    for k in ("x", "dx", "xu", "y", "dy", "yv"):
        assert bits_equal(cb.case_array(f, k), z["grid_" + k]), k


def test_reference_yaml_and_command_line(tmp_path):
    f = cases.cavity(str(tmp_path / "c"), n=32, nt=7, pois_pc="DIAGONAL")
    info = cb.case_info(f, ["-nt", "11", "-dt", "0.005", "-nu", "0.03"])
    assert info.nt == 11 and info.dt == 0.005 and info.nu == 0.03
    assert info.nx == 32 and info.ny == 32 and info.solver_type == cb.NAVIER_STOKES
    assert info.poisson_precond == 1 and info.poisson_krylov == 1  # DIAGONAL, CG


def test_bad_inputs_report_errors(tmp_path):
    with pytest.raises(cb.CuibmError) as e:
        cb.case_info(str(tmp_path / "missing"))
    assert e.value.status == cb.ERR_IO
    f = cases.cavity(str(tmp_path / "c"), n=16, nt=1)
    with open(os.path.join(f, "flow.yaml"), "a") as fh:
        fh.write("    - location: zMinus\n      u: [DIRICHLET, 0.0]\n      v: [DIRICHLET, 0.0]\n")
    with pytest.raises(cb.CuibmError) as e:
        cb.case_info(f)
    assert e.value.status == cb.ERR_BAD_INPUT and "zMinus" in str(e.value)
    with pytest.raises(cb.CuibmError):
        cb.case_info(f, ["-nt", "notanumber"])


def test_precision_option(tmp_path):
    f = cases.cavity(str(tmp_path / "m"), n=16, nt=1, precision="MIXED")
    info = cb.case_info(f)
    assert info.velocity_precision == 1 and info.poisson_precision == 1
    info = cb.case_info(cases.cavity(str(tmp_path / "d"), n=16, nt=1))
    assert info.velocity_precision == 0 and info.poisson_precision == 0
    with pytest.raises(cb.CuibmError) as e:
        cb.case_info(cases.cavity(str(tmp_path / "h"), n=16, nt=1, precision="HALF"))
    assert e.value.status == cb.ERR_BAD_INPUT and "precision" in str(e.value)


def test_strength_threshold_option(tmp_path):
    cb.case_info(cases.cavity(str(tmp_path / "s"), n=16, nt=1, strength=0.05))
    for bad in (-0.1, 1.0):
        with pytest.raises(cb.CuibmError) as e:
            cb.case_info(cases.cavity(str(tmp_path / ("b%g" % bad)), n=16, nt=1, strength=bad))
        assert e.value.status == cb.ERR_BAD_INPUT and "strengthThreshold" in str(e.value)


def test_unknown_solver_type_falls_back_to_navier_stokes(tmp_path):
    f = cases.cavity(str(tmp_path / "c"), n=16, nt=1)
    p = os.path.join(f, "simParams.yaml")
    s = open(p).read().replace("NAVIER_STOKES_SOLVER", "SOMETHING_ELSE")
    open(p, "w").write(s)
    assert cb.case_info(f).solver_type == cb.NAVIER_STOKES


def test_parses_reference_style_files(tmp_path):
    """Comments, blank lines, tabs of spacing and the reference's key layout."""
    f = tmp_path / "r"
    f.mkdir()
    (f / "simParams.yaml").write_text(
        "- type: simulation\n  dt: 0.005   # step\n  nt: 1000\n  nsave: 2000\n  SolverType: LUO\n"
        "  linearSolvers:\n    - system: velocity\n      solver: CG\n      preconditioner: DIAGONAL\n"
        "      tolerance: 1e-5\n      maxIterations: 10000\n    - system: Poisson\n      solver: CG\n"
        "      preconditioner: SMOOTHED_AGGREGATION\n      tolerance: 1e-5\n      maxIterations: 20000\n")
    (f / "flow.yaml").write_text(
        "- type: flow\n  nu: 0.025\n  initialVelocity: [1.0, 0.0]\n  boundaryConditions:\n"
        "    - location: xMinus\n      u: [DIRICHLET, 1.0]\n      v: [DIRICHLET, 0.0]\n"
        "    - location: xPlus\n      u: [CONVECTIVE, 1.0]\n      v: [CONVECTIVE, 0.0]\n"
        "    - location: yMinus\n      u: [DIRICHLET, 1.0]\n      v: [DIRICHLET, 0.0]\n"
        "    - location: yPlus\n      u: [DIRICHLET, 1.0]\n      v: [DIRICHLET, 0.0]\n")
    (f / "domain.yaml").write_text(
        "- direction: x\n  start: -15.0\n  mid_h: 0.025\n  subDomains:\n    - end: -0.6\n      stretchRatio: 1.05\n"
        "    - end: 0.6\n      stretchRatio: 1.0\n    - end: 15.0\n      stretchRatio: 1.05\n\n"
        "- direction: y\n  start: -15.0\n  mid_h: 0.025\n  subDomains:\n    - end: -0.6\n      stretchRatio: 1.05\n"
        "    - end: 0.6\n      stretchRatio: 1.0\n    - end: 15.0\n      stretchRatio: 1.05\n")
    (f / "bodies.yaml").write_text("- type: circle\n  circleOptions: [0.0, 0.0, 0.5, 126, true, 0.025]\n"
                                   "  initialOffset: [0.0, 0.0]\n")
    info = cb.case_info(str(f))
    assert info.solver_type == cb.LUO and info.poisson_precond == 2 and info.velocity_precond == 1
    assert info.total_points == 126  # selfSize: int(2*pi*0.5/0.025) = 125 -> made even
    assert info.dt == 0.005 and info.nt == 1000 and info.nsave == 2000


def test_start_step_only_with_restart(tmp_path):
    """startStep is read but not used by the reference; with restart: true it is the
    step whose saved state the run continues from."""
    f = cases.cavity(str(tmp_path / "a"), n=16, nt=20, extra={"startStep": 10})
    assert cb.case_info(f).time_step == 0
    f = cases.cavity(str(tmp_path / "b"), n=16, nt=20, extra={"startStep": 10, "restart": True})
    assert cb.case_info(f).time_step == 10
