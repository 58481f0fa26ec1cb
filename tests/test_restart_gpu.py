"""Restart that reloads the state: a run writes NNNNNNN/state beside q and lambda
every nsave steps; a run of the same case with restart: true and startStep: k reads
k/state and continues.  The continued run's fields after its steps equal, bit for
bit, those of the run that did not stop (same kernels, same inputs, deterministic
reductions), and the iteration history is appended."""
import os

import numpy as np
import pytest

cb = pytest.importorskip("cuibm_gb300")
from cuibm_gb300 import cases  # noqa: E402

pytestmark = pytest.mark.gpu


def run(folder, steps):
    with cb.NavierStokesSolver(folder) as s:
        s.initialise()
        for _ in range(steps):
            s.stepTime(1)
            s.writeData()
        forces = s.forces() if s.info.total_points else None
        return s.get("u"), s.get("p"), forces, s.timeStep


def continue_bitwise(make, tmp_path, n1=10, n2=10):
    ua, pa, fa, ta = run(make(str(tmp_path / "a"), {}), n1 + n2)
    run(make(str(tmp_path / "b"), {}), n1)
    b = make(str(tmp_path / "b"), {"restart": True, "startStep": n1})
    ub, pb, fb, tb = run(b, n2)
    assert ta == tb == n1 + n2
    assert np.array_equal(ua.view(np.uint64), ub.view(np.uint64))
    assert np.array_equal(pa.view(np.uint64), pb.view(np.uint64))
    if fa is not None:
        assert fa == fb
    with open(os.path.join(b, "iterations")) as fh:
        assert len([ln for ln in fh.read().split("\n") if ln.strip()]) == n1 + n2


def test_cavity_restart_continues_bitwise(tmp_path):
    def make(path, extra):
        return cases.cavity(path, n=32, nu=0.01, dt=0.01, nt=100, nsave=10, extra=extra)
    continue_bitwise(make, tmp_path)


@pytest.mark.parametrize("method", ["LUO", "FADLUN", "OSC_CYLINDER"])
def test_cylinder_restart_continues_bitwise(tmp_path, method):
    def make(path, extra):
        return cases.cylinder(path, h=0.05, ratio=1.1, extent=3.0, core=0.6, points=48, nu=0.025, dt=0.01, nt=100,
                              nsave=10, method=method, extra=extra)
    continue_bitwise(make, tmp_path)


def test_oscillating_restart_continues_bitwise(tmp_path):
    motion = {"xCoefficient": 0.05, "uCoefficient": 0.05 * 2 * np.pi, "xfrequency": 1.0, "xPhase": 0.0,
              "uPhase": 0.0}

    def make(path, extra):
        return cases.cylinder(path, h=0.05, ratio=1.1, extent=3.0, core=0.6, points=48, nu=0.025, dt=0.01, nt=100,
                              nsave=10, method="LUO", motion=motion, extra=extra)
    continue_bitwise(make, tmp_path)


def test_missing_state_is_an_error(tmp_path):
    f = cases.cavity(str(tmp_path / "c"), n=16, nt=20, nsave=10, extra={"restart": True, "startStep": 10})
    with cb.NavierStokesSolver(f) as s:
        with pytest.raises(cb.CuibmError) as e:
            s.initialise()
        assert "restart" in str(e.value)
