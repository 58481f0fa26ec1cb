"""Batched instances (cuibm_batch_*): independent cases of different kinds and sizes
advanced together, each on its own stream with persistent solves on a fraction of
the SMs.  Every instance ends where it ends when run alone (tight tolerances: the
solves' reduction order differs with the grid size, so fields agree to 1e-9
relative L2, not bit for bit) and where the FP64 oracle's run of the same case ends
(both solves by sparse LU), in plain FP64 and with both systems in mixed precision;
a bad case is reported with its instance index."""
import numpy as np
import pytest

import oracle

cb = pytest.importorskip("cuibm_gb300")
from cuibm_gb300 import cases  # noqa: E402

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def make(tmp_path):
    return [
        cases.cavity(str(tmp_path / "cav32"), n=32, nu=0.01, dt=0.01, nt=100, vel_tol=1e-12, pois_tol=1e-12),
        cases.cavity(str(tmp_path / "cav40"), n=40, nu=0.005, dt=0.01, nt=100, vel_tol=1e-12, pois_tol=1e-12),
        cases.cylinder(str(tmp_path / "cyl"), h=0.05, ratio=1.1, extent=3.0, core=0.6, points=48, nu=0.025, dt=0.01,
                       nt=100, vel_tol=1e-12, pois_tol=1e-12, method="LUO"),
        cases.cylinder(str(tmp_path / "emb"), h=0.05, ratio=1.1, extent=3.0, core=0.6, points=48, nu=0.025,
                       dt=0.01, nt=100, vel_tol=1e-12, pois_tol=1e-12, method="OSC_CYLINDER"),
    ]


@pytest.mark.parametrize("blocks", [None, 5])
def test_batch_matches_instances_run_alone(tmp_path, blocks):
    folders = make(tmp_path)
    alone = []
    for f in folders:
        with cb.NavierStokesSolver(f) as s:
            s.set_option("write_output", 0)
            s.initialise()
            s.stepTime(12)
            alone.append((s.get("u"), s.get("p"), s.forces() if s.info.total_points else None))
    with cb.Batch(folders, solver_blocks=blocks) as b:
        for s in b.instances:
            s.set_option("write_output", 0)
        b.initialise()
        b.stepTime(5)
        b.stepTime(7)
        for s, (u, p, f) in zip(b.instances, alone):
            assert s.timeStep == 12
            assert rel_l2(s.get("u"), u) < 1e-9
            assert rel_l2(s.get("p"), p) < 1e-8
            if f is not None:
                assert abs(s.forces()[0] - f[0]) < 1e-8


def test_autotune_keeps_every_instance_exact(tmp_path):
    folders = make(tmp_path)
    alone = []
    for f in folders:
        with cb.NavierStokesSolver(f) as s:
            s.set_option("write_output", 0)
            s.initialise()
            s.stepTime(18)
            alone.append((s.get("u"), s.get("p")))
    with cb.Batch(folders) as b:
        for s in b.instances:
            s.set_option("write_output", 0)
        b.initialise()
        nb = b.autotune(1)  # sixteen steps
        assert 1 <= nb <= 38 or nb in (-6, -8, -12, -16, -24)
        assert all(s.timeStep == 16 for s in b.instances)
        b.stepTime(2)
        for s, (u, p) in zip(b.instances, alone):
            assert rel_l2(s.get("u"), u) < 1e-9
            assert rel_l2(s.get("p"), p) < 1e-8


def test_batch_reports_the_bad_instance(tmp_path):
    folders = make(tmp_path)[:2] + [str(tmp_path / "missing")]
    with pytest.raises(cb.CuibmError) as e:
        cb.Batch(folders)
    assert "instance 2" in str(e.value)


@pytest.mark.parametrize("precision", [None, "MIXED"])
def test_batch_instances_match_the_oracle(tmp_path, precision):
    """Six steps of a batch of a cavity, an external-method cylinder and an embedded-
    method cylinder against the oracle's runs: u within 1e-9 and p within 1e-8
    relative L2 (mixed precision: its solves stop on the same FP64 residual, 1e-12)."""
    folders = [
        cases.cavity(str(tmp_path / "cav"), n=40, nu=0.005, dt=0.01, nt=100, vel_tol=1e-12, pois_tol=1e-12,
                     precision=precision),
        cases.cylinder(str(tmp_path / "cyl"), h=0.05, ratio=1.1, extent=3.0, core=0.6, points=48, nu=0.025, dt=0.01,
                       nt=100, vel_tol=1e-12, pois_tol=1e-12, method="LUO", precision=precision),
        cases.cylinder(str(tmp_path / "emb"), h=0.05, ratio=1.1, extent=3.0, core=0.6, points=48, nu=0.025,
                       dt=0.01, nt=100, vel_tol=1e-12, pois_tol=1e-12, method="OSC_CYLINDER"),
    ]
    refs = [oracle.PlainSolver(folders[0], solve="direct"), oracle.LuoSolver(folders[1], solve="direct"),
            oracle.EmbeddedSolver(folders[2], solve="direct")]
    for r in refs:
        for _ in range(6):
            r.step()
    with cb.Batch(folders) as b:
        for s in b.instances:
            s.set_option("write_output", 0)
        b.initialise()
        b.stepTime(6)
        for k, (s, r) in enumerate(zip(b.instances, refs)):
            eu, ep = rel_l2(s.get("u"), r.u), rel_l2(s.get("p"), r.p)
            print("instance %d (%s): u %.2e, p %.2e" % (k, precision or "FP64", eu, ep))
            assert eu < 1e-9 and ep < 1e-8, (k, eu, ep)
