"""The command-line program (src/cuIBM.cu main on the C ABI: cuibm_gb300/_lib/cuibm,
and python -m cuibm_gb300): a case runs to nt with the reference's outputs - the
grid, run.info, the iteration history and q/lambda every nsave steps - and a case
error is a non-zero exit status with a message, not an abort."""
import os
import struct
import subprocess
import sys

import numpy as np
import pytest

cb = pytest.importorskip("cuibm_gb300")
from cuibm_gb300 import cases  # noqa: E402

pytestmark = pytest.mark.gpu
CLI = os.path.join(os.path.dirname(cb.LIB_PATH), "cuibm")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def read_array(path):
    with open(path, "rb") as f:
        n = struct.unpack("i", f.read(4))[0]
        return np.frombuffer(f.read(8 * n), dtype=np.float64)


@pytest.mark.parametrize("how", ["binary", "python"])
def test_cli_runs_a_case_with_the_reference_outputs(tmp_path, how):
    f = cases.cavity(str(tmp_path / "cav"), n=32, nu=0.01, dt=0.01, nt=20, nsave=10)
    cmd = [CLI, "-caseFolder", f] if how == "binary" else [sys.executable, "-m", "cuibm_gb300", "-caseFolder", f]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=ROOT, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "done" in r.stdout
    for step in (10, 20):
        q = read_array(os.path.join(f, "%07d" % step, "q"))
        lam = read_array(os.path.join(f, "%07d" % step, "lambda"))
        assert q.size == 31 * 32 * 2 and lam.size == 32 * 32 and np.all(np.isfinite(q))
    info = open(os.path.join(f, "run.info")).read().splitlines()
    assert info[0] == "%20s\t%d" % ("--nx", 32) and info[5] == "%20s\t%g" % ("--dt", 0.01)
    assert len(open(os.path.join(f, "iterations")).read().splitlines()) == 20
    with cb.NavierStokesSolver(f) as s:  # the same run through the library
        s.set_option("write_output", 0)
        s.initialise()
        s.stepTime(20)
        assert np.array_equal(s.get("p"), read_array(os.path.join(f, "%07d" % 20, "lambda")))


def test_cli_reports_a_bad_case(tmp_path):
    r = subprocess.run([CLI, "-caseFolder", str(tmp_path / "missing")], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "cuibm:" in r.stderr
