"""Host-side pieces of bench.py (no GPU): the committed ncu summaries it reads the
labelled DRAM and FP64-instruction counts from, the batched workload's draws (seed 0:
sizes, Reynolds numbers and the cavities' CFL-bounded time steps) and the benchmark
cases' sizes."""
import os

import numpy as np
import pytest

import bench


def test_profiled_counts_come_from_committed_summaries():
    b, src = bench.profiled_value("dram_bytes_per_launch", "poisson_solve", "cylinder_re40")
    assert isinstance(b, int) and 1e7 < b < 1e8 and "profiles/" in src
    for wl in ("cylinder_re40", "cylinder_re550"):
        n, src = bench.profiled_value("fp64_instr_per_launch", "rhs1", wl)
        assert isinstance(n, int) and n > 0 and "not measured by this run" in src
    assert bench.profiled_value("dram_bytes_per_launch", "no_such_kernel", "cylinder_re40") == (None, None)
    # the C3 counts scale with the velocity unknowns (28 FP64 instructions each)
    n40 = bench.profiled_value("fp64_instr_per_launch", "rhs1", "cylinder_re40")[0]
    n550 = bench.profiled_value("fp64_instr_per_launch", "rhs1", "cylinder_re550")[0]
    assert abs(n40 / (2 * 269 * 270) - 28) < 0.5 and abs(n550 / (2 * 921 * 922) - 28) < 0.5


def test_batch_draws(tmp_path):
    folders = bench.batch_cases(str(tmp_path), 64)
    assert len(folders) == 64
    rng = np.random.default_rng(0)
    for k, f in enumerate(folders):
        text = open(os.path.join(f, "simParams.yaml")).read()
        if k % 2 == 0:
            N = int(rng.choice(np.arange(96, 513, 32)))
            rng.uniform(np.log(100), np.log(1000))
            assert os.path.basename(f) == "cav%02d" % k
            # the lid CFL number of every cavity is 0.32
            assert "dt: %r" % (0.01 * 32 / N) in text or str(0.01 * 32 / N) in text
        else:
            rng.choice([0.04, 0.03, 0.02])
            rng.uniform(np.log(40), np.log(300))
            assert os.path.basename(f) == "cyl%02d" % k
            assert "0.005" in text


@pytest.mark.parametrize("workload,cells", [("cavity64", 64 * 64), ("cylinder_re40", 270 * 270),
                                            ("cylinder_re550", 922 * 922)])
def test_benchmark_cases(tmp_path, workload, cells):
    f, n = bench.make_case(workload, str(tmp_path / "c"))
    assert n == cells and os.path.exists(os.path.join(f, "simParams.yaml"))
