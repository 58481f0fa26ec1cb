"""Benchmark: Mcell-steps/s of the fractional-step time step on one GB300.

A "step" is one full time step of the solver (NavierStokesSolver::stepTime /
luo_base::stepTime): explicit RHS, velocity solve, Poisson solve, projection
and, for immersed-boundary cases, the ghost-node interpolation, blending,
force, motion and tagging.  Mcell-steps/s = pressure cells x steps / seconds.

Workloads (synthetic inputs generated from the project's case presets):
  cylinder_re40  impulsively started cylinder, Re 40, external (Luo) method,
                 [-15,15]^2, h = 0.02 core stretched by 1.03 (270 x 270), 157 points,
                 dt 0.01, plain FP64 (the default: the headline configuration)
  cavity64       lid-driven cavity 64 x 64, Re 100, dt 0.01, plain FP64

Timing: W warm-up steps, then K steps, each timed with CUDA events on the
solver's stream; before every timed step a 256 MB buffer is written on that
stream (outside the events) to flush the 129 MB L2, because the whole working
set of these grids fits in L2.  --gpus N runs N independent replicas (one per
GPU, one process each under torchrun); value = total cell-steps / max time.

The line also carries "mixed_precision": the Re 550 cylinder (922 x 922) timed over
the same steps in plain FP64 and with precision MIXED (FP32 multigrid cycles inside
FP64 BiCGSTAB, FP32 inner solves under FP64 refinement), with both runs' C_D
(--no-mixed skips it; single-GPU runs only), and "batched": 64 independent cavities
and cylinders run one after another and as one batch (cuibm_batch_*), aggregate
Mcell-steps/s of both (--no-batch skips it).

--impl reference times the reference's algorithm on the host CPU cores: the
oracle port (oracle/, a C restatement of the reference's kernels and of its
BiCGSTAB / smoothed-aggregation solvers - the reference itself needs CUSP,
which is not available, and a GPU build of it cannot be made here).
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-steps/s"


# Krylov method of both solves in the cylinder workload: BICGSTAB, the
# reference's; CG (on the symmetrised operators, same stopping rule) for study -
# on this stretched grid it needs about three times as many V-cycles.
KRYLOV = os.environ.get("CUIBM_BENCH_KRYLOV", "BICGSTAB")
# Precision of both solves: FP64 (the reference's) or MIXED (FP32 multigrid cycles or
# inner solves under FP64 Krylov iterations, the same FP64 stopping rule).
PRECISION = os.environ.get("CUIBM_BENCH_PRECISION", "FP64")


def make_case(workload, folder, tight=False, precision=None, strength=None):
    from cuibm_gb300 import cases
    prec = precision or PRECISION
    prec = None if prec == "FP64" else prec
    if workload == "cavity64":
        return cases.cavity(folder, n=64, nu=0.01, dt=0.01, nt=1000000, vel_tol=1e-8, pois_tol=1e-8,
                            pois_pc="SMOOTHED_AGGREGATION", pois_krylov="CG", precision=prec), 64 * 64
    if workload == "cylinder_re40":
        k = KRYLOV
        f = cases.cylinder(folder, h=0.02, ratio=1.03, points=157, nu=1.0 / 40, dt=0.01, nt=1000000,
                           vel_tol=1e-5, pois_tol=1e-5, pois_pc="SMOOTHED_AGGREGATION", vel_krylov=k, pois_krylov=k,
                           precision=prec)
        return f, 270 * 270
    if workload == "cylinder_re550":
        k = KRYLOV
        # both solves to 1e-8: C_D then stays within 1e-6 of a tightly solved run (at 1e-5 the
        # velocity solve stops after one iteration and C_D is off by about 2e-3 at step 40)
        f = cases.cylinder(folder, h=0.005, ratio=1.01, points=629, nu=1.0 / 550, dt=0.002, nt=1000000,
                           vel_tol=1e-8, pois_tol=1e-8, pois_pc="SMOOTHED_AGGREGATION", vel_krylov=k, pois_krylov=k,
                           precision=prec, strength=strength)
        return f, 922 * 922
    raise SystemExit("unknown workload " + workload)


def workload_config(workload):
    if workload == "cavity64":
        return {"workload": "lid-driven cavity 64x64, Re 100, plain method", "nx": 64, "ny": 64, "dt": 0.01,
                "velocity": "BiCGSTAB + diagonal, rtol 1e-8", "poisson": "CG + smoothed aggregation, rtol 1e-8"}
    if workload == "cylinder_re550":
        return {"workload": "impulsively started cylinder Re 550, external (Luo) ghost-node method, " + PRECISION,
                "nx": 922, "ny": 922, "body_points": 629, "dt": 0.002,
                "velocity": KRYLOV + " + diagonal, rtol 1e-8", "poisson": KRYLOV + " + smoothed aggregation, rtol 1e-8"}
    return {"workload": "impulsively started cylinder Re 40, external (Luo) ghost-node method, plain FP64",
            "nx": 270, "ny": 270, "body_points": 157, "dt": 0.01,
            "velocity": KRYLOV + " + diagonal, rtol 1e-5", "poisson": KRYLOV + " + smoothed aggregation, rtol 1e-5"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 8 and p[0].replace(".", "").isdigit():
                    rows.append(p)
        except OSError:
            pass
        finally:
            if self.path and os.path.exists(self.path):
                os.remove(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(r[0]) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if "Active" in r[4 + k] and "Not" not in r[4 + k]})
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": float(rows[0][1]), "reasons": reasons,
                "samples": len(rows)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            return float(d.get("hbm_gbs") or d.get("hbm_GBs")), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return rank, world, local, pg


def reduce_max(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def barrier(pg):
    if pg is not None:
        pg.barrier()


def new_solver(a, local):
    import cuibm_gb300 as cb
    tmp = tempfile.mkdtemp(prefix="cuibm_bench_")
    folder, cells = make_case(a.workload, os.path.join(tmp, "case"))
    s = cb.NavierStokesSolver(folder, ["-deviceNumber", str(local)])
    s.set_option("write_output", 0)
    s.initialise()
    return s, cells


def run_ours(a, rank, world, local, pg):
    import torch

    import cuibm_gb300 as cb

    torch.cuda.set_device(local)
    s, cells = new_solver(a, local)
    stream = torch.cuda.ExternalStream(s.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    s.stepTime(a.warmup)
    torch.cuda.synchronize()
    barrier(pg)
    # Timed: steps warmup+1 .. warmup+steps of the run.  Each step is one graph
    # launch enqueued without waiting (step_sync 0) after an L2 flush on the same
    # stream; events bracket the step alone.  The solves' status is checked after.
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    s.set_option("step_sync", 0)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        barrier(pg)
        t0 = time.perf_counter()
        for k in range(a.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            evs[k][0].record(stream)
            s.stepTime(1)
            evs[k][1].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    s.set_option("step_sync", 1)
    s.stepTime(0)  # raises if a solve failed
    barrier(pg)
    dev_ms = sum(e0.elapsed_time(e1) for e0, e1 in evs)
    dev_ms = reduce_max(pg, dev_ms)
    ms_per_step = dev_ms / a.steps
    value = world * cells * a.steps / (dev_ms * 1e-3) / 1e6
    it1, it2 = s.iterations()
    fx, fy = s.forces()
    try:
        launches = s.launch_count()
    except cb.CuibmError:
        launches = None  # graphs disabled (profiling runs): no per-node count

    # roofline: the dominant kernel (the Poisson solve, one persistent launch) and the
    # others, each timed with CUDA events on the solver's stream
    peak, peak_kind = measured_peaks()
    cand = ["poisson_solve", "velocity_solve", "rhs1", "rhs2", "project"]
    prof = {}
    for k in cand:
        ms, b = s.profile_kernel(k, reps=10 if k.endswith("solve") else 50)
        prof[k] = (ms, b, s.iterations()[1 if k == "poisson_solve" else 0] if k.endswith("solve") else None)
    dom = a.roofline_kernel if a.roofline_kernel in prof else "poisson_solve"
    ms, b, its = prof[dom]
    achieved = b / (ms * 1e-3) / 1e9
    roof = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
            "bytes_per_launch": b, "ms_per_launch": round(ms, 5),
            "iterations_per_launch": its,
            "other_kernels": {k: {"ms": round(v[0], 5), "GB/s": round(v[1] / (v[0] * 1e-3) / 1e9, 1)}
                              for k, v in prof.items()}}
    roof["traffic"], roof["traffic_source"] = profiled_traffic(dom, a.workload)
    roof["fp64_issue"] = fp64_issue_roofline(s, prof, a.workload)
    s.close()

    # end to end through the public API with host buffers, on a fresh instance over
    # the same steps: every step uploads the step's boundary inputs from pinned memory
    # and reads back the velocity, pressure and forces into pinned memory, all enqueued
    # on the solver's stream (CUIBM_COPY_ASYNC, steps without per-step waits) and
    # waited for once at the end; the last step's forces are checked against the
    # synchronous read
    s, _ = new_solver(a, local)
    s.stepTime(a.warmup)
    bnames = ["bc_xminus", "bc_xplus", "bc_yminus", "bc_yplus"]
    pinned_in = {n: torch.from_numpy(s.get(n)).pin_memory() for n in bnames}
    out_u = torch.empty(s.info.numUV, dtype=torch.float64).pin_memory()
    out_p = torch.empty(s.info.numP, dtype=torch.float64).pin_memory()
    out_f = torch.empty(2, dtype=torch.float64).pin_memory()
    h2d = sum(t.numel() * 8 for t in pinned_in.values())
    d2h = (out_u.numel() + out_p.numel() + out_f.numel()) * 8
    torch.cuda.synchronize()
    s.set_option("step_sync", 0)
    barrier(pg)
    t0 = time.perf_counter()
    for k in range(a.steps):
        for n, t in pinned_in.items():
            s.set_from(n, t.data_ptr(), t.numel() * 8, asynchronous=True)
        s.stepTime(1)
        s.get_into("u", out_u.data_ptr(), out_u.numel() * 8, asynchronous=True)
        s.get_into("p", out_p.data_ptr(), out_p.numel() * 8, asynchronous=True)
        s.get_into("forces", out_f.data_ptr(), 16, asynchronous=True)
    torch.cuda.synchronize()
    e2e_s = reduce_max(pg, time.perf_counter() - t0)
    s.set_option("step_sync", 1)
    s.stepTime(0)  # raises if a solve failed
    assert tuple(out_f.tolist()) == s.forces(), "the asynchronous force read differs"
    s.close()
    e2e = {"value": round(world * cells * a.steps / e2e_s / 1e6, 3), "unit": METRIC,
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}
    return {"value": value, "ms_per_step": ms_per_step, "wall_s": wall, "roofline": roof, "e2e": e2e,
            "clocks": clk.summary(), "iterations_last_step": [it1, it2], "drag_lift_last_step": [2 * fx, 2 * fy],
            "gpu_launches": launches * a.steps if launches is not None else None}


def precision_comparison(local, warm=20, steps=20):
    """The Re 550 cylinder (922 x 922, 629 body points, dt 0.002, both solves to 1e-8),
    plain FP64 against precision MIXED on the same steps: steps warm+1 .. warm+steps of
    the impulsive start, timed with CUDA events on the solver's stream (the working set,
    several hundred MB, is larger than L2).  Each precision runs with the structured
    smoothed-aggregation hierarchy (the default at this size) and with the graph
    aggregation (-saStructured 0).  Every run's C_D at each timed step is compared with
    the FP64 oracle's (tests/golden/config_cylinder_re550.npz: the oracle's run of the
    same configuration, both systems solved by sparse LU, steps 1-40)."""
    import numpy as np
    import torch

    import cuibm_gb300 as cb
    gold = os.path.join(ROOT, "tests", "golden", "config_cylinder_re550.npz")
    cd_oracle = np.load(gold)["cd"] if os.path.exists(gold) else None
    out = {"workload": "impulsively started cylinder Re 550, external (Luo) method, 922x922, 629 points, "
                       "dt 0.002, BiCGSTAB + diagonal / smoothed aggregation, rtol 1e-8 both",
           "steps_timed": "%d-%d" % (warm + 1, warm + steps),
           "cd_reference": "FP64 oracle run (sparse LU solves), tests/golden/config_cylinder_re550.npz"}
    for prec, flags, key in (("FP64", [], "fp64"), ("MIXED", [], "mixed"),
                             ("FP64", ["-saStructured", "0"], "fp64_graph"),
                             ("MIXED", ["-saStructured", "0"], "mixed_graph")):
        with tempfile.TemporaryDirectory() as tmp:
            folder, cells = make_case("cylinder_re550", os.path.join(tmp, "case"), precision=prec)
            s = cb.NavierStokesSolver(folder, ["-deviceNumber", str(local)] + flags)
            s.set_option("write_output", 0)
            s.initialise()
            s.stepTime(warm)
            stream = torch.cuda.ExternalStream(s.stream())
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                  for _ in range(steps)]
            cds = []
            torch.cuda.synchronize()
            for k in range(steps):
                # each step bracketed by its own events (the step's forces are read between
                # steps, outside them)
                ev[k][0].record(stream)
                s.stepTime(1)
                ev[k][1].record(stream)
                cds.append(2 * s.forces()[0])
            torch.cuda.synchronize()
            ms = sum(e0.elapsed_time(e1) for e0, e1 in ev) / steps
            rec = {"ms_per_step": round(ms, 4), "value": round(cells / ms / 1e3, 3), "unit": METRIC,
                   "iterations_last_step": list(s.iterations()), "cd_last_step": cds[-1],
                   "sa_structured": s.info.sa_structured}
            if cd_oracle is not None and warm + steps <= len(cd_oracle):
                err = np.abs(np.array(cds) - cd_oracle[warm:warm + steps])
                rec["cd_error_vs_fp64_oracle_max"] = float(err.max())
            out[key] = rec
            s.close()
    base = out["fp64"]
    best64 = min(out["fp64"]["ms_per_step"], out["fp64_graph"]["ms_per_step"])
    out["speedup_mixed_over_fp64"] = round(base["ms_per_step"] / out["mixed"]["ms_per_step"], 3)
    out["speedup_mixed_over_fastest_fp64"] = round(best64 / out["mixed"]["ms_per_step"], 3)
    out["speedup_mixed_graph_over_fp64_graph"] = round(out["fp64_graph"]["ms_per_step"] /
                                                       out["mixed_graph"]["ms_per_step"], 3)
    return out


def batch_cases(tmp, n=64, seed=0, precision=None):
    """The batched workload: n instances drawn with numpy's default_rng(seed) - half
    lid-driven cavities (N from {96, 128, ..., 512}, Re log-uniform in [100, 1000]),
    half impulsively started cylinders (external method, the Re 40 case's stretching
    rule with core h from {0.04, 0.03, 0.02}, round(pi/h) body points made even, Re
    log-uniform in [40, 300], dt 0.005).  The cavities' dt is 0.01 x 32/N (a lid CFL
    number of 0.32): at dt 0.01 the finer cavities are unstable (CFL up to 5) and
    overflow within a few dozen steps, and at 0.01 x 64/N (CFL 0.64) the 480 x 480
    cavity at Re 130 still overflows by step 50.  precision MIXED: both systems of every
    instance in mixed precision (the same draws)."""
    import numpy as np
    from cuibm_gb300 import cases
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        if k % 2 == 0:
            N = int(rng.choice(np.arange(96, 513, 32)))
            Re = float(np.exp(rng.uniform(np.log(100), np.log(1000))))
            f = cases.cavity(os.path.join(tmp, "cav%02d" % k), n=N, nu=1.0 / Re, dt=0.01 * 32 / N, nt=1000000,
                             vel_tol=1e-8, pois_tol=1e-8, pois_pc="SMOOTHED_AGGREGATION", pois_krylov="CG",
                             precision=precision)
        else:
            h = float(rng.choice([0.04, 0.03, 0.02]))
            Re = float(np.exp(rng.uniform(np.log(40), np.log(300))))
            pts = int(round(np.pi / h))
            pts += pts % 2
            f = cases.cylinder(os.path.join(tmp, "cyl%02d" % k), h=h, ratio=1.03, points=pts, nu=1.0 / Re, dt=0.005,
                               nt=1000000, precision=precision)
        out.append(f)
    return out


def batch_comparison(local, n=64, warm=3, steps=20, tune_steps=2):
    """The batched workload run as one batch (cuibm_batch_*: every instance on its own
    stream, the persistent solves' block count picked by the batch autotuner during
    warm-up), in plain FP64 and in mixed precision (the configuration's), and one
    instance after another in plain FP64 (each with the whole GPU), timed over the same
    steps with wall-clock time around synchronised GPU work.  Aggregate Mcell-steps/s.
    solver_blocks is the autotuner's choice: a block count for every instance, or minus
    the rows a thread of block counts sized per instance."""
    import time as _time

    import torch

    import cuibm_gb300 as cb
    out = {"workload": "%d instances (seed 0): half lid-driven cavities N 96-512, half cylinders h 0.04-0.02, "
                       "external method" % n}
    with tempfile.TemporaryDirectory() as tmp:
        for prec, key in ((None, "batched"), ("MIXED", "batched_mixed")):
            folders = batch_cases(os.path.join(tmp, key), n, precision=prec)
            b = cb.Batch(folders, ["-deviceNumber", str(local)])
            for s in b.instances:
                s.set_option("write_output", 0)
            b.initialise()
            b.stepTime(warm)
            blocks = b.autotune(tune_steps)  # advances every instance by 16 x tune_steps
            warm_all = b.instances[0].timeStep
            cells = sum(s.info.numP for s in b.instances)
            torch.cuda.synchronize()
            t0 = _time.perf_counter()
            b.stepTime(steps)
            torch.cuda.synchronize()
            el = _time.perf_counter() - t0
            b.close()
            out["steps_timed"] = "%d-%d" % (warm_all + 1, warm_all + steps)
            out[key] = {"s": round(el, 4), "value": round(cells * steps / el / 1e6, 3), "unit": METRIC,
                        "solver_blocks": blocks, "precision": prec or "FP64"}
        folders = batch_cases(os.path.join(tmp, "sequential"), n)
        el = 0.0
        for f in folders:  # one after another, the same steps: each instance alone on the GPU
            s = cb.NavierStokesSolver(f, ["-deviceNumber", str(local)])
            s.set_option("write_output", 0)
            s.initialise()
            s.stepTime(warm_all)
            torch.cuda.synchronize()
            s.set_option("step_sync", 0)  # steps enqueued back to back, as the batch does
            t0 = _time.perf_counter()
            s.stepTime(steps)
            torch.cuda.synchronize()
            el += _time.perf_counter() - t0
            s.set_option("step_sync", 1)
            s.stepTime(0)  # raises if a solve failed
            s.close()
        out["sequential"] = {"s": round(el, 4), "value": round(cells * steps / el / 1e6, 3), "unit": METRIC}
    out["speedup_batched_over_sequential"] = round(out["sequential"]["s"] / out["batched"]["s"], 3)
    out["speedup_batched_mixed_over_sequential_fp64"] = round(out["sequential"]["s"] / out["batched_mixed"]["s"], 3)
    return out


def oscillating_case(folder, nt, tol=1e-8, nu=None, ucoef=None):
    """The oscillating cylinder at KC 10 (Re 200): [-10, 10]^2, h 0.01 in [-2, 2]^2 stretched
    by 1.02 (686 x 686), 314 points, embedded method, u_B(t) = sin(2 pi t / 10) in fluid at
    rest, dt 0.0025.  nu and the velocity amplitude uCoefficient can be changed (the path
    amplitude stays that of Um = 1)."""
    from cuibm_gb300 import cases
    period, um = 10.0, 1.0
    w = 2 * math.pi / period
    motion = {"xCoefficient": um / w, "uCoefficient": um if ucoef is None else ucoef, "xfrequency": 1.0 / period,
              "xPhase": -math.pi / 2, "uPhase": -math.pi / 2}
    return cases.cylinder(folder, h=0.01, ratio=1.02, extent=10.0, core=2.0, points=314,
                          nu=1.0 / 200 if nu is None else nu, dt=0.0025, nt=nt, method="OSC_CYLINDER", quiescent=True,
                          motion=motion, vel_tol=tol, pois_tol=tol)


def adjoint_comparison(local, steps=40, snapshots=64, tol=1e-8, fd=(), also_snapshots=(8,), run_adjoint=True):
    """The discrete adjoint on the oscillating cylinder at KC 10 (686 x 686, 314 points,
    embedded method): the gradient of the drag coefficient averaged over the first `steps`
    steps with respect to nu, the velocity amplitude and the per-point velocity offsets,
    against the forward run of the same steps (forward and transposed solves to tol).
    Times are wall-clock.  fd names the central differences of the forward run to add
    beside the gradient: "nu", "ucoef" (relative step 1e-6), "offset" (point 0's u
    offset, step 1e-6).  run_adjoint False: the forward run and the differences only."""
    import numpy as np

    import cuibm_gb300 as cb
    tmp = tempfile.mkdtemp(prefix="cuibm_adj_")

    def fresh(nu=None, ucoef=None, name="kc10", offset_u0=0.0):
        f = oscillating_case(os.path.join(tmp, name), steps, tol=tol, nu=nu, ucoef=ucoef)
        s = cb.NavierStokesSolver(f, ["-deviceNumber", str(local)])
        s.set_option("write_output", 0)
        s.set_option("adjoint_tolerance", tol)
        s.initialise()
        if offset_u0:
            off = np.zeros(2 * s.info.total_points)
            off[0] = offset_u0
            s.set("body_velocity_offset", off)
        return s

    def forward(**kw):
        s = fresh(**kw)
        t0 = time.perf_counter()
        J = 0.0
        for _ in range(steps):
            s.stepTime(1)
            J += 2.0 / steps * s.forces()[0]
        el = time.perf_counter() - t0
        s.close()
        return J, el

    s = fresh()
    info = s.info
    s.close()
    J, fwd = forward()
    out = {"workload": "oscillating cylinder KC 10, Re 200, embedded method, %dx%d, %d points, dt 0.0025"
                       % (info.nx, info.ny, info.total_points),
           "steps": steps, "tolerance": tol, "objective": "mean of C_D = 2 Fx over the steps", "J_forward": J,
           "forward_s": round(fwd, 3), "cells": info.nx * info.ny}
    for snaps in ((snapshots,) + tuple(also_snapshots)) if run_adjoint else ():
        s = fresh()
        t0 = time.perf_counter()
        Ja, grad, st = s.adjoint(steps, 2.0 / steps, snapshots=snaps)
        el = time.perf_counter() - t0
        s.close()
        out["snapshots_%d" % snaps] = {
            "adjoint_s": round(el, 3), "adjoint_over_forward": round(el / fwd, 3), "J": Ja,
            "dJ_dnu": grad[0], "dJ_duCoefficient": grad[1], "dJ_doffset_u0": grad[2],
            "dJ_doffset_v0": grad[2 + info.total_points], "stats": st}
    if fd:
        h, nu0 = 1e-6, 1.0 / 200
        g = out.get("snapshots_%d" % snapshots)
        cd = out["central_differences"] = {"step": h}
        pairs = {"nu": ("dJ_dnu", dict(nu=nu0 * (1 + h), name="nup"), dict(nu=nu0 * (1 - h), name="num"), h * nu0),
                 "ucoef": ("dJ_duCoefficient", dict(ucoef=1 + h, name="ucp"), dict(ucoef=1 - h, name="ucm"), h),
                 "offset": ("dJ_doffset_u0", dict(offset_u0=h, name="ofp"), dict(offset_u0=-h, name="ofm"), h)}
        for name in fd:
            key, plus, minus, step = pairs[name]
            cd[key] = (forward(**plus)[0] - forward(**minus)[0]) / (2 * step)
            if g is not None:
                cd["rel_err_" + key] = abs(g[key] - cd[key]) / abs(cd[key])
    return out


def fp64_issue_roofline(s, prof, workload, kernel="rhs1"):
    """The FP64-issue bound beside the HBM one.  GB300 issues about two FP64 thread
    instructions per clock per SM; the peak is measured here, in this run, by the
    library's own FP64 FMA loop (profile_kernel "fp64_fma": independent FMA chains,
    flops per launch / CUDA-event time).  The explicit right-hand-side kernel's FP64
    instruction count per launch (DADD + DMUL + DFMA thread instructions) is an ncu
    count, taken from the committed summary that holds it (a kernel's instruction
    count does not depend on the clock or the cache, only on the workload); divided
    by this run's event time it gives the achieved issue rate."""
    ms, flops = s.profile_kernel("fp64_fma", reps=3)
    peak_instr = flops / 2 / (ms * 1e-3)  # one FMA = two flops, one instruction
    out = {"peak_tflops": round(flops / (ms * 1e-3) / 1e12, 4), "peak_ginstr_per_s": round(peak_instr / 1e9, 1),
           "peak_source": "fp64_fma loop timed in this run (%.3f ms, %.4g flops)" % (ms, flops), "kernel": kernel}
    instr, src = profiled_value("fp64_instr_per_launch", kernel, workload)
    if instr is not None and kernel in prof:
        kms = prof[kernel][0]
        achieved = instr / (kms * 1e-3)
        out.update({"instr_per_launch": instr, "instr_source": src, "ms_per_launch": round(kms, 5),
                    "achieved_ginstr_per_s": round(achieved / 1e9, 1), "frac": round(achieved / peak_instr, 4)})
    return out


def profiled_value(key, kernel, workload):
    """The number on the line '<key> <kernel> <workload> <value>' of a committed ncu
    summary under profiles/, with the summary's name; (None, None) where none has it."""
    here = os.path.dirname(os.path.abspath(__file__))
    d = os.path.join(here, "profiles")
    if not os.path.isdir(d):
        return None, None
    for fn in sorted(os.listdir(d)):
        if not fn.endswith((".md", ".txt")):
            continue
        for line in open(os.path.join(d, fn)):
            f = line.strip().strip("`").split()
            if len(f) == 4 and f[0] == key and f[1] == kernel and f[2] == workload:
                return int(f[3]), "ncu capture summarised in profiles/" + fn + " (not measured by this run)"
    return None, None


def profiled_traffic(kernel, workload):
    """DRAM bytes per launch of the kernel as an ncu capture measured them: the line
    'dram_bytes_per_launch <kernel> <workload> <bytes>' of a committed summary under
    profiles/.  This run does not measure DRAM traffic (that needs ncu); the number is
    returned with the summary it comes from, which names the captured launch.  (None,
    None) where no summary has one for this kernel and workload."""
    return profiled_value("dram_bytes_per_launch", kernel, workload)


def cpu_baseline(workload, budget_s=15.0, warmup=1, max_steps=200):
    """The oracle port on the host cores (the reference's algorithm: BiCGSTAB with
    the case's preconditioners), timed over up to max_steps steps after warmup
    untimed ones, stopping early after budget_s seconds."""
    import oracle
    tmp = tempfile.mkdtemp(prefix="cuibm_cpu_")
    folder, cells = make_case(workload, os.path.join(tmp, "case"))
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    if workload == "cavity64":
        solver = oracle.PlainSolver(folder, solve="krylov")
    else:
        solver = oracle.LuoSolver(folder, solve="krylov")
    for _ in range(max(1, warmup)):
        solver.step()
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps:
        solver.step()
        steps += 1
        el = time.perf_counter() - t0
        if el > budget_s:
            break
    el = time.perf_counter() - t0
    value = cells * steps / el / 1e6
    return {"value": round(value, 4), "unit": METRIC, "cores": threads, "kind": "port",
            "sample": "steps %d-%d of the workload (%d timed, %.1f s, BiCGSTAB as configured)"
                      % (max(1, warmup) + 1, max(1, warmup) + steps, steps, el), "steps_timed": steps}


def kernel_timings(a):
    """Each named kernel launched alone three times on the workload after its warm-up
    steps, timed with CUDA events on the solver's stream (profile_kernel): ms per
    launch and its algorithmic bytes (flops for fp64_fma)."""
    import torch

    import cuibm_gb300 as cb
    with tempfile.TemporaryDirectory() as tmp:
        folder, _ = make_case(a.workload, os.path.join(tmp, "case"))
        s = cb.NavierStokesSolver(folder)
        s.set_option("write_output", 0)
        s.initialise()
        s.stepTime(a.warmup)
        torch.cuda.synchronize()
        for k in a.kernel_timings.split(","):
            ms, b = s.profile_kernel(k, reps=3)
            print(json.dumps({"workload": a.workload, "kernel": k, "ms_per_launch": round(ms, 5),
                              "bytes_or_flops": b}), flush=True)
        s.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    # default: the whole 2000-step cylinder run (3 warm-up steps, 1997 timed)
    ap.add_argument("--steps", type=int, default=1997)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=os.environ.get("CUIBM_BENCH_WORKLOAD", "cylinder_re40"))
    ap.add_argument("--roofline-kernel", default="poisson_solve")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true", help="skip the Re 550 FP64 / mixed-precision comparison")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-instances comparison")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the discrete-adjoint measurement")
    ap.add_argument("--adjoint-period", type=int, default=0, metavar="STEPS",
                    help="only the discrete-adjoint comparison over STEPS steps of the KC 10 case (4000: the "
                         "whole period), solves to --adjoint-tol, with the central differences --adjoint-fd names")
    ap.add_argument("--adjoint-tol", type=float, default=1e-10)
    ap.add_argument("--adjoint-fd", default="", metavar="NAMES",
                    help="central differences beside the gradient: a comma list of nu, ucoef, offset")
    ap.add_argument("--no-adjoint-run", action="store_true",
                    help="with --adjoint-period: the forward run and the central differences only")
    ap.add_argument("--kernel-timings", default=None, metavar="K1,K2,...",
                    help="only time these kernels (profile_kernel names) after the warm-up steps of the "
                         "workload, one JSON line each (the command the per-kernel ncu summaries capture)")
    a = ap.parse_args()
    a.warmup = max(a.warmup, 3)
    if a.kernel_timings:
        kernel_timings(a)
        return
    if a.adjoint_period:
        fd = tuple(x for x in a.adjoint_fd.split(",") if x)
        print(json.dumps(adjoint_comparison(0, steps=a.adjoint_period, tol=a.adjoint_tol, fd=fd, also_snapshots=(),
                                            run_adjoint=not a.no_adjoint_run)))
        return
    rank, world, local, pg = dist_setup(a.gpus)
    cfg = workload_config(a.workload)
    cfg.update({"l2": "flushed before every timed step (256 MB write)", "parallelism": "replicas" if world > 1
                else "single GPU"})
    if a.impl == "reference":
        if rank != 0:
            return
        # the same steps as the GPU arm times (warm-up, then K), on all host cores
        cb = cpu_baseline(a.workload, budget_s=240.0, warmup=a.warmup, max_steps=a.steps)
        line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": METRIC, "n_gpus": a.gpus,
                "steps": a.steps, "warmup": a.warmup, "higher_is_better": True, "dtype": "f64",
                "data": "synthetic", "config": cfg, "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    r = run_ours(a, rank, world, local, pg)
    if rank != 0:
        return
    line = {"metric": METRIC, "value": round(r["value"], 3), "unit": METRIC, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": round(r["ms_per_step"], 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
            "roofline": r["roofline"], "e2e": r["e2e"], "clocks": r["clocks"],
            "gpu_launches": r["gpu_launches"], "iterations_last_step": r["iterations_last_step"],
            "drag_lift_last_step": r["drag_lift_last_step"]}
    if not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(a.workload)
    if not a.no_mixed and world == 1:
        line["mixed_precision"] = precision_comparison(local)
    if not a.no_batch and world == 1:
        line["batched"] = batch_comparison(local)
    if not a.no_adjoint and world == 1:
        line["adjoint"] = adjoint_comparison(local)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
