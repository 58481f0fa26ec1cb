"""Per-phase times of the persistent solves, from their in-kernel barrier stamps.

With the option "trace_solve" on, block 0 of a persistent solve stamps the global
timer at every grid barrier together with the source line of the barrier's call
site (include/cuibm.h, CUIBM_F_SOLVE_TRACE).  The time between two stamps is the
phase that ended at the second barrier (its work, its wait for the slowest block
and the barrier itself), so summing by call site shows where a solve spends its
time without a profiler.

    python -m cuibm_gb300.trace CASE_FOLDER [--warm 20] [--system poisson] [--flags "-saStructured 0"]

runs the case for --warm steps, traces the next step and prints, per barrier site
of csrc/fused_kernels.cuh, the count, total and mean phase time.
"""
import argparse
import collections
import os

import numpy as np

SRC = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc", "fused_kernels.cuh")


def phases(trace):
    """(site line, microseconds) of every phase of one solve's trace."""
    k = int(trace[0])
    e = np.asarray(trace[1:k + 1], dtype=np.uint64)
    ts = (e & np.uint64(0xFFFFFFFFFFFF)).astype(np.int64)
    site = (e >> np.uint64(48)).astype(np.int64)
    dt = np.diff(ts) / 1000.0
    return list(zip(site[1:].tolist(), dt.tolist()))


def table(trace):
    """Per call site: [count, total us], in decreasing total."""
    agg = collections.OrderedDict()
    for line, us in phases(trace):
        a = agg.setdefault(line, [0, 0.0])
        a[0] += 1
        a[1] += us
    return sorted(agg.items(), key=lambda kv: -kv[1][1])


def main(argv=None):
    import cuibm_gb300 as cb
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("case")
    ap.add_argument("--warm", type=int, default=20)
    ap.add_argument("--system", choices=["velocity", "poisson", "both"], default="both")
    ap.add_argument("--flags", default="", help="the solver's command-line flags, e.g. \"-saStructured 0\"")
    ap.add_argument("--sequence", type=int, default=0, metavar="N",
                    help="also list the solve's phases N to 2N in order (one iteration's worth)")
    a = ap.parse_args(argv)
    src = open(SRC).read().split("\n") if os.path.exists(SRC) else []
    with cb.NavierStokesSolver(a.case, a.flags.split()) as s:
        s.set_option("write_output", 0)
        s.initialise()
        s.stepTime(a.warm)
        s.set_option("trace_solve", 1)
        s.stepTime(1)
        tr = s.get("solve_trace")
        s.set_option("trace_solve", 0)
        it = s.iterations()
        i = s.info
        print("case %s: %d x %d, SA levels %d, iterations (velocity, Poisson) %s at step %d" % (
            a.case, i.nx, i.ny, i.amg_levels, it, s.timeStep - 1))
        half = len(tr) // 2
        for name, t in (("velocity", tr[:half]), ("poisson", tr[half:])):
            if a.system not in (name, "both"):
                continue
            ph = phases(t)
            total = sum(us for _, us in ph)
            print("%s solve: %d phases, %.1f us" % (name, len(ph), total))
            for line, (n, us) in table(t):
                text = src[line - 1].strip()[:60] if 0 < line <= len(src) else ""
                print("  line %5d  n %4d  total %9.1f us  mean %7.2f us  %5.1f %%  %s" % (
                    line, n, us, us / n, 100 * us / max(total, 1e-9), text))
            if a.sequence:
                print("  phases %d-%d in order:" % (a.sequence, 2 * a.sequence - 1))
                for k, (line, us) in enumerate(ph[a.sequence:2 * a.sequence]):
                    print("    %4d  line %5d  %7.2f us" % (a.sequence + k, line, us))


if __name__ == "__main__":
    main()
