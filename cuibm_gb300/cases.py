"""Write cuIBM case folders (simParams.yaml, flow.yaml, domain.yaml, bodies.yaml).

The files follow the reference's schema (validation/**/*.yaml).  Each folder
also gets domain.json / bodies.json with the same trees, which the test
harness uses to run the reference's own grid and body parsers.

Presets reproduce the benchmark configurations of this project:
  cavity        lid-driven cavity, plain method (64x64, Re 100, dt 0.01)
  cylinder      impulsively started cylinder, external (Luo) method
                (Re 40: h 0.02 core, stretch 1.03 to [-15, 15]^2, 157 points;
                 Re 550: h 0.005, stretch 1.01, 629 points)
"""
import json
import os


def _emit(obj, indent=0):
    """Emit the YAML subset the reference uses: lists of maps, maps, [flow] lists."""
    pad = " " * indent
    lines = []
    if isinstance(obj, list):
        for item in obj:
            if isinstance(item, dict):
                first = True
                for k, v in item.items():
                    prefix = pad + ("- " if first else "  ")
                    first = False
                    lines.extend(_emit_kv(prefix, k, v, indent + 2))
            else:
                lines.append(pad + "- " + _scalar(item))
    elif isinstance(obj, dict):
        for k, v in obj.items():
            lines.extend(_emit_kv(pad, k, v, indent))
    return lines


def _scalar(v):
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, float):
        return repr(v)
    if isinstance(v, (list, tuple)):
        return "[" + ", ".join(_scalar(x) for x in v) + "]"
    return str(v)


def _emit_kv(prefix, k, v, indent):
    if isinstance(v, list) and v and isinstance(v[0], dict):
        return [prefix + "%s:" % k] + _emit(v, indent + 2)
    if isinstance(v, dict):
        return [prefix + "%s:" % k] + _emit(v, indent + 2)
    return [prefix + "%s: %s" % (k, _scalar(v))]


def write_case(folder, sim, flow, domain, bodies):
    os.makedirs(folder, exist_ok=True)
    for name, tree in (("simParams", sim), ("flow", flow), ("domain", domain), ("bodies", bodies)):
        with open(os.path.join(folder, name + ".yaml"), "w") as f:
            f.write("\n".join(_emit(tree)) + "\n" if tree else "")
        with open(os.path.join(folder, name + ".json"), "w") as f:
            json.dump(tree, f)
    return folder


def solvers(vel_pc="DIAGONAL", vel_tol=1e-5, pois_pc="SMOOTHED_AGGREGATION", pois_tol=1e-5, vel_krylov=None,
            pois_krylov=None, vel_maxit=10000, pois_maxit=20000, precision=None, strength=None):
    """The linearSolvers entries; precision "MIXED" runs both solves' multigrid cycles
    (or, without one, inner solves) in FP32 under FP64 Krylov iterations, strength sets
    the smoothed aggregation's strengthThreshold (extensions of the reference's schema)."""
    v = {"system": "velocity", "solver": "CG", "preconditioner": vel_pc, "tolerance": vel_tol,
         "maxIterations": vel_maxit}
    p = {"system": "Poisson", "solver": "CG", "preconditioner": pois_pc, "tolerance": pois_tol,
         "maxIterations": pois_maxit}
    if vel_krylov:
        v["krylov"] = vel_krylov
    if pois_krylov:
        p["krylov"] = pois_krylov
    if precision:
        v["precision"] = p["precision"] = precision
    if strength is not None:
        v["strengthThreshold"] = p["strengthThreshold"] = float(strength)
    return [v, p]


def bcs(xm, xp, ym, yp, xp_type="DIRICHLET"):
    """Each argument is (u, v) on that boundary."""
    return [
        {"location": "xMinus", "u": ["DIRICHLET", float(xm[0])], "v": ["DIRICHLET", float(xm[1])]},
        {"location": "xPlus", "u": [xp_type, float(xp[0])], "v": [xp_type, float(xp[1])]},
        {"location": "yMinus", "u": ["DIRICHLET", float(ym[0])], "v": ["DIRICHLET", float(ym[1])]},
        {"location": "yPlus", "u": ["DIRICHLET", float(yp[0])], "v": ["DIRICHLET", float(yp[1])]},
    ]


def axis(direction, start, mid_h, subs):
    return {"direction": direction, "start": float(start), "mid_h": float(mid_h),
            "subDomains": [{"end": float(e), "stretchRatio": float(r)} for e, r in subs]}


def cavity(folder, n=64, nu=0.01, dt=0.01, nt=1000, nsave=None, lid=1.0, vel_tol=1e-8, pois_tol=1e-8,
           pois_pc="SMOOTHED_AGGREGATION", pois_krylov="CG", vel_pc="DIAGONAL", vel_krylov=None, extra=None,
           precision=None, strength=None):
    """Lid-driven cavity on [0,1]^2, uniform n x n cells, fluid at rest."""
    sim = {"type": "simulation", "dt": float(dt), "nt": int(nt), "nsave": int(nsave or nt),
           "SolverType": "NAVIER_STOKES_SOLVER",
           "linearSolvers": solvers(vel_pc, vel_tol, pois_pc, pois_tol, vel_krylov, pois_krylov,
                                    precision=precision, strength=strength)}
    if extra:
        sim.update(extra)
    flow = [{"type": "flow", "nu": float(nu), "initialVelocity": [0.0, 0.0], "initialPerturbation": [0.0, 0.0],
             "boundaryConditions": bcs((0, 0), (0, 0), (0, 0), (lid, 0))}]
    h = 1.0 / n
    dom = [axis("x", 0.0, h, [(1.0, 1.0)]), axis("y", 0.0, h, [(1.0, 1.0)])]
    return write_case(folder, [sim], flow, dom, [])


def cylinder(folder, h=0.02, ratio=1.03, extent=15.0, core=0.6, points=157, nu=1.0 / 40, dt=0.01, nt=2000,
             nsave=None, method="LUO", vel_tol=1e-5, pois_tol=1e-5, pois_pc="SMOOTHED_AGGREGATION",
             pois_krylov=None, vel_krylov=None, vel_pc="DIAGONAL", radius=0.5, scaleCV=None, motion=None,
             uinf=1.0, quiescent=False, precision=None, extra=None, vinf=0.0, strength=None):
    """Circle of diameter 2*radius at the origin in [-extent, extent]^2."""
    sim = {"type": "simulation", "dt": float(dt), "nt": int(nt), "nsave": int(nsave or nt), "SolverType": method,
           "linearSolvers": solvers(vel_pc, vel_tol, pois_pc, pois_tol, vel_krylov, pois_krylov,
                                    precision=precision, strength=strength)}
    if extra:
        sim.update(extra)
    if scaleCV is not None:
        sim["scaleCV"] = float(scaleCV)
    u0 = 0.0 if quiescent else float(uinf)
    v0 = 0.0 if quiescent else float(vinf)
    flow = [{"type": "flow", "nu": float(nu), "initialVelocity": [u0, v0],
             "boundaryConditions": bcs((u0, v0), (u0, v0), (u0, v0), (u0, v0), xp_type="CONVECTIVE")}]
    subs = [(-core, ratio), (core, 1.0), (extent, ratio)]
    dom = [axis("x", -extent, h, subs), axis("y", -extent, h, subs)]
    body = {"type": "circle", "circleOptions": [0.0, 0.0, float(radius), int(points), False, float(h)]}
    if motion:
        body.update(motion)
    return write_case(folder, [sim], flow, dom, [body])
