"""The discrete adjoint of the embedded method's step (cuibm_adjoint) on the GPU, on a
reduced version of the oscillating-cylinder configuration (a cylinder of diameter 1
oscillating in fluid at rest with u_B(t) = Um sin(2 pi t / T), embedded method, a coarse
grid and a few steps):

  * the transposed operators: y . (A x) = x . (A^T y) for LHS1 and LHS2 with their
    patched rows (to rounding), at every step of a moving body's run (tags change);
  * the gradient of the period-averaged drag J = (2 / nt) sum_n Fx^n with respect to the
    viscosity, the velocity amplitude (uCoefficient) and the per-point velocity offsets,
    against the oracle's FP64 tangent-linear model (oracle/tangent.py, the restated step
    on dual numbers) and against central finite differences of the GPU's own forward
    run (relative step 1e-6);
  * binomial checkpointing with few snapshots advances the fewest steps the schedule
    allows and gives the gradient of the stored-every-step schedule;
  * a torch.autograd.Function (this file only) whose backward is cuibm_adjoint.
Forward solves run to 1e-12 and the adjoint's transposed solves to 1e-12 here, so that
the comparisons see the linearisation, not the Krylov stopping points."""
import numpy as np
import pytest

import oracle
from oracle import tangent

cb = pytest.importorskip("cuibm_gb300")
torch = pytest.importorskip("torch")
from cuibm_gb300 import cases  # noqa: E402

pytestmark = pytest.mark.gpu

NT = 12
POINTS = 48
REL_STEP = 1e-6   # central differences
RTOL_TLM = 1e-6   # adjoint vs the oracle's tangent-linear model, relative to the largest component
RTOL_FD = 1e-5    # adjoint vs central differences of the GPU forward run


def osc_case(folder, um=0.5, period=1.0, nu=0.02, ucoef=None):
    """The body path x = -(um / w) cos(w t); its velocity amplitude uCoefficient is um
    unless ucoef is given (the two are separate inputs of bodies.yaml)."""
    w = 2 * np.pi / period
    motion = {"xCoefficient": um / w, "uCoefficient": um if ucoef is None else ucoef, "xfrequency": 1.0 / period,
              "xPhase": -np.pi / 2, "uPhase": -np.pi / 2}
    return cases.cylinder(folder, h=0.05, ratio=1.1, extent=3.0, core=0.6, points=POINTS, nu=nu, dt=0.01, nt=NT,
                          method="OSC_CYLINDER", quiescent=True, motion=motion, vel_tol=1e-12, pois_tol=1e-12)


def solver(folder, offsets=None):
    s = cb.NavierStokesSolver(folder)
    s.set_option("write_output", 0)
    s.set_option("adjoint_tolerance", 1e-12)
    s.initialise()
    if offsets is not None:
        s.set("body_velocity_offset", np.concatenate(offsets))
    return s


def gpu_drag(folder, offsets=None):
    with solver(folder, offsets) as s:
        J = 0.0
        for _ in range(NT):
            s.stepTime(1)
            J += 2.0 / NT * s.forces()[0]
    return J


@pytest.fixture(scope="module")
def case(tmp_path_factory):
    return osc_case(str(tmp_path_factory.mktemp("adj") / "c"))


@pytest.fixture(scope="module")
def adjoint_run(case):
    with solver(case) as s:
        J, grad, stats = s.adjoint(NT, 2.0 / NT, snapshots=NT)
        assert s.info.time_step == 0  # back at the initial condition
    return J, grad, stats


def test_transposed_operators(case):
    with solver(case) as s:
        rng = np.random.default_rng(3)
        for step in range(NT):
            s.stepTime(1)  # the body moves: rows are patched at new nodes
            for system in (1, 2):
                n = s.info.numUV if system == 1 else s.info.numP
                m = max(s.info.numUV, s.info.numP)
                x, y = rng.standard_normal(n), rng.standard_normal(n)
                s.set("work_x", np.concatenate([x, np.zeros(m - n)]))
                s.run("apply_lhs%d" % system)
                Ax = s.get("work_y")[:n]
                s.set("work_x", np.concatenate([y, np.zeros(m - n)]))
                s.run("apply_lhs%d_t" % system)
                Aty = s.get("work_y")[:n]
                lhs, rhs = float(y @ Ax), float(x @ Aty)
                assert abs(lhs - rhs) <= 1e-12 * np.linalg.norm(y) * np.linalg.norm(Ax), (step, system, lhs, rhs)


def test_objective_matches_forward_run(case, adjoint_run):
    J, _, stats = adjoint_run
    assert abs(J - gpu_drag(case)) <= 1e-12 * max(1.0, abs(J))
    assert stats["tape_steps"] == NT
    # every step's state stored: each taped step but the last takes its solutions from the
    # snapshot of its end
    assert stats["solves_reused"] == NT - 1


def test_gradient_against_oracle_tangent(case, adjoint_run):
    _, grad, _ = adjoint_run
    unit = np.eye(POINTS)[0]
    scale = np.max(np.abs(grad))
    for k, direction in ((0, dict(d_nu=1.0)), (1, dict(d_ucoef=1.0)), (2, dict(d_offu=unit)),
                         (2 + POINTS, dict(d_offv=unit))):
        d = tangent.DualSolver(case)
        d.direction(**direction)
        for _ in range(NT):
            d.step_dual(wx=2.0 / NT)
        print("component %d: adjoint %.12g, tangent %.12g" % (k, grad[k], d.dJ))
        assert abs(grad[k] - d.dJ) <= RTOL_TLM * scale, (k, grad[k], d.dJ)
    # offsets of points other than the first: the kernels never read them
    others = np.concatenate([grad[3:2 + POINTS], grad[3 + POINTS:]])
    assert np.all(others == 0)


def test_gradient_against_finite_differences(case, adjoint_run, tmp_path):
    _, grad, _ = adjoint_run
    s0 = oracle.EmbeddedSolver(case, solve="none")
    nu0, uc0 = s0.nu, s0.coef["uCoefficient"]
    h = REL_STEP * nu0
    fd_nu = (gpu_drag(osc_case(str(tmp_path / "a"), nu=nu0 + h)) -
             gpu_drag(osc_case(str(tmp_path / "b"), nu=nu0 - h))) / (2 * h)
    h = REL_STEP * uc0
    fd_uc = (gpu_drag(osc_case(str(tmp_path / "c"), ucoef=uc0 + h)) -
             gpu_drag(osc_case(str(tmp_path / "d"), ucoef=uc0 - h))) / (2 * h)
    unit, zero = np.eye(POINTS)[0], np.zeros(POINTS)
    h = REL_STEP
    fd_off = (gpu_drag(case, (h * unit, zero)) - gpu_drag(case, (-h * unit, zero))) / (2 * h)
    print("adjoint %r, fd nu %r ucoef %r offu0 %r" % (grad[:3], fd_nu, fd_uc, fd_off))
    assert abs(grad[0] - fd_nu) <= RTOL_FD * abs(fd_nu)
    assert abs(grad[1] - fd_uc) <= RTOL_FD * abs(fd_uc)
    assert abs(grad[2] - fd_off) <= RTOL_FD * abs(fd_off)


def binomial_advances(t, snapshots):
    """The fewest forward steps that reverse t steps with the given snapshots, one of
    them holding the initial state (Griewank and Walther, revolve): r t - C(s + r, r - 1)
    with s = snapshots - 1 free slots and r the least count with C(s + r, s) >= t."""
    from math import comb
    s, r = snapshots - 1, 1
    while comb(s + r, s) < t:
        r += 1
    return r * t - comb(s + r, r - 1)


def test_checkpointing_schedule_does_not_change_the_gradient(case, adjoint_run):
    _, grad, stats_all = adjoint_run
    with solver(case) as s:
        J, g2, stats = s.adjoint(NT, 2.0 / NT, snapshots=3)
    assert stats_all["forward_steps"] == binomial_advances(NT, NT) == NT - 1
    assert stats["forward_steps"] == binomial_advances(NT, 3) == 28  # the fewest with 3 snapshots
    # every taped step but the last takes its solutions from a snapshot or the stash
    assert stats["solves_reused"] == NT - 1
    assert np.allclose(g2, grad, rtol=1e-8, atol=1e-12)


class DragFunction(torch.autograd.Function):
    """J(nu, uCoefficient, offsets) of the reduced oscillating cylinder, with the GPU
    adjoint as its backward (the tests' own wrapper; the library has no torch types)."""

    @staticmethod
    def forward(ctx, params, folder):
        offsets = params[2:].detach().cpu().numpy().astype(np.float64)
        nu, uc = float(params[0]), float(params[1])
        f = osc_case(folder, ucoef=uc, nu=nu)
        with solver(f, (offsets[:POINTS], offsets[POINTS:])) as s:
            J, grad, _ = s.adjoint(NT, 2.0 / NT, snapshots=8)
        ctx.save_for_backward(torch.from_numpy(grad))
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        (grad,) = ctx.saved_tensors
        return gJ * grad, None


def test_autograd_function(tmp_path, adjoint_run):
    _, grad, _ = adjoint_run
    params = torch.zeros(2 + 2 * POINTS, dtype=torch.float64)
    params[0], params[1] = 0.02, 0.5
    params.requires_grad_(True)
    J = DragFunction.apply(params, str(tmp_path / "f"))
    J.backward()
    g = params.grad.numpy()
    assert np.allclose(g, grad, rtol=1e-8, atol=1e-12)
