"""The solver loop (``xkgpu.solver``) against a recorded run of the reference's own
``ContactFrictionProcess`` (``tests/golden/solve7_bend.npz``).

The fixture is the 7-wire strand clamped at z = 0 and driven at z = L to the
section of a circular arc of curvature 1/(50 D), ramped over 1 ms with lumped
mass and Generalized-alpha (rho_inf 0.9), mu = 0.1, k_pen = 1e3 EA/L.  The
reference ran 14 increments (adaptive growth and shrinking, energy and force
convergence, line search); every Newton call's residual history and every
converged increment's displacements are recorded.

On the CPU the loop runs over the oracle (``tests/oracle_backend.py``), which
pins the loop itself: same increments, same attempt counts, residual
histories and displacements to rounding.  The GPU test runs the same loop over
the device engine, FP64 and mixed.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import golden

torch = pytest.importorskip("torch")

from xkgpu import solver as S  # noqa: E402


def _settings(z):
    return S.SolverSettings(dt_max_fraction=float(z["dt_max_fraction"]))


def _section(z):
    return {k: float(z[k]) for k in ("E", "G", "A", "Iy", "Iz", "J", "kappa_y", "kappa_z")}


def _compare(res, z, u_tol):
    calls = res.attempts_log
    assert len(calls) == len(z["call_frac"])
    ptr = z["call_res_ptr"]
    for k, c in enumerate(calls):
        assert abs(c.load_frac - z["call_frac"][k]) < 1e-14, k
        assert c.converged == bool(z["call_converged"][k]), k
        assert c.attempts == int(z["call_attempts"][k]), k
        want = z["call_res"][ptr[k]:ptr[k + 1]]
        got = np.asarray(c.residuals)
        assert got.shape == want.shape, k
        # residual ratios: exactly 1 at the first attempt, then within the rounding of the solves
        assert np.allclose(got, want, rtol=1e-5, atol=1e-12), (k, got, want)
    assert res.converged == bool(z["converged"])
    assert res.n_increments == int(z["n_increments"])
    assert res.n_cutbacks == int(z["n_cutbacks"])
    assert np.allclose([r.load_frac for r in res.increments], z["load_history"], rtol=0, atol=1e-14)
    U = np.array([r.u for r in res.increments])
    scale = np.max(np.abs(z["u_history"]))
    assert np.max(np.abs(U - z["u_history"])) <= u_tol * scale


def test_step_control_replays_reference_increments():
    """Fed the reference's attempt and active counts, the step control gives its load sequence."""
    z = golden("solve7_bend")
    ctl = S.StepControl(float(z["t_total"]), float(z["t_total"]), float(z["t_total"]) / 32.0,
                        float(z["dt_max_fraction"]) * float(z["t_total"]))
    prev, prev_active, fracs = 0.0, 0, []
    for k in range(len(z["call_frac"])):
        more, lf, dt = ctl.query(prev)
        assert more and abs(lf - z["call_frac"][k]) < 1e-14
        assert abs(dt - (lf - prev) * float(z["t_total"])) < 1e-18
        assert bool(z["call_converged"][k])
        ctl.success(lf, prev, int(z["call_attempts"][k]), int(z["call_active"][k]), prev_active)
        prev, prev_active = lf, int(z["call_active"][k])
        fracs.append(lf)
    assert not ctl.query(prev)[0]
    assert np.allclose(fracs, z["load_history"], rtol=0, atol=1e-14)


def test_step_control_cutback():
    """A failed step retries at the shrunk fraction, then the original target (``_adaptive_stepping.py:169-197``)."""
    ctl = S.StepControl(1.0, 1.0, 1.0 / 32.0, 0.25)
    more, lf, _ = ctl.query(0.0)
    assert lf == 0.25
    assert ctl.failure(lf, 0.0, diverged=False)
    assert ctl.query(0.0)[1] == 0.125
    assert ctl.failure(0.125, 0.0, diverged=True)  # diverged: shrink squared
    assert ctl.query(0.0)[1] == 0.125 * 0.25
    ctl.success(0.03125, 0.0, 3, 0, 0)
    assert ctl.query(0.03125)[1] == pytest.approx(0.03125 + 0.03125 * 1.5)
    tiny = S.StepControl(1.0, 1.0, 1.0 / 32.0, 1.0 / 32.0)
    _, lf, _ = tiny.query(0.0)
    assert not tiny.failure(lf, 0.0, diverged=False)  # at the minimum increment: no retry


def test_scheduled_steps():
    """A load schedule is followed exactly; a failed increment is not retried."""
    ctl = S.ScheduledSteps(2.0, (0.25, 0.5, 1.0))
    prev, seen = 0.0, []
    while True:
        more, lf, dt = ctl.query(prev)
        if not more:
            break
        assert dt == pytest.approx((lf - prev) * 2.0)
        ctl.success(lf, prev, 100, 5, 0)  # many attempts, contact change: no growth or shrink
        seen.append(lf)
        prev = lf
    assert seen == [0.25, 0.5, 1.0]
    assert not S.ScheduledSteps(1.0, (0.5, 1.0)).failure(0.5, 0.0, diverged=True)
    # with cutbacks: the failed increment is retried from the shrunk fraction, then the list continues
    ctl = S.ScheduledSteps(1.0, (0.5, 1.0), cutbacks=True, min_frac=0.01)
    assert ctl.query(0.0)[1] == 0.5
    assert ctl.failure(0.5, 0.0, diverged=False)
    assert ctl.query(0.0)[1] == 0.25
    ctl.success(0.25, 0.0, 3, 0, 0)
    assert ctl.query(0.25)[1] == 0.5
    ctl.success(0.5, 0.25, 3, 0, 0)
    assert ctl.query(0.5)[1] == 1.0
    with pytest.raises(ValueError):
        S.ScheduledSteps(1.0, (0.5, 0.4, 1.0))
    with pytest.raises(ValueError):
        S.ScheduledSteps(1.0, (0.5, 0.9))


def test_solver_loop_on_oracle_reproduces_reference_run():
    from oracle_backend import OracleBackend, TorchGA

    z = golden("solve7_bend")
    b = OracleBackend(z["X"], z["conn"], float(z["radius"]), _section(z), layer=z["elem_layer"],
                      k_pen=float(z["k_pen"]), k_t_ratio=float(z["k_t_ratio"]), mu=float(z["mu"]),
                      smoothing_delta=float(z["smoothing_delta"]))
    sol = S.ContactFrictionSolver(b, TorchGA(z["mass"], float(z["rho_inf"])), t_total=float(z["t_total"]),
                                  fixed_dofs=z["fixed"], prescribed_dofs=z["prescribed_dofs"],
                                  prescribed_values=z["prescribed_values"], settings=_settings(z))
    res = sol.run()
    _compare(res, z, 1e-8)
    # the same run, on a fresh backend, with the reference's increments given as a fixed schedule
    b = OracleBackend(z["X"], z["conn"], float(z["radius"]), _section(z), layer=z["elem_layer"],
                      k_pen=float(z["k_pen"]), k_t_ratio=float(z["k_t_ratio"]), mu=float(z["mu"]),
                      smoothing_delta=float(z["smoothing_delta"]))
    sol = S.ContactFrictionSolver(b, TorchGA(z["mass"], float(z["rho_inf"])), t_total=float(z["t_total"]),
                                  fixed_dofs=z["fixed"], prescribed_dofs=z["prescribed_dofs"],
                                  prescribed_values=z["prescribed_values"],
                                  settings=S.SolverSettings(load_schedule=tuple(z["load_history"])))
    _compare(sol.run(), z, 1e-8)


def test_block_tridiagonal_solve_matches_dense():
    """The block LU of ``xkgpu.blocktri`` on a random nonsymmetric, indefinite block-tridiagonal system."""
    from xkgpu.blocktri import blocktri_solve

    rng = np.random.default_rng(4)
    nb, b = 7, 12
    D = rng.normal(size=(nb, b, b)) + 3.0 * np.eye(b) * rng.choice([-1.0, 1.0], size=(nb, 1, b))
    Lo, Up = rng.normal(size=(nb, b, b)) * 0.5, rng.normal(size=(nb, b, b)) * 0.5
    A = np.zeros((nb * b, nb * b))
    for i in range(nb):
        A[i * b:(i + 1) * b, i * b:(i + 1) * b] = D[i]
        if i > 0:
            A[i * b:(i + 1) * b, (i - 1) * b:i * b] = Lo[i]
        if i < nb - 1:
            A[i * b:(i + 1) * b, (i + 1) * b:(i + 2) * b] = Up[i]
    rhs = rng.normal(size=nb * b)
    want = np.linalg.solve(A, rhs)
    got = blocktri_solve(torch.as_tensor(D.copy()), torch.as_tensor(Lo), torch.as_tensor(Up.copy()),
                         torch.as_tensor(rhs.reshape(nb, b, 1))).numpy().reshape(-1)
    assert np.allclose(got, want, rtol=1e-10, atol=1e-12)


def test_gmres_with_float32_block_preconditioner():
    """GMRES in FP64 preconditioned by the float32 block LU on an indefinite, badly scaled
    block-tridiagonal system (rows scaled over eight decades, condition number ~6e8): it reaches the
    attainable FP64 residual within two restart cycles and the solution of the dense solve."""
    from xkgpu.blocktri import blocktri_apply, blocktri_factor, gmres

    rng = np.random.default_rng(8)
    nb, b = 6, 10
    D = rng.normal(size=(nb, b, b)) + 4.0 * np.eye(b) * rng.choice([-1.0, 1.0], size=(nb, 1, b))
    Lo, Up = rng.normal(size=(nb, b, b)) * 0.5, rng.normal(size=(nb, b, b)) * 0.5
    scale = 10.0 ** rng.uniform(-4, 4, size=(nb, b, 1))
    D, Lo, Up = D * scale, Lo * scale, Up * scale
    A = np.zeros((nb * b, nb * b))
    for i in range(nb):
        A[i * b:(i + 1) * b, i * b:(i + 1) * b] = D[i]
        if i > 0:
            A[i * b:(i + 1) * b, (i - 1) * b:i * b] = Lo[i]
        if i < nb - 1:
            A[i * b:(i + 1) * b, (i + 1) * b:(i + 2) * b] = Up[i]
    F = tuple(torch.as_tensor(x, dtype=torch.float32) for x in (D, Lo, Up))
    blocktri_factor(*F)
    At = torch.as_tensor(A)
    rhs = torch.as_tensor(rng.normal(size=nb * b))
    x, it, rel = gmres(lambda v: At @ v, rhs,
                       lambda v: blocktri_apply(*F, v.view(nb, b, 1)).reshape(-1).double(), rtol=1e-12)
    assert rel <= 1e-8 and it <= 60
    want = np.linalg.solve(A, rhs.numpy())
    assert np.max(np.abs(x.numpy() - want)) <= 1e-7 * np.max(np.abs(want))
