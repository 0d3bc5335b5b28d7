"""The solver loop over the device engine against the reference's own solver run.

``tests/golden/solve7_bend.npz`` records the reference's ``ContactFrictionProcess``
on a bent 7-wire strand (see ``tests/test_solver_loop.py``).  The same loop
(``xkgpu.solver.ContactFrictionSolver``) over the FP64 engine and the device
Generalized-alpha integrator reproduces it: the same increments and attempt
counts, residual histories to 1e-5, every converged increment's
displacements to 1e-8 of their scale.  The mixed engine converges through the
same fixed increments to displacements within the loop's own convergence level of the FP64 run's.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("no CUDA device", allow_module_level=True)

from test_solver_loop import _compare, _section, _settings  # noqa: E402
from xkgpu import solver as S  # noqa: E402
from xkgpu.dynamics import GpuGeneralizedAlpha  # noqa: E402
from xkgpu.engine import AssemblyEngine  # noqa: E402


def _run(z, precision, settings=None):
    eng = AssemblyEngine(z["X"], z["conn"], float(z["radius"]), _section(z), layer=z["elem_layer"],
                         precision=precision, k_pen=float(z["k_pen"]), k_t_ratio=float(z["k_t_ratio"]),
                         mu=float(z["mu"]), smoothing_delta=float(z["smoothing_delta"]))
    sol = S.ContactFrictionSolver(S.EngineBackend(eng), GpuGeneralizedAlpha(z["mass"], rho_inf=float(z["rho_inf"])),
                                  t_total=float(z["t_total"]), fixed_dofs=z["fixed"],
                                  prescribed_dofs=z["prescribed_dofs"], prescribed_values=z["prescribed_values"],
                                  settings=settings or _settings(z))
    return sol.run()


def test_engine_solver_reproduces_reference_run():
    z = golden("solve7_bend")
    res = _run(z, "fp64")
    _compare(res, z, 1e-8)


def test_mixed_engine_solver_follows_fp64_run():
    """Mixed against FP64 through the reference's loop with its own convergence tests, both on the
    increments the reference run took (``load_schedule``).  The loop converges linearly (the reference's
    symmetrised CR tangent and its contact tangent are not the derivatives of the residual), and its
    energy test ends an increment at a residual near 1e-5 of the first one; FP64 with a force tolerance
    of 1e-10 stalls near that level as well.  Two runs that take different iterates therefore agree to
    the loop's own convergence level, not to the float rounding: the converged displacements of every
    increment agree within 1e-3 of their scale."""
    z = golden("solve7_bend")
    cfg = dict(dt_max_fraction=float(z["dt_max_fraction"]), load_schedule=tuple(float(f) for f in z["load_history"]))
    r64 = _run(z, "fp64", S.SolverSettings(**cfg))
    rmx = _run(z, "mixed", S.SolverSettings(**cfg))
    print("fp64 attempts", [r.attempts for r in r64.increments], "mixed attempts", [r.attempts for r in rmx.increments])
    assert r64.converged and rmx.converged
    assert [r.load_frac for r in rmx.increments] == [r.load_frac for r in r64.increments]
    diffs = [float(np.max(np.abs(a.u - b.u)) / np.max(np.abs(b.u))) for a, b in zip(rmx.increments, r64.increments)]
    print("converged displacements, mixed vs fp64 per increment:", ["%.2e" % d for d in diffs])
    assert max(diffs) <= 1e-3, diffs
